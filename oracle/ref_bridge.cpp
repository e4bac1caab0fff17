/*
 * ref_bridge.cpp -- TEST INFRASTRUCTURE ONLY.
 *
 * Compiles the reference's own CPU kernels, unmodified, from the reference
 * tree (tensor_kernels/mttkrp3_csf_cpu_taco.h, mttkrp3_csf_cpu_taco_workspace.h,
 * mttkrp4_csf_cpu_taco.h, mttkrp5_csf_cpu_taco.h, ttv_csf_cpu_taco.h) and
 * exposes them with plain-array C signatures, so tests can pin the FP64 restatement in tt_oracle.c and
 * generate golden vectors.  Built by oracle/Makefile into oracle/_ref/ only
 * where the reference sources are present.
 *
 * The kernels read indices through taco_tensor_t::indices as splatt_idx_t
 * (uint64) or long, and values as double, so the arrays passed here are int64
 * and double, with a dense root (pos of level 1 has nrows+1 entries).
 */
#include <stdint.h>
#include <string.h>
#include <vector>
#include "ds.h"
#include "timers.h"

double ref_last_ms = 0.0;

#include "mttkrp3_csf_cpu_taco.h"
#include "mttkrp3_csf_cpu_taco_workspace.h"
#include "mttkrp4_csf_cpu_taco.h"
#include "mttkrp5_csf_cpu_taco.h"
#include "ttv_csf_cpu_taco.h"

namespace {
struct Holder {
  std::vector<int32_t> dims;
  std::vector<int32_t**> lv;
  std::vector<int32_t*> slots;
  taco_tensor_t t;
  Holder(int order, const int64_t* d, double* vals) : dims(order), lv(order), slots(2 * order) {
    for (int i = 0; i < order; i++) dims[i] = (int32_t)d[i];
    memset(&t, 0, sizeof(t));
    t.order = order;
    t.dimensions = dims.data();
    for (int i = 0; i < order; i++) lv[i] = &slots[2 * i];
    t.indices = lv.data();
    t.vals = (float*)vals;
  }
  void level(int l, const int64_t* pos, const int64_t* crd) {
    lv[l][0] = (int32_t*)pos;
    lv[l][1] = (int32_t*)crd;
  }
};
struct Dense {
  int32_t dims[2];
  taco_tensor_t t;
  Dense(int64_t rows, int64_t cols, const double* v) {
    memset(&t, 0, sizeof(t));
    dims[0] = (int32_t)rows; dims[1] = (int32_t)cols;
    t.order = 2; t.dimensions = dims; t.vals = (float*)v;
  }
};
}

extern "C" {

__attribute__((visibility("default"))) double ref_last_kernel_ms(void) { return ref_last_ms; }

/* Reference TIME_COLD cache flush (timers.h:62-75): stream an 80 MB buffer. */
__attribute__((visibility("default"))) double ref_flush_cache(void) {
  static std::vector<double> dummy(10000000, 1.0);
  double s = 0.0;
#pragma omp parallel for reduction(+ : s)
  for (long i = 0; i < (long)dummy.size(); i++) s += dummy[i];
  return s;
}

__attribute__((visibility("default")))
void ref_mttkrp3(int64_t nrows, int64_t n1, int64_t n2, int64_t R,
                 const int64_t* pos1, const int64_t* crd1, const int64_t* pos2, const int64_t* crd2,
                 const double* vals, const double* C, const double* D, double* A, int workspace) {
  int64_t dims[3] = {nrows, n1, n2};
  Holder B(3, dims, (double*)vals);
  B.level(1, pos1, crd1);
  B.level(2, pos2, crd2);
  Dense Ad(nrows, R, A), Cd(n1, R, C), Dd(n2, R, D);
  if (workspace) mttkrp3_cpu_taco_workspace(&Ad.t, &B.t, &Cd.t, &Dd.t);
  else mttkrp3_cpu_taco(&Ad.t, &B.t, &Cd.t, &Dd.t);
}

__attribute__((visibility("default")))
void ref_mttkrp4(int64_t nrows, int64_t n1, int64_t n2, int64_t n3, int64_t R,
                 const int64_t* pos1, const int64_t* crd1, const int64_t* pos2, const int64_t* crd2,
                 const int64_t* pos3, const int64_t* crd3,
                 const double* vals, const double* C, const double* D, const double* E, double* A) {
  int64_t dims[4] = {nrows, n1, n2, n3};
  Holder B(4, dims, (double*)vals);
  B.level(1, pos1, crd1);
  B.level(2, pos2, crd2);
  B.level(3, pos3, crd3);
  Dense Ad(nrows, R, A), Cd(n1, R, C), Dd(n2, R, D), Ed(n3, R, E);
  mttkrp4_cpu_taco(&Ad.t, &B.t, &Cd.t, &Dd.t, &Ed.t);
}

__attribute__((visibility("default")))
void ref_mttkrp5(const int64_t* dims, int64_t R, const int64_t* const* pos, const int64_t* const* crd,
                 const double* vals, const double* const* factors, double* A) {
  Holder B(5, dims, (double*)vals);
  for (int l = 1; l < 5; l++) B.level(l, pos[l], crd[l]);
  Dense Ad(dims[0], R, A), Cd(dims[1], R, factors[0]), Dd(dims[2], R, factors[1]), Ed(dims[3], R, factors[2]),
      Fd(dims[4], R, factors[3]);
  mttkrp5_cpu_taco(&Ad.t, &B.t, &Cd.t, &Dd.t, &Ed.t, &Fd.t);
}

__attribute__((visibility("default")))
void ref_ttv(int64_t nrows, int64_t n1, int64_t n2,
             const int64_t* pos1, const int64_t* crd1, const int64_t* pos2, const int64_t* crd2,
             const double* vals, const double* c, double* y) {
  int64_t dims[3] = {nrows, n1, n2};
  Holder B(3, dims, (double*)vals);
  B.level(1, pos1, crd1);
  B.level(2, pos2, crd2);
  int32_t ydim = (int32_t)pos1[nrows];
  int32_t cdim = (int32_t)n2;
  taco_tensor_t yt, ct;
  memset(&yt, 0, sizeof(yt)); memset(&ct, 0, sizeof(ct));
  yt.order = 1; yt.dimensions = &ydim; yt.vals = (float*)y;
  ct.order = 1; ct.dimensions = &cdim; ct.vals = (float*)c;
  ttv_csf_cpu_taco(&yt, &B.t, &ct);
}

}
