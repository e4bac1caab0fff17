// tensor_main.cpp -- the tensor-eval-gpu driver on libtentaco_gb300.
//
// Same command line and CSV log as the reference's driver (tensor_main.cpp:15-43
// with tensor_experiments/mttkrp_csf_gpu.h:51-218 and timers.h:93-137):
//
//   tensor-eval-gpu [tensor_dir] [tensor_name] [experiment] [results_dir] [hardware] [feature_dim]
//                   [precision]
//
// precision (an addition; the plan experiments only): fp32 (default), bf16, bf16f
// (FP32 values, BF16 factors) or fp16 storage, FP32 accumulation.
//
// reads <tensor_dir>/<tensor_name>.tns (FROSTT), runs the experiment and appends
// one line per trial to <results_dir>/<experiment>_<feature_dim>_<hardware>.csv:
//   kernel,platform,format,library,tensor,time      (time: ms of the device work)
//
// Experiments:
//   mttkrp_csf_gpu        the reference's run: every eb_sr variant name, 25 trials
//                         each, through the reference-named entry points (host
//                         buffers in, A out; gpu_kernels.cuh)
//   mttkrp_csf_gpu_plan   plan API: upload once, learned selector (heuristic when no
//                         model is loaded), 25 trials of the device call
//   mttkrp_csf_gpu_sweep  plan API with the exhaustive sweep
//   mttkrp_csf_gpu_verify the reference's check (mttkrp_ref with all values 1):
//                         A(i,:) must equal the nonzero count of row i; exits 1 on
//                         a mismatch
//   ttv_csf_gpu           ttv_csf_gpu_taco, 25 trials
// The reference's FROSTT tensors are not shipped; tensor names of the form
// synthetic-<I>x<J>x<K>[x<L>]-<nnz>[-<seed>] generate a seeded uniform tensor
// instead of reading a file.  Factors are U(0,1) (the reference's
// rand()/RAND_MAX) from fixed seeds.
#include <sys/stat.h>
#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iostream>
#include <string>
#include <vector>
#include "tentaco/gpu_kernels.cuh"
#include "tentaco/tentaco.h"
#include "tentaco/tentaco_gen.h"

namespace {

enum { TT_LEG_TACO, TT_LEG_SR, TT_LEG_PR };
using Entry = void (*)(taco_tensor_t*, taco_tensor_t*, taco_tensor_t*, taco_tensor_t*);
struct Named {
  const char* name;
  Entry fn;
  int kind;
};
const Named kNames[] = {
#define X(name, kind, rank, tb, p1, p2) {#name, &name, kind},
#include "tentaco/tt_legacy_names.def"
#undef X
};

constexpr int kTrials = 25;  // tensor_experiments/mttkrp_csf_gpu.h:148

std::ofstream g_log;

void log_row(const std::string& kernel, const std::string& platform, const std::string& format,
             const std::string& library, const std::string& tensor, float ms) {
  g_log << kernel << "," << platform << "," << format << "," << library << "," << tensor << "," << ms << std::endl;
}

bool file_exists(const std::string& p) {
  struct stat st;
  return stat(p.c_str(), &st) == 0;
}

// synthetic-<I>x<J>x<K>[x<L>]-<nnz>[-<seed>]
taco_tensor_t* synthetic(const std::string& name) {
  const std::string pre = "synthetic-";
  if (name.compare(0, pre.size(), pre) != 0) return nullptr;
  int32_t dims[4] = {0, 0, 0, 0};
  int order = 0;
  const char* p = name.c_str() + pre.size();
  char* e = nullptr;
  while (order < 4) {
    dims[order++] = (int32_t)std::strtol(p, &e, 10);
    if (*e != 'x') break;
    p = e + 1;
  }
  if (*e != '-') return nullptr;
  const long long nnz = std::strtoll(e + 1, &e, 10);
  unsigned long long seed = 1;
  if (*e == '-') seed = std::strtoull(e + 1, &e, 10);
  if (order < 3 || nnz <= 0) return nullptr;
  double zs[4] = {0, 0, 0, 0};
  taco_tensor_t* t = nullptr;
  if (tt_gen_zipf(order, dims, zs, nnz, 0.f, 1.f, seed, 8, &t) != TT_OK) return nullptr;
  return t;
}

// A dense row-major matrix (or vector) in a taco_tensor_t.
struct Dense {
  std::vector<float> v;
  int32_t dims[2];
  int32_t ordering[2] = {0, 1};
  taco_mode_t modes[2] = {taco_mode_dense, taco_mode_dense};
  taco_tensor_t t;
  Dense(int64_t rows, int32_t cols, uint64_t seed, bool ones) : v((size_t)rows * cols) {
    dims[0] = (int32_t)rows;
    dims[1] = cols;
    if (ones) std::fill(v.begin(), v.end(), 1.f);
    else tt_gen_dense(rows, cols, 0, seed, v.data());
    std::memset(&t, 0, sizeof(t));
    t.order = 2;
    t.dimensions = dims;
    t.mode_ordering = ordering;
    t.mode_types = modes;
    t.vals = v.data();
  }
};

int fail(const char* what) {
  std::cerr << what << ": " << tt_last_error_string() << std::endl;
  return 1;
}

// Nonzeros of root row i of a 3-mode CSF with a dense root.
int64_t row_nnz(const taco_tensor_t* B, int32_t i) {
  const int32_t* p1 = B->indices[1][0];
  const int32_t* p2 = B->indices[2][0];
  return (int64_t)p2[p1[i + 1]] - p2[p1[i]];
}

}  // namespace

int main(int argc, char* argv[]) {
  const std::string tensor_dir = argc > 1 ? argv[1] : ".";
  const std::string tensor_name = argc > 2 ? argv[2] : "nell-2";
  const std::string experiment = argc > 3 ? argv[3] : "mttkrp_csf_gpu";
  const std::string results_dir = argc > 4 ? argv[4] : ".";
  const std::string hardware = argc > 5 ? argv[5] : "gb300";
  const std::string feature_dim = argc > 6 ? argv[6] : "32";
  const std::string precision = argc > 7 ? argv[7] : "fp32";
  const int R = std::atoi(feature_dim.c_str());
  if (R < 1 || R > TT_MAX_RANK) {
    std::cerr << "feature_dim must be 1.." << TT_MAX_RANK << std::endl;
    return 2;
  }
  tt_precision prec = TT_PREC_FP32;
  if (precision == "bf16") prec = TT_PREC_BF16;
  else if (precision == "bf16f") prec = TT_PREC_BF16_FACTORS;
  else if (precision == "fp16") prec = TT_PREC_FP16;
  else if (precision == "fx16") prec = TT_PREC_FX16;
  else if (precision != "fp32") {
    std::cerr << "precision must be fp32, bf16, bf16f, fp16 or fx16" << std::endl;
    return 2;
  }

  taco_tensor_t* B = nullptr;
  const std::string path = tensor_dir + "/" + tensor_name + ".tns";
  if (file_exists(path)) {
    if (tt_read_tns(path.c_str(), 0, &B) != TT_OK) return fail(path.c_str());
  } else if (!(B = synthetic(tensor_name))) {
    std::cerr << "no tensor file " << path << " (and not a synthetic-<dims>-<nnz> name)" << std::endl;
    return 2;
  }
  const int order = B->order;
  const std::string log_path = results_dir + "/" + experiment + "_" + feature_dim + "_" + hardware + ".csv";
  g_log.open(log_path, std::ofstream::app);
  if (!g_log) {
    std::cerr << "cannot open " << log_path << std::endl;
    return 2;
  }
  int rc = 0;

  if (experiment == "mttkrp_csf_gpu" || experiment == "mttkrp_csf_gpu_verify") {
    if (order != 3) {
      std::cout << "skipping as not 3 modes" << std::endl;  // as the reference does
    } else {
      const bool verify = experiment == "mttkrp_csf_gpu_verify";
      Dense A(B->dimensions[0], R, 0, false), C(B->dimensions[1], R, 12, verify), D(B->dimensions[2], R, 13, verify);
      std::vector<float> ones;
      taco_tensor_t Bv = *B;
      if (verify) {  // all values 1 (the reference's mttkrp_ref)
        const int32_t* p1 = B->indices[1][0];
        const int32_t* p2 = B->indices[2][0];
        ones.assign((size_t)p2[p1[B->dimensions[0]]], 1.f);
        Bv.vals = ones.data();
      }
      int tune = 0;
      for (const Named& n : kNames) {
        if (n.kind != TT_LEG_SR || std::strncmp(n.name, "mttkrp_32_", 10) != 0) continue;
        for (int trial = 0; trial < (verify ? 1 : kTrials); trial++) {
          n.fn(&A.t, &Bv, &C.t, &D.t);
          if (!verify) log_row("mttkrp", "eb", "sr", "tune" + std::to_string(tune), tensor_name, get_gpu_timer_result());
        }
        if (verify) {  // A(i, j) = nonzeros of row i, for every column
          int64_t bad = 0;
          for (int32_t i = 0; i < B->dimensions[0]; i++) {
            const float cnt = (float)row_nnz(B, i);
            for (int j = 0; j < R; j++) bad += A.v[(size_t)i * R + j] != cnt;
          }
          std::cout << n.name << ": " << (bad ? "MISMATCH " : "ok ") << bad << std::endl;
          if (bad) rc = 1;
        }
        tune++;
      }
    }
  } else if (experiment == "mttkrp_csf_gpu_plan" || experiment == "mttkrp_csf_gpu_sweep") {
    std::vector<Dense*> F;
    for (int m = 1; m < order; m++) F.push_back(new Dense(B->dimensions[m], R, 11 + m, false));
    std::vector<float*> dF(F.size(), nullptr);
    float* dA = nullptr;
    for (size_t m = 0; m < F.size(); m++) {
      if (tt_device_malloc((int64_t)F[m]->v.size() * 4, (void**)&dF[m]) != TT_OK) return fail("factor alloc");
      if (tt_memcpy_htod(dF[m], F[m]->v.data(), (int64_t)F[m]->v.size() * 4) != TT_OK) return fail("factor upload");
    }
    if (tt_device_malloc((int64_t)B->dimensions[0] * R * 4, (void**)&dA) != TT_OK) return fail("A alloc");
    const tt_select sel = experiment == "mttkrp_csf_gpu_sweep" ? TT_SELECT_SWEEP : TT_SELECT_MODEL;
    tt_plan* p = nullptr;
    if (tt_plan_create(B, TT_OP_MTTKRP, R, prec, sel, 0, nullptr, &p) != TT_OK) return fail("plan");
    std::vector<const float*> fp(dF.begin(), dF.end());
    if (tt_plan_set_factors(p, fp.data(), nullptr) != TT_OK) return fail("factors");
    tt_plan_set_timing(p, 2);  // the whole call (no event between the walk and the merge)
    tt_variant_info vi;
    tt_variant_get(tt_plan_variant(p), &vi);
    for (int trial = 0; trial < kTrials; trial++) {
      if (tt_plan_mttkrp(p, dA, nullptr) != TT_OK) return fail("mttkrp");
      log_row("mttkrp", "gb300", "csf", vi.name, tensor_name, tt_plan_last_ms(p));
    }
    tt_plan_destroy(p);
    for (float* d : dF) tt_device_free(d);
    tt_device_free(dA);
    for (Dense* d : F) delete d;
  } else if (experiment == "ttv_csf_gpu") {
    if (order != 3) {
      std::cout << "skipping as not 3 modes" << std::endl;
    } else {
      const int32_t* p1 = B->indices[1][0];
      const int64_t nfib = p1[B->dimensions[0]];
      std::vector<float> y((size_t)std::max<int64_t>(nfib, 1));
      int32_t ydims[1] = {(int32_t)nfib};
      taco_tensor_t Y;
      std::memset(&Y, 0, sizeof(Y));
      Y.order = 1;
      Y.dimensions = ydims;
      Y.vals = y.data();
      Dense x(B->dimensions[2], 1, 21, false);
      x.t.order = 1;
      for (int trial = 0; trial < kTrials; trial++) {
        ttv_csf_gpu_taco(&Y, B, &x.t);
        log_row("ttv", "gpu", "csf", "taco", tensor_name, get_gpu_timer_result());
      }
    }
  } else {
    std::cerr << "unknown experiment " << experiment << std::endl;
    rc = 2;
  }
  g_log.close();
  tt_tensor_free(B);
  return rc;
}
