// tt_legacy.cpp -- the reference's exported kernel names (C linkage), built on
// the plan API.  Each name maps to one variant of the MTTKRP walk family
// (see tt_legacy_names.def); the call does what the reference's wrapper does
// (tensor_kernels/mttkrp3_csf_ebpr.h:61-87, mttkrp3_csf_gpu_taco.h:73-102):
// upload, partition + clear + kernel inside the timed region, download.
#include <cstdio>
#include <cstring>
#include "tt_plan.h"
#include "../../include/tentaco/gpu_kernels.cuh"

using namespace tt;

enum { TT_LEG_TACO = 0, TT_LEG_SR = 1, TT_LEG_PR = 2 };

namespace {

int legacy_variant(int kind, int rank_in_name, int tb, int p1, int p2, int rank) {
  int G = 4, cpt = 1;
  if (kind == TT_LEG_SR) { G = p1; cpt = p2; }
  else if (kind == TT_LEG_PR) { G = 4; cpt = rank_in_name * p1 / tb; }
  else { G = 4; cpt = 1; tb = 512; }
  if (cpt < 1) cpt = 1;
  int id = variant_id(tb, G, cpt, 0);
  // the rank passed may differ from the one in the name: keep tb and G, adjust columns per lane
  for (int c = cpt; !variant_valid(id, 3, rank, (int)TT_PREC_FP32) && c <= 8; c <<= 1) id = variant_id(tb, G, c, 0);
  for (int c = cpt; !variant_valid(id, 3, rank, (int)TT_PREC_FP32) && c >= 1; c >>= 1) id = variant_id(tb, G, c, 0);
  if (!variant_valid(id, 3, rank, (int)TT_PREC_FP32)) id = default_variant(3, rank, (int)TT_PREC_FP32, 0);
  return id;
}

// The reference's to_taco_tensor (ds.h:368-384) leaves order and mode_types
// unset, so a legacy B is read as a 3-mode CSF: a compressed level 0 when
// indices[0] is set (compress_top_level), else a dense root.
taco_tensor_t legacy_view(const taco_tensor_t* B, bool dense_root) {
  taco_tensor_t v;
  std::memset(&v, 0, sizeof(v));
  v.order = 3;
  v.dimensions = B->dimensions;
  v.indices = B->indices;
  v.vals = B->vals;
  v.mode_types = nullptr;
  static thread_local int32_t** levels[3];
  static thread_local int32_t* nulls[2] = {nullptr, nullptr};
  if (dense_root) {
    levels[0] = nulls;
    levels[1] = B->indices[1];
    levels[2] = B->indices[2];
    v.indices = levels;
  }
  return v;
}

void report(const char* name, tt_status s) {
  if (s != TT_OK) std::fprintf(stderr, "%s: %s\n", name, tt_last_error_string());
}

}  // namespace

extern "C" void tt_legacy_mttkrp(const char* name, int kind, int rank_in_name, int tb, int p1, int p2,
                                 taco_tensor_t* A, taco_tensor_t* B, taco_tensor_t* C, taco_tensor_t* D) {
  if (!A || !B || !C || !D || !A->dimensions) {
    report(name, set_error(TT_ERR_INVALID_ARGUMENT, "null argument"));
    return;
  }
  const int rank = A->dimensions[1];
  const int id = legacy_variant(kind, rank_in_name, tb, p1, p2, rank);
  taco_tensor_t Bv = legacy_view(B, false);
  const taco_tensor_t* F[2] = {C, D};
  report(name, tt_mttkrp_host(A, &Bv, F, TT_PREC_FP32, TT_SELECT_FIXED, id));
}

extern "C" void tt_legacy_ttv(taco_tensor_t* A, taco_tensor_t* B, taco_tensor_t* c) {
  if (!A || !B || !c) {
    report("ttv_csf_gpu_taco", set_error(TT_ERR_INVALID_ARGUMENT, "null argument"));
    return;
  }
  taco_tensor_t Bv = legacy_view(B, true);
  report("ttv_csf_gpu_taco", tt_ttv_host(A, &Bv, c));
}

extern "C" float tt_legacy_timer_ms(void) { return legacy_last_ms(); }

extern "C" {
__attribute__((visibility("default"))) float get_gpu_timer_result(void) { return legacy_last_ms(); }
__attribute__((visibility("default"))) void ttv_csf_gpu_taco(taco_tensor_t* A, taco_tensor_t* B, taco_tensor_t* C) {
  tt_legacy_ttv(A, B, C);
}
#define X(name, kind, rank, tb, p1, p2)                                                      \
  __attribute__((visibility("default"))) void name(taco_tensor_t* A, taco_tensor_t* B,     \
                                                   taco_tensor_t* C, taco_tensor_t* D) {   \
    tt_legacy_mttkrp(#name, kind, rank, tb, p1, p2, A, B, C, D);                           \
  }
#include "../../include/tentaco/tt_legacy_names.def"
#undef X
}
