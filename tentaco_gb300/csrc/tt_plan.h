// tt_plan.h -- the plan object behind the C ABI (host-only definitions).
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include <vector>
#include "tt_internal.h"
#include "tt_kernels.h"

namespace tt {

// Kernel families of the variant table (lean, staged, TMA gather, flat, strip), 40 ids each.
constexpr int kFamilies = 5;
constexpr int kNumVariants = kFamilies * 40;

struct VariantSpec {
  int id, tb, cpt, G, staged;
};
VariantSpec variant_spec(int id);
int variant_id(int tb, int G, int cpt, int staged);
int rank_pad(int R);
int val_bytes(int prec);
bool variant_valid(int id, int order, int rank, int prec);
int default_variant(int order, int rank, int prec, int64_t nnz);
float legacy_last_ms();

}  // namespace tt

struct tt_plan {
  int device = 0;
  tt_op op = TT_OP_MTTKRP;
  int order = 0;
  int32_t dims[TT_MAX_ORDER] = {0, 0, 0, 0};
  int64_t count[TT_MAX_ORDER] = {0, 0, 0, 0};
  int64_t nnz = 0, nroot = 0, nfib_last = 0;
  bool dense_root = true;
  int rank = 0, rp = 0, prec = 0;
  cudaStream_t stream = nullptr;
  // device CSF
  int32_t* d_pos[TT_MAX_ORDER] = {nullptr, nullptr, nullptr, nullptr};
  int32_t* d_crd[TT_MAX_ORDER] = {nullptr, nullptr, nullptr, nullptr};
  void* d_vals = nullptr;
  float vinv = 1.f;  // 16-bit values: stored = value * (1/vinv)
  size_t nvals_alloc = 0;        // entries of d_vals (padded)
  float* d_vals_fx = nullptr;    // 16-bit fixed point: values times their leaf row's power of two
  int8_t* d_rowexp = nullptr;    // 16-bit fixed point: power of two of every leaf-factor row
  // factors in storage precision
  const void* fac[4] = {nullptr, nullptr, nullptr, nullptr};
  void* fac_own[4] = {nullptr, nullptr, nullptr, nullptr};
  float* d_scales = nullptr;    // per factor: colmax, scale, inv (rp each); then the output scale
  float* d_colscale = nullptr;
  bool factors_set = false;
  int32_t ttv_ru = 1, ttv_ranges = 0;  // TTV range walk: units per range, ranges
  bool broken = false;  // a device allocation failed after creation: every later call is refused
  // variant and scratch
  int variant = -1, selected_by = 0;  // 0 heuristic/fixed, 1 model, 2 sweep, 3 model's top k timed
  int tb = 0, cpt = 0, lpr = 0, G = 0, P = 0, nblocks = 0, staged = 0, wcap = 1;
  int32_t* d_err = nullptr;  // [0]: kernel error word, [1]: scratch for the window size
  tt::WalkLauncher launcher = nullptr;
  int32_t* d_part = nullptr;
  int32_t* d_kexp = nullptr;  // flat walk: level-1 coordinate of every nonzero (padded)
  int32_t* d_kexp2 = nullptr; // flat and strip walks, four or five modes: level-2 coordinate of every nonzero (padded)
  int32_t* d_kexp3 = nullptr; // strip walk, five modes: level-3 coordinate of every nonzero (padded)
  int32_t* d_rnz = nullptr;   // flat walk: first nonzero of every root position
  // the partition depends only on the CSF and the unit size: a single-slab plan
  // computes it once per variant (part_ready) and times it (part_ms)
  bool part_ready = false;
  bool variant_ready = false;  // the last use_variant succeeded
  float part_ms = 0.f;
  float* d_carry = nullptr;
  int32_t* d_meta = nullptr;     // MTTKRP: 4 ints per work unit
  double* d_segcarry = nullptr;  // MTTKRP: 2 FP64 rows per segment of work units
  int32_t* d_segmeta = nullptr;  // MTTKRP: 4 ints per segment
  int64_t scratch_blocks = 0;
  float sweep_ms[tt::kNumVariants] = {};
  // leaf-mode slabs: one walk pass per slab, adding into the output (slabs == 1:
  // slab[0] is the whole tensor)
  struct SlabDev {
    int32_t* pos[TT_MAX_ORDER] = {nullptr, nullptr, nullptr, nullptr};
    int32_t* crd[TT_MAX_ORDER] = {nullptr, nullptr, nullptr, nullptr};
    int64_t count[TT_MAX_ORDER] = {0, 0, 0, 0};  // entries per level (count[0]: root positions)
    int64_t nnz = 0, off = 0;
  };
  // entries of the nonzero-level arrays: nnz, or with slabs the slab-major
  // concatenation (each slab's run padded)
  int64_t leaf_len = 0;
  // strip walk on a slab plan: one pass over the slab-major arrays with
  // slabs * (nroot + 1) virtual rows (row nroot of each slab holds its padding),
  // written here and summed into the output by launch_virtual_rows
  float* d_vrows = nullptr;
  // plans over sorted COO input (tt_plan_create_coo): the walk streams the COO
  // columns directly, rows (MTTKRP) or fibers (TTV, TTM) are runs of coordinates
  bool coo = false;
  int32_t* d_fcoords = nullptr;  // TTV / TTM: (i, j) of every fiber
  int slabs = 1;
  int mode = 0;  // output mode (the plan's tensor is re-rooted at it when not 0)
  int gpol = 0;  // WalkArgs::gpol
  SlabDev slab[tt::kMaxSlabs];
  // timing: 0 off, 1 the call and its walk kernels, 2 the call only (no event
  // between the walk and the merge kernels, whose dependent launch it would hold back)
  int timing = 0;
  bool timed_pending = false, kernel_timed = false;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr, evk0 = nullptr, evk1 = nullptr;
  // bookkeeping
  std::vector<void*> allocs;
  int64_t device_bytes = 0;
  tt_plan() { for (auto& m : sweep_ms) m = -1.f; }
};

namespace tt {
// Learned selector: the variant the loaded model prefers for this plan, or -1.
// Valid variants for the plan's shape, ordered by the selector network's
// predicted time; TT_ERR_UNSUPPORTED when no loaded model covers the shape.
tt_status selector_rank(const tt_plan* p, const taco_tensor_t* B, std::vector<int>& ranked, bool* in_range);
}
