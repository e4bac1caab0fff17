// tt_internal.h -- host-side internals shared by the translation units of libtentaco_gb300.
#pragma once
#include <cstdint>
#include <cstdio>
#include <string>
#include <vector>
#include "../../include/tentaco/tentaco.h"

#define TT_EXPORT extern "C" __attribute__((visibility("default")))

namespace tt {

// Per-thread last error, reported by tt_last_error_string().
tt_status set_error(tt_status s, const char* fmt, ...) __attribute__((format(printf, 2, 3)));
void clear_error();
const char* g_last_error_cstr();

// A library-owned taco_tensor_t with its arrays.  `t` is the first member so the
// public pointer converts back to the owner.
struct OwnedTensor {
  taco_tensor_t t;
  uint32_t magic;
  int32_t dims[TT_MAX_ORDER];
  int32_t mode_ordering[TT_MAX_ORDER];
  taco_mode_t mode_types[TT_MAX_ORDER];
  int32_t** levels[TT_MAX_ORDER];
  int32_t* slots[2 * TT_MAX_ORDER];
  std::vector<int32_t> pos[TT_MAX_ORDER];
  std::vector<int32_t> crd[TT_MAX_ORDER];
  std::vector<float> vals;
  static constexpr uint32_t kMagic = 0x7474c5f1u;
  OwnedTensor();
  // Point the taco_tensor_t fields at the vectors (call after filling them).
  void publish(int order, const int32_t* d);
};

// Number of entries at level l of a (validated) CSF: level 0 = root positions.
struct CsfView {
  int order = 0;
  int32_t dims[TT_MAX_ORDER] = {0, 0, 0, 0};
  bool dense_root = true;
  const int32_t* root_crd = nullptr;  // compressed root ids (nullptr: dense)
  int64_t nroot = 0;                  // root positions
  const int32_t* pos[TT_MAX_ORDER] = {nullptr, nullptr, nullptr, nullptr};
  const int32_t* crd[TT_MAX_ORDER] = {nullptr, nullptr, nullptr, nullptr};
  int64_t count[TT_MAX_ORDER] = {0, 0, 0, 0};  // entries per level (count[order-1] = nnz)
  const float* vals = nullptr;
  int64_t nnz = 0;
};

// Read the CSF arrays of B (no validation).
tt_status csf_view(const taco_tensor_t* B, CsfView* v);
// Full validation (monotone pos, sorted distinct crd in range, non-empty inner fibers).
// Full host check of the structure (every level, in parallel over fibers).
tt_status csf_check(const CsfView& v);
// What the device check (launch_csf_check) leaves to the host: the compressed
// root's coordinates, the nnz limit, pos[0] of every level.
tt_status csf_check_root(const CsfView& v);
// Message for a device check result ((index << 3) | code, UINT64_MAX: none).
tt_status csf_check_error(int level, uint64_t word);
// The validated CSF v re-rooted at `mode` (level order: mode, then the other modes
// in increasing order), as a library-owned tensor (free with tt_tensor_free).
tt_status csf_reroot(const CsfView& v, int mode, taco_tensor_t** out);
// Every nonzero's coordinates (nnz x order) in the level order of the CSF rooted
// at `mode`, and the permuted dims (nd), from the validated CSF v.
tt_status csf_rerooted_coords(const CsfView& v, int mode, std::vector<int32_t>& co, int32_t* nd);

// A dense-root CSF split into leaf-mode slabs (leaf coordinate c is in slab
// c / width).  Each slab is a CSF with every row; its leaf arrays are the run
// [leaf_off, leaf_off + nnz) of leaf_crd / leaf_vals (each run padded to a
// multiple of 16 entries plus 16, zero filled).  pos[l] of a slab indexes its
// own arrays (leaf positions relative to leaf_off).
constexpr int kMaxSlabs = 16;
// TT_SELECT_MODEL: most candidates a plan may time, and how many it times when the
// tensor lies outside the range of features the network was trained on.
constexpr int kMaxTopk = 16;
constexpr int kTopkOutside = 6;
struct SlabCsf {
  struct Slab {
    std::vector<int32_t> pos[TT_MAX_ORDER], crd[TT_MAX_ORDER];
    int64_t count[TT_MAX_ORDER] = {0, 0, 0, 0};
    int64_t nnz = 0, leaf_off = 0;
  };
  int S = 1, order = 0;
  int64_t width = 0;
  Slab slab[kMaxSlabs];
  std::vector<int32_t> leaf_crd;
  std::vector<float> leaf_vals;
};
tt_status build_slabs(const CsfView& v, int S, SlabCsf& out);

// Stable parallel LSD radix sort of 64-bit keys with a 32-bit payload, on the
// low `bits` bits.
void radix_sort_pairs(std::vector<uint64_t>& keys, std::vector<uint32_t>& payload, int bits);

// Deterministic RNG: splitmix64-seeded xoshiro256**.
struct Rng {
  uint64_t s[4];
  explicit Rng(uint64_t seed, uint64_t stream = 0);
  uint64_t next();
  double uniform();  // [0,1), 53 bits
  double normal();   // Box-Muller
};

}  // namespace tt
