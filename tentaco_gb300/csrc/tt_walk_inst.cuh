// tt_walk_inst.cuh -- explicit instantiations of the MTTKRP walk kernels for one
// (order, precision): the lean warp-tile walk, shared-memory staged walk and TMA
// gather walk in tt_walk_o{3,4}_{fp32,bf16,bf16f,fp16}.cu (TT_ORDER, TT_PREC,
// TT_LOOKUP, TT_LOOKUP_FLAT and TT_LOOKUP_TMA defined), the flat, TMA and strip
// walks in the matching _flat.cu / _tma.cu / _strip.cu units (TT_FLAT_UNIT,
// TT_TMA_UNIT or TT_STRIP_UNIT, and TT_LOOKUP, defined), so the kernels compile in
// parallel.  The strip walk also has fx16 units (16-bit fixed point).  The (columns per lane, lanes per row)
// pairs cover factor ranks 8, 16, 32 and 64.
#include <atomic>
#include <mutex>
#include "tt_mttkrp.cuh"
#include "tt_kernels.h"
#ifdef TT_STRIP_UNIT
#include "tt_strip.cuh"
#endif

namespace tt {
namespace {
// fam 0: lean warp-tile walk, 1: shared-memory staged, 2 / 5: TMA-gather walk with
// 4 / 8 stages in flight per warp, 3: lean with the tighter register budget,
// 6 / 7: flat walk with the looser / tighter budget.
// units: work units of the partition (warp tiles except for fam 1, blocks there).
// Resident blocks per SM the lean kernel's registers are budgeted for: the
// variant's thread axis selects the looser (tb 256) or tighter (tb 512) budget;
// both launch 256-thread blocks.
constexpr int lean_minb(int cpt, bool tight) { return cpt >= 4 ? (tight ? 3 : 2) : (tight ? 4 : 3); }

// Dynamic shared memory one kernel is allowed, per device (the attribute is set per
// device).  Raises are serialised and never lower it, so a launch on another host
// thread keeps what it was allowed.
struct SmemLimit {
  static constexpr int kDevices = 64;
  std::atomic<size_t> bytes[kDevices];
  SmemLimit() {
    for (auto& b : bytes) b.store(48 * 1024);
  }
};
inline std::mutex& smem_limit_mutex() {
  static std::mutex m;
  return m;
}

// One launch: warp-unit kernels run 256-thread blocks; `lim` is the calling
// kernel's own record of the dynamic shared memory it was allowed.
template <typename K>
cudaError_t launch_k(K k, const WalkArgs& a, int units, int tb, size_t smem, cudaStream_t s, bool warp_units,
                     SmemLimit& lim) {
  if (warp_units) tb = 256;  // lean, TMA and flat: one work unit per warp, 256-thread blocks
  const int grid = warp_units ? (units + tb / 32 - 1) / (tb / 32) : units;
  if (smem > 48 * 1024) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= SmemLimit::kDevices) return cudaErrorInvalidDevice;
    if (smem > lim.bytes[dev].load(std::memory_order_acquire)) {
      std::lock_guard<std::mutex> lk(smem_limit_mutex());
      if (smem > lim.bytes[dev].load(std::memory_order_relaxed)) {
        e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        lim.bytes[dev].store(smem, std::memory_order_release);
      }
    }
  }
  k<<<grid, tb, smem, s>>>(a);
  return cudaGetLastError();
}

#if !defined(TT_FLAT_UNIT) && !defined(TT_TMA_UNIT)
// lean (families 0 / 3) and staged (family 1) walks
template <int CPT, int LPR, int FAM>
cudaError_t launch_walk(const WalkArgs& a, int units, int tb, size_t smem, cudaStream_t s) {
  constexpr bool kTight = FAM == 3;  // lean with the tighter register budget
  auto k = FAM == 1 ? mttkrp_stage_kernel<TT_ORDER, TT_PREC, CPT, LPR>
                    : mttkrp_lean_kernel<TT_ORDER, TT_PREC, CPT, LPR, lean_minb(CPT, kTight)>;
  static SmemLimit configured;
  return launch_k(k, a, units, tb, smem, s, FAM != 1, configured);
}
#endif

#ifdef TT_TMA_UNIT
// TMA gather walk (families 2 / 5: 4 / 8 stages in flight per warp)
template <int CPT, int LPR, int FAM>
cudaError_t launch_tma(const WalkArgs& a, int units, int tb, size_t smem, cudaStream_t s) {
  auto k = mttkrp_tma_kernel<TT_ORDER, TT_PREC, CPT, LPR, FAM == 5 ? 8 : 4>;
  static SmemLimit configured;
  return launch_k(k, a, units, tb, smem, s, true, configured);
}
#endif

#ifdef TT_FLAT_UNIT
// flat walk (families 6 / 7: looser / tighter register budget)
template <int CPT, int LPR, int FAM>
cudaError_t launch_flat(const WalkArgs& a, int units, int tb, size_t smem, cudaStream_t s) {
  auto k = mttkrp_flat_kernel<TT_ORDER, TT_PREC, CPT, LPR, lean_minb(CPT, FAM == 7)>;
  static SmemLimit configured;
  return launch_k(k, a, units, tb, smem, s, true, configured);
}
#endif  // TT_FLAT_UNIT

#ifdef TT_STRIP_UNIT
// strip walk (families 8 / 9: four nonzeros per team and step with registers for
// two resident blocks, or two with registers for three)
template <int CPT, int LPR, int FAM>
cudaError_t launch_strip(const WalkArgs& a, int units, int tb, size_t smem, cudaStream_t s) {
  auto k = mttkrp_strip_kernel<TT_ORDER, TT_PREC, CPT, LPR, FAM == 9 ? 2 : 4, FAM == 9 ? 3 : 2>;
  static SmemLimit configured;
  return launch_k(k, a, units, tb, smem, s, true, configured);
}
#endif  // TT_STRIP_UNIT
}  // namespace

#if defined(TT_STRIP_UNIT)
// the strip walk's launchers (families 8 and 9); two or more columns per lane
WalkLauncher TT_LOOKUP(int cpt, int lpr, int fam) {
#define TT_CASE(C, L) \
  if (cpt == C && lpr == L) return fam == 8 ? &launch_strip<C, L, 8> : fam == 9 ? &launch_strip<C, L, 9> : nullptr;
  TT_CASE(2, 4) TT_CASE(4, 2) TT_CASE(8, 1)      // rank 8
  TT_CASE(2, 8) TT_CASE(4, 4) TT_CASE(8, 2)      // rank 16
  TT_CASE(2, 16) TT_CASE(4, 8) TT_CASE(8, 4)     // rank 32
  TT_CASE(2, 32) TT_CASE(4, 16) TT_CASE(8, 8)    // rank 64
#undef TT_CASE
  return nullptr;
}
#elif defined(TT_TMA_UNIT)
// the TMA walk's launchers (families 2 and 5), in their own translation unit
WalkLauncher TT_LOOKUP(int cpt, int lpr, int fam) {
#define TT_CASE(C, L) \
  if (cpt == C && lpr == L) return fam == 2 ? &launch_tma<C, L, 2> : fam == 5 ? &launch_tma<C, L, 5> : nullptr;
  TT_CASE(1, 8) TT_CASE(2, 4) TT_CASE(4, 2) TT_CASE(8, 1)     // rank 8
  TT_CASE(1, 16) TT_CASE(2, 8) TT_CASE(4, 4) TT_CASE(8, 2)    // rank 16
  TT_CASE(1, 32) TT_CASE(2, 16) TT_CASE(4, 8) TT_CASE(8, 4)   // rank 32
  TT_CASE(2, 32) TT_CASE(4, 16) TT_CASE(8, 8)                 // rank 64
#undef TT_CASE
  return nullptr;
}
#elif defined(TT_FLAT_UNIT)
// the flat walk's launchers (families 6 and 7), in their own translation unit
WalkLauncher TT_LOOKUP(int cpt, int lpr, int fam) {
#define TT_CASE(C, L) \
  if (cpt == C && lpr == L) return fam == 6 ? &launch_flat<C, L, 6> : fam == 7 ? &launch_flat<C, L, 7> : nullptr;
  TT_CASE(1, 8) TT_CASE(2, 4) TT_CASE(4, 2) TT_CASE(8, 1)     // rank 8
  TT_CASE(1, 16) TT_CASE(2, 8) TT_CASE(4, 4) TT_CASE(8, 2)    // rank 16
  TT_CASE(1, 32) TT_CASE(2, 16) TT_CASE(4, 8) TT_CASE(8, 4)   // rank 32
  TT_CASE(2, 32) TT_CASE(4, 16) TT_CASE(8, 8)                 // rank 64
#undef TT_CASE
  return nullptr;
}
#else
WalkLauncher TT_LOOKUP_FLAT(int cpt, int lpr, int fam);  // the _flat translation unit
WalkLauncher TT_LOOKUP_TMA(int cpt, int lpr, int fam);   // the _tma translation unit

WalkLauncher TT_LOOKUP(int cpt, int lpr, int fam) {
  if (fam == 6 || fam == 7) return TT_LOOKUP_FLAT(cpt, lpr, fam);
  if (fam == 2 || fam == 5) return TT_LOOKUP_TMA(cpt, lpr, fam);
#define TT_CASE(C, L)                                                                   \
  if (cpt == C && lpr == L)                                                             \
    return fam == 3 ? &launch_walk<C, L, 3> : fam == 1 ? &launch_walk<C, L, 1> : &launch_walk<C, L, 0>;
  TT_CASE(1, 8) TT_CASE(2, 4) TT_CASE(4, 2) TT_CASE(8, 1)     // rank 8
  TT_CASE(1, 16) TT_CASE(2, 8) TT_CASE(4, 4) TT_CASE(8, 2)    // rank 16
  TT_CASE(1, 32) TT_CASE(2, 16) TT_CASE(4, 8) TT_CASE(8, 4)   // rank 32
  TT_CASE(2, 32) TT_CASE(4, 16) TT_CASE(8, 8)                 // rank 64
#undef TT_CASE
  return nullptr;
}
#endif
}  // namespace tt
