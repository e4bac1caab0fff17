// tt_walk_inst.cuh -- explicit instantiations of the MTTKRP walk kernels for one
// (order, precision) -- lean warp-tile walk, shared-memory staged walk and ring
// walk --, included by tt_walk_o{3,4}_{fp32,bf16,bf16f,fp16}.cu with TT_ORDER,
// TT_PREC and TT_LOOKUP defined.  The (columns per lane, lanes per row)
// pairs cover factor ranks 8, 16, 32 and 64.
#include "tt_mttkrp.cuh"
#include "tt_kernels.h"

namespace tt {
namespace {
// fam 0: lean warp-tile walk, 1: shared-memory staged, 2: register walk with a
// per-lane cp.async ring.  units: work units of the partition (warp tiles for
// fam 0, blocks otherwise).
template <int CPT, int LPR, int FAM>
cudaError_t launch_walk(const WalkArgs& a, int units, int tb, size_t smem, cudaStream_t s) {
  auto k = FAM == 1 ? mttkrp_stage_kernel<TT_ORDER, TT_PREC, CPT, LPR>
         : FAM == 2 ? mttkrp_walk_kernel<TT_ORDER, TT_PREC, CPT, LPR, false, true>
                    : mttkrp_lean_kernel<TT_ORDER, TT_PREC, CPT, LPR>;
  const int grid = FAM == 0 ? (units + tb / 32 - 1) / (tb / 32) : units;
  static size_t configured = 48 * 1024;
  if (smem > configured) {
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    configured = smem;
  }
  k<<<grid, tb, smem, s>>>(a);
  return cudaGetLastError();
}
}  // namespace

WalkLauncher TT_LOOKUP(int cpt, int lpr, int fam) {
#define TT_CASE(C, L)                                                        \
  if (cpt == C && lpr == L)                                                  \
    return fam == 2 ? &launch_walk<C, L, 2> : fam == 1 ? &launch_walk<C, L, 1> : &launch_walk<C, L, 0>;
  TT_CASE(1, 8) TT_CASE(2, 4) TT_CASE(4, 2) TT_CASE(8, 1)     // rank 8
  TT_CASE(1, 16) TT_CASE(2, 8) TT_CASE(4, 4) TT_CASE(8, 2)    // rank 16
  TT_CASE(1, 32) TT_CASE(2, 16) TT_CASE(4, 8) TT_CASE(8, 4)   // rank 32
  TT_CASE(2, 32) TT_CASE(4, 16) TT_CASE(8, 8)                 // rank 64
#undef TT_CASE
  return nullptr;
}
}  // namespace tt
