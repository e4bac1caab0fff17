// tt_ttv.cuh -- tensor-times-vector over the last mode of a CSF tensor, sm_103a.
//
//   y(f) = sum_{p in fiber f} vals[p] * x[crd[p]]      f = fibers of level order-2
//
// Replaces the reference's ttv_kernel / ttv_csf_gpu_taco
// (tensor_kernels/ttv_csf_gpu_taco.h:2-121).  The output is indexed by fiber
// position, as in the reference (A_vals[j_pos] there), so only the last two CSF
// levels are read: the kernels see a 2-level CSF (WalkArgs with pos[1] = fiber
// starts, crd[1] = last-mode coordinates, nrows = fibers, one output column).
// Unlike the reference, every output is written exactly once (no memset, no
// float atomics):
//   * a warp owns kTtvNpt * 32 consecutive nonzeros (its work unit); it stages
//     their coordinates and values with 128-bit loads into shared memory (each
//     lane's run padded by 16 bytes against bank conflicts) and the fiber
//     window, then every lane walks kTtvNpt nonzeros with its x gathers issued
//     before use;
//   * fibers complete inside a lane are stored directly; the lanes' first and
//     last partial fibers are merged by the warp's shuffle tree, and fibers
//     shared between warps go through the unit carry slots and the two-level
//     merge of tt_mttkrp.cuh (FP32 Kahan inside a segment of units, FP64 across).
// x is read through L1 (it is small for the reference's workloads); the streams
// are evict_first in L2.
#pragma once
#include "tt_mttkrp.cuh"

namespace tt {

constexpr int kTtvNpt = 16;  // nonzeros per lane

// Shared memory of one warp: coordinate runs 32 x (kTtvNpt + 4) int32, value runs
// 32 x (kTtvNpt * vbytes + 16) bytes, fiber window starts (at most 32*kTtvNpt + 2).
__host__ __device__ inline size_t ttv_warp_bytes(int vbytes) {
  const size_t pu = (size_t)32 * kTtvNpt;
  size_t b = (size_t)32 * (kTtvNpt + 4) * 4 + (size_t)32 * ((size_t)kTtvNpt * vbytes + 16);
  b += (pu + 2) * 4;
  return (b + 15) & ~(size_t)15;
}

#ifndef TT_ARGS_ONLY
template <int VK>
__global__ void __launch_bounds__(256, 4) ttv_lean_kernel(const __grid_constant__ WalkArgs a) {
  constexpr int VB = VK == kF32 ? 4 : 2;
  constexpr int NPT = kTtvNpt;
  using WK = Walk<3, kFP32, 1, 1>;  // the merge helpers for one output column
  extern __shared__ __align__(16) unsigned char smem[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int u = blockIdx.x * (blockDim.x >> 5) + warp;
  if (u >= a.nblocks) return;  // whole warp
  const int PU = a.P;          // 32 * NPT
  unsigned char* ws = smem + (size_t)warp * ttv_warp_bytes(VB);
  int32_t* s_lc = reinterpret_cast<int32_t*>(ws);
  unsigned char* s_val = ws + (size_t)32 * (NPT + 4) * 4;
  int32_t* s_pos = reinterpret_cast<int32_t*>(s_val + (size_t)32 * (NPT * VB + 16));

  const int64_t ustart64 = (int64_t)u * PU;
  const int ustart = (int)ustart64;
  const int cnt = (int)min((int64_t)PU, a.nnz - ustart64);
  const int fs = a.part[u];
  const int W = a.part[u + 1] - fs + 1;
  {
    // chunk c (entries 4c..4c+3) belongs to lane c / (NPT/4); the arrays are padded
    // so the rounded-up last chunk stays in bounds
    const uint64_t polF = policy_evict_first();
    const int n4 = (cnt + 3) >> 2;
    const int32_t* gl = a.crd[1] + ustart64;
    stage_runs<VB>(gl, a.vals, ustart64, n4, 2, lane, s_lc, s_val, polF);  // runs of NPT = 16 entries
    stage_ints(a.pos[1] + fs, W + 1, lane, s_pos);
  }
  __syncwarp();

  WK wk(a, 0);
  Summ<1> X;
  X.h = kEmpty;
  X.t = kNone;
  const int s = ustart + lane * NPT;
  if (s < ustart + cnt) {
    const int n = min(NPT, ustart + cnt - s);
    const int32_t* lc = s_lc + lane * (NPT + 4);
    const unsigned char* vt = s_val + lane * (NPT * VB + 16);
    const float* xv_g = static_cast<const float*>(a.fac[0]);
    float xv[NPT], v[NPT];
#pragma unroll
    for (int k = 0; k < NPT; k++) xv[k] = __ldg(xv_g + (k < n ? lc[k] : 0));
    if constexpr (VB == 4) {
#pragma unroll
      for (int k = 0; k < NPT / 4; k++) {
        const float4 f = reinterpret_cast<const float4*>(vt)[k];
        v[4 * k] = f.x; v[4 * k + 1] = f.y; v[4 * k + 2] = f.z; v[4 * k + 3] = f.w;
      }
    } else {
#pragma unroll
      for (int k = 0; k < NPT / 8; k++) {
        const uint4 w = reinterpret_cast<const uint4*>(vt)[k];
        const float2 p0 = pair16<VK>(w.x), p1 = pair16<VK>(w.y), p2 = pair16<VK>(w.z), p3 = pair16<VK>(w.w);
        v[8 * k] = p0.x; v[8 * k + 1] = p0.y; v[8 * k + 2] = p1.x; v[8 * k + 3] = p1.y;
        v[8 * k + 4] = p2.x; v[8 * k + 5] = p2.y; v[8 * k + 6] = p3.x; v[8 * k + 7] = p3.y;
      }
#pragma unroll
      for (int k = 0; k < NPT; k++) v[k] *= a.vscale;
    }
    // a nonzero ends at most one fiber (fibers are not empty): emit the fiber at
    // its last nonzero, with a short body the compiler can predicate
    int x = (int)search_le(s_pos, 0, W - 1, s);
    int fend = s_pos[x + 1];
    float acc = 0.f;
    bool flushed = false, open = false;
#pragma unroll
    for (int k = 0; k < NPT; k++) {
      if (k < n) {
        acc = fmaf(v[k], xv[k], acc);
        open = true;
        if (s + k + 1 == fend) {  // fiber fs + x ends here
          const int f = fs + x;
          if (flushed) {
            a.out[f] = acc;
          } else {
            X.h = f;
            X.ha[0] = acc;
          }
          flushed = true;
          open = false;
          acc = 0.f;
          x++;
          // past the window's last fiber (the tensor's last unit) there is no next end
          fend = x < W ? s_pos[x + 1] : INT32_MAX;
        }
      }
    }
    if (open) {  // the lane's last fiber continues past it
      if (!flushed) {
        X.h = fs + x;
        X.t = kNone;
        X.ha[0] = acc;
      } else {
        X.t = fs + x;
        X.ta[0] = acc;
      }
    }  // else: X.h is the first fiber and nothing is left open (X.t stays kNone)
  }
  warp_tree(wk, X);
  if (lane == 0) settle_unit(a, wk, X, (int64_t)fs, (int64_t)fs, (int64_t)s_pos[0], ustart64, a.part[u + 1], u, 0);
}
#endif  // TT_ARGS_ONLY
}  // namespace tt
