// tt_ttv.cuh -- tensor-times-vector over the last mode of a CSF tensor, sm_103a.
//
//   y(f) = sum_{p in fiber f} vals[p] * x[crd[p]]      f = fibers of level order-2
//
// Replaces the reference's ttv_kernel / ttv_csf_gpu_taco
// (tensor_kernels/ttv_csf_gpu_taco.h:2-121).  The output is indexed by fiber
// position, as in the reference (A_vals[j_pos] there), so only the last two CSF
// levels are read.  Unlike the reference, every output is written exactly once
// (no memset, no float atomics):
//   * block b owns nonzeros [b*P, (b+1)*P); each thread walks NPT consecutive
//     nonzeros with 128-bit streaming loads of crd and vals;
//   * fibers complete inside a thread are stored directly; the first and last
//     partial fibers of every thread are merged by a warp shuffle tree and
//     across warps in shared memory;
//   * fibers that span blocks go through a carry buffer and a per-chain ticket
//     (indexed by the chain's first block, reset by the last arriver), and the
//     last block sums the partials in FP64 in block order.
// x is gathered through L1 (it is small for the reference's workloads); the
// streams are evict_first in L2.
#pragma once
#include "tt_common.cuh"

namespace tt {

struct TtvArgs {
  const int32_t* pos;   // nfib+1
  const int32_t* crd;   // nnz (padded)
  const void* vals;     // FP32 or BF16 (padded)
  const float* x;
  float* y;             // nfib
  const int32_t* part;  // nblocks+1 fiber ids
  float* carry;         // 2*nblocks
  int32_t* tickets;     // nblocks, zero between calls
  float vscale;         // value scale (BF16 values), 1 otherwise
  int64_t nnz;
  int64_t nfib;
  int32_t P;
  int32_t NPT;          // nonzeros per thread, multiple of 4
  int32_t nblocks;
  int32_t vals_kind;    // kF32, kB16 or kH16
};

struct TSumm {
  int64_t h, t;
  float ha, ta;
};

__host__ __device__ inline size_t ttv_smem_bytes(int P, int tb) {
  size_t b = (size_t)(P + 2) * sizeof(int32_t);
  b = (b + 15) & ~(size_t)15;
  b += (size_t)(tb / 32) * (2 * sizeof(int64_t) + 2 * sizeof(float));
  b = (b + 15) & ~(size_t)15;
  b += (size_t)tb * sizeof(double) + 8 * sizeof(int64_t);
  return b;
}

#ifndef TT_ARGS_ONLY
__device__ __forceinline__ void ttv_combine(TSumm& X, const TSumm& Y, float* y) {
  if (Y.h == kEmpty) return;
  if (X.h == kEmpty) { X = Y; return; }
  const bool xs = X.t == kNone, ys = Y.t == kNone;
  const int64_t xl = xs ? X.h : X.t;
  if (xl == Y.h) {
    if (xs) { X.ha += Y.ha; if (!ys) { X.t = Y.t; X.ta = Y.ta; } }
    else if (ys) X.ta += Y.ha;
    else { y[X.t] = X.ta + Y.ha; X.t = Y.t; X.ta = Y.ta; }
  } else {
    if (!xs) y[X.t] = X.ta;
    if (ys) { X.t = Y.h; X.ta = Y.ha; }
    else { y[Y.h] = Y.ha; X.t = Y.t; X.ta = Y.ta; }
  }
}

__global__ void __launch_bounds__(512) ttv_walk_kernel(const __grid_constant__ TtvArgs a) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int tb = blockDim.x, nw = tb / 32, warp = threadIdx.x / 32, lane = threadIdx.x % 32;
  const int b = blockIdx.x;
  const int P = a.P;
  int32_t* s_pos = reinterpret_cast<int32_t*>(smem);
  size_t off = ((size_t)(P + 2) * 4 + 15) & ~(size_t)15;
  int64_t* s_wh = reinterpret_cast<int64_t*>(smem + off);
  int64_t* s_wt = s_wh + nw;
  float* s_wha = reinterpret_cast<float*>(s_wt + nw);
  float* s_wta = s_wha + nw;
  off += (size_t)nw * (2 * sizeof(int64_t) + 2 * sizeof(float));
  off = (off + 15) & ~(size_t)15;
  double* s_dbl = reinterpret_cast<double*>(smem + off);
  int64_t* s_ctl = reinterpret_cast<int64_t*>(s_dbl + tb);

  const int64_t bstart = (int64_t)b * P;
  const int64_t bend = min(bstart + (int64_t)P, a.nnz);
  const int64_t fs = a.part[b];
  const int W = (int)(a.part[b + 1] - fs + 1);
  for (int x = threadIdx.x; x <= W; x += tb) s_pos[x] = a.pos[fs + x];
  __syncthreads();

  const uint64_t polF = policy_evict_first();
  TSumm X;
  X.h = kEmpty; X.t = kNone; X.ha = 0.f; X.ta = 0.f;
  const int64_t s = bstart + (int64_t)threadIdx.x * a.NPT;
  if (s < bend) {
    const int64_t e = min(s + (int64_t)a.NPT, bend);
    int xw = (int)search_le(s_pos, 0, W - 1, s);
    int64_t fend = s_pos[xw + 1];
    float acc = 0.f;
    bool flushed = false;
    for (int64_t p = s; p < e; p += 4) {
      const int4 l4 = ld_stream_i4(a.crd + p, polF);
      float v[4];
      if (a.vals_kind == kB16) {
        uint2 w = ld_stream_u2(static_cast<const uint16_t*>(a.vals) + p, polF);
        v[0] = bf16lo(w.x) * a.vscale; v[1] = bf16hi(w.x) * a.vscale;
        v[2] = bf16lo(w.y) * a.vscale; v[3] = bf16hi(w.y) * a.vscale;
      } else if (a.vals_kind == kH16) {
        uint2 w = ld_stream_u2(static_cast<const uint16_t*>(a.vals) + p, polF);
        v[0] = h16lo(w.x) * a.vscale; v[1] = h16hi(w.x) * a.vscale;
        v[2] = h16lo(w.y) * a.vscale; v[3] = h16hi(w.y) * a.vscale;
      } else {
        float4 w = ld_stream_f4(static_cast<const float*>(a.vals) + p, polF);
        v[0] = w.x; v[1] = w.y; v[2] = w.z; v[3] = w.w;
      }
      const float xv[4] = {__ldg(a.x + l4.x), __ldg(a.x + l4.y), __ldg(a.x + l4.z), __ldg(a.x + l4.w)};
#pragma unroll
      for (int u = 0; u < 4; u++) {
        const int64_t pp = p + u;
        if (pp < e) {
          while (pp >= fend) {
            const int64_t f = fs + xw;
            if (!flushed) { X.h = f; X.ha = acc; flushed = true; }
            else a.y[f] = acc;
            acc = 0.f;
            xw++;
            fend = s_pos[xw + 1];
          }
          acc = fmaf(v[u], xv[u], acc);
        }
      }
    }
    const int64_t f = fs + xw;
    if (!flushed) { X.h = f; X.ha = acc; X.t = kNone; }
    else { X.t = f; X.ta = acc; }
  }
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    TSumm Y;
    Y.h = __shfl_down_sync(0xffffffffu, X.h, d);
    Y.t = __shfl_down_sync(0xffffffffu, X.t, d);
    Y.ha = __shfl_down_sync(0xffffffffu, X.ha, d);
    Y.ta = __shfl_down_sync(0xffffffffu, X.ta, d);
    if ((lane & (2 * d - 1)) == 0 && lane + d < 32) ttv_combine(X, Y, a.y);
  }
  if (lane == 0) { s_wh[warp] = X.h; s_wt[warp] = X.t; s_wha[warp] = X.ha; s_wta[warp] = X.ta; }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < nw; w++) {
      TSumm Y;
      Y.h = s_wh[w]; Y.t = s_wt[w]; Y.ha = s_wha[w]; Y.ta = s_wta[w];
      ttv_combine(X, Y, a.y);
    }
    for (int slot = 0; slot < 2; slot++) {
      const int64_t f = slot == 0 ? X.h : X.t;
      int64_t last = -1, b0 = 0, b1 = 0;
      if (f >= 0) {
        b0 = (int64_t)a.pos[f] / P;
        b1 = ((int64_t)a.pos[f + 1] - 1) / P;
        const float v = slot == 0 ? X.ha : X.ta;
        if (b0 == b1) a.y[f] = v;
        else {
          a.carry[2 * (size_t)b + slot] = v;
          __threadfence();
          const int t = atomicAdd(a.tickets + b0, 1);
          if (t == (int)(b1 - b0)) { a.tickets[b0] = 0; __threadfence(); last = f; }
        }
      }
      s_ctl[slot] = last; s_ctl[2 + slot] = b0; s_ctl[4 + slot] = b1;
    }
  }
  __syncthreads();
  for (int slot = 0; slot < 2; slot++) {
    const int64_t f = s_ctl[slot];
    if (f < 0) continue;
    const int64_t b0 = s_ctl[2 + slot], b1 = s_ctl[4 + slot];
    double acc = 0.0;
    for (int64_t bb = b0 + threadIdx.x; bb <= b1; bb += tb) {
      const int sb = (a.part[bb] == f) ? 0 : 1;
      acc += (double)__ldcg(a.carry + 2 * bb + sb);
    }
    s_dbl[threadIdx.x] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
      double tot = 0.0;
      for (int k = 0; k < tb; k++) tot += s_dbl[k];
      a.y[f] = (float)tot;
    }
    __syncthreads();
  }
}

__global__ void ttv_partition_kernel(const __grid_constant__ TtvArgs a) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b > a.nblocks) return;
  const int64_t s = (b < a.nblocks) ? (int64_t)b * a.P : a.nnz - 1;
  const_cast<int32_t*>(a.part)[b] = (int32_t)search_le(a.pos, 0, a.nfib - 1, s);
}

#endif  // TT_ARGS_ONLY
}  // namespace tt
