// tt_mttkrp.cuh -- mode-0 MTTKRP over a CSF tensor (3 or 4 modes) on sm_103a.
//
//   A(i,:) = sum_{k,l}   B(i,k,l)   C(k,:) .* D(l,:)             (order 3)
//   A(i,:) = sum_{k,l,m} B(i,k,l,m) C(k,:) .* D(l,:) .* E(m,:)    (order 4)
//
// Replaces the reference's GPU MTTKRP family (tensor_kernels/mttkrp3_csf_gpu_taco.h:4-71,
// tensor_kernels/mttkrp3_csf_ebsr.h:4-152, tensor_kernels/mttkrp3_csf_ebpr.h:4-59) and adds
// the first GPU MTTKRP4 (the reference has only tensor_kernels/mttkrp4_csf_cpu_taco.h).
//
// Work decomposition (element-balanced, like the reference's EB kernels):
//   * block b owns nonzeros [b*P, (b+1)*P);  P = teams * G.
//   * a team is LPR lanes; lane q owns factor columns [q*CPT, q*CPT+CPT).  Team t
//     walks G consecutive nonzeros serially (the EBSR idea), in the factored
//     order of the reference's workspace kernel: per fiber t = sum v * D(l,:),
//     then row += t .* C(k,:).  A team row that starts and ends inside its
//     range is complete and is stored directly.
//   * the first and last (partial) rows of every team are merged across the
//     warp by a shuffle tree keyed by row (the EBPR idea, segmented by output
//     row, so it crosses fiber boundaries), then across warps in shared memory.
//   * the block's first and last rows, if they extend into other blocks, go to
//     a carry buffer; the last block to arrive at a row (a per-row ticket,
//     reset by that block) sums all of the row's block partials in FP64, in
//     block order.  No float atomics on A: every output is written once and the
//     result is bitwise reproducible run to run.
//
// Data layout in HBM (owned by the plan): int32 pos/crd per level, values FP32 or
// BF16, factors row-major with RP = CPT*LPR entries per row (FP32 or BF16), every
// stream padded with zeros to a multiple of 16 entries so 128-bit loads never read
// past the end.  Dynamic shared memory holds the block's tile of coordinates and
// values and its window of last-level fiber boundaries, both staged with
// coalesced 128-bit loads (evict_first in L2), and the merge scratch.  The walk
// then reads only shared memory and the factor rows; the factor-row gathers of
// the next four nonzeros are issued before the current four are consumed, and
// the next fiber's factor row is requested when the current fiber starts.
#pragma once
#include "tt_common.cuh"

namespace tt {

struct WalkArgs {
  const int32_t* pos[4];  // pos[l], l = 1..order-1 (pos[1] indexed by root position)
  const int32_t* crd[4];  // crd[l], l = 1..order-1; crd[0] = root ids (nullptr: dense root)
  const void* vals;       // FP32 or BF16, padded
  const void* fac[3];     // factors of modes 1..order-1, RP entries per row
  const float* colscale;  // RP output scales (nullptr: all 1)
  float* out;             // output rows (row id = crd[0][ip] or ip), ldo floats apart
  const int32_t* part;    // (nblocks+1) x (order-1): root position, then fiber ids per level
  float* carry;           // 2 * nblocks * RP
  int32_t* tickets;       // one per root position, zero between calls
  int64_t nnz;
  int32_t nrows;
  int32_t R;              // columns stored (<= RP)
  int32_t ldo;
  int32_t P;              // nonzeros per block
  int32_t G;              // nonzeros per team, multiple of 4
  int32_t nblocks;
};

constexpr int kEmpty = -2;  // summary of a team that owns no nonzeros
constexpr int kNone = -1;   // single-row summary: no tail

template <int CPT>
struct Summ {
  int h, t;
  float ha[CPT], ta[CPT];
};

// Bytes of dynamic shared memory a launch needs.
__host__ __device__ inline size_t walk_tile_bytes(int P, int vbytes) {
  return (size_t)P * 4 + (((size_t)P * vbytes + 15) & ~(size_t)15);  // crd + vals tile
}
__host__ __device__ inline size_t walk_smem_bytes(int P, int tb, int rp, int vbytes) {
  size_t nw = (size_t)tb / 32;
  size_t b = walk_tile_bytes(P, vbytes);
  b += (size_t)(2 * P + 4) * sizeof(int32_t);         // fiber window
  b += nw * 2 * sizeof(int32_t);                      // warp summary rows
  b += nw * 2 * (size_t)rp * sizeof(float);           // warp summary accs
  b = (b + 15) & ~(size_t)15;
  b += (size_t)tb * sizeof(double);                   // FP64 merge partials
  b += 8 * sizeof(int32_t);                           // merge control
  return b;
}

template <int ORDER, int PREC, int CPT, int LPR>
struct Walk {
  static constexpr int RP = CPT * LPR;
  static constexpr int FK = fac_kind(PREC);
  static constexpr int VK = val_kind(PREC);
  static constexpr int VB = VK == kF32 ? 4 : 2;  // bytes per stored value
  // gathers of the next chunk in flight while the current one is consumed
  static constexpr bool PIPE = CPT <= 4;

  const WalkArgs& a;
  int q;
  float sc[CPT];

  __device__ __forceinline__ Walk(const WalkArgs& args, int lane_in_team) : a(args), q(lane_in_team) {
#pragma unroll
    for (int c = 0; c < CPT; c++) sc[c] = a.colscale ? a.colscale[q * CPT + c] : 1.0f;
  }

  __device__ __forceinline__ int64_t row_id(int ip) const {
    return a.crd[0] ? (int64_t)a.crd[0][ip] : (int64_t)ip;
  }

  // Store a finished output row (scaled).
  __device__ __forceinline__ void store_row(int ip, const float (&acc)[CPT]) const {
    float* o = a.out + row_id(ip) * a.ldo + q * CPT;
    if (CPT == 4 && a.R == RP && (a.ldo & 3) == 0) {
      *reinterpret_cast<float4*>(o) = make_float4(acc[0] * sc[0], acc[1] * sc[1], acc[2] * sc[2], acc[3] * sc[3]);
    } else {
#pragma unroll
      for (int c = 0; c < CPT; c++)
        if (q * CPT + c < a.R) o[c] = acc[c] * sc[c];
    }
  }

  // Four coordinates and values of the staged tile (offset i, a multiple of 4).
  __device__ __forceinline__ void tile4(const int32_t* s_lc, const unsigned char* s_val, int i,
                                        int4& l4, float (&v)[4]) const {
    l4 = *reinterpret_cast<const int4*>(s_lc + i);
    if constexpr (VK == kF32) {
      const float4 w = *reinterpret_cast<const float4*>(reinterpret_cast<const float*>(s_val) + i);
      v[0] = w.x; v[1] = w.y; v[2] = w.z; v[3] = w.w;
    } else {
      const uint2 w = *reinterpret_cast<const uint2*>(reinterpret_cast<const uint16_t*>(s_val) + i);
      v[0] = lo16<VK>(w.x); v[1] = hi16<VK>(w.x); v[2] = lo16<VK>(w.y); v[3] = hi16<VK>(w.y);
    }
  }

  __device__ __forceinline__ void frow(int m, int64_t row, uint64_t pol, float (&v)[CPT]) const {
    row_load<FK, CPT>(a.fac[m], row * RP + q * CPT, pol, v);
  }

  __device__ __forceinline__ void gather4(const int4& l4, uint64_t pol, float (&g)[4][CPT]) const {
    frow(ORDER - 2, l4.x, pol, g[0]);
    frow(ORDER - 2, l4.y, pol, g[1]);
    frow(ORDER - 2, l4.z, pol, g[2]);
    frow(ORDER - 2, l4.w, pol, g[3]);
  }

  // Combine summary Y (to the right) into X, storing rows that become complete.
  __device__ __forceinline__ void combine(Summ<CPT>& X, const Summ<CPT>& Y) const {
    if (Y.h == kEmpty) return;
    if (X.h == kEmpty) { X = Y; return; }
    const bool xs = X.t == kNone, ys = Y.t == kNone;
    const int xl = xs ? X.h : X.t;
    if (xl == Y.h) {
      if (xs) {
#pragma unroll
        for (int c = 0; c < CPT; c++) X.ha[c] += Y.ha[c];
        if (!ys) {
          X.t = Y.t;
#pragma unroll
          for (int c = 0; c < CPT; c++) X.ta[c] = Y.ta[c];
        }
      } else if (ys) {
#pragma unroll
        for (int c = 0; c < CPT; c++) X.ta[c] += Y.ha[c];
      } else {
        float m[CPT];
#pragma unroll
        for (int c = 0; c < CPT; c++) m[c] = X.ta[c] + Y.ha[c];
        store_row(X.t, m);
        X.t = Y.t;
#pragma unroll
        for (int c = 0; c < CPT; c++) X.ta[c] = Y.ta[c];
      }
    } else {
      if (!xs) store_row(X.t, X.ta);
      if (ys) {
        X.t = Y.h;
#pragma unroll
        for (int c = 0; c < CPT; c++) X.ta[c] = Y.ha[c];
      } else {
        store_row(Y.h, Y.ha);
        X.t = Y.t;
#pragma unroll
        for (int c = 0; c < CPT; c++) X.ta[c] = Y.ta[c];
      }
    }
  }

  // A row ended inside the walk: the first one is the team's head (maybe
  // partial), later ones started and ended inside the team's range.
  __device__ __forceinline__ void flush(int ip, float (&ra)[CPT], bool& flushed, Summ<CPT>& X) const {
    if (!flushed) {
      X.h = ip;
#pragma unroll
      for (int c = 0; c < CPT; c++) X.ha[c] = ra[c];
      flushed = true;
    } else {
      store_row(ip, ra);
    }
#pragma unroll
    for (int c = 0; c < CPT; c++) ra[c] = 0.f;
  }

  // Serial walk of nonzeros [s, e) of the block (tile offsets relative to bstart).
  __device__ __forceinline__ void walk(int64_t s, int64_t e, int64_t bstart, const int32_t* s_lc,
                                       const unsigned char* s_val, const int32_t* s_pos,
                                       const int32_t* s_fcrd, int W, int64_t fs, const int32_t* pb,
                                       const int32_t* pn, Summ<CPT>& X) const {
    const uint64_t polL = policy_evict_last();
    const int32_t* pos1 = a.pos[1];

    int x = (int)search_le(s_pos, 0, W - 1, s);
    int64_t fend = s_pos[x + 1];
    int64_t f1 = 0, kend = 0;  // order 4: level-1 fiber and its end (in level-2 fibers)
    int ip;
    // cur: factor row of the current window fiber; nxt: of the next one (prefetched)
    float cur[CPT], nxt[CPT], crow[CPT];
    if constexpr (ORDER == 3) {
      ip = (int)search_le(pos1, pb[0], pn[0], fs + x);
    } else {
      f1 = search_le(a.pos[2], pb[1], pn[1], fs + x);
      kend = a.pos[2][f1 + 1];
      ip = (int)search_le(pos1, pb[0], pn[0], f1);
      frow(0, a.crd[1][f1], polL, crow);
    }
    frow(ORDER == 3 ? 0 : 1, s_fcrd[x], polL, cur);
    if (x + 1 < W) frow(ORDER == 3 ? 0 : 1, s_fcrd[x + 1], polL, nxt);
    int64_t rend = pos1[ip + 1];

    float f3[CPT], f2[CPT], ra[CPT];
#pragma unroll
    for (int c = 0; c < CPT; c++) { f3[c] = 0.f; f2[c] = 0.f; ra[c] = 0.f; }
    bool flushed = false;

    int4 l4;
    float v4[4];
    float g[4][CPT];
    tile4(s_lc, s_val, (int)(s - bstart), l4, v4);
    gather4(l4, polL, g);
    for (int64_t p = s; p < e; p += 4) {
      int4 ln;
      float vn[4];
      float gn[PIPE ? 4 : 1][CPT];
      if constexpr (PIPE) {
        if (p + 4 < e) {
          tile4(s_lc, s_val, (int)(p + 4 - bstart), ln, vn);
          gather4(ln, polL, gn);
        }
      }
#pragma unroll
      for (int u = 0; u < 4; u++) {
        const int64_t pp = p + u;
        if (pp < e) {
          while (pp >= fend) {
            // the last-level fiber ended: fold it into its parent
            if constexpr (ORDER == 3) {
#pragma unroll
              for (int c = 0; c < CPT; c++) { ra[c] = fmaf(f3[c], cur[c], ra[c]); f3[c] = 0.f; }
            } else {
#pragma unroll
              for (int c = 0; c < CPT; c++) { f2[c] = fmaf(f3[c], cur[c], f2[c]); f3[c] = 0.f; }
            }
            x++;
            fend = s_pos[x + 1];
            const int64_t fg = fs + x;
            if constexpr (ORDER == 4) {
              while (fg >= kend) {
#pragma unroll
                for (int c = 0; c < CPT; c++) { ra[c] = fmaf(f2[c], crow[c], ra[c]); f2[c] = 0.f; }
                f1++;
                kend = a.pos[2][f1 + 1];
                while (f1 >= rend) { flush(ip, ra, flushed, X); ip++; rend = pos1[ip + 1]; }
                frow(0, a.crd[1][f1], polL, crow);
              }
            } else {
              while (fg >= rend) { flush(ip, ra, flushed, X); ip++; rend = pos1[ip + 1]; }
            }
#pragma unroll
            for (int c = 0; c < CPT; c++) cur[c] = nxt[c];
            if (x + 1 < W) frow(ORDER == 3 ? 0 : 1, s_fcrd[x + 1], polL, nxt);
          }
#pragma unroll
          for (int c = 0; c < CPT; c++) f3[c] = fmaf(v4[u], g[u][c], f3[c]);
        }
      }
      if constexpr (PIPE) {
#pragma unroll
        for (int u = 0; u < 4; u++) {
          v4[u] = vn[u];
#pragma unroll
          for (int c = 0; c < CPT; c++) g[u][c] = gn[u][c];
        }
      } else {
        if (p + 4 < e) {
          tile4(s_lc, s_val, (int)(p + 4 - bstart), l4, v4);
          gather4(l4, polL, g);
        }
      }
    }
    if constexpr (ORDER == 3) {
#pragma unroll
      for (int c = 0; c < CPT; c++) ra[c] = fmaf(f3[c], cur[c], ra[c]);
    } else {
#pragma unroll
      for (int c = 0; c < CPT; c++) { f2[c] = fmaf(f3[c], cur[c], f2[c]); ra[c] = fmaf(f2[c], crow[c], ra[c]); }
    }
    if (!flushed) {
      X.h = ip; X.t = kNone;
#pragma unroll
      for (int c = 0; c < CPT; c++) X.ha[c] = ra[c];
    } else {
      X.t = ip;
#pragma unroll
      for (int c = 0; c < CPT; c++) X.ta[c] = ra[c];
    }
  }

  // First and one-past-last nonzero of root position r.
  __device__ __forceinline__ void row_span(int r, int64_t& n0, int64_t& n1) const {
    int64_t f0 = a.pos[1][r], f1 = a.pos[1][r + 1];
    if constexpr (ORDER == 4) { f0 = a.pos[2][f0]; f1 = a.pos[2][f1]; }
    n0 = a.pos[ORDER - 1][f0];
    n1 = a.pos[ORDER - 1][f1];
  }
};

#ifndef TT_ARGS_ONLY
// EXACT = true: the nonzero-level crd/vals arrays are read only up to nnz (the
// caller's own unpadded arrays); false: the plan's padded copies are read in
// whole 128-bit words.
template <int ORDER, int PREC, int CPT, int LPR, bool EXACT = false>
__global__ void __launch_bounds__(512) mttkrp_walk_kernel(const __grid_constant__ WalkArgs a) {
  using WK = Walk<ORDER, PREC, CPT, LPR>;
  constexpr int RP = WK::RP;
  constexpr int VB = WK::VB;
  static_assert(!EXACT || VB == 4, "exact-length staging is built for FP32 values");
  constexpr int TW = 32 / LPR;  // teams per warp
  extern __shared__ __align__(16) unsigned char smem[];

  const int tb = blockDim.x;
  const int nw = tb / 32;
  const int b = blockIdx.x;
  const int P = a.P;
  int32_t* s_lc = reinterpret_cast<int32_t*>(smem);
  unsigned char* s_val = smem + (size_t)P * 4;
  int32_t* s_pos = reinterpret_cast<int32_t*>(smem + walk_tile_bytes(P, VB));
  int32_t* s_fcrd = s_pos + (P + 2);
  int32_t* s_wh = s_fcrd + (P + 2);
  int32_t* s_wt = s_wh + nw;
  float* s_wha = reinterpret_cast<float*>(s_wt + nw);
  float* s_wta = s_wha + nw * RP;
  size_t off = walk_tile_bytes(P, VB) + (size_t)(2 * P + 4) * 4 + (size_t)nw * 8 + (size_t)nw * 2 * RP * 4;
  off = (off + 15) & ~(size_t)15;
  double* s_dbl = reinterpret_cast<double*>(smem + off);
  int32_t* s_ctl = reinterpret_cast<int32_t*>(s_dbl + tb);

  const int32_t* pb = a.part + (size_t)b * (ORDER - 1);
  const int32_t* pn = pb + (ORDER - 1);
  const int64_t bstart = (int64_t)b * P;
  const int64_t bend = min(bstart + (int64_t)P, a.nnz);

  // Stage the block's coordinates and values (128-bit streaming loads; the
  // arrays are padded so the rounded-up tail stays in bounds) and its window of
  // last-level fibers.
  const int64_t fs = pb[ORDER - 2];
  const int W = (int)(pn[ORDER - 2] - fs + 1);
  {
    const uint64_t polF = policy_evict_first();
    const int n4 = (int)((bend - bstart + 3) >> 2);
    const int32_t* gl = a.crd[ORDER - 1] + bstart;
    if constexpr (EXACT) {
      // whole words below nnz, element loads (zero filled) for the ragged end
      const int nt = (int)(bend - bstart);
      for (int i = threadIdx.x; i < n4; i += tb) {
        if (4 * i + 4 <= nt) {
          reinterpret_cast<int4*>(s_lc)[i] = ld_stream_i4(gl + 4 * i, polF);
          reinterpret_cast<float4*>(s_val)[i] = ld_stream_f4(static_cast<const float*>(a.vals) + bstart + 4 * i, polF);
        } else {
          for (int k = 0; k < 4; k++) {
            const bool in = 4 * i + k < nt;
            s_lc[4 * i + k] = in ? gl[4 * i + k] : 0;
            reinterpret_cast<float*>(s_val)[4 * i + k] = in ? static_cast<const float*>(a.vals)[bstart + 4 * i + k] : 0.f;
          }
        }
      }
    } else {
    for (int i = threadIdx.x; i < n4; i += tb)
      reinterpret_cast<int4*>(s_lc)[i] = ld_stream_i4(gl + 4 * i, polF);
    if constexpr (VB == 4) {
      const float* gv = static_cast<const float*>(a.vals) + bstart;
      for (int i = threadIdx.x; i < n4; i += tb)
        reinterpret_cast<float4*>(s_val)[i] = ld_stream_f4(gv + 4 * i, polF);
    } else {
      const uint16_t* gv = static_cast<const uint16_t*>(a.vals) + bstart;
      for (int i = threadIdx.x; i < n4; i += tb)
        reinterpret_cast<uint2*>(s_val)[i] = ld_stream_u2(gv + 4 * i, polF);
    }
    }
    const int32_t* gpos = a.pos[ORDER - 1] + fs;
    const int32_t* gcrd = a.crd[ORDER - 2] + fs;
    for (int x = threadIdx.x; x <= W; x += tb) s_pos[x] = gpos[x];
    for (int x = threadIdx.x; x < W; x += tb) s_fcrd[x] = gcrd[x];
  }
  __syncthreads();

  const int team = threadIdx.x / LPR;
  const int q = threadIdx.x % LPR;
  const int tw = team % TW;       // team index inside its warp
  const int warp = threadIdx.x / 32;
  WK wk(a, q);

  Summ<CPT> X;
  X.h = kEmpty;
  X.t = kNone;
  const int64_t s = bstart + (int64_t)team * a.G;
  if (s < bend)
    wk.walk(s, min(s + (int64_t)a.G, bend), bstart, s_lc, s_val, s_pos, s_fcrd, W, fs, pb, pn, X);

  // Warp-level merge of team summaries (tree over teams, keyed by row).
#pragma unroll
  for (int d = 1; d < TW; d <<= 1) {
    Summ<CPT> Y;
    Y.h = __shfl_down_sync(0xffffffffu, X.h, d * LPR);
    Y.t = __shfl_down_sync(0xffffffffu, X.t, d * LPR);
#pragma unroll
    for (int c = 0; c < CPT; c++) {
      Y.ha[c] = __shfl_down_sync(0xffffffffu, X.ha[c], d * LPR);
      Y.ta[c] = __shfl_down_sync(0xffffffffu, X.ta[c], d * LPR);
    }
    if ((tw & (2 * d - 1)) == 0 && tw + d < TW) wk.combine(X, Y);
  }
  if (tw == 0) {
    if (q == 0) { s_wh[warp] = X.h; s_wt[warp] = X.t; }
#pragma unroll
    for (int c = 0; c < CPT; c++) {
      s_wha[warp * RP + q * CPT + c] = X.ha[c];
      s_wta[warp * RP + q * CPT + c] = X.ta[c];
    }
  }
  __syncthreads();

  // Block-level merge by the first team, then the cross-block protocol.
  if (threadIdx.x < LPR) {
    for (int w = 1; w < nw; w++) {
      Summ<CPT> Y;
      Y.h = s_wh[w];
      Y.t = s_wt[w];
#pragma unroll
      for (int c = 0; c < CPT; c++) {
        Y.ha[c] = s_wha[w * RP + q * CPT + c];
        Y.ta[c] = s_wta[w * RP + q * CPT + c];
      }
      wk.combine(X, Y);
    }
    // Up to two boundary rows: slot 0 = the block's first row, slot 1 = its last.
#pragma unroll
    for (int slot = 0; slot < 2; slot++) {
      const int r = slot == 0 ? X.h : X.t;
      int last = -1;
      int64_t n0 = 0, n1 = 0;
      if (r >= 0) {
        wk.row_span(r, n0, n1);
        const int64_t b0 = n0 / P, b1 = (n1 - 1) / P;
        if (b0 == b1) {
          if (slot == 0) wk.store_row(r, X.ha); else wk.store_row(r, X.ta);
        } else {
          float* cp = a.carry + ((size_t)(2 * b + slot)) * RP + q * CPT;
#pragma unroll
          for (int c = 0; c < CPT; c++) cp[c] = (slot == 0 ? X.ha[c] : X.ta[c]) * wk.sc[c];
          __threadfence();
          __syncwarp((LPR == 32) ? 0xffffffffu : ((1u << LPR) - 1u));
          int t = 0;
          if (q == 0) {
            t = atomicAdd(a.tickets + r, 1);
            if (t == (int)(b1 - b0)) { a.tickets[r] = 0; __threadfence(); }
          }
          t = __shfl_sync((LPR == 32) ? 0xffffffffu : ((1u << LPR) - 1u), t, 0, LPR);
          if (t == (int)(b1 - b0)) last = r;
        }
      }
      if (q == 0) {
        s_ctl[slot] = last;
        s_ctl[2 + slot] = (int)(n0 / P);
        s_ctl[4 + slot] = (int)((n1 - 1) / P);
      }
    }
  }
  __syncthreads();

  // The last block to reach a boundary row sums its block partials in FP64, in block order.
#pragma unroll
  for (int slot = 0; slot < 2; slot++) {
    const int r = s_ctl[slot];
    if (r < 0) continue;  // uniform across the block
    const int b0 = s_ctl[2 + slot], b1 = s_ctl[4 + slot];
    const int j = threadIdx.x % RP;
    const int sl = threadIdx.x / RP, ns = tb / RP;
    double acc = 0.0;
    for (int bb = b0 + sl; bb <= b1; bb += ns) {
      const int sb = (a.part[(size_t)bb * (ORDER - 1)] == r) ? 0 : 1;
      acc += (double)__ldcg(a.carry + ((size_t)(2 * bb + sb)) * RP + j);
    }
    s_dbl[threadIdx.x] = acc;
    __syncthreads();
    if (threadIdx.x < RP) {
      double tot = 0.0;
      for (int k = 0; k < ns; k++) tot += s_dbl[k * RP + threadIdx.x];
      if (threadIdx.x < a.R) a.out[wk.row_id(r) * a.ldo + threadIdx.x] = (float)tot;
    }
    __syncthreads();
  }
}

// Partition: for each block boundary b in [0, nblocks], the root position and
// the fiber id at every level that contain nonzero min(b*P, nnz-1).
// Same role as the reference's taco_binarySearchBeforeBlock +
// taco_binarySearchIndirectBeforeBlock pair (gpu_library.h:206-256), fused.
template <int ORDER>
__global__ void partition_kernel(const __grid_constant__ WalkArgs a) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b > a.nblocks) return;
  const int64_t s = (b < a.nblocks) ? (int64_t)b * a.P : a.nnz - 1;
  int32_t* out = const_cast<int32_t*>(a.part) + (size_t)b * (ORDER - 1);
  // number of fibers at level ORDER-2 = last entry index of pos[ORDER-1] minus one
  int64_t hi = 0;
  // fibers at level 1: pos[1][nrows]; level 2: pos[2][#level1]
  int64_t nf1 = a.pos[1][a.nrows];
  int64_t f1;
  if constexpr (ORDER == 3) {
    f1 = search_le(a.pos[2], 0, nf1 - 1, s);
    out[1] = (int32_t)f1;
  } else {
    int64_t nf2 = a.pos[2][nf1];
    int64_t f2 = search_le(a.pos[3], 0, nf2 - 1, s);
    f1 = search_le(a.pos[2], 0, nf1 - 1, f2);
    out[1] = (int32_t)f1;
    out[2] = (int32_t)f2;
  }
  (void)hi;
  out[0] = (int32_t)search_le(a.pos[1], 0, a.nrows - 1, f1);
}

#endif  // TT_ARGS_ONLY
}  // namespace tt
