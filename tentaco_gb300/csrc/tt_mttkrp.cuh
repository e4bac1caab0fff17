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
//     the block's two carry slots; after the walk, seg_fold_kernel sums each
//     row's carries inside a segment of 32 blocks (FP32, Kahan-compensated) and
//     seg_chain_kernel sums the FP64 partials of rows crossing segments, both in
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
#include <cuda.h>  // CUtensorMap (the TMA walk's descriptor of the leaf factor)
#include "tt_common.cuh"

namespace tt {

struct alignas(64) WalkArgs {
  CUtensorMap tmap;       // TMA walk: 2-D map of the leaf factor (RP columns x rows, box RP x 1)
  const int32_t* pos[5];  // pos[l], l = 1..order-1 (pos[1] indexed by root position)
  const int32_t* crd[5];  // crd[l], l = 1..order-1; crd[0] = root ids (nullptr: dense root)
  const void* vals;       // FP32 or BF16, padded
  const void* fac[4];     // factors of modes 1..order-1, RP entries per row
  const float* colscale;  // RP output scales (nullptr: all 1)
  float* out;             // output rows (row id = crd[0][ip] or ip), ldo floats apart
  const int32_t* part;    // (nblocks+1) x (order-1): root position, then fiber ids per level
  float* carry;           // 2 * nblocks * RP: partial rows shared with other blocks
  int32_t* meta;          // 4 ints per block: first row, last row, flags (see block_merge)
  int64_t nnz;
  int32_t nrows;
  int32_t R;              // columns stored (<= RP)
  int32_t ldo;
  int32_t P;              // nonzeros per block
  int32_t G;              // nonzeros per team, a power of two >= 4
  int32_t lgG;            // log2(G)
  int32_t nblocks;
  int32_t rp;             // factor row width the kernels were compiled for
  int32_t fac_rows[4];    // rows of each factor (bounds for checked builds)
  int32_t smem_bytes;     // dynamic shared memory of the launch (bounds for checked builds)
  int32_t accum;          // 1: add rows into out (slab passes), 0: overwrite
  int32_t gpol;           // L2 policy of the lean walk's factor-row gathers: 0 evict_last, 1 evict_normal
  float vscale;           // TTV: scale of the stored values (1 for FP32 values)
  double* segcarry;       // cross-unit rows: 2 FP64 partial rows per segment of kSeg units
  int32_t* segmeta;       // 4 ints per segment
  int32_t wcap;           // staged kernels: window fibers per block the shared memory holds
  int32_t* err;           // staged kernels: set nonzero if a block's window exceeds wcap
  const int32_t* kexp;    // flat walk: the level-1 coordinate of every nonzero (padded)
  const int32_t* kexp2;   // flat and strip walks, four or five modes: the level-2 coordinate of every nonzero (padded)
  const int32_t* kexp3;   // strip walk, five modes: the level-3 coordinate of every nonzero (padded)
  const int32_t* rnz;     // flat and strip walks: first nonzero of every row (nrows + 1); null otherwise
  uint32_t wait_ns;       // TMA walk: bound on each wait for a stage's barrier, ns (0: 5 ms)
  int32_t tma_withhold;   // TMA walk, test hook: 1 arms every stage's barrier but issues no copy
  int32_t unit_lo;        // strip walk: first unit of this launch (units arriving in chunks)
  int32_t unit_hi;        // strip walk: end of this launch's units (0: nblocks)
};

constexpr int kEmpty = -2;  // summary of a team that owns no nonzeros
constexpr int kNone = -1;   // single-row summary: no tail

template <int CPT>
struct Summ {
  int h, t;
  float ha[CPT], ta[CPT];
};

// Work units per segment of the two-level cross-unit row merge.
constexpr int kSeg = 32;
__host__ __device__ inline int num_segments(int units) { return (units + kSeg - 1) / kSeg; }

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
  return (b + 15) & ~(size_t)15;
}

// Lean kernel, shared memory of one warp: coordinate runs TW x (G+4) int32,
// value runs TW x (G*vbytes + 16) bytes, window starts and coordinates (a
// warp's window has at most TW*G + 1 fibers).
// Shared memory of one flat-walk warp: leaf and upper coordinate runs (order - 1
// sets of tw runs of G + 4 int32 each) and value runs (tw runs of G * vbytes + 16
// bytes).
__host__ __device__ inline size_t flat_warp_bytes(int G, int tw, int vbytes, int order = 3) {
  size_t b = (size_t)(order - 1) * tw * (G + 4) * 4 + (size_t)tw * ((size_t)G * vbytes + 16);
  return (b + 15) & ~(size_t)15;
}

__host__ __device__ inline size_t lean_warp_bytes(int G, int tw, int vbytes) {
  const size_t pu = (size_t)tw * G;
  size_t b = (size_t)tw * (G + 4) * 4 + (size_t)tw * ((size_t)G * vbytes + 16);
  b += (pu + 2) * 4 * 2;
  return (b + 15) & ~(size_t)15;
}

// TMA walk, shared memory of one warp: a ring of ns stages of kTmaRows factor rows
// (rb bytes each), ns mbarriers, then the lean layout; rounded to 128 bytes so every
// warp's ring starts 128-byte aligned.
constexpr int kTmaRows = 32;  // factor rows per stage: 8 gather4 copies
__host__ __device__ inline size_t tma_warp_bytes(int G, int tw, int vbytes, int rb, int ns) {
  size_t b = (size_t)ns * kTmaRows * rb + (size_t)ns * 8;
  b = (b + 15) & ~(size_t)15;
  b += lean_warp_bytes(G, tw, vbytes);
  return (b + 127) & ~(size_t)127;
}

// Staged kernels: the tile, the gathered factor rows (one per nonzero, one per
// window fiber) and the window, then the same merge scratch.
__host__ __device__ inline size_t stage_off_rows(int P, int vbytes) {
  return (walk_tile_bytes(P, vbytes) + 15) & ~(size_t)15;
}
__host__ __device__ inline size_t stage_smem_bytes(int P, int wcap, int tb, int rp, int vbytes, int fbytes) {
  const size_t rb = (size_t)rp * fbytes;
  size_t b = stage_off_rows(P, vbytes) + (size_t)P * rb + (size_t)wcap * rb;
  b += (size_t)(2 * wcap + 4) * sizeof(int32_t);
  const size_t nw = (size_t)tb / 32;
  b += nw * 2 * sizeof(int32_t) + nw * 2 * (size_t)rp * sizeof(float);
  return (b + 15) & ~(size_t)15;
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

  __device__ __forceinline__ Walk(const WalkArgs& args, int lane_in_team) : a(args), q(lane_in_team) {}

  // Output scale of this lane's column c (16-bit storage), read when a row is
  // written rather than held in registers through the walk.
  __device__ __forceinline__ float sc(int c) const { return a.colscale ? a.colscale[q * CPT + c] : 1.0f; }

  __device__ __forceinline__ int64_t row_id(int ip) const {
    return a.crd[0] ? (int64_t)a.crd[0][ip] : (int64_t)ip;
  }

  // Store a finished output row (scaled).
  // Store a finished output row (scaled); slab passes add into the row (each
  // row has one writer per pass, and passes run in order on one stream).
  __device__ __forceinline__ void store_row(int ip, const float (&acc)[CPT]) const {
    float* o = a.out + row_id(ip) * a.ldo + q * CPT;
    if (CPT == 4 && a.R == RP && (a.ldo & 3) == 0) {
      float4 r = make_float4(acc[0] * sc(0), acc[1] * sc(1), acc[2] * sc(2), acc[3] * sc(3));
      if (a.accum) {
        const float4 o4 = *reinterpret_cast<const float4*>(o);
        r.x += o4.x; r.y += o4.y; r.z += o4.z; r.w += o4.w;
      }
      *reinterpret_cast<float4*>(o) = r;
    } else {
#pragma unroll
      for (int c = 0; c < CPT; c++)
        if (q * CPT + c < a.R) o[c] = acc[c] * sc(c) + (a.accum ? o[c] : 0.f);
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

  // Bytes of its factor row one lane loads per nonzero (its CPT columns).
  static constexpr int LB = CPT * (FK == kF32 ? 4 : 2);

  // ---- lean walk (family 0) ------------------------------------------------
  static constexpr int NWD = LB >= 4 ? LB / 4 : 1;  // 32-bit words of a lane's row piece
  static constexpr int MWD = ORDER == 4 ? NWD : 1;    // words of a level-2 piece (flat walk, four modes)
  static constexpr int FRB = RP * (FK == kF32 ? 4 : 2);  // bytes per factor row

  // The lane's piece (LB bytes) of a factor row, as raw words: the load is
  // issued now, the conversion happens when the words are used.
  // L1: allocate the piece in L1 (rows that the next nonzeros of the same fiber
  // read again: the flat walk's upper-level rows); otherwise L1 is bypassed.
  template <bool L1 = false>
  __device__ __forceinline__ static void piece_load(const unsigned char* p, uint64_t pol, uint32_t (&w)[NWD]) {
    if constexpr (LB == 32) {
      const uint4 x = L1 ? ld_gather_16(p, pol) : ld_gather_16_na(p, pol);
      const uint4 y = L1 ? ld_gather_16(p + 16, pol) : ld_gather_16_na(p + 16, pol);
      w[0] = x.x; w[1] = x.y; w[2] = x.z; w[3] = x.w; w[4] = y.x; w[5] = y.y; w[6] = y.z; w[7] = y.w;
    } else if constexpr (LB == 16) {
      const uint4 x = L1 ? ld_gather_16(p, pol) : ld_gather_16_na(p, pol);
      w[0] = x.x; w[1] = x.y; w[2] = x.z; w[3] = x.w;
    } else if constexpr (LB == 8) {
      const uint2 x = L1 ? ld_gather_8(p, pol) : ld_gather_8_na(p, pol);
      w[0] = x.x; w[1] = x.y;
    } else if constexpr (LB == 4) {
      w[0] = L1 ? ld_gather_4(p, pol) : ld_gather_4_na(p, pol);
    } else {
      w[0] = L1 ? ld_gather_2(p, pol) : ld_gather_2_na(p, pol);
    }
  }
  __device__ __forceinline__ static void piece_cvt(const uint32_t (&w)[NWD], float (&g)[CPT]) {
    if constexpr (FK == kF32) {
#pragma unroll
      for (int c = 0; c < CPT; c++) g[c] = __uint_as_float(w[c]);
    } else if constexpr (CPT == 1) {
      g[0] = lo16<FK>(w[0]);
    } else {
#pragma unroll
      for (int c = 0; c < CPT; c += 2) {
        const float2 f = pair16<FK>(w[c >> 1]);
        g[c] = f.x;
        g[c + 1] = f.y;
      }
    }
  }
  // U consecutive stored values of a team's run (runs of 4 or more start 16-byte aligned).
  template <int U>
  __device__ __forceinline__ static void vals_load(const unsigned char* vt, float (&v)[U]) {
    if constexpr (VK == kF32 && U % 4 == 0) {
#pragma unroll
      for (int k = 0; k < U / 4; k++) {
        const float4 f = reinterpret_cast<const float4*>(vt)[k];
        v[4 * k] = f.x; v[4 * k + 1] = f.y; v[4 * k + 2] = f.z; v[4 * k + 3] = f.w;
      }
    } else if constexpr (VK != kF32 && U % 8 == 0) {
#pragma unroll
      for (int k = 0; k < U / 8; k++) {
        const uint4 w = reinterpret_cast<const uint4*>(vt)[k];
        const float2 a = pair16<VK>(w.x), b = pair16<VK>(w.y), c = pair16<VK>(w.z), d = pair16<VK>(w.w);
        v[8 * k] = a.x; v[8 * k + 1] = a.y; v[8 * k + 2] = b.x; v[8 * k + 3] = b.y;
        v[8 * k + 4] = c.x; v[8 * k + 5] = c.y; v[8 * k + 6] = d.x; v[8 * k + 7] = d.y;
      }
    } else if constexpr (VK != kF32 && U == 4) {
      const uint2 w = *reinterpret_cast<const uint2*>(vt);
      const float2 a = pair16<VK>(w.x), b = pair16<VK>(w.y);
      v[0] = a.x; v[1] = a.y; v[2] = b.x; v[3] = b.y;
    } else {  // 1 or 2 values
#pragma unroll
      for (int u = 0; u < U; u++) v[u] = val_one(vt, u);
    }
  }
  // 16-bit storage whose values and factors share a kind: the walk's products
  // use the mixed-precision FMA on the raw 16-bit words (same result as fmaf on
  // the converted operands, without the conversions).
  static constexpr bool MIXED = VK == FK && VK != kF32;
  // f3 += (half HV of value word v) * (the lane's piece w of a factor row)
  template <int HV>
  __device__ __forceinline__ static void acc_mixed(float (&f3)[CPT], const uint32_t (&w)[NWD], uint32_t v) {
    if constexpr (CPT == 1) {
      mfma1<FK, HV>(f3[0], w[0], v);
    } else {
#pragma unroll
      for (int k = 0; k < CPT / 2; k++) mfma2<FK, HV>(f3[2 * k], f3[2 * k + 1], w[k], v);
    }
  }
  // U consecutive stored 16-bit values as raw words, two per word (U % 4 == 0 or
  // U == 2; runs start 16-byte aligned and batches at multiples of U).
  template <int U>
  __device__ __forceinline__ static void vals_raw(const unsigned char* vt, uint32_t (&w)[U / 2]) {
    static_assert(U % 4 == 0 || U == 2, "raw values come in 4- or 8-byte pieces");
    if constexpr (U == 2) {
      w[0] = *reinterpret_cast<const uint32_t*>(vt);
    } else if constexpr (U % 8 == 0) {
#pragma unroll
      for (int k = 0; k < U / 8; k++) {
        const uint4 x = reinterpret_cast<const uint4*>(vt)[k];
        w[4 * k] = x.x; w[4 * k + 1] = x.y; w[4 * k + 2] = x.z; w[4 * k + 3] = x.w;
      }
    } else {
      const uint2 x = *reinterpret_cast<const uint2*>(vt);
      w[0] = x.x; w[1] = x.y;
    }
  }
  __device__ __forceinline__ static float val_one(const unsigned char* vt, int j) {
    if constexpr (VK == kF32) return reinterpret_cast<const float*>(vt)[j];
    else return lo16<VK>((uint32_t)reinterpret_cast<const uint16_t*>(vt)[j]);
  }

  // Serial walk of this team's n nonzeros starting at absolute position s.
  //   lc, vt: the team's coordinate / value run in shared memory (entry 0 = s)
  // Nonzero-level factor rows are gathered U nonzeros per batch into registers,
  // one batch ahead of use (two register buffers); the window-level factor row
  // of the next fiber is loaded when the current one starts.  The fold of a
  // finished fiber and the row bookkeeping are the only branches.
  template <int U>
  __device__ __forceinline__ void walk_lean(int s, int n, const int32_t* lc, const unsigned char* vt,
                                            const int32_t* s_pos, const int32_t* s_fcrd, int W, int fs,
                                            const int32_t* pb, const int32_t* pn, Summ<CPT>& X) const {
    const uint64_t pol = a.gpol == 1 ? policy_evict_normal() : policy_evict_last();
    const int32_t* pos1 = a.pos[1];
    const unsigned char* fz = static_cast<const unsigned char*>(a.fac[ORDER - 2]) + q * LB;
    const unsigned char* fw = static_cast<const unsigned char*>(a.fac[ORDER == 3 ? 0 : 1]) + q * LB;
    int x = (int)search_le(s_pos, 0, W - 1, s);
    int fend = s_pos[x + 1];
    int f1 = 0, kend = 0, ip;
    float crow[CPT];
    if constexpr (ORDER == 3) {
      ip = (int)search_le(pos1, pb[0], pn[0], fs + x);
    } else {
      f1 = (int)search_le(a.pos[2], pb[1], pn[1], fs + x);
      kend = a.pos[2][f1 + 1];
      ip = (int)search_le(pos1, pb[0], pn[0], f1);
      frow(0, a.crd[1][f1], pol, crow);
    }
    int rend = pos1[ip + 1];
    uint32_t wc[NWD], wn[NWD];
    piece_load(fw + (size_t)(uint32_t)s_fcrd[x] * FRB, pol, wc);
    if (x + 1 < W) piece_load(fw + (size_t)(uint32_t)s_fcrd[x + 1] * FRB, pol, wn);
    float f3[CPT], f2[CPT], ra[CPT];
#pragma unroll
    for (int c = 0; c < CPT; c++) { f3[c] = 0.f; f2[c] = 0.f; ra[c] = 0.f; }
    bool flushed = false;

    // the current window fiber ended: fold its partial into the parent level
    auto fold = [&]() {
      float cw[CPT];
      piece_cvt(wc, cw);
      if constexpr (ORDER == 3) {
#pragma unroll
        for (int c = 0; c < CPT; c++) { ra[c] = fmaf(f3[c], cw[c], ra[c]); f3[c] = 0.f; }
      } else {
#pragma unroll
        for (int c = 0; c < CPT; c++) { f2[c] = fmaf(f3[c], cw[c], f2[c]); f3[c] = 0.f; }
      }
      x++;
      fend = s_pos[x + 1];
#pragma unroll
      for (int k = 0; k < NWD; k++) wc[k] = wn[k];
      if (x + 1 < W) piece_load(fw + (size_t)(uint32_t)s_fcrd[x + 1] * FRB, pol, wn);
      const int fg = fs + x;
      if constexpr (ORDER == 4) {
        while (fg >= kend) {
#pragma unroll
          for (int c = 0; c < CPT; c++) { ra[c] = fmaf(f2[c], crow[c], ra[c]); f2[c] = 0.f; }
          f1++;
          kend = a.pos[2][f1 + 1];
          while (f1 >= rend) { flush(ip, ra, flushed, X); ip++; rend = pos1[ip + 1]; }
          frow(0, a.crd[1][f1], pol, crow);
        }
      } else {
        while (fg >= rend) { flush(ip, ra, flushed, X); ip++; rend = pos1[ip + 1]; }
      }
    };
    auto load = [&](uint32_t (&g)[U][NWD], int j) {
      int32_t l[U];
#pragma unroll
      for (int k = 0; k < U / 4; k++) {
        const int4 c4 = reinterpret_cast<const int4*>(lc + j)[k];
        l[4 * k] = c4.x; l[4 * k + 1] = c4.y; l[4 * k + 2] = c4.z; l[4 * k + 3] = c4.w;
      }
#pragma unroll
      for (int u = 0; u < U; u++) piece_load(fz + (size_t)(uint32_t)l[u] * FRB, pol, g[u]);
    };
    auto consume = [&](const uint32_t (&g)[U][NWD], int j) {
      if constexpr (MIXED) {
        uint32_t vw[U / 2];
        vals_raw<U>(vt + (size_t)j * VB, vw);
        if (s + j + U <= fend) {
#pragma unroll
          for (int u = 0; u < U; u += 2) {
            acc_mixed<0>(f3, g[u], vw[u >> 1]);
            acc_mixed<1>(f3, g[u + 1], vw[u >> 1]);
          }
          return;
        }
#pragma unroll
        for (int u = 0; u < U; u += 2) {
          while (s + j + u >= fend) fold();
          acc_mixed<0>(f3, g[u], vw[u >> 1]);
          while (s + j + u + 1 >= fend) fold();
          acc_mixed<1>(f3, g[u + 1], vw[u >> 1]);
        }
        return;
      }
      float v[U];
      vals_load<U>(vt + (size_t)j * VB, v);
      if (s + j + U <= fend) {
        // the whole batch lies in the current fiber: no boundary checks
#pragma unroll
        for (int u = 0; u < U; u++) {
          float d[CPT];
          piece_cvt(g[u], d);
#pragma unroll
          for (int c = 0; c < CPT; c++) f3[c] = fmaf(v[u], d[c], f3[c]);
        }
        return;
      }
#pragma unroll
      for (int u = 0; u < U; u++) {
        while (s + j + u >= fend) fold();
        float d[CPT];
        piece_cvt(g[u], d);
#pragma unroll
        for (int c = 0; c < CPT; c++) f3[c] = fmaf(v[u], d[c], f3[c]);
      }
    };
    const int nb = n / U;
    uint32_t gA[U][NWD], gB[U][NWD];
    if (nb > 0) load(gA, 0);
    for (int b = 0; b < nb; b += 2) {
      if (b + 1 < nb) load(gB, (b + 1) * U);
      consume(gA, b * U);
      if (b + 1 < nb) {
        if (b + 2 < nb) load(gA, (b + 2) * U);
        consume(gB, (b + 1) * U);
      }
    }
    for (int j = nb * U; j < n; j++) {  // ragged end (the tensor's last tile only)
      uint32_t g[NWD];
      piece_load(fz + (size_t)(uint32_t)lc[j] * FRB, pol, g);
      if constexpr (MIXED) {
        const uint32_t vr = reinterpret_cast<const uint16_t*>(vt)[j];
        while (s + j >= fend) fold();
        acc_mixed<0>(f3, g, vr);
      } else {
        const float v = val_one(vt, j);
        while (s + j >= fend) fold();
        float d[CPT];
        piece_cvt(g, d);
#pragma unroll
        for (int c = 0; c < CPT; c++) f3[c] = fmaf(v, d[c], f3[c]);
      }
    }
    {
      float cw[CPT];
      piece_cvt(wc, cw);
      if constexpr (ORDER == 3) {
#pragma unroll
        for (int c = 0; c < CPT; c++) ra[c] = fmaf(f3[c], cw[c], ra[c]);
      } else {
#pragma unroll
        for (int c = 0; c < CPT; c++) { f2[c] = fmaf(f3[c], cw[c], f2[c]); ra[c] = fmaf(f2[c], crow[c], ra[c]); }
      }
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

  // ---- flat walk (family 3) --------------------------------------------------
  // Every nonzero carries its upper coordinates (a.kexp: level 1, a.kexp2: level 2
  // for four modes), so a team accumulates A(i,:) += ((v * C(k,:)) [* D(l,:)]) *
  // last(m,:) per nonzero with every factor row gathered (the upper factors are
  // small and stay in L2): the reference's own loop arithmetic
  // (tensor_kernels/mttkrp3_csf_cpu_taco.h:45, mttkrp4_csf_cpu_taco.h:53), with no
  // fiber boundaries in the walk; only row ends (a.rnz) are checked, per batch.
  //   lc, kc, k2c, vt: the team's leaf coordinates, level-1 coordinates, level-2
  //   coordinates (four modes) and values
  //   rlo, rhi: rows holding the unit's first nonzero and the next unit's
  template <int U>
  __device__ __forceinline__ void walk_flat(int s, int n, const int32_t* lc, const int32_t* kc, const int32_t* k2c,
                                            const unsigned char* vt, int rlo, int rhi, Summ<CPT>& X) const {
    const uint64_t pol = a.gpol == 1 ? policy_evict_normal() : policy_evict_last();
    const int32_t* rnz = a.rnz;
    const unsigned char* fd = static_cast<const unsigned char*>(a.fac[ORDER - 2]) + q * LB;  // leaf factor
    const unsigned char* fc = static_cast<const unsigned char*>(a.fac[0]) + q * LB;          // level-1 factor
    const unsigned char* fm = static_cast<const unsigned char*>(a.fac[1]) + q * LB;          // level-2 factor (four modes)
    int ip = (int)search_le(rnz, rlo, rhi, s);
    int rend = rnz[ip + 1];
    float ra[CPT];
#pragma unroll
    for (int c = 0; c < CPT; c++) ra[c] = 0.f;
    bool flushed = false;
    // one nonzero: ra += v * (c * d) (three modes) or (c * d) * (v * m) (four),
    // value half HV of word vw.  The 16-bit products c * d and v * m are exact in
    // FP32 (mixed-precision FMA with a zero addend), so each column takes one
    // rounding per nonzero, as (v * c) * d does; the FP32 FMAs go two columns per
    // instruction.
    auto acc16 = [&](const uint32_t (&gc)[NWD], const uint32_t (&gm)[MWD], const uint32_t (&gd)[NWD], uint32_t vw,
                     auto hv) {
      constexpr int HV = decltype(hv)::value;
      if constexpr (CPT == 1) {
        const float p = hprod1<FK, 0, 0>(gc[0], gd[0]);
        if constexpr (ORDER == 4) ra[0] = fmaf(p, hprod1<FK, HV, 0>(vw, gm[0]), ra[0]);
        else ra[0] = fmaf(HV ? hi16<VK>(vw) : lo16<VK>(vw), p, ra[0]);
      } else {
        const float v = HV ? hi16<VK>(vw) : lo16<VK>(vw);
        const uint32_t vv = HV ? (vw >> 16) | (vw & 0xffff0000u) : (vw << 16) | (vw & 0xffffu);  // v in both halves
#pragma unroll
        for (int k = 0; k < CPT / 2; k++) {
          const float2 p = hprod2<FK>(gc[k], gd[k]);
          if constexpr (ORDER == 4) {
            const float2 t = hprod2<FK>(vv, gm[k]);
            ffma2(ra[2 * k], ra[2 * k + 1], p.x, p.y, t.x, t.y);
          } else {
            (void)vv;
            ffma2(ra[2 * k], ra[2 * k + 1], v, v, p.x, p.y);
          }
        }
      }
    };
    auto acc32 = [&](const uint32_t (&gc)[NWD], const uint32_t (&gm)[MWD], const uint32_t (&gd)[NWD], float v) {
      float c[CPT], d[CPT], mm[CPT];
      piece_cvt(gc, c);
      piece_cvt(gd, d);
      if constexpr (ORDER == 4) piece_cvt(gm, mm);
      else (void)gm;
      if constexpr (CPT == 1) {
        float t = v * c[0];
        if constexpr (ORDER == 4) t = t * mm[0];
        ra[0] = fmaf(t, d[0], ra[0]);
      } else {
#pragma unroll
        for (int k = 0; k < CPT; k += 2) {
          float2 t = fmul2(v, v, c[k], c[k + 1]);
          if constexpr (ORDER == 4) t = fmul2(t.x, t.y, mm[k], mm[k + 1]);
          ffma2(ra[k], ra[k + 1], t.x, t.y, d[k], d[k + 1]);
        }
      }
    };
    auto next_row = [&]() {
      flush(ip, ra, flushed, X);
      ip++;
      rend = rnz[ip + 1];
    };
    auto load = [&](uint32_t (&gc)[U][NWD], uint32_t (&gm)[U][MWD], uint32_t (&gd)[U][NWD], int j) {
      int32_t l[U], k[U], k2[U];
      if constexpr (U == 2) {  // 8-byte coordinate pairs
        const int2 l2 = *reinterpret_cast<const int2*>(lc + j);
        const int2 kk = *reinterpret_cast<const int2*>(kc + j);
        l[0] = l2.x; l[1] = l2.y; k[0] = kk.x; k[1] = kk.y;
        if constexpr (ORDER == 4) {
          const int2 m2 = *reinterpret_cast<const int2*>(k2c + j);
          k2[0] = m2.x; k2[1] = m2.y;
        }
      }
#pragma unroll
      for (int w = 0; w < U / 4; w++) {
        const int4 l4 = reinterpret_cast<const int4*>(lc + j)[w];
        const int4 k4 = reinterpret_cast<const int4*>(kc + j)[w];
        l[4 * w] = l4.x; l[4 * w + 1] = l4.y; l[4 * w + 2] = l4.z; l[4 * w + 3] = l4.w;
        k[4 * w] = k4.x; k[4 * w + 1] = k4.y; k[4 * w + 2] = k4.z; k[4 * w + 3] = k4.w;
        if constexpr (ORDER == 4) {
          const int4 m4 = reinterpret_cast<const int4*>(k2c + j)[w];
          k2[4 * w] = m4.x; k2[4 * w + 1] = m4.y; k2[4 * w + 2] = m4.z; k2[4 * w + 3] = m4.w;
        }
      }
#pragma unroll
      for (int u = 0; u < U; u++) {
        piece_load<true>(fc + (size_t)(uint32_t)k[u] * FRB, pol, gc[u]);
        if constexpr (ORDER == 4) piece_load<true>(fm + (size_t)(uint32_t)k2[u] * FRB, pol, gm[u]);
        piece_load(fd + (size_t)(uint32_t)l[u] * FRB, pol, gd[u]);
      }
      if constexpr (ORDER != 4) {
#pragma unroll
        for (int u = 0; u < U; u++) gm[u][0] = 0u;
      }
    };
    auto consume = [&](const uint32_t (&gc)[U][NWD], const uint32_t (&gm)[U][MWD], const uint32_t (&gd)[U][NWD], int j) {
      const bool inside = s + j + U <= rend;  // the batch lies in one row
      if constexpr (MIXED) {
        uint32_t vw[U / 2];
        vals_raw<U>(vt + (size_t)j * VB, vw);
#pragma unroll
        for (int u = 0; u < U; u += 2) {
          if (!inside) while (s + j + u >= rend) next_row();
          acc16(gc[u], gm[u], gd[u], vw[u >> 1], std::integral_constant<int, 0>{});
          if (!inside) while (s + j + u + 1 >= rend) next_row();
          acc16(gc[u + 1], gm[u + 1], gd[u + 1], vw[u >> 1], std::integral_constant<int, 1>{});
        }
      } else {
        float v[U];
        vals_load<U>(vt + (size_t)j * VB, v);
#pragma unroll
        for (int u = 0; u < U; u++) {
          if (!inside) while (s + j + u >= rend) next_row();
          acc32(gc[u], gm[u], gd[u], v[u]);
        }
      }
    };
    const int nb = n / U;
    uint32_t cA[U][NWD], mA[U][MWD], dA[U][NWD], cB[U][NWD], mB[U][MWD], dB[U][NWD];
    if (nb > 0) load(cA, mA, dA, 0);
    for (int b = 0; b < nb; b += 2) {
      if (b + 1 < nb) load(cB, mB, dB, (b + 1) * U);
      consume(cA, mA, dA, b * U);
      if (b + 1 < nb) {
        if (b + 2 < nb) load(cA, mA, dA, (b + 2) * U);
        consume(cB, mB, dB, (b + 1) * U);
      }
    }
    for (int j = nb * U; j < n; j++) {  // ragged end (the tensor's last tile only)
      uint32_t gc[NWD], gd[NWD], gm[MWD];
      piece_load<true>(fc + (size_t)(uint32_t)kc[j] * FRB, pol, gc);
      if constexpr (ORDER == 4) piece_load<true>(fm + (size_t)(uint32_t)k2c[j] * FRB, pol, gm);
      else gm[0] = 0u;
      piece_load(fd + (size_t)(uint32_t)lc[j] * FRB, pol, gd);
      while (s + j >= rend) next_row();
      if constexpr (MIXED) acc16(gc, gm, gd, (uint32_t)reinterpret_cast<const uint16_t*>(vt)[j], std::integral_constant<int, 0>{});
      else acc32(gc, gm, gd, val_one(vt, j));
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

  // Walk like walk_lean, but the nonzero-level factor rows arrive by TMA: for
  // every stage k of the warp (U nonzeros of each of its TW teams, kTmaRows rows),
  // lanes 0..7 issue one tile::gather4 copy each into ring slot k % NS, completing
  // on that slot's mbarrier; NS stages are in flight.  All lanes of the warp call
  // this (teams without nonzeros pass n = 0) because the stage loop is warp-wide.
  //   s_lcw: the warp's coordinate runs (team t at t * (G + 4)); cnt: the warp
  //   tile's nonzeros; nst: stages (ceil(min(G, cnt) / U)); ring/bar_sa: the warp's
  //   ring and barriers.  A barrier that does not complete within a.wait_ns sets
  //   the error word (301) and the warp stops walking: it waits (bounded again) for
  //   the copies it has in flight and returns false (warp-uniform) without a summary.
  template <int U, int NS>
  __device__ __forceinline__ bool walk_tma(int s, int n, int team, int nst, const int32_t* s_lcw, int G, int cnt,
                                           const unsigned char* vt, const int32_t* s_pos,
                                           const int32_t* s_fcrd, int W, int fs, const int32_t* pb,
                                           const int32_t* pn, const unsigned char* ring, uint32_t bar_sa,
                                           Summ<CPT>& X) const {
    constexpr int TW = 32 / LPR;
    constexpr int SR = kTmaRows;
    static_assert(U * TW == SR, "a stage holds U nonzeros of every team");
    const int lane = threadIdx.x & 31;
    const uint32_t ring_sa = (uint32_t)__cvta_generic_to_shared(ring);
    const uint64_t pol = a.gpol == 1 ? policy_evict_normal() : policy_evict_last();
    const int32_t* pos1 = a.pos[1];
    const unsigned char* fw = static_cast<const unsigned char*>(a.fac[ORDER == 3 ? 0 : 1]) + q * LB;
    const bool active = n > 0;
    int x = 0, fend = 0, f1 = 0, kend = 0, ip = 0, rend = 0;
    float crow[CPT];
    uint32_t wc[NWD], wn[NWD];
    float f3[CPT], f2[CPT], ra[CPT];
#pragma unroll
    for (int c = 0; c < CPT; c++) { f3[c] = 0.f; f2[c] = 0.f; ra[c] = 0.f; crow[c] = 0.f; }
#pragma unroll
    for (int k = 0; k < NWD; k++) { wc[k] = 0u; wn[k] = 0u; }
    bool flushed = false;
    if (active) {
      x = (int)search_le(s_pos, 0, W - 1, s);
      fend = s_pos[x + 1];
      if constexpr (ORDER == 3) {
        ip = (int)search_le(pos1, pb[0], pn[0], fs + x);
      } else {
        f1 = (int)search_le(a.pos[2], pb[1], pn[1], fs + x);
        kend = a.pos[2][f1 + 1];
        ip = (int)search_le(pos1, pb[0], pn[0], f1);
        frow(0, a.crd[1][f1], pol, crow);
      }
      rend = pos1[ip + 1];
      piece_load(fw + (size_t)(uint32_t)s_fcrd[x] * FRB, pol, wc);
      if (x + 1 < W) piece_load(fw + (size_t)(uint32_t)s_fcrd[x + 1] * FRB, pol, wn);
    }
    auto fold = [&]() {
      float cw[CPT];
      piece_cvt(wc, cw);
      if constexpr (ORDER == 3) {
#pragma unroll
        for (int c = 0; c < CPT; c++) { ra[c] = fmaf(f3[c], cw[c], ra[c]); f3[c] = 0.f; }
      } else {
#pragma unroll
        for (int c = 0; c < CPT; c++) { f2[c] = fmaf(f3[c], cw[c], f2[c]); f3[c] = 0.f; }
      }
      x++;
      fend = s_pos[x + 1];
#pragma unroll
      for (int k = 0; k < NWD; k++) wc[k] = wn[k];
      if (x + 1 < W) piece_load(fw + (size_t)(uint32_t)s_fcrd[x + 1] * FRB, pol, wn);
      const int fg = fs + x;
      if constexpr (ORDER == 4) {
        while (fg >= kend) {
#pragma unroll
          for (int c = 0; c < CPT; c++) { ra[c] = fmaf(f2[c], crow[c], ra[c]); f2[c] = 0.f; }
          f1++;
          kend = a.pos[2][f1 + 1];
          while (f1 >= rend) { flush(ip, ra, flushed, X); ip++; rend = pos1[ip + 1]; }
          frow(0, a.crd[1][f1], pol, crow);
        }
      } else {
        while (fg >= rend) { flush(ip, ra, flushed, X); ip++; rend = pos1[ip + 1]; }
      }
    };
    // producer: stage k into slot k % NS (lane 0 arms the barrier first)
    auto issue = [&](int k) {
      const int slot = k % NS;
      const uint32_t bar = bar_sa + (uint32_t)slot * 8u;
      if (lane == 0) mbar_arrive_expect_tx(bar, (uint32_t)(SR * FRB));
      __syncwarp();
      if (lane < SR / 4 && !a.tma_withhold) {
        int r[4];
#pragma unroll
        for (int i = 0; i < 4; i++) {
          const int j = 4 * lane + i;
          const int tt = j % TW, u = j / TW;
          const int p = k * U + u;
          const int nt = min(max(cnt - tt * G, 0), G);
          r[i] = p < nt ? s_lcw[tt * (G + 4) + p] : 0;
        }
        tma_gather4(ring_sa + (uint32_t)(slot * SR * FRB + 4 * lane * FRB), &a.tmap, 0, r[0], r[1], r[2], r[3], bar);
      }
    };
    // the team's piece of row slot u of a stage
    auto piece = [&](int slot, int u, uint32_t (&w)[NWD]) {
      const unsigned char* p = ring + (size_t)slot * SR * FRB + (size_t)(u * TW + team) * FRB + q * LB;
      if constexpr (LB >= 16) {
#pragma unroll
        for (int k = 0; k < LB / 16; k++) {
          const uint4 v4 = reinterpret_cast<const uint4*>(p)[k];
          w[4 * k] = v4.x; w[4 * k + 1] = v4.y; w[4 * k + 2] = v4.z; w[4 * k + 3] = v4.w;
        }
      } else if constexpr (LB == 8) {
        const uint2 v2 = *reinterpret_cast<const uint2*>(p);
        w[0] = v2.x; w[1] = v2.y;
      } else if constexpr (LB == 4) {
        w[0] = *reinterpret_cast<const uint32_t*>(p);
      } else {
        w[0] = *reinterpret_cast<const uint16_t*>(p);
      }
    };
    auto consume = [&](int slot, int j) {
      float v[U];
      vals_load<U>(vt + (size_t)j * VB, v);
      if (j + U <= n && s + j + U <= fend) {
#pragma unroll
        for (int u = 0; u < U; u++) {
          uint32_t w[NWD];
          piece(slot, u, w);
          float d[CPT];
          piece_cvt(w, d);
#pragma unroll
          for (int c = 0; c < CPT; c++) f3[c] = fmaf(v[u], d[c], f3[c]);
        }
        return;
      }
#pragma unroll
      for (int u = 0; u < U; u++) {
        if (j + u < n) {
          while (s + j + u >= fend) fold();
          uint32_t w[NWD];
          piece(slot, u, w);
          float d[CPT];
          piece_cvt(w, d);
#pragma unroll
          for (int c = 0; c < CPT; c++) f3[c] = fmaf(v[u], d[c], f3[c]);
        }
      }
    };
    const uint64_t kWaitNs = a.wait_ns ? a.wait_ns : 5000000u;  // a stage normally lands within microseconds
    bool ok = true;
    for (int k = 0; k < NS && k < nst; k++) issue(k);
    int k = 0;
    for (; k < nst && ok; k++) {
      const int slot = k % NS;
      const uint32_t bar = bar_sa + (uint32_t)slot * 8u;
      const uint32_t parity = (uint32_t)((k / NS) & 1);
      const bool landed = mbar_wait_bounded(bar, parity, kWaitNs);
      if (__any_sync(0xffffffffu, !landed)) {
        if (lane == 0) atomicCAS(a.err, 0, 301);
        ok = false;
        break;
      }
      if (active && k * U < n) consume(slot, k * U);
      fence_proxy_async_smem();  // this slot's reads before the TMA refills it
      __syncwarp();
      if (k + NS < nst) issue(k + NS);
    }
    if (!ok) {
      // wait (bounded) for every copy still in flight before the warp leaves
      for (int kk = k; kk < nst && kk < k + NS; kk++)
        mbar_wait_bounded(bar_sa + (uint32_t)(kk % NS) * 8u, (uint32_t)((kk / NS) & 1), kWaitNs);
      return false;
    }
    if (!active) return true;
    {
      float cw[CPT];
      piece_cvt(wc, cw);
      if constexpr (ORDER == 3) {
#pragma unroll
        for (int c = 0; c < CPT; c++) ra[c] = fmaf(f3[c], cw[c], ra[c]);
      } else {
#pragma unroll
        for (int c = 0; c < CPT; c++) { f2[c] = fmaf(f3[c], cw[c], f2[c]); ra[c] = fmaf(f2[c], crow[c], ra[c]); }
      }
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
    return true;
  }

  // Serial walk of nonzeros [s, e) reading only shared memory: values and the
  // gathered nonzero-level factor rows by tile offset, window-fiber factor rows
  // by window offset.  Global reads remain only at row boundaries (and, for
  // order 4, at level-1 fiber boundaries).
  __device__ __forceinline__ void walk_staged(int64_t s, int64_t e, int64_t bstart, const unsigned char* s_val,
                                              const unsigned char* s_rows, const unsigned char* s_wrows,
                                              const int32_t* s_pos, int W, int64_t fs, const int32_t* pb,
                                              const int32_t* pn, Summ<CPT>& X) const {
    constexpr int RB = RP * (FK == kF32 ? 4 : 2);
    const uint64_t polL = policy_evict_last();
    const int32_t* pos1 = a.pos[1];
    int x = (int)search_le(s_pos, 0, W - 1, s);
    int64_t fend = s_pos[x + 1];
    int64_t f1 = 0, kend = 0;
    int ip;
    float crow[CPT];
    if constexpr (ORDER == 3) {
      ip = (int)search_le(pos1, pb[0], pn[0], fs + x);
    } else {
      f1 = search_le(a.pos[2], pb[1], pn[1], fs + x);
      kend = a.pos[2][f1 + 1];
      ip = (int)search_le(pos1, pb[0], pn[0], f1);
      frow(0, a.crd[1][f1], polL, crow);
    }
    int64_t rend = pos1[ip + 1];
    float f3[CPT], f2[CPT], ra[CPT];
#pragma unroll
    for (int c = 0; c < CPT; c++) { f3[c] = 0.f; f2[c] = 0.f; ra[c] = 0.f; }
    bool flushed = false;
#pragma unroll 4
    for (int64_t p = s; p < e; p++) {
      while (p >= fend) {
        float cur[CPT];
        smem_row<FK, CPT>(s_wrows + (size_t)x * RB, q, cur);
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
      }
      const int i = (int)(p - bstart);
      float v;
      if constexpr (VK == kF32) v = reinterpret_cast<const float*>(s_val)[i];
      else v = VK == kB16 ? bf16lo(reinterpret_cast<const uint16_t*>(s_val)[i]) : h16lo(reinterpret_cast<const uint16_t*>(s_val)[i]);
      float g[CPT];
      smem_row<FK, CPT>(s_rows + (size_t)i * RB, q, g);
#pragma unroll
      for (int c = 0; c < CPT; c++) f3[c] = fmaf(v, g[c], f3[c]);
    }
    {
      float cur[CPT];
      smem_row<FK, CPT>(s_wrows + (size_t)x * RB, q, cur);
      if constexpr (ORDER == 3) {
#pragma unroll
        for (int c = 0; c < CPT; c++) ra[c] = fmaf(f3[c], cur[c], ra[c]);
      } else {
#pragma unroll
        for (int c = 0; c < CPT; c++) { f2[c] = fmaf(f3[c], cur[c], f2[c]); ra[c] = fmaf(f2[c], crow[c], ra[c]); }
      }
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
// Merge the teams' summaries of one block (warp shuffle tree, then the first
// team over the warps), then settle the block's first and last rows: a row that
// starts and ends inside the block is stored; a row shared with a neighbouring
// block is written to the block's carry slot (0: first row, 1: last row) for
// the segment fold.  No fence, atomic or second barrier: the block ends here.
//   head_ff  first window-level fiber of the block's first row (loaded at start)
//   meta[b]  {first row, last row, flags}: bit0 first row started before the
//            block, bit1 last row continues after it, bit2 single-row block
// Warp-level merge of the team summaries (tree over teams, keyed by row); the
// result is left in the first team's lanes.
template <int ORDER, int PREC, int CPT, int LPR>
__device__ __forceinline__ void warp_tree(const Walk<ORDER, PREC, CPT, LPR>& wk, Summ<CPT>& X) {
  constexpr int TW = 32 / LPR;
  const int tw = (threadIdx.x & 31) / LPR;
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
}

// Settle the first and last rows of work unit b (a block, or a warp's tile in
// the lean kernel) from its merged summary X; run by the LPR lanes holding X.
// A row that starts and ends inside the unit is stored; a row shared with a
// neighbouring unit is written to the unit's carry slot (0: first row, 1: last
// row) for the segment fold (seg_fold_kernel / seg_chain_kernel).
//   head_ff  first window-level fiber of the unit's first row
//   meta[b]  {first row, last row, flags}: bit0 first row started before the
//            unit, bit1 last row continues after it, bit2 single-row unit
template <int ORDER, int PREC, int CPT, int LPR>
__device__ __forceinline__ void settle_unit(const WalkArgs& a, const Walk<ORDER, PREC, CPT, LPR>& wk,
                                            const Summ<CPT>& X, int64_t head_ff, int64_t fs, int64_t win0,
                                            int64_t bstart, int next_row, int b, int q) {
  constexpr int RP = CPT * LPR;
  const bool single = X.t == kNone;
  const int last = single ? X.h : X.t;
  const bool h_before = head_ff < fs || (head_ff == fs && win0 < bstart);
  const bool l_after = b + 1 < a.nblocks && next_row == last;
  float* c0 = a.carry + ((size_t)(2 * b)) * RP + q * CPT;
  float* c1 = c0 + RP;
  if (single) {
    if (h_before || l_after) {
#pragma unroll
      for (int c = 0; c < CPT; c++) c0[c] = X.ha[c] * wk.sc(c);
    } else {
      wk.store_row(X.h, X.ha);
    }
  } else {
    if (h_before) {
#pragma unroll
      for (int c = 0; c < CPT; c++) c0[c] = X.ha[c] * wk.sc(c);
    } else {
      wk.store_row(X.h, X.ha);
    }
    if (l_after) {
#pragma unroll
      for (int c = 0; c < CPT; c++) c1[c] = X.ta[c] * wk.sc(c);
    } else {
      wk.store_row(X.t, X.ta);
    }
  }
  if (q == 0)
    reinterpret_cast<int4*>(a.meta)[b] =
        make_int4(X.h, last, (h_before ? 1 : 0) | (l_after ? 2 : 0) | (single ? 4 : 0), 0);
}

// Merge the teams' summaries of one block (warp trees, then the first team over
// the warps) and settle the block's rows.  No fence, atomic or second barrier:
// the block ends here.
template <int ORDER, int PREC, int CPT, int LPR>
__device__ __forceinline__ void block_merge(const WalkArgs& a, const Walk<ORDER, PREC, CPT, LPR>& wk,
                                            Summ<CPT>& X, int32_t* s_wh, int32_t* s_wt, float* s_wha,
                                            float* s_wta, int64_t head_ff, int64_t fs, int64_t win0,
                                            int64_t bstart, int next_row, int b) {
  constexpr int RP = CPT * LPR;
  constexpr int TW = 32 / LPR;
  const int tb = blockDim.x, nw = tb / 32;
  const int team = threadIdx.x / LPR, q = threadIdx.x % LPR, tw = team % TW, warp = threadIdx.x / 32;
  warp_tree(wk, X);
  if (tw == 0) {
    if (q == 0) { s_wh[warp] = X.h; s_wt[warp] = X.t; }
#pragma unroll
    for (int c = 0; c < CPT; c++) {
      s_wha[warp * RP + q * CPT + c] = X.ha[c];
      s_wta[warp * RP + q * CPT + c] = X.ta[c];
    }
  }
  __syncthreads();
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
    settle_unit(a, wk, X, head_ff, fs, win0, bstart, next_row, b, q);
  }
}

// First window-level fiber of root position r (level 1 for order 3, level 2 for order 4).
template <int ORDER>
__device__ __forceinline__ int64_t row_first_window_fiber(const WalkArgs& a, int r) {
  int64_t f = a.pos[1][r];
  if constexpr (ORDER == 4) f = a.pos[2][f];
  return f;
}

#ifndef TT_ARGS_ONLY
// ---------------------------------------------------------------------------
// Cross-unit rows.  Each work unit left at most two carry entries (settle_unit):
// a partial of its first row (it started in an earlier unit) and/or of its last
// row (it continues in a later unit).  In unit order the entries of one row are
// consecutive, so every shared row is a run of entries.  The runs are summed in
// two levels, each in a fixed order (bitwise reproducible):
//   seg_fold_kernel   one warp per segment of kSeg units, lanes over columns:
//                     sums each run inside the segment (FP32 with Kahan
//                     compensation; at most 2*kSeg terms); a run that starts and
//                     ends in the segment is final and written to the output,
//                     the segment's first/last run, if it crosses the segment's
//                     edge, goes to the segment's FP64 carry slot (same meta
//                     layout as the units', one level up);
//   seg_chain_kernel  one warp per segment where a crossing row starts: sums the
//                     row's segment partials (lane = column for short chains,
//                     lane = segment stripe plus a fixed butterfly for long ones).
// ---------------------------------------------------------------------------
// Final value of output row r, column j (slab passes add into the row).
__device__ __forceinline__ void put_row_value(const WalkArgs& a, int r, int j, double v) {
  const int64_t row = a.crd[0] ? (int64_t)a.crd[0][r] : (int64_t)r;
  float* o = a.out + row * a.ldo + j;
  *o = (float)(a.accum ? v + (double)*o : v);
}
// The same for a Kahan pair (s, c) with |c| <= ulp(s): without slab accumulation
// the FP32 sum s + c rounds the exact value once, which is what the FP64 route
// gives (the FP64 sum of the pair is exact), and it keeps the FP64 pipe free.
__device__ __forceinline__ void put_row_pair(const WalkArgs& a, int r, int j, float s, float c) {
  if (a.accum) {
    put_row_value(a, r, j, (double)s + (double)c);
    return;
  }
  const int64_t row = a.crd[0] ? (int64_t)a.crd[0][r] : (int64_t)r;
  a.out[row * a.ldo + j] = __fadd_rn(s, c);
}

template <int ORDER>  // (the fold itself does not depend on the order)
__global__ void __launch_bounds__(256, 2) seg_fold_kernel(const __grid_constant__ WalkArgs a) {
  grid_dependency_wait();  // the walk's carries and metadata
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int sg = blockIdx.x * (blockDim.x >> 5) + warp;
  if (sg >= num_segments(a.nblocks)) return;
  // a walk that gave up (error word set) left some units' entries unwritten
  if (a.err && *reinterpret_cast<volatile const int32_t*>(a.err) != 0) return;
  const int u0 = sg * kSeg, n = min(kSeg, a.nblocks - u0);
  const int rp = a.rp;
  int4 mine = make_int4(-1, -1, 0, 0);
  if (lane < n) mine = reinterpret_cast<const int4*>(a.meta)[u0 + lane];
  double* sc0 = a.segcarry + (size_t)(2 * sg) * rp;
  double* sc1 = sc0 + rp;
  int sfirst = -1, slast = -1, sflags = 0, nruns = 0;
  // one column (TTV): every lane loads its own unit's two carries at once, and the
  // fold takes them by shuffle (no load waits inside the fold)
  const bool one_col = rp == 1;
  float lane_c0 = 0.f, lane_c1 = 0.f;
  if (one_col && lane < n) {
    lane_c0 = a.carry[(size_t)(2 * (u0 + lane))];
    lane_c1 = a.carry[(size_t)(2 * (u0 + lane)) + 1];
  }
  // one pass per 32 columns (lane = column); the run structure is the same in every pass
  for (int c0 = 0; c0 < rp; c0 += 32) {
    const int col = c0 + lane;
    const bool live = col < rp;
    int cur = -1;
    bool cur_before = false, cur_after = false, first_run = true;
    // the run's sum in FP32 with Kahan compensation (a run has at most 64 terms);
    // what leaves the segment is kept in FP64
    float acc = 0.f, comp = 0.f;
    int runs = 0;
    auto close_run = [&]() {
      runs++;
      if (!cur_before && !cur_after) {
        if (col < a.R) put_row_pair(a, cur, col, acc, comp);
      } else if (cur_before) {  // necessarily the segment's first run
        if (c0 == 0) { sfirst = cur; sflags |= 1; if (cur_after) { slast = cur; sflags |= 2; } }
        if (live) sc0[col] = (double)acc + (double)comp;
      } else {  // cur_after only: the segment's last run (slot 0 when it is the only run)
        if (c0 == 0) { slast = cur; sflags |= 2; }
        if (live) (first_run ? sc0 : sc1)[col] = (double)acc + (double)comp;
      }
      if (c0 == 0 && first_run && sfirst < 0) sfirst = cur;
      first_run = false;
    };
    auto entry = [&](int r, float v, bool before, bool after) {
      if (r != cur) {
        if (cur >= 0) close_run();
        cur = r;
        cur_before = before;
        acc = 0.f;
        comp = 0.f;
      }
      // Kahan (1965): y = v - c; t = s + y; c = (t - s) - y; s = t  (comp holds -c)
      const float y = v + comp;
      const float t = acc + y;
      comp = y - (t - acc);
      acc = t;
      cur_after = after;
    };
    // units in groups of kG, the loop kept rolled (a small body stays in the
    // instruction cache); the next group's carries are loaded before the current
    // group is folded
    constexpr int kG = 4;
    auto load_group = [&](int g, float (&w0)[kG], float (&w1)[kG]) {
#pragma unroll
      for (int k = 0; k < kG; k++) {
        const int uu = g * kG + k;
        w0[k] = 0.f;
        w1[k] = 0.f;
        if (one_col) {  // warp-uniform
          const float x0 = __shfl_sync(0xffffffffu, lane_c0, uu & 31);
          const float x1 = __shfl_sync(0xffffffffu, lane_c1, uu & 31);
          if (uu < n && live) { w0[k] = x0; w1[k] = x1; }
        } else if (uu < n && live) {
          const float* c = a.carry + (size_t)(2 * (u0 + uu)) * rp + col;
          w0[k] = c[0];
          w1[k] = c[rp];
        }
      }
    };
    float c0v[kG], c1v[kG];
    load_group(0, c0v, c1v);
#pragma unroll 1
    for (int g = 0; g * kG < n; g++) {
      float n0[kG], n1[kG];
      load_group(g + 1, n0, n1);
#pragma unroll
      for (int k = 0; k < kG; k++) {
        const int uu = g * kG + k;
        if (uu < n) {  // warp-uniform
          const int mx = __shfl_sync(0xffffffffu, mine.x, uu);
          const int my = __shfl_sync(0xffffffffu, mine.y, uu);
          const int mz = __shfl_sync(0xffffffffu, mine.z, uu);
          const bool hb = mz & 1, la = mz & 2, single = mz & 4;
          // slot 0: the unit's first row (a single-row unit's only entry); slot 1:
          // its last row when that differs
          if (single ? (hb || la) : hb) entry(mx, c0v[k], hb, single && la);
          if (!single && la) entry(my, c1v[k], false, true);
        }
      }
#pragma unroll
      for (int k = 0; k < kG; k++) { c0v[k] = n0[k]; c1v[k] = n1[k]; }
    }
    if (cur >= 0) close_run();
    if (c0 == 0) {
      nruns = runs;
      if (slast < 0) slast = cur;
    }
  }
  if (lane == 0) {
    // bit2: one run in the segment (its partial, if any, is in slot 0)
    reinterpret_cast<int4*>(a.segmeta)[sg] = make_int4(sfirst, slast, sflags | (nruns == 1 ? 4 : 0), 0);
  }
}

template <int ORDER>
__global__ void __launch_bounds__(256) seg_chain_kernel(const __grid_constant__ WalkArgs a) {
  grid_dependency_wait();  // the fold's segment partials
  constexpr int kShort = 16;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int sg = blockIdx.x * (blockDim.x >> 5) + warp;
  if (sg >= num_segments(a.nblocks)) return;
  if (a.err && *reinterpret_cast<volatile const int32_t*>(a.err) != 0) return;  // (as seg_fold_kernel)
  const int4 m = reinterpret_cast<const int4*>(a.segmeta)[sg];
  const bool before = m.z & 1, after = m.z & 2, single = m.z & 4;
  if (!after || (single && before)) return;  // warp-uniform: no crossing row starts here
  const int r = m.y;
  // end of row r: through rnz for the flat and strip walks (whose rows may be a
  // slab plan's virtual rows, with no pos arrays), else through the pos levels;
  // ORDER 2: the "rows" are TTV fibers (pos[1] = fiber starts)
  int64_t n1;
  if (a.rnz) {
    n1 = a.rnz[r + 1];
  } else {
    int64_t f1 = ORDER == 2 ? (int64_t)r + 1 : (int64_t)a.pos[1][r + 1];
    for (int l = 2; l < ORDER - 1; l++) f1 = a.pos[l][f1];
    n1 = a.pos[ORDER - 1][f1];
  }
  const int s1 = (int)((n1 - 1) / a.P) / kSeg;  // segment holding the row's last nonzero
  const int rp = a.rp;
  const int slot0 = single ? 0 : 1;  // this segment's slot; later segments hold the row in slot 0
  auto src = [&](int sgi) { return a.segcarry + (size_t)(2 * sgi + (sgi == sg ? slot0 : 0)) * rp; };
  if (s1 - sg < kShort) {
    for (int j = lane; j < rp; j += 32) {
      double acc = 0.0;
      for (int t = sg; t <= s1; t++) acc += src(t)[j];
      if (j < a.R) put_row_value(a, r, j, acc);
    }
    return;
  }
  for (int c0 = 0; c0 < rp; c0 += 32) {  // at most 32 columns per pass
    const int nc = rp - c0 < 32 ? rp - c0 : 32;
    double acc[32];
#pragma unroll
    for (int c = 0; c < 32; c++) acc[c] = 0.0;
    for (int t = sg + lane; t <= s1; t += 32) {
      const double* v = src(t) + c0;
#pragma unroll
      for (int c = 0; c < 32; c++)
        if (c < nc) acc[c] += v[c];
    }
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) {
#pragma unroll
      for (int c = 0; c < 32; c++) acc[c] += __shfl_xor_sync(0xffffffffu, acc[c], d);
    }
    // every lane holds the same totals; lane c writes column c0 + c
#pragma unroll
    for (int c = 0; c < 32; c++)
      if (lane == c && c < nc && c0 + c < a.R) put_row_value(a, r, c0 + c, acc[c]);
  }
}

#endif  // TT_ARGS_ONLY

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
  const int TE = P;
  int32_t* s_lc = reinterpret_cast<int32_t*>(smem);
  unsigned char* s_val = smem + (size_t)TE * 4;
  int32_t* s_pos = reinterpret_cast<int32_t*>(smem + walk_tile_bytes(TE, VB));
  int32_t* s_fcrd = s_pos + (P + 2);
  int32_t* s_wh = s_fcrd + (P + 2);
  int32_t* s_wt = s_wh + nw;
  float* s_wha = reinterpret_cast<float*>(s_wt + nw);
  float* s_wta = s_wha + nw * RP;

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
    auto dst4 = [&](int i) { return i; };
    for (int i = threadIdx.x; i < n4; i += tb)
      reinterpret_cast<int4*>(s_lc)[dst4(i)] = ld_stream_i4(gl + 4 * i, polF);
    if constexpr (VB == 4) {
      const float* gv = static_cast<const float*>(a.vals) + bstart;
      for (int i = threadIdx.x; i < n4; i += tb)
        reinterpret_cast<float4*>(s_val)[dst4(i)] = ld_stream_f4(gv + 4 * i, polF);
    } else {
      const uint16_t* gv = static_cast<const uint16_t*>(a.vals) + bstart;
      for (int i = threadIdx.x; i < n4; i += tb)
        reinterpret_cast<uint2*>(s_val)[dst4(i)] = ld_stream_u2(gv + 4 * i, polF);
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

  // the first team settles the block's rows at the end; its loads start now
  const int64_t head_ff = threadIdx.x < LPR ? row_first_window_fiber<ORDER>(a, pb[0]) : 0;
  Summ<CPT> X;
  X.h = kEmpty;
  X.t = kNone;
  const int64_t s = bstart + (int64_t)team * a.G;
  if (s < bend) {
    wk.walk(s, min(s + (int64_t)a.G, bend), bstart, s_lc, s_val, s_pos, s_fcrd, W, fs, pb, pn, X);
  }

  block_merge<ORDER, PREC, CPT, LPR>(a, wk, X, s_wh, s_wt, s_wha, s_wta, head_ff, fs, s_pos[0], bstart, pn[0], blockIdx.x);
}

// Warp staging of a tile's coordinate and value streams into per-run shared
// memory: 16-byte chunk c (entries 4c..4c+3) goes to run c >> lg_cpr, each run
// followed by 16 bytes of padding (bank skew).  All loads of a round (up to
// four chunks per lane) are issued before any store, so a lane has several
// DRAM round trips in flight instead of one.  The streams are padded, so the
// rounded-up last chunk stays in bounds.
template <int VB>
__device__ __forceinline__ void stage_runs(const int32_t* gl, const void* vals, int64_t base, int n4, int lg_cpr,
                                           int lane, int32_t* s_lc, unsigned char* s_val, uint64_t pol) {
  constexpr int R = 4;
  for (int c0 = lane; c0 < n4; c0 += 32 * R) {
    int4 li[R];
    float4 vf[R];
    uint2 vh[R];
#pragma unroll
    for (int r = 0; r < R; r++) {
      const int c = c0 + 32 * r;
      if (c < n4) {
        li[r] = ld_stream_i4(gl + 4 * c, pol);
        if constexpr (VB == 4)
          vf[r] = ld_stream_f4(static_cast<const float*>(vals) + base + 4 * c, pol);
        else
          vh[r] = ld_stream_u2(static_cast<const uint16_t*>(vals) + base + 4 * c, pol);
      }
    }
#pragma unroll
    for (int r = 0; r < R; r++) {
      const int c = c0 + 32 * r;
      if (c < n4) {
        const int t = c >> lg_cpr;
        reinterpret_cast<int4*>(s_lc)[c + t] = li[r];
        if constexpr (VB == 4)
          reinterpret_cast<float4*>(s_val)[c + t] = vf[r];
        else
          reinterpret_cast<uint2*>(s_val)[c + 2 * t] = vh[r];
      }
    }
  }
}

// A tile's int32 stream alone into per-run shared memory (the layout of
// stage_runs' coordinate runs).
__device__ __forceinline__ void stage_int_runs(const int32_t* g, int n4, int lg_cpr, int lane, int32_t* sdst,
                                               uint64_t pol) {
  constexpr int R = 4;
  for (int c0 = lane; c0 < n4; c0 += 32 * R) {
    int4 li[R];
#pragma unroll
    for (int r = 0; r < R; r++) {
      const int c = c0 + 32 * r;
      if (c < n4) li[r] = ld_stream_i4(g + 4 * c, pol);
    }
#pragma unroll
    for (int r = 0; r < R; r++) {
      const int c = c0 + 32 * r;
      if (c < n4) reinterpret_cast<int4*>(sdst)[c + (c >> lg_cpr)] = li[r];
    }
  }
}

// A tile's fiber window: W + 1 fiber starts and W fiber coordinates, all loads
// of a round issued before its stores.
__device__ __forceinline__ void stage_window(const int32_t* gpos, const int32_t* gcrd, int W, int lane,
                                             int32_t* s_pos, int32_t* s_fcrd) {
  constexpr int R = 2;
  for (int x0 = lane; x0 <= W; x0 += 32 * R) {
    int p[R], c[R];
#pragma unroll
    for (int r = 0; r < R; r++) {
      const int x = x0 + 32 * r;
      if (x <= W) p[r] = gpos[x];
      if (x < W) c[r] = gcrd[x];
    }
#pragma unroll
    for (int r = 0; r < R; r++) {
      const int x = x0 + 32 * r;
      if (x <= W) s_pos[x] = p[r];
      if (x < W) s_fcrd[x] = c[r];
    }
  }
}

// n consecutive int32 from global into shared memory, four loads per lane in
// flight per round.
__device__ __forceinline__ void stage_ints(const int32_t* g, int n, int lane, int32_t* sdst) {
  constexpr int R = 4;
  for (int x0 = lane; x0 < n; x0 += 32 * R) {
    int v[R];
#pragma unroll
    for (int r = 0; r < R; r++) {
      const int x = x0 + 32 * r;
      if (x < n) v[r] = g[x];
    }
#pragma unroll
    for (int r = 0; r < R; r++) {
      const int x = x0 + 32 * r;
      if (x < n) sdst[x] = v[r];
    }
  }
}

// Lean kernel (family 0): every warp owns a tile of TW*G consecutive nonzeros
// (TW = 32/LPR teams of G), which is the unit of the partition, of the carry
// slots and of chain_fixup_kernel.  A warp stages its own tile and window with
// 128-bit loads, walks it (walk_lean) and settles its rows: no block barrier,
// so a warp waiting on its gathers never holds up another.
// MINB: resident 256-thread blocks per SM the register budget is cut for
// (2: up to 128 registers a thread, 3: 80, 4: 64).
template <int ORDER, int PREC, int CPT, int LPR, int MINB = 2, bool EXACT = false>
__global__ void __launch_bounds__(256, MINB) mttkrp_lean_kernel(const __grid_constant__ WalkArgs a) {
  using WK = Walk<ORDER, PREC, CPT, LPR>;
  constexpr int VB = WK::VB;
  constexpr int TW = 32 / LPR;
  constexpr int U = WK::LB >= 16 ? 4 : 8;  // nonzeros per gather batch (two batches in registers)
  static_assert(!EXACT || VB == 4, "exact-length staging is built for FP32 values");
  extern __shared__ __align__(16) unsigned char smem[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int u = blockIdx.x * (blockDim.x >> 5) + warp;
  if (u >= a.nblocks) return;  // whole warp: nothing below synchronises the block
  const int G = a.G, PU = a.P;
  unsigned char* ws = smem + (size_t)warp * lean_warp_bytes(G, TW, VB);
  int32_t* s_lc = reinterpret_cast<int32_t*>(ws);
  unsigned char* s_val = ws + (size_t)TW * (G + 4) * 4;
  int32_t* s_pos = reinterpret_cast<int32_t*>(s_val + (size_t)TW * (G * VB + 16));
  int32_t* s_fcrd = s_pos + (PU + 2);

  const int32_t* pb = a.part + (size_t)u * (ORDER - 1);
  const int32_t* pn = pb + (ORDER - 1);
  const int64_t ustart64 = (int64_t)u * PU;
  const int ustart = (int)ustart64;
  const int cnt = (int)min((int64_t)PU, a.nnz - ustart64);
  const int fs = pb[ORDER - 2];
  const int W = pn[ORDER - 2] - fs + 1;
  {
    // chunk c (entries 4c..4c+3) belongs to team 4c >> lgG; each team's runs of
    // coordinates and values are followed by 16 bytes of padding (bank skew)
    const uint64_t polF = policy_evict_first();
    const int n4 = (cnt + 3) >> 2;
    const int32_t* gl = a.crd[ORDER - 1] + ustart64;
    if constexpr (!EXACT) stage_runs<VB>(gl, a.vals, ustart64, n4, a.lgG - 2, lane, s_lc, s_val, polF);
    for (int c = lane; EXACT && c < n4; c += 32) {
      const int t = (4 * c) >> a.lgG;
      if (4 * c + 4 <= cnt) {
        reinterpret_cast<int4*>(s_lc)[c + t] = ld_stream_i4(gl + 4 * c, polF);
        if constexpr (VB == 4)
          reinterpret_cast<float4*>(s_val)[c + t] = ld_stream_f4(static_cast<const float*>(a.vals) + ustart64 + 4 * c, polF);
        else
          reinterpret_cast<uint2*>(s_val)[c + 2 * t] = ld_stream_u2(static_cast<const uint16_t*>(a.vals) + ustart64 + 4 * c, polF);
      } else {
        for (int k = 0; k < 4; k++) {
          const bool in = 4 * c + k < cnt;
          s_lc[4 * (c + t) + k] = in ? gl[4 * c + k] : 0;
          reinterpret_cast<float*>(s_val)[4 * (c + t) + k] = in ? static_cast<const float*>(a.vals)[ustart64 + 4 * c + k] : 0.f;
        }
      }
    }
    stage_window(a.pos[ORDER - 1] + fs, a.crd[ORDER - 2] + fs, W, lane, s_pos, s_fcrd);
  }
  __syncwarp();

  const int team = lane / LPR, q = lane % LPR;
  WK wk(a, q);
  const int64_t head_ff = lane < LPR ? row_first_window_fiber<ORDER>(a, pb[0]) : 0;
  Summ<CPT> X;
  X.h = kEmpty;
  X.t = kNone;
  const int s = ustart + team * G;
  if (s < ustart + cnt)
    wk.template walk_lean<U>(s, min(G, ustart + cnt - s), s_lc + team * (G + 4), s_val + (size_t)team * (G * VB + 16),
                             s_pos, s_fcrd, W, fs, pb, pn, X);
  warp_tree(wk, X);
  if (lane < LPR) settle_unit(a, wk, X, head_ff, fs, s_pos[0], ustart64, pn[0], u, q);
}

// Flat kernel (family 3): the lean kernel's warp tiles and merge, with the upper
// coordinates of every nonzero staged beside its leaf coordinate and value; teams
// run walk_flat (row ends only).
template <int ORDER, int PREC, int CPT, int LPR, int MINB>
__global__ void __launch_bounds__(256, MINB) mttkrp_flat_kernel(const __grid_constant__ WalkArgs a) {
  using WK = Walk<ORDER, PREC, CPT, LPR>;
  constexpr int VB = WK::VB;
  constexpr int TW = 32 / LPR;
  // nonzeros per gather batch (two batches of ORDER - 1 rows each in registers):
  // 16-byte pieces under the tighter register budget take pairs
  constexpr int U = WK::LB >= 16 && MINB >= 3 ? 2 : WK::LB >= 8 ? 4 : 8;
  extern __shared__ __align__(16) unsigned char smem[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int u = blockIdx.x * (blockDim.x >> 5) + warp;
  if (u >= a.nblocks) return;  // whole warp
  const int G = a.G, PU = a.P;
  unsigned char* ws = smem + (size_t)warp * flat_warp_bytes(G, TW, VB, ORDER);
  int32_t* s_lc = reinterpret_cast<int32_t*>(ws);
  int32_t* s_kc = s_lc + TW * (G + 4);
  int32_t* s_k2c = s_kc + TW * (G + 4);  // four modes only
  unsigned char* s_val = reinterpret_cast<unsigned char*>(s_lc + (ORDER - 1) * TW * (G + 4));
  const int32_t* pb = a.part + (size_t)u * (ORDER - 1);
  const int32_t* pn = pb + (ORDER - 1);
  const int64_t ustart64 = (int64_t)u * PU;
  const int ustart = (int)ustart64;
  const int cnt = (int)min((int64_t)PU, a.nnz - ustart64);
  {
    const uint64_t polF = policy_evict_first();
    const int n4 = (cnt + 3) >> 2;
    stage_runs<VB>(a.crd[ORDER - 1] + ustart64, a.vals, ustart64, n4, a.lgG - 2, lane, s_lc, s_val, polF);
    stage_int_runs(a.kexp + ustart64, n4, a.lgG - 2, lane, s_kc, polF);
    if constexpr (ORDER == 4) stage_int_runs(a.kexp2 + ustart64, n4, a.lgG - 2, lane, s_k2c, polF);
  }
  __syncwarp();
  const int team = lane / LPR, q = lane % LPR;
  WK wk(a, q);
  Summ<CPT> X;
  X.h = kEmpty;
  X.t = kNone;
  const int s = ustart + team * G;
  if (s < ustart + cnt)
    wk.template walk_flat<U>(s, min(G, ustart + cnt - s), s_lc + team * (G + 4), s_kc + team * (G + 4),
                             s_k2c + team * (G + 4), s_val + (size_t)team * (G * VB + 16), pb[0], pn[0], X);
  warp_tree(wk, X);
  // the unit's first row started before it when its first nonzero lies earlier
  if (lane < LPR) settle_unit(a, wk, X, 0, 0, a.rnz[pb[0]], ustart64, pn[0], u, q);
}

// TMA kernel (family 2): the lean kernel's warp tiles, with the nonzero-level
// factor rows fetched by TMA tile::gather4 into a per-warp ring (walk_tma).
// NS: stages in flight per warp.
template <int ORDER, int PREC, int CPT, int LPR, int NS>
__global__ void __launch_bounds__(256, 1) mttkrp_tma_kernel(const __grid_constant__ WalkArgs a) {
  using WK = Walk<ORDER, PREC, CPT, LPR>;
  constexpr int VB = WK::VB;
  constexpr int TW = 32 / LPR;
  constexpr int U = kTmaRows / TW;
  extern __shared__ __align__(128) unsigned char smem[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int u = blockIdx.x * (blockDim.x >> 5) + warp;
  if (u >= a.nblocks) return;  // whole warp
  // after a recorded device error, later warps skip their tiles (the call fails)
  if (*reinterpret_cast<volatile const int32_t*>(a.err) != 0) return;
  const int G = a.G, PU = a.P;
  unsigned char* ws = smem + (size_t)warp * tma_warp_bytes(G, TW, VB, WK::FRB, NS);
  unsigned char* ring = ws;
  const uint32_t bar_sa = (uint32_t)__cvta_generic_to_shared(ws + (size_t)NS * kTmaRows * WK::FRB);
  unsigned char* lw = ws + ((((size_t)NS * kTmaRows * WK::FRB + (size_t)NS * 8) + 15) & ~(size_t)15);
  int32_t* s_lc = reinterpret_cast<int32_t*>(lw);
  unsigned char* s_val = lw + (size_t)TW * (G + 4) * 4;
  int32_t* s_pos = reinterpret_cast<int32_t*>(s_val + (size_t)TW * (G * VB + 16));
  int32_t* s_fcrd = s_pos + (PU + 2);

  const int32_t* pb = a.part + (size_t)u * (ORDER - 1);
  const int32_t* pn = pb + (ORDER - 1);
  const int64_t ustart64 = (int64_t)u * PU;
  const int ustart = (int)ustart64;
  const int cnt = (int)min((int64_t)PU, a.nnz - ustart64);
  const int fs = pb[ORDER - 2];
  const int W = pn[ORDER - 2] - fs + 1;
  if (lane == 0) {
    for (int k = 0; k < NS; k++) mbar_init(bar_sa + 8u * k, 1);
    fence_mbar_init();
  }
  {
    const uint64_t polF = policy_evict_first();
    const int n4 = (cnt + 3) >> 2;
    const int32_t* gl = a.crd[ORDER - 1] + ustart64;
    stage_runs<VB>(gl, a.vals, ustart64, n4, a.lgG - 2, lane, s_lc, s_val, polF);
    stage_window(a.pos[ORDER - 1] + fs, a.crd[ORDER - 2] + fs, W, lane, s_pos, s_fcrd);
  }
  __syncwarp();

  const int team = lane / LPR, q = lane % LPR;
  WK wk(a, q);
  const int64_t head_ff = lane < LPR ? row_first_window_fiber<ORDER>(a, pb[0]) : 0;
  Summ<CPT> X;
  X.h = kEmpty;
  X.t = kNone;
  const int s = ustart + team * G;
  const int n = s < ustart + cnt ? min(G, ustart + cnt - s) : 0;
  const int nst = (min(G, cnt) + U - 1) / U;
  // a wait that ran out (error word 301): no summary, the unit's merge entries are
  // left unwritten (the merge kernels skip once the error word is set)
  if (!wk.template walk_tma<U, NS>(s, n, team, nst, s_lc, G, cnt, s_val + (size_t)team * (G * VB + 16), s_pos,
                                   s_fcrd, W, fs, pb, pn, ring, bar_sa, X))
    return;
  warp_tree(wk, X);
  if (lane < LPR) settle_unit(a, wk, X, head_ff, fs, s_pos[0], ustart64, pn[0], u, q);
}

// Staged kernel: every factor row the block needs is gathered into shared memory
// with cp.async before the walk (one row per nonzero of the tile and one per
// window fiber), so thousands of row gathers per SM are in flight at once and the
// walk itself reads only shared memory.  Layout of the dynamic shared memory:
//   [crd tile P][vals tile P][rows P x RB][window rows wcap x RB][window bounds]
//   [window coords][warp summaries][FP64 merge partials][control]
template <int ORDER, int PREC, int CPT, int LPR, bool EXACT = false>
__global__ void __launch_bounds__(512) mttkrp_stage_kernel(const __grid_constant__ WalkArgs a) {
  using WK = Walk<ORDER, PREC, CPT, LPR>;
  constexpr int RP = WK::RP;
  constexpr int VB = WK::VB;
  constexpr int FB = WK::FK == kF32 ? 4 : 2;
  constexpr int RB = RP * FB;    // bytes per factor row
  constexpr int CPR = RB / 16;   // 16-byte copies per row
  static_assert(RB % 16 == 0, "factor rows must be whole 16-byte chunks");
  static_assert(!EXACT || VB == 4, "exact-length staging is built for FP32 values");
  extern __shared__ __align__(16) unsigned char smem[];

  const int tb = blockDim.x, nw = tb / 32, b = blockIdx.x, P = a.P, wcap = a.wcap;
  int32_t* s_lc = reinterpret_cast<int32_t*>(smem);
  unsigned char* s_val = smem + (size_t)P * 4;
  unsigned char* s_rows = smem + stage_off_rows(P, VB);
  unsigned char* s_wrows = s_rows + (size_t)P * RB;
  int32_t* s_pos = reinterpret_cast<int32_t*>(s_wrows + (size_t)wcap * RB);
  int32_t* s_fcrd = s_pos + (wcap + 2);
  int32_t* s_wh = s_fcrd + (wcap + 2);
  int32_t* s_wt = s_wh + nw;
  float* s_wha = reinterpret_cast<float*>(s_wt + nw);
  float* s_wta = s_wha + nw * RP;

  const int32_t* pb = a.part + (size_t)b * (ORDER - 1);
  const int32_t* pn = pb + (ORDER - 1);
  const int64_t bstart = (int64_t)b * P;
  const int64_t bend = min(bstart + (int64_t)P, a.nnz);
  const int nt = (int)(bend - bstart);
  const int64_t fs = pb[ORDER - 2];
  const int W = (int)(pn[ORDER - 2] - fs + 1);
  if (W > wcap) {  // the plan sized wcap from this partition; never expected
    if (threadIdx.x == 0) atomicExch(a.err, 1);
    return;
  }
  const uint64_t polF = policy_evict_first();
  const uint64_t polL = policy_evict_last();
  const int64_t head_ff = threadIdx.x < LPR ? row_first_window_fiber<ORDER>(a, pb[0]) : 0;

  // 1. tile of coordinates and values (async), window bounds and coordinates
  {
    const int n4 = (nt + 3) >> 2;
    const int32_t* gl = a.crd[ORDER - 1] + bstart;
    const unsigned char* gv = static_cast<const unsigned char*>(a.vals) + (size_t)bstart * VB;
    for (int i = threadIdx.x; i < n4; i += tb) {
      if (!EXACT || 4 * i + 4 <= nt) cp_async16(s_lc + 4 * i, gl + 4 * i, polF);
      else cp_async16_part(s_lc + 4 * i, gl + 4 * i, 4 * (nt - 4 * i));
    }
    const int nvb = (nt * VB + 15) >> 4;  // 16-byte chunks of values
    for (int i = threadIdx.x; i < nvb; i += tb) {
      if (!EXACT || 16 * i + 16 <= nt * VB) cp_async16(s_val + 16 * i, gv + 16 * i, polF);
      else cp_async16_part(s_val + 16 * i, gv + 16 * i, nt * VB - 16 * i);
    }
    const int32_t* gpos = a.pos[ORDER - 1] + fs;
    const int32_t* gcrd = a.crd[ORDER - 2] + fs;
    for (int x = threadIdx.x; x <= W; x += tb) s_pos[x] = gpos[x];
    for (int x = threadIdx.x; x < W; x += tb) s_fcrd[x] = gcrd[x];
  }
  cp_async_wait_all();
  __syncthreads();

  // 2. gather the factor rows: nonzero-level factor for each tile entry, the
  //    window factor for each window fiber
  {
    const unsigned char* fz = static_cast<const unsigned char*>(a.fac[ORDER - 2]);
    const unsigned char* fw = static_cast<const unsigned char*>(a.fac[ORDER - 3]);
    for (int j = threadIdx.x; j < nt * CPR; j += tb) {
      const int i = j / CPR, c = j - i * CPR;
      cp_async16(s_rows + (size_t)i * RB + 16 * c, fz + (size_t)s_lc[i] * RB + 16 * c, polL);
    }
    for (int j = threadIdx.x; j < W * CPR; j += tb) {
      const int x = j / CPR, c = j - x * CPR;
      cp_async16(s_wrows + (size_t)x * RB + 16 * c, fw + (size_t)s_fcrd[x] * RB + 16 * c, polL);
    }
  }
  cp_async_wait_all();
  __syncthreads();

  const int team = threadIdx.x / LPR;
  const int q = threadIdx.x % LPR;
  WK wk(a, q);
  Summ<CPT> X;
  X.h = kEmpty;
  X.t = kNone;
  const int64_t s = bstart + (int64_t)team * a.G;
  if (s < bend)
    wk.walk_staged(s, min(s + (int64_t)a.G, bend), bstart, s_val, s_rows, s_wrows, s_pos, W, fs, pb, pn, X);
  block_merge<ORDER, PREC, CPT, LPR>(a, wk, X, s_wh, s_wt, s_wha, s_wta, head_ff, fs, s_pos[0], bstart, pn[0], blockIdx.x);
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
  if constexpr (ORDER == 2) {  // TTV: the fiber holding the unit's first nonzero (nrows = fibers)
    out[0] = (int32_t)search_le(a.pos[1], 0, a.nrows - 1, s);
  } else {
    // fibers at level 1: pos[1][nrows]; level 2: pos[2][#level1]
    const int64_t nf1 = a.pos[1][a.nrows];
    int64_t f1;
    if constexpr (ORDER == 3) {
      f1 = search_le(a.pos[2], 0, nf1 - 1, s);
      out[1] = (int32_t)f1;
    } else {
      const int64_t nf2 = a.pos[2][nf1];
      const int64_t f2 = search_le(a.pos[3], 0, nf2 - 1, s);
      f1 = search_le(a.pos[2], 0, nf1 - 1, f2);
      out[1] = (int32_t)f1;
      out[2] = (int32_t)f2;
    }
    out[0] = (int32_t)search_le(a.pos[1], 0, a.nrows - 1, f1);
  }
}


#endif  // TT_ARGS_ONLY
}  // namespace tt
