// tt_strip.cuh -- the strip walk (family 4): mode-0 MTTKRP over a CSF tensor whose
// rows are long compared with a warp's step of nonzeros (3, 4 or 5 modes).
//
//   A(i,:) = sum_{k,l}   B(i,k,l)   C(k,:) .* D(l,:)             (order 3)
//   A(i,:) = sum_{k,l,m} B(i,k,l,m) C(k,:) .* D(l,:) .* E(m,:)    (order 4)
//   A(i,:) = sum B(i,k,l,m,n) C(k,:) .* D(l,:) .* E(m,:) .* F(n,:)  (order 5)
//   Y(f,:) = sum_l B(f,l) U(:,l)                                   (order 2: TTM,
//            the rows being a 3-mode tensor's fibers and U^T the one factor)
//
// Every nonzero carries its upper coordinates (kexp, kexp2, kexp3: built once per plan),
// so a nonzero is one independent product of gathered factor rows, the reference's
// own loop arithmetic (tensor_kernels/mttkrp3_csf_cpu_taco.h:45,
// mttkrp4_csf_cpu_taco.h:53; five modes: the product of tensor_kernels/
// mttkrp5_csf_cpu_taco.h:35-95, summed per nonzero instead of level by level).  The walk is warp-synchronous:
//
//   * a warp owns a tile of P consecutive nonzeros (the work unit of the partition
//     and of the cross-unit row merge), staged into shared memory in order with
//     coalesced 16-byte loads;
//   * the tile is walked in steps of TW * U nonzeros: team t (LPR lanes, CPT factor
//     columns each) takes nonzeros t*U .. t*U+U-1 of the step, so the warp's teams
//     always work on neighbouring nonzeros and row ends are decided once per step
//     for the whole warp, with no divergence;
//   * a step inside one output row (all of them on tensors with long rows) is only
//     loads and FMAs: each team adds its nonzeros' products into its partial row;
//   * a step holding a row end adds each nonzero to the row it belongs to (masked
//     passes over the step, one per row piece); the teams' partials of a finished
//     row are summed by a fixed reduce-scatter of shuffles that leaves each lane a
//     few of the row's columns to store (one coalesced store per row), or, for the
//     unit's first row, by a full butterfly that keeps the row for the unit's merge;
//     the end of the next row is loaded ahead, so a row end waits on no search
//     unless empty rows follow.
//
// The gathered rows of the next step are in flight while the current step is
// consumed (two register buffers).  Upper-level rows are gathered through L1 (the
// next nonzeros of a fiber read the same row); leaf rows bypass L1.  16-bit
// factors multiply in pairs by the mixed-precision FMA (exact products); the FP32
// FMAs go two columns per instruction (fma.rn.f32x2).
//
// The unit's first and last rows go through settle_unit and the two-level
// fixed-order merge of tt_mttkrp.cuh, as for the other families, so results are
// bitwise reproducible.  Rows are found through rnz (first nonzero of every row);
// a plan may lay the nonzeros out slab-major, with slabs * (rows + 1) "virtual"
// rows, and sum the slabs' rows afterwards (launch_virtual_rows).
#pragma once
#include "tt_mttkrp.cuh"

namespace tt {

// Element kinds of the strip walk's arrays per storage precision:
// V values, U upper-level factors, L leaf-level factor.
template <int PREC>
struct StripKinds;
template <>
struct StripKinds<kFP32> { static constexpr int V = kF32, U = kF32, L = kF32; };
template <>
struct StripKinds<kBF16> { static constexpr int V = kB16, U = kB16, L = kB16; };
template <>
struct StripKinds<kBF16F> { static constexpr int V = kF32, U = kB16, L = kB16; };
template <>
struct StripKinds<kFP16> { static constexpr int V = kH16, U = kH16, L = kH16; };
template <>
struct StripKinds<kFX16> { static constexpr int V = kF32, U = kF32, L = kI16; };

// Shared memory of one strip warp: leaf, level-1 (and level-2) coordinates, then
// the values, all in nonzero order.
__host__ __device__ inline size_t strip_warp_bytes(int P, int vbytes, int order) {
  return (size_t)(order - 1) * P * 4 + (((size_t)P * vbytes + 15) & ~(size_t)15);
}

#ifndef TT_ARGS_ONLY

// One lane's piece of a factor row (BYTES: 4, 8, 16 or 32), as raw words.
template <int BYTES, bool L1>
__device__ __forceinline__ void strip_piece(const unsigned char* p, uint64_t pol, uint32_t (&w)[(BYTES + 3) / 4]) {
  if constexpr (BYTES == 32) {
    const uint4 x = L1 ? ld_gather_16(p, pol) : ld_gather_16_na(p, pol);
    const uint4 y = L1 ? ld_gather_16(p + 16, pol) : ld_gather_16_na(p + 16, pol);
    w[0] = x.x; w[1] = x.y; w[2] = x.z; w[3] = x.w; w[4] = y.x; w[5] = y.y; w[6] = y.z; w[7] = y.w;
  } else if constexpr (BYTES == 16) {
    const uint4 x = L1 ? ld_gather_16(p, pol) : ld_gather_16_na(p, pol);
    w[0] = x.x; w[1] = x.y; w[2] = x.z; w[3] = x.w;
  } else if constexpr (BYTES == 8) {
    const uint2 x = L1 ? ld_gather_8(p, pol) : ld_gather_8_na(p, pol);
    w[0] = x.x; w[1] = x.y;
  } else {
    w[0] = L1 ? ld_gather_4(p, pol) : ld_gather_4_na(p, pol);
  }
}

// n16 16-byte chunks of a stream into shared memory, four loads per lane in
// flight per round (the streams are padded, so whole chunks stay in bounds).
__device__ __forceinline__ void strip_stage(const void* g, void* s, int n16, int lane, uint64_t pol) {
  constexpr int R = 4;
  const int32_t* gi = static_cast<const int32_t*>(g);
  int4* si = static_cast<int4*>(s);
  for (int c0 = lane; c0 < n16; c0 += 32 * R) {
    int4 x[R];
#pragma unroll
    for (int r = 0; r < R; r++)
      if (c0 + 32 * r < n16) x[r] = ld_stream_i4(gi + 4 * (c0 + 32 * r), pol);
#pragma unroll
    for (int r = 0; r < R; r++)
      if (c0 + 32 * r < n16) si[c0 + 32 * r] = x[r];
  }
}

template <int ORDER, int PREC, int CPT, int LPR, int U>
struct Strip {
  using K = StripKinds<PREC>;
  static constexpr int TW = 32 / LPR;  // teams per warp
  static constexpr int STEP = TW * U;  // nonzeros per warp step
  static constexpr int VB = K::V == kF32 ? 4 : 2;
  static constexpr int UB = CPT * (K::U == kF32 ? 4 : 2);  // bytes of a lane's upper-row piece
  static constexpr int LB = CPT * (K::L == kF32 ? 4 : 2);  // bytes of a lane's leaf-row piece
  static constexpr int UW = UB / 4, LW = LB / 4;
  static constexpr int MW = ORDER >= 4 ? UW : 1;
  static constexpr int EW = ORDER == 5 ? UW : 1;
  // bytes per factor row (the kernel is compiled for rows of RP = CPT * LPR entries)
  static constexpr uint32_t URB = (uint32_t)LPR * UB, LRB = (uint32_t)LPR * LB;
  static_assert(CPT >= 2 && CPT % 2 == 0, "the strip walk works on column pairs");

  // gathered pieces of one step's U nonzeros of a team, and their values
  struct Batch {
    uint32_t c[U][UW];  // level-1 factor
    uint32_t m[U][MW];  // level-2 factor (four and five modes)
    uint32_t e[U][EW];  // level-3 factor (five modes)
    uint32_t d[U][LW];  // leaf factor
    uint32_t v[U * VB / 4 > 0 ? U * VB / 4 : 1];  // raw values (U * VB bytes)
  };

  const unsigned char *fc, *fm, *fe, *fd;  // this lane's piece of row 0 of each factor
  uint64_t pol_u, pol_l;

  __device__ __forceinline__ void load(Batch& b, const int32_t* s_l, const int32_t* s_k, const int32_t* s_k2,
                                       const int32_t* s_k3, const unsigned char* s_v, int p0) const {
    int32_t l[U], k[U], k2[U], k3[U];
    if constexpr (U == 4) {
      const int4 a = *reinterpret_cast<const int4*>(s_l + p0);
      l[0] = a.x; l[1] = a.y; l[2] = a.z; l[3] = a.w;
      if constexpr (ORDER >= 3) {
        const int4 c = *reinterpret_cast<const int4*>(s_k + p0);
        k[0] = c.x; k[1] = c.y; k[2] = c.z; k[3] = c.w;
      }
      if constexpr (ORDER >= 4) {
        const int4 e = *reinterpret_cast<const int4*>(s_k2 + p0);
        k2[0] = e.x; k2[1] = e.y; k2[2] = e.z; k2[3] = e.w;
      }
      if constexpr (ORDER == 5) {
        const int4 e = *reinterpret_cast<const int4*>(s_k3 + p0);
        k3[0] = e.x; k3[1] = e.y; k3[2] = e.z; k3[3] = e.w;
      }
    } else if constexpr (U == 2) {
      const int2 a = *reinterpret_cast<const int2*>(s_l + p0);
      l[0] = a.x; l[1] = a.y;
      if constexpr (ORDER >= 3) {
        const int2 c = *reinterpret_cast<const int2*>(s_k + p0);
        k[0] = c.x; k[1] = c.y;
      }
      if constexpr (ORDER >= 4) {
        const int2 e = *reinterpret_cast<const int2*>(s_k2 + p0);
        k2[0] = e.x; k2[1] = e.y;
      }
      if constexpr (ORDER == 5) {
        const int2 e = *reinterpret_cast<const int2*>(s_k3 + p0);
        k3[0] = e.x; k3[1] = e.y;
      }
    } else {
      l[0] = s_l[p0];
      if constexpr (ORDER >= 3) k[0] = s_k[p0];
      if constexpr (ORDER >= 4) k2[0] = s_k2[p0];
      if constexpr (ORDER == 5) k3[0] = s_k3[p0];
    }
    constexpr int NVW = U * VB / 4;
    if constexpr (NVW == 4) {
      const uint4 w = *reinterpret_cast<const uint4*>(s_v + (size_t)p0 * VB);
      b.v[0] = w.x; b.v[1] = w.y; b.v[2] = w.z; b.v[3] = w.w;
    } else if constexpr (NVW == 2) {
      const uint2 w = *reinterpret_cast<const uint2*>(s_v + (size_t)p0 * VB);
      b.v[0] = w.x; b.v[1] = w.y;
    } else if constexpr (NVW == 1) {
      b.v[0] = *reinterpret_cast<const uint32_t*>(s_v + (size_t)p0 * VB);
    } else {  // one 16-bit value
      b.v[0] = *reinterpret_cast<const uint16_t*>(s_v + (size_t)p0 * VB);
    }
#pragma unroll
    for (int u = 0; u < U; u++) {
      if constexpr (ORDER >= 3) strip_piece<UB, true>(fc + (uint64_t)(uint32_t)k[u] * URB, pol_u, b.c[u]);
      if constexpr (ORDER >= 4) strip_piece<UB, true>(fm + (uint64_t)(uint32_t)k2[u] * URB, pol_u, b.m[u]);
      if constexpr (ORDER == 5) strip_piece<UB, true>(fe + (uint64_t)(uint32_t)k3[u] * URB, pol_u, b.e[u]);
      strip_piece<LB, false>(fd + (uint64_t)(uint32_t)l[u] * LRB, pol_l, b.d[u]);
    }
  }

  // value u of the batch as FP32 (the stored number, before the output scale)
  __device__ __forceinline__ static float value(const Batch& b, int u) {
    if constexpr (K::V == kF32) return __uint_as_float(b.v[u]);
    else {
      const uint32_t w = b.v[u >> 1];
      return (u & 1) ? hi16<K::V>(w) : lo16<K::V>(w);
    }
  }

  // acc += product of nonzero u of the batch
  __device__ __forceinline__ static void add(float (&acc)[CPT], const Batch& b, int u) {
    const float v = value(b, u);
    if constexpr (ORDER == 2) {
      // one factor: acc += v * d (FP32 storage)
      static_assert(K::U == kF32 && K::L == kF32, "the two-level walk (TTM) is built for FP32 storage");
#pragma unroll
      for (int j = 0; j < CPT / 2; j++)
        ffma2(acc[2 * j], acc[2 * j + 1], v, v, __uint_as_float(b.d[u][2 * j]), __uint_as_float(b.d[u][2 * j + 1]));
    } else if constexpr (K::U != kF32) {
      // 16-bit upper and leaf rows of one kind: c * d (and v * m, or v converted
      // times m) exact in FP32, then one FMA per column
      constexpr int FK = K::U;
#pragma unroll
      for (int j = 0; j < CPT / 2; j++) {
        const float2 p = hprod2<FK>(b.c[u][j], b.d[u][j]);
        if constexpr (ORDER >= 4) {
          float2 t;
          if constexpr (K::V == FK) {
            const uint32_t w = b.v[u >> 1];
            const uint32_t vv = (u & 1) ? (w >> 16) | (w & 0xffff0000u) : (w << 16) | (w & 0xffffu);
            t = hprod2<FK>(vv, b.m[u][j]);
          } else {
            const float2 mm = pair16<FK>(b.m[u][j]);
            t = fmul2(v, v, mm.x, mm.y);
          }
          if constexpr (ORDER == 5) {  // times the level-3 row (one rounding more)
            const float2 ee = pair16<FK>(b.e[u][j]);
            t = fmul2(t.x, t.y, ee.x, ee.y);
          }
          ffma2(acc[2 * j], acc[2 * j + 1], p.x, p.y, t.x, t.y);
        } else {
          ffma2(acc[2 * j], acc[2 * j + 1], v, v, p.x, p.y);
        }
      }
    } else {
      // FP32 upper rows: t = v * c [* m], then acc += t * d with d FP32 or 16-bit fixed point
#pragma unroll
      for (int j = 0; j < CPT / 2; j++) {
        float2 t = fmul2(v, v, __uint_as_float(b.c[u][2 * j]), __uint_as_float(b.c[u][2 * j + 1]));
        if constexpr (ORDER >= 4) t = fmul2(t.x, t.y, __uint_as_float(b.m[u][2 * j]), __uint_as_float(b.m[u][2 * j + 1]));
        if constexpr (ORDER == 5) t = fmul2(t.x, t.y, __uint_as_float(b.e[u][2 * j]), __uint_as_float(b.e[u][2 * j + 1]));
        float2 dd;
        if constexpr (K::L == kF32) dd = make_float2(__uint_as_float(b.d[u][2 * j]), __uint_as_float(b.d[u][2 * j + 1]));
        else dd = i16pair(b.d[u][j]);
        ffma2(acc[2 * j], acc[2 * j + 1], t.x, t.y, dd.x, dd.y);
      }
    }
  }
};

// Sum of the teams' partial rows (a fixed xor butterfly: every lane ends with the
// same total for its columns).
template <int CPT, int LPR>
__device__ __forceinline__ void strip_team_sum(const float (&acc)[CPT], float (&r)[CPT]) {
#pragma unroll
  for (int c = 0; c < CPT; c++) r[c] = acc[c];
#pragma unroll
  for (int d = LPR; d < 32; d <<= 1)
#pragma unroll
    for (int c = 0; c < CPT; c++) r[c] += __shfl_xor_sync(0xffffffffu, r[c], d);
}

// Reduce-scatter of the teams' partial rows: split butterfly levels halve the
// columns a lane keeps (lanes exchange the half they give away), then plain
// levels sum what is left across the remaining teams.  Lane (team, q) ends with W
// columns' totals, columns q*CPT + off(lane) + [0, W); among lanes that differ only
// in the plain levels' bits, the one with those bits clear stores them.  Fixed
// order: bitwise reproducible.
template <int CPT, int LPR>
struct TeamScatter {
  static constexpr int lg(int x) { return x <= 1 ? 0 : 1 + lg(x / 2); }
  static constexpr int TW = 32 / LPR;
  static constexpr int NS = lg(CPT) < lg(TW) ? lg(CPT) : lg(TW);  // split levels
  static constexpr int NP = lg(TW) - NS;                           // plain levels
  static constexpr int W = CPT >> NS;                              // columns kept per lane
  __device__ __forceinline__ static int offset(int lane) {
    int off = 0;
#pragma unroll
    for (int k = 0; k < NS; k++)
      if (lane & (LPR << k)) off += CPT >> (k + 1);
    return off;
  }
  __device__ __forceinline__ static bool stores(int lane) {
    bool st = true;
#pragma unroll
    for (int k = NS; k < NS + NP; k++)
      if (lane & (LPR << k)) st = false;
    return st;
  }
  __device__ __forceinline__ static void run(const float (&acc)[CPT], float (&r)[CPT], int lane) {
#pragma unroll
    for (int c = 0; c < CPT; c++) r[c] = acc[c];
#pragma unroll
    for (int k = 0; k < NS; k++) {
      const int d = LPR << k;
      const bool hi = (lane & d) != 0;
      const int half = (CPT >> k) / 2;
#pragma unroll
      for (int c = 0; c < CPT / 2; c++) {
        if (c < half) {
          const float send = hi ? r[c] : r[c + half];
          const float keep = hi ? r[c + half] : r[c];
          r[c] = keep + __shfl_xor_sync(0xffffffffu, send, d);
        }
      }
    }
#pragma unroll
    for (int k = NS; k < NS + NP; k++)
#pragma unroll
      for (int c = 0; c < W; c++) r[c] += __shfl_xor_sync(0xffffffffu, r[c], LPR << k);
  }
};

// Strip kernel: one work unit (P = TW * G nonzeros) per warp, 256-thread blocks;
// a launch covers units [unit_lo, unit_hi) of the nblocks (the one-shot call walks
// the units whose nonzeros have arrived while later ones are still being copied).
// part[u * (ORDER - 1)]: the row holding unit u's first nonzero (launch_partition_rows).
template <int ORDER, int PREC, int CPT, int LPR, int U, int MINB>
__global__ void __launch_bounds__(256, MINB) mttkrp_strip_kernel(const __grid_constant__ WalkArgs a) {
  using ST = Strip<ORDER, PREC, CPT, LPR, U>;
  using WK = Walk<ORDER, PREC, CPT, LPR>;
  constexpr int STEP = ST::STEP, VB = ST::VB;
  extern __shared__ __align__(16) unsigned char smem[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int unit = a.unit_lo + blockIdx.x * (blockDim.x >> 5) + warp;
  if (unit >= (a.unit_hi > 0 ? a.unit_hi : a.nblocks)) return;  // whole warp: nothing below synchronises the block
  const int P = a.P;
  unsigned char* ws = smem + (size_t)warp * strip_warp_bytes(P, VB, ORDER);
  int32_t* s_l = reinterpret_cast<int32_t*>(ws);
  int32_t* s_k = s_l + P;
  int32_t* s_k2 = s_k + P;   // four and five modes
  int32_t* s_k3 = s_k2 + P;  // five modes
  unsigned char* s_v = reinterpret_cast<unsigned char*>(s_l + (size_t)(ORDER - 1) * P);
  const int64_t ustart = (int64_t)unit * P;
  const int cnt = (int)min((int64_t)P, a.nnz - ustart);
  {
    const uint64_t polF = policy_evict_first();
    const int n4 = (cnt + 3) >> 2;
    strip_stage(a.crd[ORDER - 1] + ustart, s_l, n4, lane, polF);
    if constexpr (ORDER >= 3) strip_stage(a.kexp + ustart, s_k, n4, lane, polF);
    if constexpr (ORDER >= 4) strip_stage(a.kexp2 + ustart, s_k2, n4, lane, polF);
    if constexpr (ORDER == 5) strip_stage(a.kexp3 + ustart, s_k3, n4, lane, polF);
    strip_stage(static_cast<const unsigned char*>(a.vals) + ustart * VB, s_v, (cnt * VB + 15) >> 4, lane, polF);
    // the tensor's last unit: the steps past its end still gather (masked out
    // later), so their coordinates must be valid rows
    for (int p = 4 * n4 + lane; p < (cnt + STEP - 1) / STEP * STEP; p += 32) {
      s_l[p] = 0;
      if constexpr (ORDER >= 3) s_k[p] = 0;
      if constexpr (ORDER >= 4) s_k2[p] = 0;
      if constexpr (ORDER == 5) s_k3[p] = 0;
    }
  }
  __syncwarp();

  const int team = lane / LPR, q = lane % LPR;
  WK wk(a, q);
  ST st;
  st.fc = static_cast<const unsigned char*>(a.fac[0]) + q * ST::UB;
  st.fm = static_cast<const unsigned char*>(a.fac[1]) + q * ST::UB;
  st.fe = static_cast<const unsigned char*>(a.fac[2]) + q * ST::UB;
  st.fd = static_cast<const unsigned char*>(a.fac[ORDER - 2]) + q * ST::LB;
  st.pol_u = policy_evict_last();
  st.pol_l = a.gpol == 1 ? policy_evict_normal() : policy_evict_last();

  const int32_t* rnz = a.rnz;
  const int32_t* pb = a.part + (size_t)unit * (ORDER - 1);
  const int rhi = pb[ORDER - 1];  // row of the next unit's first nonzero
  const int first_row = (int)search_le(rnz, pb[0], rhi, ustart);
  // positions below are relative to the unit's start (32-bit); a row end past the
  // unit is clamped to it (only "inside the unit or not" matters)
  auto rel = [&](int64_t abs_pos) { return (int)min(abs_pos - ustart, (int64_t)cnt + STEP); };
  int ip = first_row;
  int rend = rel(rnz[ip + 1]);
  int64_t rnext = rnz[min(ip + 2, a.nrows)];  // end of the next row (loaded ahead)
  bool first_done = false;
  // interior rows leave through the reduce-scatter: this lane's columns, and their
  // output scales, are fixed for the whole walk
  using TS = TeamScatter<CPT, LPR>;
  const int scol = q * CPT + TS::offset(lane);
  const bool sstore = TS::stores(lane);
  float sscale[TS::W];
#pragma unroll
  for (int c = 0; c < TS::W; c++) sscale[c] = a.colscale && scol + c < a.R ? a.colscale[scol + c] : 1.f;
  Summ<CPT> X;
  X.h = kEmpty;
  X.t = kNone;
  float acc[CPT];
#pragma unroll
  for (int c = 0; c < CPT; c++) acc[c] = 0.f;

  // row ip ends inside the step: its total goes to the unit's summary (first row)
  // or straight to the output, then the walk moves to the row holding `at`
  auto row_end = [&](int at_rel) {
    const int64_t at = ustart + at_rel;
    float r[CPT];
    if (!first_done) {
      strip_team_sum<CPT, LPR>(acc, r);
      X.h = ip;
#pragma unroll
      for (int c = 0; c < CPT; c++) X.ha[c] = r[c];
      first_done = true;
    } else {
      // a row that starts and ends inside the unit: complete, stored once
      TS::run(acc, r, lane);
      if (sstore) {
        float* o = a.out + (int64_t)wk.row_id(ip) * a.ldo + scol;
#pragma unroll
        for (int c = 0; c < TS::W; c++)
          if (scol + c < a.R) o[c] = r[c] * sscale[c];
      }
    }
#pragma unroll
    for (int c = 0; c < CPT; c++) acc[c] = 0.f;
    // the next row holds `at` unless it is empty (then search past the empty rows)
    int nip = ip + 1;
    int64_t nend = rnext;
    if (nend <= at) {
      nip = (int)search_le(rnz, ip + 1, rhi, at);
      nend = rnz[nip + 1];
    }
    ip = nip;
    rend = rel(nend);
    rnext = rnz[min(ip + 2, a.nrows)];
  };
  auto consume = [&](const typename ST::Batch& b, int s) {
    const int sb = s * STEP;
    const int se = min(sb + STEP, cnt);
    if (se <= rend && se == sb + STEP) {
#pragma unroll
      for (int u = 0; u < U; u++) ST::add(acc, b, u);
      return;
    }
    const int mine = sb + team * U;  // this team's first nonzero of the step
    int lo = sb;
    while (true) {
      const int hi = min(rend, se);
#pragma unroll
      for (int u = 0; u < U; u++)
        if (mine + u >= lo && mine + u < hi) ST::add(acc, b, u);
      if (hi == se) break;
      row_end(hi);
      lo = hi;
    }
  };

  const int nsteps = (cnt + STEP - 1) / STEP;
  typename ST::Batch bA, bB;
  const int toff = team * U;
  if (nsteps > 0) st.load(bA, s_l, s_k, s_k2, s_k3, s_v, toff);
  for (int s = 0; s < nsteps; s += 2) {
    if (s + 1 < nsteps) st.load(bB, s_l, s_k, s_k2, s_k3, s_v, (s + 1) * STEP + toff);
    consume(bA, s);
    if (s + 1 < nsteps) {
      if (s + 2 < nsteps) st.load(bA, s_l, s_k, s_k2, s_k3, s_v, (s + 2) * STEP + toff);
      consume(bB, s + 1);
    }
  }
  {
    float r[CPT];
    strip_team_sum<CPT, LPR>(acc, r);
    if (!first_done) {
      X.h = ip;
      X.t = kNone;
#pragma unroll
      for (int c = 0; c < CPT; c++) X.ha[c] = r[c];
    } else {
      X.t = ip;
#pragma unroll
      for (int c = 0; c < CPT; c++) X.ta[c] = r[c];
    }
  }
  // the unit's first row started before it when its first nonzero lies earlier
  if (lane < LPR) settle_unit(a, wk, X, 0, 0, rnz[first_row], ustart, rhi, unit, q);
}

#endif  // TT_ARGS_ONLY
}  // namespace tt
