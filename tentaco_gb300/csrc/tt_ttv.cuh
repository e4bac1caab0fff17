// tt_ttv.cuh -- tensor-times-vector over the last mode of a CSF tensor, sm_103a.
//
//   y(f) = sum_{p in fiber f} vals[p] * x[crd[p]]      f = fibers of level order-2
//
// Replaces the reference's ttv_kernel / ttv_csf_gpu_taco
// (tensor_kernels/ttv_csf_gpu_taco.h:2-121).  The output is indexed by fiber
// position, as in the reference (A_vals[j_pos] there), so only the last two CSF
// levels are read: the kernel sees a 2-level CSF (WalkArgs with pos[1] = fiber
// starts, crd[1] = last-mode coordinates, nrows = fibers, one output column).
// Unlike the reference, every output is written exactly once (no memset, no
// float atomics).  Work: 512-nonzero units (the partition's), grouped into ranges
// of RU consecutive units; warp w of the grid walks range w in order.
//   * per unit, lane L owns the 16 nonzeros from 16 L and loads its coordinates,
//     values and (XS) x entries; the unit's fiber ends are byte flags in shared
//     memory (flag e: nonzero e ends a fiber), set by plain byte stores from the
//     fiber starts of the unit's window, then packed into a 16-bit mask per lane;
//     a lane's first fiber is fs + the ends before it (a warp prefix sum);
//   * the per-nonzero loop has no branches: an FMA, a predicated shared-memory
//     store of a fiber that starts and ends in the lane, and selects;
//   * the lanes are merged by a segmented scan of their open tail sums (a lane
//     where a fiber ends starts a segment); the unit's finished fibers, staged in
//     shared memory, leave in one coalesced store (not one 32-byte sector write
//     per fiber);
//   * a fiber crossing a unit boundary inside the range is carried in registers;
//     the range's first and last fibers go through the carry slots and the
//     two-level merge of tt_mttkrp.cuh (FP32 Kahan inside a segment, FP64 across).
// Fibers are never empty (canonical CSF), so a nonzero ends at most one fiber.
#pragma once
#include "tt_mttkrp.cuh"

namespace tt {

constexpr int kTtvNpt = 16;  // nonzeros per lane (the mask holds 16 bits per lane)
// range walk (ttv_range_kernel)
constexpr int kTtvWarps = 24;  // warps per block
constexpr int kTtvYStage = 520;  // floats per warp staging a unit's finished fibers (at most 512)
constexpr int kTtvPre = 8;     // fiber starts per lane loaded with the unit (256 per unit)
constexpr int kTtvMaxRU = 62;  // units per range (the partition entries fit two per lane)

#ifndef TT_ARGS_ONLY
// The range walk.  Ranges instead of single units cut the merge's work units from
// about 98,000 to 3,600 on 50M nonzeros.  One block of kTtvWarps warps per SM (80
// registers a thread).  x sits in shared memory when it fits (XS): the 16 gathers
// per lane and unit are then shared-memory loads instead of L1 tag lookups (a
// walk gathering x through L1 spent 72% of the L1's throughput on them).  The
// range's unit boundaries come from one load of its partition entries per lane; a
// unit's coordinates, values and first 256 fiber starts are loaded together, the
// first unit's while x is being staged.
// Measured on 50M nonzeros (x of 30,000 entries): 24 warps per SM without loads
// ahead, 16 warps with the next unit's loads in a second register set, and 32
// warps (spilling) take 139, 139 and 162 us; with the loads coalesced in chunks of
// 128 nonzeros (four lane merges per unit) 195 us; the staged fiber stores, 134 us.
// a.P = RU * 512 and a.nblocks = ranges (the merge's units), a.wcap = RU,
// a.part = the 512-nonzero partition, a.fac_rows[0] = length of x.

// V8: the lane's 64 bytes of coordinates (and of values) as 32-byte loads, half the
// load instructions and L1 wavefronts of 16-byte ones (the streams must be 32-byte
// aligned; the launcher checks).
template <int VK, bool XS, bool V8>
__global__ void __launch_bounds__(32 * kTtvWarps, 1) ttv_range_kernel(const __grid_constant__ WalkArgs a) {
  constexpr int NPT = kTtvNpt;
  constexpr int UN = 32 * NPT;                    // nonzeros per unit
  constexpr int NW = VK == kF32 ? NPT : NPT / 2;  // value words per lane
  using WK = Walk<3, kFP32, 1, 1>;
  extern __shared__ __align__(16) unsigned char smem[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  uint8_t* s_end = smem + warp * UN;  // one flag per nonzero of the unit
  float* s_y = reinterpret_cast<float*>(smem + kTtvWarps * UN) + warp * kTtvYStage;  // the unit's finished fibers
  float* s_x = reinterpret_cast<float*>(smem + kTtvWarps * UN) + kTtvWarps * kTtvYStage;
  const int nunits = (int)((a.nnz + UN - 1) / UN);
  const int RU = a.wcap;
  const int r = blockIdx.x * kTtvWarps + warp;
  const int ub = min(r * RU, nunits), ue = min(ub + RU, nunits);
  const float* xg = static_cast<const float*>(a.fac[0]);
  const uint64_t polF = policy_evict_first();

  // the range's partition entries part[ub .. ue] (at most 63), two per lane
  const int np = ue - ub + 1;
  const int pr0 = lane < np ? a.part[ub + lane] : 0;
  const int pr1 = 32 + lane < np ? a.part[ub + 32 + lane] : 0;
  auto partv = [&](int i) {  // part[ub + i], i warp-uniform
    const int v0 = __shfl_sync(0xffffffffu, pr0, i & 31), v1 = __shfl_sync(0xffffffffu, pr1, i & 31);
    return i < 32 ? v0 : v1;
  };

  struct Set {
    int32_t lc[NPT];
    uint32_t vw[NW];
    int32_t pw[kTtvPre];
  };
  // loads of unit u (ub <= u < ue) into S
  auto issue = [&](int u, Set& S) {
    const int64_t s64 = (int64_t)u * UN + (int64_t)lane * NPT;
    if (s64 < a.nnz) {  // runs are padded past the last 16-entry run
      const int32_t* gl = a.crd[1] + s64;
      const unsigned char* gv = static_cast<const unsigned char*>(a.vals) + s64 * (VK == kF32 ? 4 : 2);
      if constexpr (V8) {
#pragma unroll
        for (int k = 0; k < NPT / 8; k++) {
          uint32_t w[8];
          ld_stream_l1_v8(gl + 8 * k, polF, w);
#pragma unroll
          for (int j = 0; j < 8; j++) S.lc[8 * k + j] = (int32_t)w[j];
        }
#pragma unroll
        for (int k = 0; k < NW / 8; k++) {
          uint32_t w[8];
          ld_stream_l1_v8(gv + 32 * k, polF, w);
#pragma unroll
          for (int j = 0; j < 8; j++) S.vw[8 * k + j] = w[j];
        }
      } else {
#pragma unroll
        for (int k = 0; k < NPT / 4; k++) {
          const uint4 c4 = ld_stream_l1_u4(gl + 4 * k, polF);
          S.lc[4 * k] = (int32_t)c4.x; S.lc[4 * k + 1] = (int32_t)c4.y;
          S.lc[4 * k + 2] = (int32_t)c4.z; S.lc[4 * k + 3] = (int32_t)c4.w;
        }
#pragma unroll
        for (int k = 0; k < NW / 4; k++) {
          const uint4 w = ld_stream_l1_u4(gv + 16 * k, polF);
          S.vw[4 * k] = w.x; S.vw[4 * k + 1] = w.y; S.vw[4 * k + 2] = w.z; S.vw[4 * k + 3] = w.w;
        }
      }
    } else {
#pragma unroll
      for (int k = 0; k < NPT; k++) S.lc[k] = 0;
#pragma unroll
      for (int k = 0; k < NW; k++) S.vw[k] = 0u;
    }
    const int fs = partv(u - ub);
    const int W = partv(u - ub + 1) - fs + 1;
    const int32_t* gpos = a.pos[1] + fs;
#pragma unroll
    for (int j = 0; j < kTtvPre; j++) {
      const int x = 1 + lane + 32 * j;
      S.pw[j] = x <= W ? gpos[x] : 0;
    }
  };

  Set A;
  if (ub < ue) issue(ub, A);
  if constexpr (XS) {
    // x into shared memory (all threads of the block; overlaps the first unit's loads)
    const int nx = a.fac_rows[0];
    if ((reinterpret_cast<uintptr_t>(xg) & 15) == 0) {
      for (int i = threadIdx.x; i < nx / 4; i += blockDim.x)
        reinterpret_cast<float4*>(s_x)[i] = __ldg(reinterpret_cast<const float4*>(xg) + i);
      for (int i = (nx & ~3) + threadIdx.x; i < nx; i += blockDim.x) s_x[i] = __ldg(xg + i);
    } else {
      for (int i = threadIdx.x; i < nx; i += blockDim.x) s_x[i] = __ldg(xg + i);
    }
    __syncthreads();
  }
  if (ub >= ue) return;  // whole warp

  const int head = __shfl_sync(0xffffffffu, pr0, 0);  // part[ub]: the range's head fiber
  const int next_row = partv(ue - ub);                 // part[ue]: the fiber after the range
  const int64_t win0 = lane == 0 ? (int64_t)a.pos[1][head] : 0;                   // start of the head fiber
  bool head_done = false;
  float head_acc = 0.f;
  int carry_f = -1;  // fiber open at the end of the last unit walked (warp-uniform)
  float carry_v = 0.f;

  auto walk = [&](int u, const Set& S) {
    const int64_t ustart64 = (int64_t)u * UN;
    const int ustart = (int)ustart64;
    const int cnt = (int)min((int64_t)UN, a.nnz - ustart64);
    const int n = max(0, min(NPT, cnt - lane * NPT));
    const int fs = partv(u - ub);
    const int W = partv(u - ub + 1) - fs + 1;
    float xv[NPT];
#pragma unroll
    for (int k = 0; k < NPT; k++) xv[k] = XS ? s_x[S.lc[k]] : __ldg(xg + S.lc[k]);
    // fiber ends as byte flags, then the lane's 16 flags as a mask
    reinterpret_cast<uint4*>(s_end)[lane] = make_uint4(0u, 0u, 0u, 0u);
    __syncwarp();
#pragma unroll
    for (int j = 0; j < kTtvPre; j++) {
      const int x = 1 + lane + 32 * j;
      const int e = S.pw[j] - 1 - ustart;
      if (x <= W && e >= 0 && e < cnt) s_end[e] = 1;
    }
    for (int x = 1 + 32 * kTtvPre + lane; x <= W; x += 32) {  // windows of more than 256 fibers
      const int e = a.pos[1][fs + x] - 1 - ustart;
      if (e >= 0 && e < cnt) s_end[e] = 1;
    }
    __syncwarp();
    uint32_t m = 0u;
    {
      const uint4 b = reinterpret_cast<const uint4*>(s_end)[lane];
      const uint32_t w[4] = {b.x, b.y, b.z, b.w};
#pragma unroll
      for (int k = 0; k < 4; k++)
        m |= ((w[k] & 1u) | ((w[k] >> 7) & 2u) | ((w[k] >> 14) & 4u) | ((w[k] >> 21) & 8u)) << (4 * k);
    }
    int incl = __popc(m);
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const int t = __shfl_up_sync(0xffffffffu, incl, d);
      if (lane >= d) incl += t;
    }
    const int f0 = fs + incl - __popc(m);  // fiber of the lane's first nonzero
    float v[NPT];
    if constexpr (VK == kF32) {
#pragma unroll
      for (int k = 0; k < NPT; k++) v[k] = __uint_as_float(S.vw[k]);
    } else {
#pragma unroll
      for (int k = 0; k < NPT / 2; k++) {
        const float2 p = pair16<VK>(S.vw[k]);
        v[2 * k] = p.x * a.vscale;
        v[2 * k + 1] = p.y * a.vscale;
      }
    }
    float acc = 0.f, hacc = 0.f;
    bool hset = false;
    int f = f0;
    auto step = [&](int k) {
      acc = fmaf(v[k], xv[k], acc);
      const bool e = (m >> k) & 1u;
      if (e && hset) s_y[f - fs] = acc;  // a fiber that started and ended in this lane
      hacc = (e && !hset) ? acc : hacc;
      hset = hset || e;
      f += e ? 1 : 0;
      acc = e ? 0.f : acc;
    };
    if (cnt == UN) {
#pragma unroll
      for (int k = 0; k < NPT; k++) step(k);
    } else {
#pragma unroll
      for (int k = 0; k < NPT; k++)
        if (k < n) step(k);
    }
    // the lanes' open tail sums, merged by a segmented inclusive scan (as in the
    // unit walk)
    const bool active = n > 0;
    float val = active ? acc : 0.f;
    bool hd = active && hset;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const float vu = __shfl_up_sync(0xffffffffu, val, d);
      const int hu = __shfl_up_sync(0xffffffffu, hd ? 1 : 0, d);
      if (lane >= d) {
        if (!hd) val = vu + val;
        hd = hd || hu;
      }
    }
    float cin = __shfl_up_sync(0xffffffffu, val, 1);
    if (lane == 0) cin = 0.f;
    const float total = cin + hacc;
    const unsigned ends = __ballot_sync(0xffffffffu, active && hset);
    const int lstar = ends ? __ffs((int)ends) - 1 : -1;
    if (active && hset && lane != lstar) s_y[f0 - fs] = total;
    // fibers fs + 1 .. fs + E - 1 start and end in the unit: one coalesced store
    __syncwarp();
    const int E = __shfl_sync(0xffffffffu, incl, 31);  // fiber ends in the unit
    for (int i = 1 + lane; i < E; i += 32) a.out[fs + i] = s_y[i];
    const int la = (cnt - 1) / NPT;
    const float tot_first = __shfl_sync(0xffffffffu, total, lstar < 0 ? 0 : lstar);
    const float out_last = __shfl_sync(0xffffffffu, val, la);
    const int f_last = __shfl_sync(0xffffffffu, f, la);
    const uint32_t m_last = __shfl_sync(0xffffffffu, m, la);
    const bool open = !((m_last >> (cnt - la * NPT - 1)) & 1u);
    // the unit's first fiber fs continues the fiber carried from the previous unit
    // (if one is open); until the range's head fiber ends, every unit lies in it
    const float cin0 = carry_f == fs ? carry_v : 0.f;
    if (lstar >= 0) {
      const float T = cin0 + tot_first;
      if (!head_done) {
        head_acc = T;
        head_done = true;
      } else if (lane == 0) {
        a.out[fs] = T;
      }
      carry_f = open ? f_last : -1;
      carry_v = open ? out_last : 0.f;
    } else {
      carry_f = fs;
      carry_v = cin0 + out_last;
    }
  };

  walk(ub, A);
  for (int u = ub + 1; u < ue; u++) {
    issue(u, A);
    walk(u, A);
  }
  if (lane == 0) {
    // the range's summary: its head fiber and, if different, the fiber open at its end
    Summ<1> X;
    X.h = head;
    X.t = kNone;
    if (!head_done) {
      X.ha[0] = carry_v;  // the whole range lies in the head fiber
    } else {
      X.ha[0] = head_acc;
      if (carry_f >= 0) {
        X.t = carry_f;
        X.ta[0] = carry_v;
      }
    }
    WK wk(a, 0);
    settle_unit(a, wk, X, (int64_t)head, (int64_t)head, win0, (int64_t)ub * UN, next_row, r, 0);
  }
}
#endif  // TT_ARGS_ONLY
}  // namespace tt
