// tt_misc.cu -- partition, TTV and storage-conversion kernels of libtentaco_gb300.
#include <cuda_bf16.h>
#include <algorithm>
#include <atomic>
#include <utility>
#include <cuda_fp16.h>
#include "tt_kernels.h"
#include "tt_mttkrp.cuh"
#include "tt_ttv.cuh"
#include "tt_strip.cuh"

namespace tt {

// A launch of a kernel that begins with grid_dependency_wait(): with programmatic
// stream serialization, so it starts as the previous kernel's blocks finish instead
// of after a launch gap.
template <typename... P, typename... A>
cudaError_t launch_dependent(void (*k)(P...), int grid, int block, cudaStream_t s, A&&... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)grid);
  cfg.blockDim = dim3((unsigned)block);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, k, std::forward<A>(args)...);
}


WalkLauncher walk_launcher(int order, int prec, int cpt, int lpr, int staged) {
  if (staged == 8 || staged == 9) {  // strip walk (U = 4 / 2 nonzeros per team and step)
    if (order == 3) {
      if (prec == kFP32) return walk_launcher_o3_fp32_strip(cpt, lpr, staged);
      if (prec == kBF16) return walk_launcher_o3_bf16_strip(cpt, lpr, staged);
      if (prec == kBF16F) return walk_launcher_o3_bf16f_strip(cpt, lpr, staged);
      if (prec == kFP16) return walk_launcher_o3_fp16_strip(cpt, lpr, staged);
      if (prec == kFX16) return walk_launcher_o3_fx16_strip(cpt, lpr, staged);
    } else if (order == 4) {
      if (prec == kFP32) return walk_launcher_o4_fp32_strip(cpt, lpr, staged);
      if (prec == kBF16) return walk_launcher_o4_bf16_strip(cpt, lpr, staged);
      if (prec == kBF16F) return walk_launcher_o4_bf16f_strip(cpt, lpr, staged);
      if (prec == kFP16) return walk_launcher_o4_fp16_strip(cpt, lpr, staged);
      if (prec == kFX16) return walk_launcher_o4_fx16_strip(cpt, lpr, staged);
    } else if (order == 2) {  // TTM (fibers times one matrix): FP32
      if (prec == kFP32) return walk_launcher_o2_fp32_strip(cpt, lpr, staged);
    } else if (order == 5) {  // five modes: FP32, FP16 and 16-bit fixed point
      if (prec == kFP32) return walk_launcher_o5_fp32_strip(cpt, lpr, staged);
      if (prec == kFP16) return walk_launcher_o5_fp16_strip(cpt, lpr, staged);
      if (prec == kFX16) return walk_launcher_o5_fx16_strip(cpt, lpr, staged);
    }
    return nullptr;
  }
  if (order > 4 || order < 3) return nullptr;  // five modes and TTM: strip walk only
  if (prec == kFX16) return nullptr;  // 16-bit fixed point: strip walk only
  if (order == 3) {
    if (prec == kFP32) return walk_launcher_o3_fp32(cpt, lpr, staged);
    if (prec == kBF16) return walk_launcher_o3_bf16(cpt, lpr, staged);
    if (prec == kBF16F) return walk_launcher_o3_bf16f(cpt, lpr, staged);
    if (prec == kFP16) return walk_launcher_o3_fp16(cpt, lpr, staged);
  } else if (order == 4) {
    if (prec == kFP32) return walk_launcher_o4_fp32(cpt, lpr, staged);
    if (prec == kBF16) return walk_launcher_o4_bf16(cpt, lpr, staged);
    if (prec == kBF16F) return walk_launcher_o4_bf16f(cpt, lpr, staged);
    if (prec == kFP16) return walk_launcher_o4_fp16(cpt, lpr, staged);
  }
  return nullptr;
}

cudaError_t launch_partition(int order, const WalkArgs& a, cudaStream_t s) {
  const int n = a.nblocks + 1;
  const int tb = 256, grid = (n + tb - 1) / tb;
  if (order == 2) partition_kernel<2><<<grid, tb, 0, s>>>(a);
  else if (order == 3) partition_kernel<3><<<grid, tb, 0, s>>>(a);
  else if (order == 4) partition_kernel<4><<<grid, tb, 0, s>>>(a);
  else return cudaErrorInvalidValue;  // five modes: launch_partition_rows (strip walk)
  return cudaGetLastError();
}

// Partition for the strip walk: for each unit boundary b in [0, nblocks], the row
// (through rnz) holding nonzero min(b * P, nnz - 1), at stride `stride` in part.
__global__ void partition_rows_kernel(const __grid_constant__ WalkArgs a, int stride) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b > a.nblocks) return;
  const int64_t s = (b < a.nblocks) ? (int64_t)b * a.P : a.nnz - 1;
  const_cast<int32_t*>(a.part)[(size_t)b * stride] = (int32_t)search_le(a.rnz, 0, a.nrows - 1, s);
}

cudaError_t launch_partition_rows(int order, const WalkArgs& a, cudaStream_t s) {
  const int n = a.nblocks + 1;
  partition_rows_kernel<<<(n + 255) / 256, 256, 0, s>>>(a, order - 1);
  return cudaGetLastError();
}

// A(i, j) = sum over slabs k, in slab order, of V(k * vstride + i, j): the virtual
// rows of a slab-major plan summed into the output in FP32 with Kahan compensation
// (at most 16 terms: within an ulp or two of the exact sum; GB300's FP64 pipe runs at
// 1/64 of the FP32 rate and would bound this kernel).  A
// virtual row without nonzeros (rnz[r] == rnz[r + 1]) was never written and
// counts as zero.  One thread per 4 columns of a row: every load of a row is
// issued before any is used (the emptiness test selects, it does not branch, and
// V is allocated for every virtual row).  ldv: row stride of V, a multiple of 4;
// lda: row stride of A.
constexpr int kVirtMaxSlabs = 16;
// One instance per slab count S (registers for S rows, not for the maximum): with
// four slabs a thread holds 16 loaded words and the SMs stay fully occupied.
template <int S>
__global__ void __launch_bounds__(256) virtual_rows_kernel(const float* __restrict__ V, const int32_t* __restrict__ rnz,
                                                           int64_t nrows, int64_t vstride, int ldv, int lda, int R,
                                                           float* __restrict__ A) {
  grid_dependency_wait();       // the walk's and the merge's virtual rows
  const int q4 = (R + 3) >> 2;  // 4-column groups per row
  const int64_t n = nrows * q4;
  const bool narrow = n <= 0x7fffffff;  // 32-bit index arithmetic
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
    int64_t i;
    int j;
    if (narrow) {
      const int i32 = (int)e / q4;
      i = i32;
      j = ((int)e - i32 * q4) * 4;
    } else {
      i = e / q4;
      j = (int)(e - i * q4) * 4;
    }
    float4 v[S];
    bool live[S];
#pragma unroll
    for (int k = 0; k < S; k++) {
      const int64_t r = (int64_t)k * vstride + i;
      live[k] = rnz[r + 1] > rnz[r];
      v[k] = *reinterpret_cast<const float4*>(V + r * ldv + j);
    }
    float sum[4] = {0.f, 0.f, 0.f, 0.f}, cmp[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
    for (int k = 0; k < S; k++) {
      if (live[k]) {
        const float x[4] = {v[k].x, v[k].y, v[k].z, v[k].w};
#pragma unroll
        for (int c = 0; c < 4; c++) {  // Kahan: cmp holds the low part lost so far
          const float y = __fsub_rn(x[c], cmp[c]);
          const float t = __fadd_rn(sum[c], y);
          cmp[c] = __fsub_rn(__fsub_rn(t, sum[c]), y);
          sum[c] = t;
        }
      }
    }
    float* o = A + i * lda + j;
    if (j + 3 < R && (lda & 3) == 0) {
      *reinterpret_cast<float4*>(o) = make_float4(sum[0], sum[1], sum[2], sum[3]);
    } else {
      for (int c = 0; c < 4 && j + c < R; c++) o[c] = sum[c];
    }
  }
}

template <int S>
cudaError_t launch_virtual_rows_s(const float* V, const int32_t* rnz, int64_t nrows, int64_t vstride, int ldv, int lda,
                                  int R, float* A, int grid, cudaStream_t s) {
  const cudaError_t e = launch_dependent(virtual_rows_kernel<S>, grid, 256, s, V, rnz, nrows, vstride, ldv, lda, R, A);
  return e != cudaSuccess ? e : cudaGetLastError();
}

cudaError_t launch_virtual_rows(const float* V, const int32_t* rnz, int S, int64_t nrows, int64_t vstride, int ldv,
                                int lda, int R, float* A, cudaStream_t s) {
  if (nrows == 0 || R == 0) return cudaSuccess;
  if (S < 1 || S > kVirtMaxSlabs || (ldv & 3) != 0 || ldv < ((R + 3) & ~3) || lda < R) return cudaErrorInvalidValue;
  const int64_t n = nrows * ((R + 3) / 4);
  const int grid = (int)std::min<int64_t>((n + 255) / 256, 152 * 8);
  using L = cudaError_t (*)(const float*, const int32_t*, int64_t, int64_t, int, int, int, float*, int, cudaStream_t);
  static const L table[kVirtMaxSlabs] = {
      launch_virtual_rows_s<1>,  launch_virtual_rows_s<2>,  launch_virtual_rows_s<3>,  launch_virtual_rows_s<4>,
      launch_virtual_rows_s<5>,  launch_virtual_rows_s<6>,  launch_virtual_rows_s<7>,  launch_virtual_rows_s<8>,
      launch_virtual_rows_s<9>,  launch_virtual_rows_s<10>, launch_virtual_rows_s<11>, launch_virtual_rows_s<12>,
      launch_virtual_rows_s<13>, launch_virtual_rows_s<14>, launch_virtual_rows_s<15>, launch_virtual_rows_s<16>};
  return table[S - 1](V, rnz, nrows, vstride, ldv, lda, R, A, grid, s);
}

__global__ void window_max_kernel(const __grid_constant__ WalkArgs a, int lvl, int stride, int* out) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= a.nblocks) return;
  const int w = a.part[(size_t)(b + 1) * stride + lvl] - a.part[(size_t)b * stride + lvl] + 1;
  atomicMax(out, w);
}

cudaError_t launch_window_max(int order, const WalkArgs& a, int* out, cudaStream_t s) {
  cudaError_t e = cudaMemsetAsync(out, 0, sizeof(int), s);
  if (e != cudaSuccess) return e;
  if (a.nblocks == 0) return cudaSuccess;
  window_max_kernel<<<(a.nblocks + 255) / 256, 256, 0, s>>>(a, order - 2, order - 1, out);
  return cudaGetLastError();
}

template <int ORDER>
cudaError_t launch_fold_chain(const WalkArgs& a, int grid, cudaStream_t s) {
  cudaError_t e = launch_dependent(seg_fold_kernel<ORDER>, grid, 256, s, a);
  if (e == cudaSuccess) e = launch_dependent(seg_chain_kernel<ORDER>, grid, 256, s, a);
  return e;
}

cudaError_t launch_chain_fixup(int order, const WalkArgs& a, cudaStream_t s) {
  if (a.nblocks == 0) return cudaSuccess;
  const int grid = (num_segments(a.nblocks) + 7) / 8;  // one warp per segment
  cudaError_t e;
  if (order == 2) e = launch_fold_chain<2>(a, grid, s);
  else if (order == 3) e = launch_fold_chain<3>(a, grid, s);
  else if (order == 4) e = launch_fold_chain<4>(a, grid, s);
  else e = launch_fold_chain<5>(a, grid, s);
  if (e != cudaSuccess) return e;
  return cudaGetLastError();
}

// one warp per chunk of kKexpChunk consecutive nonzeros, lane i taking nonzeros
// i, i+32, ... of it (stores of a warp instruction are consecutive): a lane finds
// the fiber of its first nonzero by binary search over pos2, then moves forward
// through the fiber ends (a fiber of any length is spread over many warps)
constexpr int kKexpChunk = 2048;
__global__ void flat_kexp_kernel(const int32_t* __restrict__ crd1, const int32_t* __restrict__ pos2, int64_t nf1,
                                 int32_t* __restrict__ kexp) {
  const int64_t nnz = pos2[nf1];
  const int64_t nchunks = (nnz + kKexpChunk - 1) / kKexpChunk;
  const int lane = threadIdx.x & 31;
  const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t ch = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); ch < nchunks; ch += warps) {
    const int64_t p0 = ch * kKexpChunk + lane, p1 = min(nnz, (ch + 1) * kKexpChunk);
    if (p0 >= p1) continue;
    int64_t f = search_le(pos2, 0, nf1 - 1, p0);  // last fiber starting at or before p0
    int64_t fend = pos2[f + 1];
    for (int64_t p = p0; p < p1; p += 32) {
      while (p >= fend) {  // empty fibers are skipped too
        f++;
        fend = pos2[f + 1];
      }
      kexp[p] = crd1[f];
    }
  }
}

__global__ void flat_rnz_kernel(const int32_t* __restrict__ pos1, const int32_t* __restrict__ pos2,
                                const int32_t* __restrict__ pos3, const int32_t* __restrict__ pos4, int64_t nroot,
                                int32_t* __restrict__ rnz, int64_t off) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i <= nroot; i += (int64_t)gridDim.x * blockDim.x) {
    int32_t f = pos2[pos1[i]];
    if (pos3) f = pos3[f];
    if (pos4) f = pos4[f];
    rnz[i] = (int32_t)(off + f);
  }
}

namespace {
int flat_grid(int64_t m) { return (int)std::max<int64_t>(1, std::min<int64_t>((m + 255) / 256, 152 * 16)); }
}  // namespace

cudaError_t launch_expand(const int32_t* per_fiber, const int32_t* pos, int64_t nf, int64_t n, int32_t* out,
                          cudaStream_t s) {
  if (nf > 0 && n > 0)  // one warp per chunk: 8 chunks per 256-thread block
    flat_kexp_kernel<<<flat_grid(((n + kKexpChunk - 1) / kKexpChunk) * 32), 256, 0, s>>>(per_fiber, pos, nf, out);
  return cudaGetLastError();
}

cudaError_t launch_row_starts(const int32_t* pos1, const int32_t* pos2, const int32_t* pos3, int64_t nroot,
                              int32_t* rnz, cudaStream_t s, int64_t off, const int32_t* pos4) {
  flat_rnz_kernel<<<flat_grid(nroot + 1), 256, 0, s>>>(pos1, pos2, pos3, pos4, nroot, rnz, off);
  return cudaGetLastError();
}

// Dynamic shared memory above 48 KB needs a per-kernel, per-device opt-in: recorded
// per instantiation so that it is asked for once.
template <int VK, bool XS, bool V8>
cudaError_t launch_ttv_range_k(const WalkArgs& a, size_t smem, int grid, cudaStream_t s) {
  static std::atomic<size_t> allowed[64];
  auto k = ttv_range_kernel<VK, XS, V8>;
  if (smem > 48 * 1024) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
    if (allowed[dev].load(std::memory_order_acquire) < smem) {
      e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      if (e != cudaSuccess) return e;
      allowed[dev].store(smem, std::memory_order_release);
    }
  }
  k<<<grid, 32 * kTtvWarps, smem, s>>>(a);
  return cudaGetLastError();
}

template <int VK>
cudaError_t launch_ttv_range_vk(const WalkArgs& a, bool xs, size_t smem, int grid, cudaStream_t s) {
  // 32-byte stream loads when both streams start on 32-byte boundaries (every
  // lane's run then does: it begins a multiple of 16 entries in)
  const bool v8 = ((uintptr_t)a.crd[1] & 31) == 0 && ((uintptr_t)a.vals & 31) == 0;
  if (v8) return xs ? launch_ttv_range_k<VK, true, true>(a, smem, grid, s) : launch_ttv_range_k<VK, false, true>(a, smem, grid, s);
  return xs ? launch_ttv_range_k<VK, true, false>(a, smem, grid, s) : launch_ttv_range_k<VK, false, false>(a, smem, grid, s);
}

// The range walk: a.nblocks ranges of a.wcap units, kTtvWarps ranges per block; x
// goes to shared memory when it fits beside the flags.
cudaError_t launch_ttv_ranges(const WalkArgs& a, int vals_kind, cudaStream_t s) {
  if (a.nblocks == 0) return cudaSuccess;
  if (a.wcap < 1 || a.wcap > kTtvMaxRU) return cudaErrorInvalidValue;
  int dev = 0, optin = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  if (e != cudaSuccess) return e;
  const size_t flags = (size_t)kTtvWarps * (32 * kTtvNpt + kTtvYStage * sizeof(float));  // flags and fiber stages
  const size_t with_x = flags + (size_t)a.fac_rows[0] * sizeof(float);
  const bool xs = with_x <= (size_t)optin;
  const size_t smem = xs ? with_x : flags;
  const int grid = (a.nblocks + kTtvWarps - 1) / kTtvWarps;
  if (vals_kind == kB16) return launch_ttv_range_vk<kB16>(a, xs, smem, grid, s);
  if (vals_kind == kH16) return launch_ttv_range_vk<kH16>(a, xs, smem, grid, s);
  return launch_ttv_range_vk<kF32>(a, xs, smem, grid, s);
}


// ---------------------------------------------------------------------------
// CSF structure check of one level on the plan's device copies (after upload;
// the host checks the compressed root and every pos[0]).  err[0] keeps the first
// pos violation, err[1] the first crd violation, each as (index << 3) | code
// (atomicMin: the lowest index wins; UINT64_MAX: none):
//   1 pos[f + 1] < pos[f]   2 empty inner fiber   (index: fiber f)
//   3 crd outside [0, dim)  4 crd not increasing inside a fiber   (index: position p)
// The pos pass marks every fiber start in [0, n) in a bit mask; the crd pass
// compares crd[p] with crd[p - 1] where p starts no fiber.  Every access is in
// bounds whatever the arrays hold.
// ---------------------------------------------------------------------------
__global__ void csf_pos_check_kernel(const int32_t* __restrict__ pos, int64_t nf, int64_t n, int inner,
                                     uint32_t* __restrict__ starts, unsigned long long* __restrict__ err) {
  for (int64_t f = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; f < nf; f += (int64_t)gridDim.x * blockDim.x) {
    const int32_t a = pos[f], b = pos[f + 1];
    if (b < a) atomicMin(err, ((unsigned long long)f << 3) | 1ull);
    else if (inner && b == a) atomicMin(err, ((unsigned long long)f << 3) | 2ull);
    if (a >= 0 && (int64_t)a < n) atomicOr(&starts[a >> 5], 1u << (a & 31));
  }
}

__global__ void csf_crd_check_kernel(const int32_t* __restrict__ crd, int64_t n, int32_t dim,
                                     const uint32_t* __restrict__ starts, unsigned long long* __restrict__ err) {
  for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < n; p += (int64_t)gridDim.x * blockDim.x) {
    const int32_t c = crd[p];
    if (c < 0 || c >= dim) {
      atomicMin(err, ((unsigned long long)p << 3) | 3ull);
    } else if (p > 0 && !((starts[p >> 5] >> (p & 31)) & 1u) && c <= crd[p - 1]) {
      atomicMin(err, ((unsigned long long)p << 3) | 4ull);
    }
  }
}

// The crd pass over positions [p0, p1) of a level that arrives in pieces (the
// one-shot call's leaf coordinates): the same checks, and with `clamp` an
// out-of-range coordinate is also overwritten with 0, so that a walk launched
// after this pass on the same stream gathers only rows inside the factor (the
// call then reports the recorded violation and discards its result).  Position
// p0 - 1 must have arrived (and been checked) before.
__global__ void csf_crd_check_range_kernel(int32_t* __restrict__ crd, int64_t p0, int64_t p1, int32_t dim,
                                           const uint32_t* __restrict__ starts, unsigned long long* __restrict__ err,
                                           int clamp) {
  for (int64_t p = p0 + (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < p1; p += (int64_t)gridDim.x * blockDim.x) {
    const int32_t c = crd[p];
    if (c < 0 || c >= dim) {
      atomicMin(err, ((unsigned long long)p << 3) | 3ull);
      if (clamp) crd[p] = 0;
    } else if (p > 0 && !((starts[p >> 5] >> (p & 31)) & 1u) && c <= crd[p - 1]) {
      atomicMin(err, ((unsigned long long)p << 3) | 4ull);
    }
  }
}

static int check_grid(int64_t m) { return (int)std::min<int64_t>((m + 255) / 256, 152 * 16); }

cudaError_t launch_csf_pos_check(const int32_t* pos, int64_t nf, int inner, int64_t n, uint32_t* starts,
                                 unsigned long long* err, cudaStream_t s) {
  cudaError_t e = cudaMemsetAsync(starts, 0, sizeof(uint32_t) * (size_t)((n + 31) / 32 + 1), s);
  if (e != cudaSuccess) return e;
  if (nf > 0) csf_pos_check_kernel<<<check_grid(nf), 256, 0, s>>>(pos, nf, n, inner, starts, err);
  return cudaGetLastError();
}

cudaError_t launch_csf_crd_check_range(int32_t* crd, int64_t p0, int64_t p1, int32_t dim, const uint32_t* starts,
                                       unsigned long long* err, int clamp, cudaStream_t s) {
  if (p1 > p0) csf_crd_check_range_kernel<<<check_grid(p1 - p0), 256, 0, s>>>(crd, p0, p1, dim, starts, err, clamp);
  return cudaGetLastError();
}

cudaError_t launch_csf_check(const int32_t* pos, int64_t nf, int inner, const int32_t* crd, int64_t n, int32_t dim,
                             uint32_t* starts, unsigned long long* err, cudaStream_t s) {
  cudaError_t e = launch_csf_pos_check(pos, nf, inner, n, starts, err, s);
  if (e != cudaSuccess) return e;
  if (n > 0) csf_crd_check_kernel<<<check_grid(n), 256, 0, s>>>(crd, n, dim, starts, err + 1);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// storage conversion (factors to BF16 with power-of-two column scales)
// ---------------------------------------------------------------------------
__global__ void colmax_kernel(const float* __restrict__ x, int64_t rows, int cols, float* colmax) {
  // one thread per (row-slab, column); the block's slabs are reduced in shared
  // memory first, so each block adds one atomic per column (|x| >= 0, so the
  // unsigned compare of the bits orders it)
  __shared__ float s_m[256];
  const int j = threadIdx.x % cols;
  const int lanes = blockDim.x / cols;
  const int l = threadIdx.x / cols;
  float m = 0.f;
  if (l < lanes) {
    for (int64_t r = (int64_t)blockIdx.x * lanes + l; r < rows; r += (int64_t)gridDim.x * lanes) {
      const float v = fabsf(x[r * cols + j]);
      m = v > m ? v : m;  // NaN ignored
    }
  }
  s_m[threadIdx.x] = m;
  __syncthreads();
  for (int h = lanes / 2; h > 0; h >>= 1) {  // lanes is a power of two
    if (l < h) {
      const float o = s_m[threadIdx.x + h * cols];
      if (o > s_m[threadIdx.x]) s_m[threadIdx.x] = o;
    }
    __syncthreads();
  }
  if (l == 0) atomicMax(reinterpret_cast<unsigned int*>(colmax) + j, __float_as_uint(s_m[threadIdx.x]));
}

cudaError_t launch_colmax(const float* x, int64_t rows, int cols, float* colmax, cudaStream_t s) {
  cudaError_t e = cudaMemsetAsync(colmax, 0, sizeof(float) * (size_t)cols, s);
  if (e != cudaSuccess) return e;
  if (rows == 0) return cudaSuccess;
  if (cols < 1 || cols > 256) return cudaErrorInvalidValue;  // one block holds every column
  int lanes = 1;  // rows per block pass: the largest power of two with lanes * cols <= 256
  while (2 * lanes * cols <= 256) lanes *= 2;
  const int tb = lanes * cols;
  int64_t grid = (rows + lanes * 32 - 1) / (lanes * 32);
  if (grid > 4096) grid = 4096;
  colmax_kernel<<<(int)grid, tb, 0, s>>>(x, rows, cols, colmax);
  return cudaGetLastError();
}

__global__ void pow2_scales_kernel(const float* colmax, int cols, int target_exp, float* scale, float* inv) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= cols) return;
  const uint32_t bits = __float_as_uint(colmax[j]);
  const int ex = (int)((bits >> 23) & 0xff);  // biased exponent of the column max
  float sc = 1.f, iv = 1.f;
  if (ex != 0 && ex != 0xff) {
    // column max in [2^E, 2^(E+1)), E = ex - 127: scale = 2^(T-E) puts it in
    // [2^T, 2^(T+1)), inv = 2^(E-T) undoes it.  Both exact powers of two in FP32.
    const int es = 127 + target_exp - (ex - 127);  // biased exponent of 2^(T-E)
    const int ei = ex - target_exp;                 // biased exponent of 2^(E-T)
    if (es >= 1 && es <= 254 && ei >= 1 && ei <= 254) {
      sc = __uint_as_float((uint32_t)es << 23);
      iv = __uint_as_float((uint32_t)ei << 23);
    }
  }
  scale[j] = sc;
  inv[j] = iv;
}

cudaError_t launch_pow2_scales(const float* colmax, int cols, int target_exp, float* scale, float* inv,
                               cudaStream_t s) {
  pow2_scales_kernel<<<(cols + 63) / 64, 64, 0, s>>>(colmax, cols, target_exp, scale, inv);
  return cudaGetLastError();
}

__global__ void to_16_kernel(const float* __restrict__ src, int64_t rows, int cols, int rp,
                             const float* __restrict__ scale, int kind, uint16_t* __restrict__ dst) {
  const int64_t n = rows * rp;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = i / rp;
    const int j = (int)(i - r * rp);
    const float v = j < cols ? src[r * cols + j] * (scale ? scale[j] : 1.f) : 0.f;
    dst[i] = kind == 2 ? __half_as_ushort(__float2half_rn(v)) : __bfloat16_as_ushort(__float2bfloat16_rn(v));
  }
}

// Full-range fixed-point scales: scale[j] = 32767 / colmax[j], inv[j] = colmax[j] / 32767
// (1 where colmax is 0 or not finite), so each column's max maps to 32767.
__global__ void fullrange_scales_kernel(const float* colmax, int cols, float* scale, float* inv) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= cols) return;
  const float m = colmax[j];
  const bool ok = m > 0.f && m <= 3.4e38f;
  scale[j] = ok ? (float)(32767.0 / (double)m) : 1.f;
  inv[j] = ok ? (float)((double)m / 32767.0) : 1.f;
}

cudaError_t launch_fullrange_scales(const float* colmax, int cols, float* scale, float* inv, cudaStream_t s) {
  fullrange_scales_kernel<<<(cols + 63) / 64, 64, 0, s>>>(colmax, cols, scale, inv);
  return cudaGetLastError();
}

// 16-bit fixed point of the leaf factor, one warp per row: x = src * scale[col]
// (column max -> 32767), then the row's power of two e (0..40) that puts its
// largest |x| in [16384, 32767]; q = rint(x * 2^e) stored offset-binary (q + 32768),
// zero for cols <= j < rp; rowexp[r] = e.
__global__ void fx16_rows_kernel(const float* __restrict__ src, int64_t rows, int cols, int rp,
                                 const float* __restrict__ scale, uint16_t* __restrict__ dst,
                                 int8_t* __restrict__ rowexp) {
  const int lane = threadIdx.x & 31;
  const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t r = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); r < rows; r += warps) {
    float x[2];
    float m = 0.f;
#pragma unroll
    for (int h = 0; h < 2; h++) {
      const int j = lane + 32 * h;
      x[h] = j < cols ? src[r * cols + j] * scale[j] : 0.f;
      if (!(fabsf(x[h]) <= 3.4e38f)) x[h] = 0.f;  // non-finite entries are stored as 0
      m = fmaxf(m, fabsf(x[h]));
    }
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, d));
    int e = 0;
    while (e < 40 && m > 0.f && m * 2.f <= 32767.f) {
      m *= 2.f;
      e++;
    }
    const float f = __uint_as_float((uint32_t)(127 + e) << 23);  // 2^e
#pragma unroll
    for (int h = 0; h < 2; h++) {
      const int j = lane + 32 * h;
      if (j < rp) {
        const float q = fminf(fmaxf(rintf(x[h] * f), -32767.f), 32767.f);
        dst[r * rp + j] = (uint16_t)((int)q + 32768);
      }
    }
    if (lane == 0) rowexp[r] = (int8_t)e;
  }
}

cudaError_t launch_fx16_rows(const float* src, int64_t rows, int cols, int rp, const float* scale, uint16_t* dst,
                             int8_t* rowexp, cudaStream_t s) {
  if (rows == 0) return cudaSuccess;
  if (cols < 1 || cols > 64 || rp > 64) return cudaErrorInvalidValue;
  fx16_rows_kernel<<<(int)std::min<int64_t>((rows + 7) / 8, 152 * 64), 256, 0, s>>>(src, rows, cols, rp, scale, dst,
                                                                                    rowexp);
  return cudaGetLastError();
}

// out[p] = vals[p] * 2^-rowexp[leaf[p]]: an exact power-of-two scaling (padding
// entries have value 0 and leaf coordinate 0).
__global__ void fx16_values_kernel(const float* __restrict__ vals, const int32_t* __restrict__ leaf,
                                   const int8_t* __restrict__ rowexp, int64_t n, float* __restrict__ out) {
  for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < n; p += (int64_t)gridDim.x * blockDim.x)
    out[p] = ldexpf(vals[p], -(int)rowexp[leaf[p]]);
}

cudaError_t launch_fx16_values(const float* vals, const int32_t* leaf, const int8_t* rowexp, int64_t n, float* out,
                               cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  fx16_values_kernel<<<(int)std::min<int64_t>((n + 255) / 256, 152 * 32), 256, 0, s>>>(vals, leaf, rowexp, n, out);
  return cudaGetLastError();
}

cudaError_t launch_to_16(const float* src, int64_t rows, int cols, int rp, const float* scale, int kind,
                         uint16_t* dst, cudaStream_t s) {
  const int64_t n = rows * rp;
  if (n == 0) return cudaSuccess;
  int64_t grid = (n + 255) / 256;
  if (grid > 152 * 32) grid = 152 * 32;
  to_16_kernel<<<(int)grid, 256, 0, s>>>(src, rows, cols, rp, scale, kind, dst);
  return cudaGetLastError();
}

__global__ void pad_fp32_kernel(const float* __restrict__ src, int64_t rows, int cols, int rp, float* __restrict__ dst) {
  const int64_t n = rows * rp;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = i / rp;
    const int j = (int)(i - r * rp);
    dst[i] = j < cols ? src[r * cols + j] : 0.f;
  }
}

cudaError_t launch_pad_fp32(const float* src, int64_t rows, int cols, int rp, float* dst, cudaStream_t s) {
  const int64_t n = rows * rp;
  if (n == 0) return cudaSuccess;
  int64_t grid = (n + 255) / 256;
  if (grid > 152 * 32) grid = 152 * 32;
  pad_fp32_kernel<<<(int)grid, 256, 0, s>>>(src, rows, cols, rp, dst);
  return cudaGetLastError();
}

struct InvPtrs { const float* p[4]; };

__global__ void scale_product_kernel(InvPtrs inv, int nm, int rp, float vinv, float* out) {
  const int j = threadIdx.x;
  if (j >= rp) return;
  float v = vinv;
  for (int m = 0; m < nm; m++) v *= inv.p[m] ? inv.p[m][j] : 1.f;
  out[j] = v;
}

cudaError_t launch_scale_product(const float* const* inv, int nm, int rp, float vinv, float* out, cudaStream_t s) {
  InvPtrs ip{};
  for (int m = 0; m < nm && m < 4; m++) ip.p[m] = inv[m];
  scale_product_kernel<<<1, 64, 0, s>>>(ip, nm, rp, vinv, out);
  return cudaGetLastError();
}

}  // namespace tt
