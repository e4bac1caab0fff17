// tt_build.cu -- the canonical CSF built on the GPU from COO coordinates.
//
// Same result as the host builder (tt_csf_from_coo in tt_host.cpp), bit for bit:
// coordinates packed into 64-bit keys (mode 0 most significant), a stable LSD
// radix sort of (key, input index), duplicates summed in FP64 in input order,
// then every CSF level from prefix sums of "a new fiber starts here" flags.
// It replaces the reference's SPLATT loader step (splatt_csf_load, ds.h:351-366)
// in a file-to-CSF pipeline: FROSTT coordinates in, canonical CSF out.
//
// Every kernel indexes through grid-stride loops or tiles bounded by n; the radix
// scatter also checks each target position against n and records a violation
// instead of writing.
#include <cuda_runtime.h>
#include <algorithm>
#include <cstring>
#include <vector>
#include "tt_internal.h"
#include "tt_kernels.h"

namespace tt {
namespace {

constexpr int kThreads = 256;
constexpr int kRounds = 16;                  // keys per thread per tile
constexpr int kTile = kThreads * kRounds;    // keys per block tile
constexpr unsigned kFull = 0xffffffffu;

struct PackDev {
  int order;
  int shift[TT_MAX_ORDER];
  int bits[TT_MAX_ORDER];
  int32_t dims[TT_MAX_ORDER];
};

__device__ __forceinline__ int32_t key_get(uint64_t k, const PackDev& pk, int m) {
  return (int32_t)((k >> pk.shift[m]) & ((1ull << pk.bits[m]) - 1));
}

int grid_for(int64_t n) { return (int)std::max<int64_t>(1, std::min<int64_t>((n + kThreads - 1) / kThreads, 152 * 16)); }

// keys[p] = packed coordinates of nonzero p, idx[p] = p; a coordinate outside
// [0, dims[m]) sets err[0] (the keys are then not used)
__global__ void pack_kernel(const int32_t* __restrict__ coords, int64_t n, PackDev pk, uint64_t* __restrict__ keys,
                            uint32_t* __restrict__ idx, int* err) {
  for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < n; p += (int64_t)gridDim.x * blockDim.x) {
    uint64_t k = 0;
    bool ok = true;
    for (int m = 0; m < pk.order; m++) {
      const int32_t c = coords[p * pk.order + m];
      ok = ok && c >= 0 && c < pk.dims[m];
      k |= (uint64_t)(uint32_t)c << pk.shift[m];
    }
    if (!ok) atomicExch(err, 1);
    keys[p] = k;
    idx[p] = (uint32_t)p;
  }
}

// ---- stable LSD radix sort, 8-bit digits -------------------------------------
// hist[d * nblocks + b]: keys of tile b with digit d
__global__ void radix_hist_kernel(const uint64_t* __restrict__ keys, int64_t n, int shift, uint32_t* __restrict__ hist) {
  __shared__ uint32_t h[256];
  h[threadIdx.x] = 0;
  __syncthreads();
  const int64_t base = (int64_t)blockIdx.x * kTile;
  for (int r = 0; r < kRounds; r++) {
    const int64_t p = base + (int64_t)r * kThreads + threadIdx.x;
    if (p < n) atomicAdd(&h[(keys[p] >> shift) & 255u], 1u);
  }
  __syncthreads();
  hist[(size_t)threadIdx.x * gridDim.x + blockIdx.x] = h[threadIdx.x];
}

// offs: exclusive scan of hist in digit-major order.  Round r of tile b places
// keys base + r*256 + t in t order: rank inside the warp from __match_any_sync,
// warps in order through per-warp digit counts, rounds in order through run[].
__global__ void radix_scatter_kernel(const uint64_t* __restrict__ kin, const uint32_t* __restrict__ vin, int64_t n,
                                     int shift, const uint32_t* __restrict__ offs, uint64_t* __restrict__ kout,
                                     uint32_t* __restrict__ vout, int* err) {
  __shared__ uint32_t wc[kThreads / 32][256];
  __shared__ uint32_t run[256];
  const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
  run[t] = offs[(size_t)t * gridDim.x + blockIdx.x];
  const int64_t base = (int64_t)blockIdx.x * kTile;
  for (int r = 0; r < kRounds; r++) {
#pragma unroll
    for (int w = 0; w < kThreads / 32; w++) wc[w][t] = 0;
    __syncthreads();
    const int64_t p = base + (int64_t)r * kThreads + t;
    const bool valid = p < n;
    const uint64_t k = valid ? kin[p] : 0ull;
    const uint32_t v = valid ? vin[p] : 0u;
    const int d = valid ? (int)((k >> shift) & 255u) : 256 + lane;  // lanes past n match nobody
    const unsigned peers = __match_any_sync(kFull, d);
    const int lower = __popc(peers & ((1u << lane) - 1u));
    if (valid && lower == 0) wc[warp][d] = (uint32_t)__popc(peers);
    __syncthreads();
    uint32_t acc = 0;  // this thread's digit t: exclusive prefix over the warps
#pragma unroll
    for (int w = 0; w < kThreads / 32; w++) {
      const uint32_t c = wc[w][t];
      wc[w][t] = acc;
      acc += c;
    }
    __syncthreads();
    if (valid) {
      const uint64_t q = (uint64_t)run[d] + wc[warp][d] + (uint32_t)lower;
      if (q < (uint64_t)n) {
        kout[q] = k;
        vout[q] = v;
      } else {
        atomicExch(err, 2);
      }
    }
    __syncthreads();
    run[t] += acc;
  }
}

// ---- exclusive prefix sum of uint32 (totals below 2^32) ----------------------
__global__ void scan_tile_sums_kernel(const uint32_t* __restrict__ in, int64_t n, uint32_t* __restrict__ sums) {
  __shared__ uint32_t s[kThreads];
  const int64_t base = (int64_t)blockIdx.x * kTile + (int64_t)threadIdx.x * kRounds;
  uint32_t a = 0;
  for (int i = 0; i < kRounds; i++)
    if (base + i < n) a += in[base + i];
  s[threadIdx.x] = a;
  __syncthreads();
  for (int h = kThreads / 2; h > 0; h >>= 1) {
    if (threadIdx.x < h) s[threadIdx.x] += s[threadIdx.x + h];
    __syncthreads();
  }
  if (threadIdx.x == 0) sums[blockIdx.x] = s[0];
}

// one block of 1024 threads: sums[0..nb) -> exclusive prefixes, total in sums[nb]
__global__ void scan_sums_kernel(uint32_t* sums, int64_t nb) {
  __shared__ uint32_t s[1024];
  const int t = threadIdx.x;
  const int64_t per = (nb + 1023) / 1024;
  const int64_t lo = std::min<int64_t>(nb, t * per), hi = std::min<int64_t>(nb, lo + per);
  uint32_t a = 0;
  for (int64_t i = lo; i < hi; i++) a += sums[i];
  s[t] = a;
  __syncthreads();
  for (int d = 1; d < 1024; d <<= 1) {  // inclusive Hillis-Steele scan
    const uint32_t u = t >= d ? s[t - d] : 0u;
    __syncthreads();
    s[t] += u;
    __syncthreads();
  }
  uint32_t run = s[t] - a;
  for (int64_t i = lo; i < hi; i++) {
    const uint32_t c = sums[i];
    sums[i] = run;
    run += c;
  }
  if (t == 1023) sums[nb] = s[1023];
}

__global__ void scan_tile_kernel(const uint32_t* __restrict__ in, int64_t n, const uint32_t* __restrict__ sums,
                                 uint32_t* __restrict__ out) {
  __shared__ uint32_t s[kThreads];
  const int64_t base = (int64_t)blockIdx.x * kTile + (int64_t)threadIdx.x * kRounds;
  uint32_t a = 0;
  for (int i = 0; i < kRounds; i++)
    if (base + i < n) a += in[base + i];
  s[threadIdx.x] = a;
  __syncthreads();
  for (int d = 1; d < kThreads; d <<= 1) {
    const uint32_t u = threadIdx.x >= (unsigned)d ? s[threadIdx.x - d] : 0u;
    __syncthreads();
    s[threadIdx.x] += u;
    __syncthreads();
  }
  uint32_t run = sums[blockIdx.x] + s[threadIdx.x] - a;
  for (int i = 0; i < kRounds; i++)
    if (base + i < n) {
      const uint32_t c = in[base + i];
      out[base + i] = run;
      run += c;
    }
}

// ---- CSF construction -----------------------------------------------------------
__global__ void run_flags_kernel(const uint64_t* __restrict__ keys, int64_t n, uint32_t* __restrict__ first) {
  for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < n; p += (int64_t)gridDim.x * blockDim.x)
    first[p] = (p == 0 || keys[p] != keys[p - 1]) ? 1u : 0u;
}

// each run of equal keys: its values (input order) summed in FP64
__global__ void runs_kernel(const uint64_t* __restrict__ keys, const uint32_t* __restrict__ idx,
                            const float* __restrict__ vals, const uint32_t* __restrict__ first,
                            const uint32_t* __restrict__ ridx, int64_t n, uint64_t* __restrict__ ukeys,
                            float* __restrict__ uvals) {
  for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < n; p += (int64_t)gridDim.x * blockDim.x) {
    if (!first[p]) continue;
    double s = 0.0;
    int64_t q = p;
    do {
      s += (double)vals[idx[q]];
      q++;
    } while (q < n && !first[q]);
    ukeys[ridx[p]] = keys[p];
    uvals[ridx[p]] = (float)s;
  }
}

// flags[l][r] = 1 when unique key r opens a new fiber at level l (1 <= l < order):
// it differs from key r-1 at some level <= l
__global__ void level_flags_kernel(const uint64_t* __restrict__ ukeys, int64_t m, PackDev pk, uint32_t* __restrict__ flags) {
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < m; r += (int64_t)gridDim.x * blockDim.x) {
    int nl = 0;
    if (r > 0) {
      nl = pk.order;
      const uint64_t diff = ukeys[r] ^ ukeys[r - 1];
      for (int l = 0; l < pk.order; l++)
        if ((diff >> pk.shift[l]) & ((1ull << pk.bits[l]) - 1)) { nl = l; break; }
    }
    for (int l = 1; l < pk.order; l++) flags[(size_t)(l - 1) * m + r] = nl <= l ? 1u : 0u;
  }
}

// crd[l][fidx_l[r]] = coordinate l; pos[l+1][fidx_l[r]] = fidx_{l+1}[r]; frow
// (root coordinate of every level-1 fiber)
__global__ void levels_kernel(const uint64_t* __restrict__ ukeys, int64_t m, PackDev pk, const uint32_t* __restrict__ flags,
                              const uint32_t* __restrict__ fidx, int32_t* crd1, int32_t* crd2, int32_t* crd3,
                              int32_t* crd4, int32_t* pos2, int32_t* pos3, int32_t* pos4, int32_t* __restrict__ frow) {
  int32_t* crd[TT_MAX_ORDER] = {nullptr, crd1, crd2, crd3, crd4};
  int32_t* pos[TT_MAX_ORDER] = {nullptr, nullptr, pos2, pos3, pos4};
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < m; r += (int64_t)gridDim.x * blockDim.x) {
    for (int l = 1; l < pk.order; l++) {
      if (!flags[(size_t)(l - 1) * m + r]) continue;
      const uint32_t f = fidx[(size_t)(l - 1) * m + r];
      crd[l][f] = key_get(ukeys[r], pk, l);
      if (l == 1) frow[f] = key_get(ukeys[r], pk, 0);
      if (l + 1 < pk.order) pos[l + 1][f] = (int32_t)fidx[(size_t)l * m + r];
    }
  }
}

// pos1[i] = level-1 fibers in rows below i (frow is sorted)
__global__ void root_pos_kernel(const int32_t* __restrict__ frow, int64_t nf, int32_t rows, int32_t* __restrict__ pos1) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i <= rows; i += (int64_t)gridDim.x * blockDim.x) {
    int64_t lo = 0, hi = nf;
    while (lo < hi) {
      const int64_t mid = (lo + hi) >> 1;
      if (frow[mid] < (int32_t)i) lo = mid + 1;
      else hi = mid;
    }
    pos1[i] = (int32_t)lo;
  }
}

// Device buffers from the library's pool (on the legacy default stream, which the
// builder works on), handed back at scope exit, like all of the library's device
// memory: driver-level allocation and release between plans (measured on the
// candidate timing's placeholders) slowed the kernels of a later plan.
struct DevBufs {
  std::vector<void*> p;
  template <typename T>
  cudaError_t get(T** out, size_t count) {
    *out = nullptr;
    cudaError_t e = device_pool_alloc((void**)out, std::max<size_t>(count, 1) * sizeof(T), nullptr);
    if (e == cudaSuccess) p.push_back((void*)*out);
    return e;
  }
  ~DevBufs() {
    for (void* q : p) device_pool_free(q, nullptr);
    cudaStreamSynchronize(nullptr);
  }
};

// Exclusive scan of n uint32 into out; *total gets the sum.
cudaError_t exclusive_scan(const uint32_t* in, int64_t n, uint32_t* out, uint32_t* sums, uint32_t* total, cudaStream_t st) {
  const int64_t nb = (n + kTile - 1) / kTile;
  if (nb == 0) { *total = 0; return cudaSuccess; }
  scan_tile_sums_kernel<<<(unsigned)nb, kThreads, 0, st>>>(in, n, sums);
  scan_sums_kernel<<<1, 1024, 0, st>>>(sums, nb);
  scan_tile_kernel<<<(unsigned)nb, kThreads, 0, st>>>(in, n, sums, out);
  cudaError_t e = cudaMemcpyAsync(total, sums + nb, sizeof(uint32_t), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  return e == cudaSuccess ? cudaGetLastError() : e;
}

}  // namespace

// Exclusive scan of n uint32 on the device (out may alias in); *total (host) gets
// the sum; sums: scratch of scan_scratch_entries(n) uint32.  Synchronises st.
int64_t scan_scratch_entries(int64_t n) { return (n + kTile - 1) / kTile + 1; }
cudaError_t device_exclusive_scan(const uint32_t* in, int64_t n, uint32_t* out, uint32_t* sums, uint32_t* total,
                                  cudaStream_t st) {
  return exclusive_scan(in, n, out, sums, total, st);
}
}  // namespace tt

using namespace tt;

#define CKB(expr)                                                                                    \
  do {                                                                                               \
    cudaError_t e_ = (expr);                                                                         \
    if (e_ != cudaSuccess)                                                                           \
      return set_error(e_ == cudaErrorMemoryAllocation ? TT_ERR_OUT_OF_MEMORY : TT_ERR_CUDA, "%s: %s", \
                       #expr, cudaGetErrorString(e_));                                                \
  } while (0)

TT_EXPORT tt_status tt_csf_from_coo_gpu(int32_t order, const int32_t* dims, int64_t nnz, const int32_t* coords,
                                        const float* vals, taco_tensor_t** out) {
  clear_error();
  if (!out || !dims || (nnz > 0 && (!coords || !vals))) return set_error(TT_ERR_INVALID_ARGUMENT, "null argument");
  *out = nullptr;
  if (order < 2 || order > TT_MAX_ORDER) return set_error(TT_ERR_UNSUPPORTED, "order %d", order);
  if (nnz < 0 || nnz > 0x7fffffffLL) return set_error(TT_ERR_UNSUPPORTED, "nnz %lld (int32 positions)", (long long)nnz);
  for (int m = 0; m < order; m++)
    if (dims[m] <= 0) return set_error(TT_ERR_INVALID_ARGUMENT, "dims[%d] = %d", m, dims[m]);
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    return set_error(TT_ERR_NO_DEVICE, "no CUDA device visible");
  }
  PackDev pk{};
  pk.order = order;
  {
    int total = 0;
    for (int m = order - 1; m >= 0; m--) {
      int b = 1;
      while ((1ll << b) < dims[m]) b++;
      pk.bits[m] = b;
      pk.shift[m] = total;
      pk.dims[m] = dims[m];
      total += b;
    }
    if (total > 63) return set_error(TT_ERR_UNSUPPORTED, "coordinates need %d bits (> 63)", total);
  }
  const int key_bits = pk.shift[0] + pk.bits[0];
  const int64_t n = nnz;
  cudaStream_t st = nullptr;
  DevBufs db;
  int32_t* dco = nullptr;
  float* dvals = nullptr;
  uint64_t *k0 = nullptr, *k1 = nullptr;
  uint32_t *i0 = nullptr, *i1 = nullptr;
  int* derr = nullptr;
  CKB(db.get(&dco, (size_t)n * order));
  CKB(db.get(&dvals, (size_t)n));
  CKB(db.get(&k0, (size_t)n));
  CKB(db.get(&k1, (size_t)n));
  CKB(db.get(&i0, (size_t)n));
  CKB(db.get(&i1, (size_t)n));
  CKB(db.get(&derr, 1));
  CKB(cudaMemsetAsync(derr, 0, sizeof(int), st));
  if (n > 0) {
    CKB(cudaMemcpyAsync(dco, coords, sizeof(int32_t) * (size_t)n * order, cudaMemcpyHostToDevice, st));
    CKB(cudaMemcpyAsync(dvals, vals, sizeof(float) * (size_t)n, cudaMemcpyHostToDevice, st));
    pack_kernel<<<grid_for(n), kThreads, 0, st>>>(dco, n, pk, k0, i0, derr);
    CKB(cudaGetLastError());
    int herr = 0;
    CKB(cudaMemcpyAsync(&herr, derr, sizeof(int), cudaMemcpyDeviceToHost, st));
    CKB(cudaStreamSynchronize(st));
    if (herr) return set_error(TT_ERR_INVALID_ARGUMENT, "a coordinate is out of range");
  }
  // radix sort passes over the key's bits
  const int64_t nb = (n + kTile - 1) / kTile;
  uint32_t *hist = nullptr, *sums = nullptr;
  CKB(db.get(&hist, (size_t)nb * 256));
  CKB(db.get(&sums, (size_t)(nb * 256 + kTile - 1) / kTile + 1));
  uint32_t total = 0;
  for (int shift = 0; n > 1 && shift < key_bits; shift += 8) {
    radix_hist_kernel<<<(unsigned)nb, kThreads, 0, st>>>(k0, n, shift, hist);
    CKB(cudaGetLastError());
    CKB(exclusive_scan(hist, nb * 256, hist, sums, &total, st));
    radix_scatter_kernel<<<(unsigned)nb, kThreads, 0, st>>>(k0, i0, n, shift, hist, k1, i1, derr);
    CKB(cudaGetLastError());
    std::swap(k0, k1);
    std::swap(i0, i1);
  }
  // runs of equal keys -> unique keys with FP64 sums
  uint32_t *first = nullptr, *ridx = nullptr, *rsums = nullptr;
  CKB(db.get(&first, (size_t)n));
  CKB(db.get(&ridx, (size_t)n));
  CKB(db.get(&rsums, (size_t)(n + kTile - 1) / kTile + 1));
  uint32_t m = 0;
  if (n > 0) {
    run_flags_kernel<<<grid_for(n), kThreads, 0, st>>>(k0, n, first);
    CKB(exclusive_scan(first, n, ridx, rsums, &m, st));
  }
  uint64_t* uk = k1;  // the other sort buffer holds the unique keys
  float* uv = nullptr;
  CKB(db.get(&uv, (size_t)m));
  if (n > 0) runs_kernel<<<grid_for(n), kThreads, 0, st>>>(k0, i0, dvals, first, ridx, n, uk, uv);
  // levels
  const int L = order - 1;
  uint32_t *flags = nullptr, *fidx = nullptr, *lsums = nullptr;
  CKB(db.get(&flags, (size_t)L * m));
  CKB(db.get(&fidx, (size_t)L * m));
  CKB(db.get(&lsums, (size_t)(m + kTile - 1) / kTile + 1));
  uint32_t cnt[TT_MAX_ORDER] = {0, 0, 0, 0};
  if (m > 0) {
    level_flags_kernel<<<grid_for(m), kThreads, 0, st>>>(uk, m, pk, flags);
    for (int l = 1; l <= L; l++)
      CKB(exclusive_scan(flags + (size_t)(l - 1) * m, m, fidx + (size_t)(l - 1) * m, lsums, &cnt[l], st));
  }
  int32_t* dcrd[TT_MAX_ORDER] = {nullptr, nullptr, nullptr, nullptr};
  int32_t* dpos[TT_MAX_ORDER] = {nullptr, nullptr, nullptr, nullptr};
  int32_t* frow = nullptr;
  for (int l = 1; l <= L; l++) {
    CKB(db.get(&dcrd[l], (size_t)cnt[l]));
    CKB(db.get(&dpos[l], l == 1 ? (size_t)dims[0] + 1 : (size_t)cnt[l - 1] + 1));
  }
  CKB(db.get(&frow, (size_t)cnt[1]));
  if (m > 0) {
    levels_kernel<<<grid_for(m), kThreads, 0, st>>>(uk, m, pk, flags, fidx, dcrd[1], dcrd[2], dcrd[3], dcrd[4],
                                                     dpos[2], dpos[3], dpos[4], frow);
    CKB(cudaGetLastError());
  }
  root_pos_kernel<<<grid_for((int64_t)dims[0] + 1), kThreads, 0, st>>>(frow, cnt[1], dims[0], dpos[1]);
  CKB(cudaGetLastError());
  int herr = 0;
  CKB(cudaMemcpyAsync(&herr, derr, sizeof(int), cudaMemcpyDeviceToHost, st));
  CKB(cudaStreamSynchronize(st));
  if (herr) return set_error(TT_ERR_CUDA, "radix sort placed a key outside the array (code %d)", herr);

  auto* o = new OwnedTensor();
  o->pos[1].resize((size_t)dims[0] + 1);
  cudaError_t e = cudaMemcpy(o->pos[1].data(), dpos[1], sizeof(int32_t) * ((size_t)dims[0] + 1), cudaMemcpyDeviceToHost);
  for (int l = 1; l <= L && e == cudaSuccess; l++) {
    o->crd[l].resize((size_t)cnt[l]);
    if (cnt[l] > 0) e = cudaMemcpy(o->crd[l].data(), dcrd[l], sizeof(int32_t) * cnt[l], cudaMemcpyDeviceToHost);
    if (l >= 2 && e == cudaSuccess) {
      o->pos[l].resize((size_t)cnt[l - 1] + 1);
      if (cnt[l - 1] > 0)
        e = cudaMemcpy(o->pos[l].data(), dpos[l], sizeof(int32_t) * cnt[l - 1], cudaMemcpyDeviceToHost);
      o->pos[l][cnt[l - 1]] = (int32_t)cnt[l];
    }
  }
  o->vals.resize(m);
  if (e == cudaSuccess && m > 0) e = cudaMemcpy(o->vals.data(), uv, sizeof(float) * m, cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) {
    delete o;
    return set_error(TT_ERR_CUDA, "download CSF: %s", cudaGetErrorString(e));
  }
  // compressed-root arrays for reference callers, as the host builder fills them
  o->pos[0] = {0, dims[0]};
  o->crd[0].resize((size_t)dims[0]);
  for (int32_t i = 0; i < dims[0]; i++) o->crd[0][(size_t)i] = i;
  o->publish(order, dims);
  *out = &o->t;
  return TT_OK;
}
