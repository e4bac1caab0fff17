// tt_plan.cu -- plan API of libtentaco_gb300 (see include/tentaco/tentaco.h).
//
// A plan replaces the reference's per-call staging (copy_to_device_mttkrp /
// copy_from_device_mttkrp / free_tensors_mttkrp, gpu_library.h:780-945, which
// cudaMalloc and upload every array on every call and publish the pointers in
// process-global __device__ symbols).  Here the CSF is uploaded once, into
// plan-owned buffers padded for 128-bit loads; per call only the partition
// (inside the timed region, as the reference's TIME_GPU does), the output clear
// and the walk kernel run, on the caller's stream.
#include <cuda_runtime.h>
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <vector>
#include <nvtx3/nvToolsExt.h>
#include "tt_internal.h"
#include "tt_kernels.h"
#define TT_ARGS_ONLY
#include "tt_mttkrp.cuh"
#include "tt_ttv.cuh"
#include "tt_strip.cuh"
#include "tt_plan.h"

using namespace tt;

namespace tt {

// ---------------------------------------------------------------------------
// variant table: family {lean warp tile, staged, TMA gather, flat, strip} x threads
// {256,512} x nonzeros per team (5 values per family) x columns per lane {8,4,2,1}
// ---------------------------------------------------------------------------
static const int kTB[2] = {256, 512};
static const int kGF[kFamilies][5] = {{16, 32, 64, 128, 256}, {4, 8, 16, 32, 64}, {16, 32, 64, 128, 256},
                                      {16, 32, 64, 128, 256}, {16, 32, 64, 128, 256}};
static const int kCPT[4] = {8, 4, 2, 1};
constexpr int kPerFamily = 2 * 5 * 4;
constexpr size_t kSmemLimit = (size_t)227 * 1024;

VariantSpec variant_spec(int id) {
  VariantSpec v{};
  if (id < 0 || id >= kNumVariants) return v;
  v.id = id;
  v.staged = id / kPerFamily;
  const int b = id % kPerFamily;
  v.cpt = kCPT[b % 4];
  v.G = kGF[v.staged][(b / 4) % 5];
  v.tb = kTB[b / 20];
  return v;
}

// Nearest table entry for (tb, G, cpt) in a family (G rounded to the family's list).
int variant_id(int tb, int G, int cpt, int staged) {
  int ti = tb == 512 ? 1 : 0, gi = 0, ci = 0;
  for (int i = 0; i < 5; i++) if (kGF[staged][i] <= G) gi = i;
  for (int i = 0; i < 4; i++) if (kCPT[i] == cpt) ci = i;
  return staged * kPerFamily + (ti * 5 + gi) * 4 + ci;
}

// Kernel family a variant launches: the lean family's second thread value selects
// its tighter register budget (family 3); both launch 256-thread blocks.
// The TMA family's second value selects 8 stages in flight per warp instead of 4 (family 5).
// The flat family launches family 6, or 7 with the tighter register budget.
int launch_family(const VariantSpec& v) {
  if (v.staged == 0) return v.tb == 512 ? 3 : 0;
  if (v.staged == 2) return v.tb == 512 ? 5 : 2;
  if (v.staged == 3) return v.tb == 512 ? 7 : 6;
  if (v.staged == 4) return v.tb == 512 ? 9 : 8;
  return v.staged;
}
int tma_stages(const VariantSpec& v) { return v.tb == 512 ? 8 : 4; }

// Resident 256-thread blocks a lean (or flat) variant's registers are budgeted for;
// a strip variant's: 2 (four nonzeros per team and step) or 3 (two).
int lean_blocks(const VariantSpec& v) {
  if (v.staged == 4) return v.tb == 512 ? 3 : 2;
  return v.cpt >= 4 ? (v.tb == 512 ? 3 : 2) : (v.tb == 512 ? 4 : 3);
}

// Nonzeros of one work unit: a warp's tile for the lean family, a block's tile otherwise.
int variant_unit(const VariantSpec& v, int rp) {
  const int lpr = rp / v.cpt;
  return (v.staged != 1 ? 32 / lpr : v.tb / lpr) * v.G;
}

int fac_bytes(int prec) { return fac_kind(prec) == kF32 ? 4 : 2; }

size_t variant_smem(const VariantSpec& v, int rp, int prec, int wcap, int order) {
  const int lpr = rp / v.cpt;
  const int P = (v.tb / lpr) * v.G;
  if (v.staged == 0) return (size_t)(256 / 32) * lean_warp_bytes(v.G, 32 / lpr, val_bytes(prec));
  if (v.staged == 3) return (size_t)(256 / 32) * flat_warp_bytes(v.G, 32 / lpr, val_bytes(prec), order);
  if (v.staged == 4) return (size_t)(256 / 32) * strip_warp_bytes((32 / lpr) * v.G, val_bytes(prec), order);
  if (v.staged == 2)  // TMA gather: 8 warps, each with its ring of row stages and its lean tile
    return (size_t)(256 / 32) * tma_warp_bytes(v.G, 32 / lpr, val_bytes(prec), rp * fac_bytes(prec), tma_stages(v));
  return v.staged ? stage_smem_bytes(P, wcap, v.tb, rp, val_bytes(prec), fac_bytes(prec))
                  : walk_smem_bytes(P, v.tb, rp, val_bytes(prec));
}

int val_bytes(int prec) { return val_kind(prec) == kF32 ? 4 : 2; }

int rank_pad(int R) {
  if (R <= 8) return 8;
  if (R <= 16) return 16;
  if (R <= 32) return 32;
  return 64;
}

bool variant_valid(int id, int order, int rank, int prec) {
  VariantSpec v = variant_spec(id);
  if (v.tb == 0) return false;
  const int rp = rank_pad(rank);
  if (rp % v.cpt) return false;
  const int lpr = rp / v.cpt;
  if (lpr < 1 || lpr > 32) return false;
  // the strip walk works on column pairs; 16-bit fixed point is strip-only
  if (v.staged == 4 && v.cpt < 2) return false;
  if (prec == kFX16 && v.staged != 4) return false;
  // shared memory must fit the 227 KB opt-in limit (staged: with the smallest
  // window; a plan checks its own tensor's largest window)
  if (variant_smem(v, rp, prec, 1, order) > kSmemLimit) return false;
  if (v.staged && v.staged != 4 && (rp * fac_bytes(prec)) % 16) return false;
  // TMA gather: four rows per copy land on 128-byte boundaries (rows of 32-byte
  // multiples), and a team's G nonzeros are whole stages of U = lanes-per-row rows
  if (v.staged == 2 && ((rp * fac_bytes(prec)) % 32 != 0 || v.G % lpr != 0)) return false;
  return walk_launcher(order, prec, v.cpt, lpr, launch_family(v)) != nullptr;
}

int lean_default_variant(int order, int rank, int prec);
int strip_default_variant(int order, int rank, int prec);

int default_variant(int order, int rank, int prec, int64_t nnz) {
  (void)nnz;
  // four and five modes and 16-bit fixed point: the strip rule (the fastest family
  // on the 80M-nonzero 4-mode tensor in every storage precision; the only one for
  // five modes)
  if (order >= 4 || prec == kFX16) {
    const int id = strip_default_variant(order, rank, prec);
    if (id >= 0) return id;
  }
  if (order == 3) {
    // flat family, 256 threads: the best single flat variant per (storage, rank)
    // over the training split of the selector corpus (12-28% mean regret against
    // the per-tensor sweep optimum): 4 columns per lane, or 8 for 16-bit factor
    // rows of 32 columns and more
    const int rp3 = rank_pad(rank);
    const bool f32 = fac_kind(prec) == kF32;
    const int cpt = (!f32 && rp3 >= 32) ? 8 : 4;
    const int G = rp3 <= 8 ? 16 : rp3 <= 16 ? 32 : (f32 ? 64 : 32);
    const int id = variant_id(256, G, cpt, 3);
    if (variant_valid(id, order, rank, prec)) return id;
  }
  return lean_default_variant(order, rank, prec);
}

int lean_default_variant(int order, int rank, int prec) {
  // lean family, looser register budget, 16 bytes of a factor row per lane (4 FP32
  // or 8 16-bit columns), G growing with the rank: before the flat family, the best
  // single variant per (storage, rank) over the training split of the selector
  // corpus; the rule for four modes and for slab plans
  const int rp = rank_pad(rank);
  int cpt = fac_kind(prec) == kF32 ? 4 : 8;
  while (cpt > 1 && rp / cpt < 1) cpt >>= 1;
  while (rp / cpt > 32) cpt <<= 1;
  const int G = rp <= 8 ? 16 : rp <= 16 ? 32 : rp == 32 ? (fac_kind(prec) == kF32 ? 64 : 32) : 64;
  const int id = variant_id(256, G, cpt, 0);
  if (variant_valid(id, order, rank, prec)) return id;
  for (int i = 0; i < kNumVariants; i++)
    if (variant_valid(i, order, rank, prec)) return i;
  return -1;
}

// The strip rule: G 128 with four nonzeros per team and step, 8 columns per lane
// for 16-bit factors (16 bytes of a factor row), else 4.
int strip_default_variant(int order, int rank, int prec) {
  const int rp = rank_pad(rank);
  int cpt = fac_kind(prec) == kF32 || prec == kFX16 ? 4 : 8;
  while (cpt > 2 && rp / cpt < 1) cpt >>= 1;
  const int id = variant_id(256, 128, cpt, 4);
  if (variant_valid(id, order, rank, prec)) return id;
  for (int i = 4 * kPerFamily; i < kNumVariants; i++)
    if (variant_valid(i, order, rank, prec)) return i;
  return -1;
}

// Leaf-mode slabs chosen automatically: when the leaf factor (as stored) exceeds
// 48 MB, slices of at most 44 MB, so that the slab being walked stays L2-resident
// beside the streams (129 MB of L2).  Smaller slices keep more of it resident but
// split every output row once more per slab (more row ends in the walk, more rows
// to sum): on the 100M-nonzero headline tensor 3 slabs of the 128 MB FP16 factor
// beat 2 and 4 (0.940 ms per call against 0.996 and 0.988), 6 slabs of the 256 MB
// FP32 factor beat 5 and 8 (1.386 ms against 1.428 and 1.429).  The strip walk runs
// all slabs in one launch in slab-major order (virtual rows, summed afterwards);
// the lean, staged and TMA walks run one pass per slab; the flat walk does not run
// on slab plans.
int auto_slabs(int order, int64_t leaf_dim, int rp, int prec) {
  if (order > 4) return 1;  // slab-major layouts are built for three and four modes
  const int64_t bytes = leaf_dim * (int64_t)rp * fac_bytes(prec);
  constexpr int64_t kMB = 1 << 20;
  if (bytes <= 48 * kMB) return 1;
  return (int)std::min<int64_t>(kMaxSlabs, (bytes + 44 * kMB - 1) / (44 * kMB));
}

}  // namespace tt

// ---------------------------------------------------------------------------
// helpers
// ---------------------------------------------------------------------------
#define CK(expr)                                                                          \
  do {                                                                                    \
    cudaError_t e_ = (expr);                                                              \
    if (e_ != cudaSuccess) {                                                              \
      return set_error(e_ == cudaErrorMemoryAllocation ? TT_ERR_OUT_OF_MEMORY : TT_ERR_CUDA, \
                       "%s: %s", #expr, cudaGetErrorString(e_));                         \
    }                                                                                     \
  } while (0)

namespace {

// NVTX range over a public entry point (or a phase of one): shows in Nsight
// Systems / Nsight Compute (--nvtx) when a tool is attached, a no-op otherwise.
struct NvtxRange {
  explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
  ~NvtxRange() { nvtxRangePop(); }
  NvtxRange(const NvtxRange&) = delete;
  NvtxRange& operator=(const NvtxRange&) = delete;
};

std::atomic<float> g_legacy_ms{-1.0f};

// ---------------------------------------------------------------------------
// Device memory of plans and one-shot calls comes from one stream-ordered pool
// per device, owned by the library, that keeps freed memory for reuse (release
// threshold unlimited): repeated calls on tensors of similar size then pay no
// cudaMalloc / cudaFree.  tt_release_cached_memory() hands it back.
// ---------------------------------------------------------------------------
constexpr int kMaxDevices = 64;
std::mutex g_pool_mu;
cudaMemPool_t g_pool[kMaxDevices] = {};

cudaError_t pool_of(cudaMemPool_t* out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lk(g_pool_mu);
  if (!g_pool[dev]) {
    cudaMemPoolProps props = {};
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = dev;
    cudaMemPool_t pool;
    if ((e = cudaMemPoolCreate(&pool, &props)) != cudaSuccess) return e;
    uint64_t keep = UINT64_MAX;
    if ((e = cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep)) != cudaSuccess) {
      cudaMemPoolDestroy(pool);
      return e;
    }
    g_pool[dev] = pool;
  }
  *out = g_pool[dev];
  return cudaSuccess;
}

// Failure injection and accounting of the pool (tt_debug_fail_pool_alloc,
// tt_debug_pool_live): g_fail_countdown > 0 counts allocations down to the one
// that fails; g_pool_live counts the allocations held.
std::atomic<int64_t> g_fail_countdown{0};
std::atomic<int64_t> g_pool_live{0};
std::atomic<int32_t> g_tma_withhold{0};
std::atomic<int64_t> g_tma_wait_ns{0};

tt_status broken_error() {
  return set_error(TT_ERR_INVALID_ARGUMENT, "plan unusable: a device allocation failed in an earlier call (destroy it)");
}

bool injected_failure() {
  static const bool env_read = [] {
    const char* v = getenv("TT_FAIL_POOL_ALLOC_AT");
    if (v && atoll(v) > 0) g_fail_countdown.store(atoll(v));
    return true;
  }();
  (void)env_read;
  int64_t c = g_fail_countdown.load();
  while (c > 0 && !g_fail_countdown.compare_exchange_weak(c, c - 1)) {
  }
  return c == 1;
}

// Stream-ordered allocation from the pool: usable on `st` at once, on other
// streams after `st` is synchronised.
cudaError_t pool_alloc(void** ptr, size_t bytes, cudaStream_t st) {
  *ptr = nullptr;
  if (injected_failure()) return cudaErrorMemoryAllocation;
  cudaMemPool_t pool;
  cudaError_t e = pool_of(&pool);
  if (e != cudaSuccess) return e;
  e = cudaMallocFromPoolAsync(ptr, bytes, pool, st);
  if (e == cudaSuccess) g_pool_live.fetch_add(1);
  return e;
}

void pool_free(void* ptr, cudaStream_t st) {
  if (!ptr) return;
  cudaFreeAsync(ptr, st);
  g_pool_live.fetch_sub(1);
}

template <typename T>
tt_status dev_alloc(tt_plan* p, T** ptr, size_t count) {
  *ptr = nullptr;
  if (count == 0) count = 1;
  if (pool_alloc((void**)ptr, count * sizeof(T), p->stream) != cudaSuccess) {
    // whatever the plan was building is incomplete: it refuses every later call
    p->broken = true;
    return set_error(TT_ERR_OUT_OF_MEMORY, "device allocation of %zu bytes", count * sizeof(T));
  }
  p->allocs.push_back((void*)*ptr);
  p->device_bytes += (int64_t)(count * sizeof(T));
  return TT_OK;
}

// Host-to-device copy that reads host memory from a 128-byte boundary: GB300's copy
// engines read host memory at 211 GB/s from 128-byte-aligned addresses and at
// 185-190 GB/s otherwise (the destination's alignment does not matter), and large
// host allocations commonly start 16 bytes past a page.  A misaligned source's
// first bytes therefore go in a copy of their own.
cudaError_t htod_async(void* dst, const void* src, size_t n, cudaStream_t st) {
  const size_t mis = (uintptr_t)src & 127;
  if (mis == 0 || n <= 65536) return cudaMemcpyAsync(dst, src, n, cudaMemcpyHostToDevice, st);
  const size_t head = 128 - mis;
  const cudaError_t e = cudaMemcpyAsync(dst, src, head, cudaMemcpyHostToDevice, st);
  if (e != cudaSuccess) return e;
  return cudaMemcpyAsync(static_cast<char*>(dst) + head, static_cast<const char*>(src) + head, n - head,
                         cudaMemcpyHostToDevice, st);
}

// Like cudaFree, waits for the device before the memory goes back to the pool.
void dev_free(tt_plan* p, void* ptr) {
  if (!ptr) return;
  auto it = std::find(p->allocs.begin(), p->allocs.end(), ptr);
  if (it != p->allocs.end()) p->allocs.erase(it);
  cudaDeviceSynchronize();
  pool_free(ptr, p->stream);
}


int64_t pad16(int64_t n) { return ((n + 15) / 16) * 16 + 16; }

// Work units of the plan's walk: the nonzeros (slab passes: the largest slab is
// no larger), or for the strip walk on a slab plan the slab-major arrays.
int64_t walk_units(const tt_plan* p, int P) {
  const int64_t n = p->staged == 4 && p->slabs > 1 ? p->leaf_len : p->nnz;
  return (n + P - 1) / P;
}

tt_status alloc_walk_scratch(tt_plan* p, int P) {
  const int64_t nb = walk_units(p, P);
  if (nb > p->scratch_blocks) {
    struct SyncAtEnd {  // pool memory becomes usable on every stream
      cudaStream_t st;
      ~SyncAtEnd() { cudaStreamSynchronize(st); }
    } sync_at_end{p->stream};
    dev_free(p, p->d_part);
    dev_free(p, p->d_carry);
    p->d_part = nullptr;
    p->d_carry = nullptr;
    dev_free(p, p->d_meta);
    p->d_meta = nullptr;
    dev_free(p, p->d_segcarry);
    p->d_segcarry = nullptr;
    dev_free(p, p->d_segmeta);
    p->d_segmeta = nullptr;
    tt_status s = dev_alloc(p, &p->d_part, (size_t)(nb + 1) * (size_t)(p->order - 1));
    if (s != TT_OK) return s;
    s = dev_alloc(p, &p->d_carry, (size_t)(2 * nb) * (size_t)p->rp);
    if (s != TT_OK) return s;
    s = dev_alloc(p, &p->d_meta, (size_t)nb * 4);
    if (s != TT_OK) return s;
    const int64_t ns = num_segments((int)nb);
    s = dev_alloc(p, &p->d_segcarry, (size_t)(2 * ns) * (size_t)p->rp);
    if (s != TT_OK) return s;
    s = dev_alloc(p, &p->d_segmeta, (size_t)ns * 4);
    if (s != TT_OK) return s;
    p->scratch_blocks = nb;
  }
  return TT_OK;
}

WalkArgs walk_args(const tt_plan* p, float* A, int q);
WalkArgs ttv_args(const tt_plan* p, const float* x, float* y);

// Compute the work-unit partition of a single-slab plan once, on the plan's
// stream, timed with events (the legacy timer adds it back, so that it covers
// what the reference's per-call timer covers); later calls reuse it.
tt_status prepare_partition(tt_plan* p) {
  p->part_ready = false;
  p->part_ms = 0.f;
  // the strip walk (MTTKRP and COO TTM plans) partitions by rows through rnz
  const bool strip = p->op != TT_OP_TTV && p->staged == 4;
  if ((p->slabs != 1 && !strip) || p->nnz == 0) return TT_OK;
  const WalkArgs a = p->op == TT_OP_TTV ? ttv_args(p, nullptr, nullptr) : walk_args(p, nullptr, 0);
  cudaEvent_t e0, e1;
  CK(cudaEventCreate(&e0));
  if (cudaEventCreate(&e1) != cudaSuccess) {
    cudaEventDestroy(e0);
    return set_error(TT_ERR_CUDA, "partition timer");
  }
  cudaError_t e = cudaEventRecord(e0, p->stream);
  if (e == cudaSuccess) e = strip ? launch_partition_rows(p->order, a, p->stream)
                                 : launch_partition(p->op == TT_OP_TTV ? 2 : p->order, a, p->stream);
  if (e == cudaSuccess) e = cudaEventRecord(e1, p->stream);
  if (e == cudaSuccess) e = cudaEventSynchronize(e1);
  float ms = 0.f;
  if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (e != cudaSuccess) return set_error(TT_ERR_CUDA, "partition: %s", cudaGetErrorString(e));
  p->part_ms = ms;
  p->part_ready = true;
  return TT_OK;
}

// Structure check of every level on the plan's device copies (launch_csf_check),
// before anything reads the arrays.
tt_status device_csf_check(tt_plan* p, const CsfView& v, cudaStream_t st) {
  const int L = v.order - 1;
  int64_t maxn = 1;
  for (int l = 1; l <= L; l++) maxn = std::max<int64_t>(maxn, v.count[l]);
  uint32_t* starts = nullptr;
  unsigned long long* err = nullptr;
  CK(pool_alloc((void**)&starts, sizeof(uint32_t) * (size_t)((maxn + 31) / 32 + 1), st));
  cudaError_t e = pool_alloc((void**)&err, sizeof(unsigned long long) * 2 * (size_t)L, st);
  unsigned long long h[2 * TT_MAX_ORDER];
  if (e == cudaSuccess) e = cudaMemsetAsync(err, 0xff, sizeof(unsigned long long) * 2 * (size_t)L, st);
  for (int l = 1; l <= L && e == cudaSuccess; l++)
    e = launch_csf_check(p->d_pos[l], v.count[l - 1], l >= 2 ? 1 : 0, p->d_crd[l], v.count[l], v.dims[l], starts,
                         err + 2 * (l - 1), st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(h, err, sizeof(unsigned long long) * 2 * (size_t)L, cudaMemcpyDeviceToHost, st);
  pool_free(err, st);
  pool_free(starts, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return set_error(TT_ERR_CUDA, "structure check: %s", cudaGetErrorString(e));
  for (int l = 1; l <= L; l++) {
    tt_status s = csf_check_error(l, h[2 * (l - 1)]);  // pos first: the crd pass trusts its marks
    if (s == TT_OK) s = csf_check_error(l, h[2 * (l - 1) + 1]);
    if (s != TT_OK) return s;
  }
  return TT_OK;
}

// Variants next to `id` in its family: one step in G, one step in columns per
// lane, or the other thread value (register budget).
std::vector<int> variant_neighbours(int id) {
  std::vector<int> out;
  const VariantSpec v = variant_spec(id);
  if (v.tb == 0) return out;
  const int ti = v.tb == 512 ? 1 : 0;
  int gi = 0, ci = 0;
  for (int i = 0; i < 5; i++) if (kGF[v.staged][i] == v.G) gi = i;
  for (int i = 0; i < 4; i++) if (kCPT[i] == v.cpt) ci = i;
  const int d[4][2] = {{-1, 0}, {1, 0}, {0, -1}, {0, 1}};
  for (const auto& dd : d) {
    const int g = gi + dd[0], c = ci + dd[1];
    if (g >= 0 && g < 5 && c >= 0 && c < 4) out.push_back(v.staged * kPerFamily + (ti * 5 + g) * 4 + c);
  }
  out.push_back(v.staged * kPerFamily + ((1 - ti) * 5 + gi) * 4 + ci);
  return out;
}

// The fixed heuristic for this plan: slab plans and 16-bit fixed point take the
// strip rule (one launch over the slab-major layout; the flat family has no slab
// passes), other plans the shape rule.
int plan_default_variant(const tt_plan* p) {
  if (p->slabs > 1 || p->prec == kFX16) {
    const int id = strip_default_variant(p->order, p->rank, p->prec);
    if (id >= 0) return id;
    return lean_default_variant(p->order, p->rank, p->prec);
  }
  return default_variant(p->order, p->rank, p->prec, p->nnz);
}

// Builds the flat and strip families' per-nonzero upper coordinates and per-row
// first nonzero (once per plan).  On a slab plan (strip walk only) the arrays follow
// the slab-major layout: slab q's nonzeros at slab[q].off, and rnz over
// slabs * (nroot + 1) virtual rows, row nroot of each slab covering its padding.
// All or nothing: on failure no array is kept.
tt_status build_slab_flat_arrays(tt_plan* p);
tt_status build_flat_arrays5(tt_plan* p);
tt_status build_flat_arrays(tt_plan* p) {
  if (p->slabs > 1) return build_slab_flat_arrays(p);
  if (p->order == 5) return build_flat_arrays5(p);
  const size_t np = (size_t)pad16(p->nnz);
  int32_t *kexp = nullptr, *kexp2 = nullptr, *rnz = nullptr, *k1f2 = nullptr;
  auto undo = [&](tt_status s) {
    cudaStreamSynchronize(p->stream);
    dev_free(p, k1f2);
    dev_free(p, kexp2);
    dev_free(p, rnz);
    dev_free(p, kexp);
    return s;
  };
  auto ck = [&](cudaError_t e, const char* what) {
    return e == cudaSuccess ? TT_OK
                            : set_error(e == cudaErrorMemoryAllocation ? TT_ERR_OUT_OF_MEMORY : TT_ERR_CUDA,
                                        "%s: %s", what, cudaGetErrorString(e));
  };
  tt_status s;
  if ((s = dev_alloc(p, &kexp, np)) != TT_OK) return undo(s);
  if ((s = dev_alloc(p, &rnz, (size_t)p->nroot + 1)) != TT_OK) return undo(s);
  if ((s = ck(cudaMemsetAsync(kexp, 0, sizeof(int32_t) * np, p->stream), "kexp clear")) != TT_OK) return undo(s);
  if (p->order == 3) {
    if ((s = ck(launch_expand(p->d_crd[1], p->d_pos[2], p->count[1], p->nnz, kexp, p->stream), "expand")) != TT_OK)
      return undo(s);
    if ((s = ck(launch_row_starts(p->d_pos[1], p->d_pos[2], nullptr, p->nroot, rnz, p->stream), "row starts")) != TT_OK)
      return undo(s);
  } else {
    if ((s = dev_alloc(p, &kexp2, np)) != TT_OK) return undo(s);
    // level-1 coordinate of every level-2 fiber
    if ((s = dev_alloc(p, &k1f2, (size_t)p->count[2] + 1)) != TT_OK) return undo(s);
    if ((s = ck(cudaMemsetAsync(kexp2, 0, sizeof(int32_t) * np, p->stream), "kexp2 clear")) != TT_OK) return undo(s);
    if ((s = ck(launch_expand(p->d_crd[1], p->d_pos[2], p->count[1], p->count[2], k1f2, p->stream), "expand")) != TT_OK ||
        (s = ck(launch_expand(k1f2, p->d_pos[3], p->count[2], p->nnz, kexp, p->stream), "expand")) != TT_OK ||
        (s = ck(launch_expand(p->d_crd[2], p->d_pos[3], p->count[2], p->nnz, kexp2, p->stream), "expand")) != TT_OK ||
        (s = ck(launch_row_starts(p->d_pos[1], p->d_pos[2], p->d_pos[3], p->nroot, rnz, p->stream), "row starts")) !=
            TT_OK)
      return undo(s);
  }
  if ((s = ck(cudaStreamSynchronize(p->stream), "flat arrays")) != TT_OK) return undo(s);
  dev_free(p, k1f2);
  p->d_kexp = kexp;
  p->d_kexp2 = kexp2;
  p->d_rnz = rnz;
  return TT_OK;
}

// Five modes (strip walk): the level-1, level-2 and level-3 coordinates of every
// nonzero, each carried down the levels by launch_expand, and the row starts.
tt_status build_flat_arrays5(tt_plan* p) {
  const size_t np = (size_t)pad16(p->nnz);
  int32_t *k1 = nullptr, *k2 = nullptr, *k3 = nullptr, *rnz = nullptr, *a2 = nullptr, *a31 = nullptr, *a32 = nullptr;
  auto undo = [&](tt_status s) {
    cudaStreamSynchronize(p->stream);
    for (int32_t* d : {a32, a31, a2, rnz, k3, k2, k1}) dev_free(p, d);
    return s;
  };
  auto ck = [&](cudaError_t e, const char* what) {
    return e == cudaSuccess ? TT_OK
                            : set_error(e == cudaErrorMemoryAllocation ? TT_ERR_OUT_OF_MEMORY : TT_ERR_CUDA,
                                        "%s: %s", what, cudaGetErrorString(e));
  };
  tt_status s;
  for (int32_t** d : {&k1, &k2, &k3}) {
    if ((s = dev_alloc(p, d, np)) != TT_OK) return undo(s);
    if ((s = ck(cudaMemsetAsync(*d, 0, sizeof(int32_t) * np, p->stream), "clear")) != TT_OK) return undo(s);
  }
  if ((s = dev_alloc(p, &rnz, (size_t)p->nroot + 1)) != TT_OK) return undo(s);
  if ((s = dev_alloc(p, &a2, (size_t)p->count[2] + 1)) != TT_OK) return undo(s);
  if ((s = dev_alloc(p, &a31, (size_t)p->count[3] + 1)) != TT_OK) return undo(s);
  if ((s = dev_alloc(p, &a32, (size_t)p->count[3] + 1)) != TT_OK) return undo(s);
  // a2: level-1 coordinate of each level-2 fiber; a31 / a32: level-1 / level-2
  // coordinate of each level-3 fiber
  if ((s = ck(launch_expand(p->d_crd[1], p->d_pos[2], p->count[1], p->count[2], a2, p->stream), "expand")) != TT_OK ||
      (s = ck(launch_expand(a2, p->d_pos[3], p->count[2], p->count[3], a31, p->stream), "expand")) != TT_OK ||
      (s = ck(launch_expand(p->d_crd[2], p->d_pos[3], p->count[2], p->count[3], a32, p->stream), "expand")) != TT_OK ||
      (s = ck(launch_expand(a31, p->d_pos[4], p->count[3], p->nnz, k1, p->stream), "expand")) != TT_OK ||
      (s = ck(launch_expand(a32, p->d_pos[4], p->count[3], p->nnz, k2, p->stream), "expand")) != TT_OK ||
      (s = ck(launch_expand(p->d_crd[3], p->d_pos[4], p->count[3], p->nnz, k3, p->stream), "expand")) != TT_OK ||
      (s = ck(launch_row_starts(p->d_pos[1], p->d_pos[2], p->d_pos[3], p->nroot, rnz, p->stream, 0, p->d_pos[4]),
              "row starts")) != TT_OK)
    return undo(s);
  if ((s = ck(cudaStreamSynchronize(p->stream), "flat arrays")) != TT_OK) return undo(s);
  for (int32_t* d : {a32, a31, a2}) dev_free(p, d);
  p->d_kexp = k1;
  p->d_kexp2 = k2;
  p->d_kexp3 = k3;
  p->d_rnz = rnz;
  return TT_OK;
}

tt_status build_slab_flat_arrays(tt_plan* p) {
  const int S = p->slabs;
  const int64_t I = p->nroot;
  const size_t np = (size_t)pad16(p->leaf_len);
  int32_t *kexp = nullptr, *kexp2 = nullptr, *rnz = nullptr, *k1f2 = nullptr;
  auto undo = [&](tt_status s) {
    cudaStreamSynchronize(p->stream);
    dev_free(p, k1f2);
    dev_free(p, kexp2);
    dev_free(p, rnz);
    dev_free(p, kexp);
    return s;
  };
  auto ck = [&](cudaError_t e, const char* what) {
    return e == cudaSuccess ? TT_OK
                            : set_error(e == cudaErrorMemoryAllocation ? TT_ERR_OUT_OF_MEMORY : TT_ERR_CUDA,
                                        "%s: %s", what, cudaGetErrorString(e));
  };
  tt_status s;
  const int64_t nv = (int64_t)S * (I + 1);
  if (nv + 1 > INT32_MAX || p->leaf_len > INT32_MAX)
    return set_error(TT_ERR_UNSUPPORTED, "slab-major strip layout: %lld virtual rows", (long long)nv);
  if ((s = dev_alloc(p, &kexp, np)) != TT_OK) return undo(s);
  if ((s = dev_alloc(p, &rnz, (size_t)nv + 1)) != TT_OK) return undo(s);
  if ((s = ck(cudaMemsetAsync(kexp, 0, sizeof(int32_t) * np, p->stream), "kexp clear")) != TT_OK) return undo(s);
  if (p->order == 4) {
    if ((s = dev_alloc(p, &kexp2, np)) != TT_OK) return undo(s);
    if ((s = ck(cudaMemsetAsync(kexp2, 0, sizeof(int32_t) * np, p->stream), "kexp2 clear")) != TT_OK) return undo(s);
    int64_t m2 = 1;
    for (int q = 0; q < S; q++) m2 = std::max<int64_t>(m2, p->slab[q].count[2] + 1);
    if ((s = dev_alloc(p, &k1f2, (size_t)m2)) != TT_OK) return undo(s);
  }
  for (int q = 0; q < S; q++) {
    const tt_plan::SlabDev& sl = p->slab[q];
    int32_t* rq = rnz + (size_t)q * (size_t)(I + 1);
    if (p->order == 3) {
      if ((s = ck(launch_expand(sl.crd[1], sl.pos[2], sl.count[1], sl.nnz, kexp + sl.off, p->stream), "expand")) != TT_OK ||
          (s = ck(launch_row_starts(sl.pos[1], sl.pos[2], nullptr, I, rq, p->stream, sl.off), "row starts")) != TT_OK)
        return undo(s);
    } else {
      if ((s = ck(launch_expand(sl.crd[1], sl.pos[2], sl.count[1], sl.count[2], k1f2, p->stream), "expand")) != TT_OK ||
          (s = ck(launch_expand(k1f2, sl.pos[3], sl.count[2], sl.nnz, kexp + sl.off, p->stream), "expand")) != TT_OK ||
          (s = ck(launch_expand(sl.crd[2], sl.pos[3], sl.count[2], sl.nnz, kexp2 + sl.off, p->stream), "expand")) != TT_OK ||
          (s = ck(launch_row_starts(sl.pos[1], sl.pos[2], sl.pos[3], I, rq, p->stream, sl.off), "row starts")) != TT_OK)
        return undo(s);
    }
  }
  const int32_t end = (int32_t)p->leaf_len;
  if ((s = ck(cudaMemcpyAsync(rnz + nv, &end, sizeof(int32_t), cudaMemcpyHostToDevice, p->stream), "rnz end")) != TT_OK)
    return undo(s);
  if ((s = ck(cudaStreamSynchronize(p->stream), "slab flat arrays")) != TT_OK) return undo(s);
  dev_free(p, k1f2);
  p->d_kexp = kexp;
  p->d_kexp2 = kexp2;
  p->d_rnz = rnz;
  return TT_OK;
}

tt_status set_variant(tt_plan* p, int id) {
  VariantSpec v = variant_spec(id);
  p->variant = id;
  p->staged = v.staged;
  p->tb = v.tb;
  p->cpt = v.cpt;
  p->lpr = p->rp / v.cpt;
  p->G = v.G;
  p->P = variant_unit(v, p->rp);
  p->nblocks = (int)walk_units(p, p->P);
  p->launcher = walk_launcher(p->order, p->prec, p->cpt, p->lpr, launch_family(v));
  if (!p->launcher) return set_error(TT_ERR_UNSUPPORTED, "variant %d not compiled for this shape", id);
  if (v.staged == 3 && p->slabs != 1) return set_error(TT_ERR_UNSUPPORTED, "the flat walk runs without slabs");
  tt_status s = alloc_walk_scratch(p, p->P);
  if (s != TT_OK) return s;
  p->part_ready = false;
  if (p->coo && v.staged != 4) return set_error(TT_ERR_UNSUPPORTED, "COO plans run the strip walk");
  if ((v.staged == 3 || v.staged == 4) && !p->coo && !p->d_kexp && p->nnz > 0 && (s = build_flat_arrays(p)) != TT_OK)
    return s;
  if (v.staged == 4 && p->slabs > 1 && !p->d_vrows && p->nnz > 0 &&
      (s = dev_alloc(p, &p->d_vrows, (size_t)p->slabs * (size_t)(p->nroot + 1) * (size_t)p->rp)) != TT_OK)
    return s;
  p->wcap = 1;
  if (p->staged == 1 && p->nnz > 0) {
    // size the window-row region from this tensor's partition (computed once here)
    int wmax = 1;
    for (int q = 0; q < p->slabs; q++) {
      if (p->slab[q].nnz == 0) continue;
      WalkArgs a = walk_args(p, nullptr, q);
      CK(launch_partition(p->order, a, p->stream));
      CK(launch_window_max(p->order, a, p->d_err + 1, p->stream));
      int w = 0;
      CK(cudaMemcpyAsync(&w, p->d_err + 1, sizeof(int), cudaMemcpyDeviceToHost, p->stream));
      CK(cudaStreamSynchronize(p->stream));
      wmax = std::max(wmax, w);
    }
    p->wcap = wmax;
    const size_t need = variant_smem(v, p->rp, p->prec, p->wcap, p->order);
    if (need > kSmemLimit)
      return set_error(TT_ERR_UNSUPPORTED, "variant %d needs %zu bytes of shared memory for this tensor", id, need);
  }
  return prepare_partition(p);
}

// Switches the plan to variant `id`.  Until a switch succeeds the plan has no
// usable variant, and calls on it report an error instead of launching a walk
// whose scratch, tables or shared memory were not set up for it.
tt_status use_variant(tt_plan* p, int id) {
  p->variant_ready = false;
  const tt_status s = set_variant(p, id);
  p->variant_ready = s == TT_OK;
  return s;
}

WalkArgs strip_slab_args(const tt_plan* p);

// Arguments of one walk pass over slab q (the whole tensor when slabs == 1).
WalkArgs walk_args(const tt_plan* p, float* A, int q) {
  if (p->staged == 4 && p->slabs > 1) return strip_slab_args(p);
  WalkArgs a{};
  const tt_plan::SlabDev& sl = p->slab[q];
  for (int l = 0; l < TT_MAX_ORDER; l++) { a.pos[l] = sl.pos[l]; a.crd[l] = sl.crd[l]; }
  a.crd[0] = p->dense_root ? nullptr : p->d_crd[0];
  // 16-bit fixed point reads the values scaled by their leaf rows' powers of two,
  // which exist once factors are set (the unscaled values before: placeholder runs)
  a.vals = static_cast<const unsigned char*>(p->prec == kFX16 && p->d_vals_fx ? (const void*)p->d_vals_fx : p->d_vals) +
           (size_t)sl.off * (size_t)val_bytes(p->prec);
  a.accum = p->slabs > 1 ? 1 : 0;
  a.gpol = p->gpol;
  for (int m = 0; m < 4; m++) a.fac[m] = p->fac[m];
  a.colscale = p->d_colscale;
  a.out = A;
  a.part = p->d_part;
  a.carry = p->d_carry;
  a.meta = p->d_meta;
  a.segcarry = p->d_segcarry;
  a.segmeta = p->d_segmeta;
  a.nnz = sl.nnz;
  a.nrows = (int32_t)p->nroot;
  a.rp = p->rp;
  a.R = p->rank;
  a.ldo = p->rank;
  a.P = p->P;
  a.G = p->G;
  a.lgG = 0;
  while ((1 << a.lgG) < p->G) a.lgG++;
  a.nblocks = (int)((sl.nnz + p->P - 1) / p->P);
  a.wcap = p->wcap;
  a.err = p->d_err;
  a.kexp = p->d_kexp;
  a.kexp2 = p->d_kexp2;
  a.kexp3 = p->d_kexp3;
  // rows through rnz only for the families that walk by it (the row merge uses it too)
  a.rnz = p->staged == 3 || p->staged == 4 ? p->d_rnz : nullptr;
  for (int m = 0; m < 4; m++) a.fac_rows[m] = m + 1 < p->order ? (int32_t)p->dims[m + 1] : 0;
  a.wait_ns = (uint32_t)g_tma_wait_ns.load(std::memory_order_relaxed);
  a.tma_withhold = g_tma_withhold.load(std::memory_order_relaxed);
  return a;
}

// The strip walk's single pass over a slab plan's slab-major arrays: virtual rows
// q * (nroot + 1) + i, written once each into d_vrows.
WalkArgs strip_slab_args(const tt_plan* p) {
  WalkArgs a{};
  const int L = p->order - 1;
  a.crd[L] = p->d_crd[L];
  a.vals = p->prec == kFX16 && p->d_vals_fx ? (const void*)p->d_vals_fx : p->d_vals;
  a.accum = 0;
  a.gpol = p->gpol;
  for (int m = 0; m < 4; m++) a.fac[m] = p->fac[m];
  a.colscale = p->d_colscale;
  a.out = p->d_vrows;
  a.part = p->d_part;
  a.carry = p->d_carry;
  a.meta = p->d_meta;
  a.segcarry = p->d_segcarry;
  a.segmeta = p->d_segmeta;
  a.nnz = p->leaf_len;
  a.nrows = (int32_t)((int64_t)p->slabs * (p->nroot + 1));
  a.rp = p->rp;
  a.R = p->rank;
  a.ldo = p->rp;  // virtual rows RP floats apart (16-byte rows for the slab sum)
  a.P = p->P;
  a.G = p->G;
  a.lgG = 0;
  while ((1 << a.lgG) < p->G) a.lgG++;
  a.nblocks = p->nblocks;
  a.err = p->d_err;
  a.kexp = p->d_kexp;
  a.kexp2 = p->d_kexp2;
  a.kexp3 = p->d_kexp3;
  a.rnz = p->d_rnz;
  for (int m = 0; m < 4; m++) a.fac_rows[m] = m + 1 < p->order ? (int32_t)p->dims[m + 1] : 0;
  return a;
}

// The TMA walk's descriptor of the leaf factor: RP columns x dims[leaf] rows of the
// stored type, one-row boxes (tile::gather4 fetches four rows of the box width).
using EncodeTiledFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                   const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                   CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encode_tiled() {
  static EncodeTiledFn fn = []() -> EncodeTiledFn {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess) {
      cudaGetLastError();
      return nullptr;
    }
    return reinterpret_cast<EncodeTiledFn>(f);
  }();
  return fn;
}

tt_status encode_leaf_tmap(const tt_plan* p, CUtensorMap* m) {
  const int leaf = p->order - 1;
  const void* base = p->fac[p->order - 2];
  const int fb = fac_bytes(p->prec);
  if (reinterpret_cast<uintptr_t>(base) % 16)
    return set_error(TT_ERR_UNSUPPORTED, "TMA walk: the last factor is not 16-byte aligned");
  EncodeTiledFn fn = encode_tiled();
  if (!fn) return set_error(TT_ERR_UNSUPPORTED, "TMA walk: cuTensorMapEncodeTiled is not available");
  const cuuint64_t dims[2] = {(cuuint64_t)p->rp, (cuuint64_t)p->dims[leaf]};
  const cuuint64_t strides[1] = {(cuuint64_t)p->rp * (cuuint64_t)fb};
  const cuuint32_t box[2] = {(cuuint32_t)p->rp, 1u};
  const cuuint32_t estr[2] = {1u, 1u};
  const CUresult r = fn(m, fb == 2 ? CU_TENSOR_MAP_DATA_TYPE_UINT16 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2,
                        const_cast<void*>(base), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                        CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_NONE, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return set_error(TT_ERR_UNSUPPORTED, "TMA walk: cuTensorMapEncodeTiled returned %d", (int)r);
  return TT_OK;
}

tt_status run_mttkrp(tt_plan* p, float* A, cudaStream_t st) {
  const size_t outbytes = (size_t)p->dims[0] * (size_t)p->rank * sizeof(float);
  if (!p->variant_ready)
    return set_error(TT_ERR_INVALID_ARGUMENT, "the plan's last variant switch failed: select a variant");
  // the device error word reports this call only: a bounded wait that ran out in an
  // earlier call (or in a variant timed at plan creation) does not stop this one
  if (p->d_err) CK(cudaMemsetAsync(p->d_err, 0, sizeof(int32_t), st));
  if (p->nnz > 0 && p->staged == 4 && p->slabs > 1) {
    // strip walk over the slab-major layout: one launch, the virtual rows' merge,
    // then the slabs' rows summed into A (every row of A written, no clear)
    WalkArgs a = walk_args(p, A, 0);
    const size_t smem = variant_smem(variant_spec(p->variant), p->rp, p->prec, p->wcap, p->order);
    a.smem_bytes = (int32_t)smem;
    if (!p->part_ready) CK(launch_partition_rows(p->order, a, st));
    if (p->timing == 1) CK(cudaEventRecord(p->evk0, st));
    CK(p->launcher(a, a.nblocks, p->tb, smem, st));
    if (p->timing == 1) CK(cudaEventRecord(p->evk1, st));
    CK(launch_chain_fixup(p->order, a, st));
    CK(launch_virtual_rows(p->d_vrows, p->d_rnz, p->slabs, p->nroot, p->nroot + 1, p->rp, p->rank, p->rank, A, st));
    return TT_OK;
  }
  CK(cudaMemsetAsync(A, 0, outbytes, st));
  if (p->nnz == 0) return TT_OK;
  // one pass per slab, in slab order, each adding its rows into A; the kernel
  // timer spans the first pass's walk to the last one's
  const size_t smem = variant_smem(variant_spec(p->variant), p->rp, p->prec, p->wcap, p->order);
  int first = -1, last = -1;
  for (int q = 0; q < p->slabs; q++)
    if (p->slab[q].nnz > 0) { if (first < 0) first = q; last = q; }
  for (int q = first; q >= 0 && q <= last; q++) {
    WalkArgs a = walk_args(p, A, q);
    if (a.nnz == 0) continue;
    a.smem_bytes = (int32_t)smem;
    if (p->staged == 2) {
      const tt_status s2 = encode_leaf_tmap(p, &a.tmap);
      if (s2 != TT_OK) return s2;
    }
    if (!p->part_ready) CK(p->staged == 4 ? launch_partition_rows(p->order, a, st) : launch_partition(p->order, a, st));
    if (p->timing == 1 && q == first) CK(cudaEventRecord(p->evk0, st));
    CK(p->launcher(a, a.nblocks, p->tb, smem, st));
    if (p->timing == 1 && q == last) CK(cudaEventRecord(p->evk1, st));
    CK(launch_chain_fixup(p->order, a, st));
  }
  return TT_OK;
}

// TTV sees the last two levels as a 2-level CSF: "rows" are the fibers, one
// output column.
WalkArgs ttv_args(const tt_plan* p, const float* x, float* y) {
  WalkArgs a{};
  a.pos[1] = p->d_pos[p->order - 1];
  a.crd[1] = p->d_crd[p->order - 1];
  a.vals = p->d_vals;
  a.fac[0] = x;
  a.out = y;
  a.part = p->d_part;
  a.carry = p->d_carry;
  a.meta = p->d_meta;
  a.segcarry = p->d_segcarry;
  a.segmeta = p->d_segmeta;
  a.vscale = val_kind(p->prec) != kF32 ? p->vinv : 1.f;
  a.nnz = p->nnz;
  a.nrows = (int32_t)p->nfib_last;
  a.R = 1;
  a.rp = 1;
  a.ldo = 1;
  a.P = p->P;
  a.G = kTtvNpt;
  a.nblocks = p->nblocks;
  a.fac_rows[0] = (int32_t)p->dims[p->order - 1];  // length of x
  return a;
}

// The range walk's view: the merge's units are ranges of ttv_ru partition units.
WalkArgs ttv_range_args(const tt_plan* p, const float* x, float* y) {
  WalkArgs a = ttv_args(p, x, y);
  a.wcap = p->ttv_ru;
  a.P = p->ttv_ru * p->P;
  a.nblocks = p->ttv_ranges;
  return a;
}

// Ranges for the TTV walk: one per resident warp (kTtvWarps per SM) while a range
// holds at most kTtvMaxRU units, more ranges (in waves) beyond that.
tt_status set_ttv_ranges(tt_plan* p) {
  int dev = 0, sms = 0;
  CK(cudaGetDevice(&dev));
  CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  const int64_t units = p->nblocks;
  const int64_t warps = (int64_t)std::max(sms, 1) * kTtvWarps;
  p->ttv_ru = (int32_t)std::min<int64_t>(kTtvMaxRU, std::max<int64_t>(1, (units + warps - 1) / warps));
  p->ttv_ranges = (int32_t)((units + p->ttv_ru - 1) / p->ttv_ru);
  return TT_OK;
}

tt_status run_ttv(tt_plan* p, const float* x, float* y, cudaStream_t st) {
  if (p->nnz == 0) {
    if (p->nfib_last > 0) CK(cudaMemsetAsync(y, 0, sizeof(float) * (size_t)p->nfib_last, st));
    return TT_OK;
  }
  if (!p->part_ready) CK(launch_partition(2, ttv_args(p, x, y), st));
  const WalkArgs a = ttv_range_args(p, x, y);
  if (p->timing == 1) CK(cudaEventRecord(p->evk0, st));
  CK(launch_ttv_ranges(a, val_kind(p->prec), st));
  if (p->timing == 1) CK(cudaEventRecord(p->evk1, st));
  CK(launch_chain_fixup(2, a, st));
  return TT_OK;
}

tt_status time_variants(tt_plan* p, cudaStream_t st, const std::vector<int>& cands, int max_timed, int extra);

// Values on the device: FP32 as given, or 16-bit with one power-of-two scale
// (max in [1,2) for BF16, [2^14,2^15) for FP16), found and applied on the device;
// nvals_alloc - nvals entries of zero padding.
tt_status upload_values(tt_plan* p, const float* hvals, int64_t nvals, size_t nvals_alloc, cudaStream_t st) {
  tt_status s;
  p->nvals_alloc = nvals_alloc;
  const size_t n = nvals_alloc;
  if (val_kind(p->prec) != kF32) {
    // values: one power-of-two scale (max in [1,2) for BF16, [2^14,2^15) for FP16),
    // found and applied on the device (absolute max, scale, round-to-nearest-even)
    const bool h16 = p->prec == kFP16;
    p->vinv = h16 ? 1.f / 16384.f : 1.f;  // (no values: never used)
    uint16_t* d = nullptr;
    if ((s = dev_alloc(p, &d, n)) != TT_OK) return s;
    p->d_vals = d;
    if (n > (size_t)nvals && cudaMemsetAsync(d + nvals, 0, (n - (size_t)nvals) * 2, st) != cudaSuccess)
      return (set_error(TT_ERR_CUDA, "clear vals"));
    if (nvals > 0) {
      float* tmp = nullptr;
      if (pool_alloc((void**)&tmp, (size_t)nvals * 4 + 64, st) != cudaSuccess)
        return (set_error(TT_ERR_OUT_OF_MEMORY, "value staging"));
      float* cmax = reinterpret_cast<float*>(((uintptr_t)(tmp + nvals) + 15) & ~(uintptr_t)15);
      float* scl = cmax + 1;
      float* inv = cmax + 2;
      float vinv = 1.f;
      cudaError_t e = htod_async(tmp, hvals, (size_t)nvals * 4, st);
      if (e == cudaSuccess) e = launch_colmax(tmp, nvals, 1, cmax, st);
      if (e == cudaSuccess) e = launch_pow2_scales(cmax, 1, h16 ? 14 : 0, scl, inv, st);
      if (e == cudaSuccess) e = launch_to_16(tmp, nvals, 1, 1, scl, h16 ? 2 : 1, d, st);
      if (e == cudaSuccess) e = cudaMemcpyAsync(&vinv, inv, 4, cudaMemcpyDeviceToHost, st);
      pool_free(tmp, st);
      const cudaError_t e2 = cudaStreamSynchronize(st);
      if (e != cudaSuccess || e2 != cudaSuccess)
        return (set_error(TT_ERR_CUDA, "value conversion: %s", cudaGetErrorString(e != cudaSuccess ? e : e2)));
      p->vinv = vinv;
    }
  } else {
    float* d = nullptr;
    if ((s = dev_alloc(p, &d, n)) != TT_OK) return s;
    p->d_vals = d;
    if (n > (size_t)nvals && cudaMemsetAsync(d + nvals, 0, (n - (size_t)nvals) * 4, st) != cudaSuccess)
      return (set_error(TT_ERR_CUDA, "clear vals"));
    if (nvals > 0 && htod_async(d, hvals, (size_t)nvals * 4, st) != cudaSuccess)
      return (set_error(TT_ERR_CUDA, "upload vals"));
  }
  return TT_OK;
}


}  // namespace

// ---------------------------------------------------------------------------
// public API
// ---------------------------------------------------------------------------
TT_EXPORT const char* tt_status_string(tt_status s) {
switch (s) {
  case TT_OK: return "TT_OK";
  case TT_ERR_INVALID_ARGUMENT: return "TT_ERR_INVALID_ARGUMENT";
  case TT_ERR_INVALID_CSF: return "TT_ERR_INVALID_CSF";
  case TT_ERR_UNSUPPORTED: return "TT_ERR_UNSUPPORTED";
  case TT_ERR_CUDA: return "TT_ERR_CUDA";
  case TT_ERR_OUT_OF_MEMORY: return "TT_ERR_OUT_OF_MEMORY";
  case TT_ERR_NO_DEVICE: return "TT_ERR_NO_DEVICE";
  case TT_ERR_DEVICE_WAIT: return "TT_ERR_DEVICE_WAIT";
}
return "TT_ERR_UNKNOWN";
}

TT_EXPORT int32_t tt_abi_version(void) { return TT_ABI_VERSION; }
TT_EXPORT int32_t tt_num_variants(void) { return kNumVariants; }

TT_EXPORT tt_status tt_variant_get(int32_t id, tt_variant_info* info) {
clear_error();
if (!info || id < 0 || id >= kNumVariants) return set_error(TT_ERR_INVALID_ARGUMENT, "variant %d", id);
VariantSpec v = variant_spec(id);
std::memset(info, 0, sizeof(*info));
info->id = id;
info->threads = v.tb;
info->cols_per_lane = v.cpt;
info->nnz_per_team = v.G;
info->rank_pad = 32;
info->lanes_per_row = 32 / v.cpt;
info->nnz_per_block = v.tb / info->lanes_per_row * v.G;
info->staged = v.staged;
static const char* fam[kFamilies] = {"lean", "stage", "tma", "flat", "strip"};
if (v.staged == 0 || v.staged == 3 || v.staged == 4) {  // lean / flat / strip: 256-thread blocks, budget for b resident blocks per SM
  info->threads = 256;
  info->nnz_per_block = 256 / info->lanes_per_row * v.G;
  std::snprintf(info->name, sizeof(info->name), "%s_b%d_g%d_c%d", fam[v.staged], lean_blocks(v), v.G, v.cpt);
} else if (v.staged == 2) {  // TMA gather: 256-thread blocks, s stages in flight per warp
  info->threads = 256;
  info->nnz_per_block = 256 / info->lanes_per_row * v.G;
  std::snprintf(info->name, sizeof(info->name), "tma_s%d_g%d_c%d", tma_stages(v), v.G, v.cpt);
} else {
  std::snprintf(info->name, sizeof(info->name), "%s_t%d_g%d_c%d", fam[v.staged], v.tb, v.G, v.cpt);
}
  return TT_OK;
}

TT_EXPORT int32_t tt_variant_default(int32_t order, int32_t rank, tt_precision prec, int64_t nnz) {
  return default_variant(order, rank, (int)prec, nnz);
}

TT_EXPORT int32_t tt_variant_valid(int32_t id, int32_t order, int32_t rank, tt_precision prec) {
  return variant_valid(id, order, rank, (int)prec) ? 1 : 0;
}

TT_EXPORT tt_status tt_plan_create(const taco_tensor_t* B, tt_op op, int32_t rank, tt_precision prec,
                                   tt_select select, int32_t variant, void* stream, tt_plan** out) {
  return tt_plan_create_ex(B, op, rank, prec, select, variant, nullptr, stream, out);
}

TT_EXPORT tt_status tt_plan_create_ex(const taco_tensor_t* B, tt_op op, int32_t rank, tt_precision prec,
                                      tt_select select, int32_t variant, const tt_plan_options* opts,
                                      void* stream, tt_plan** out) {
  NvtxRange nvtx_range("tt_plan_create");
  clear_error();
  if (opts && (opts->slabs < 0 || opts->slabs > kMaxSlabs))
    return set_error(TT_ERR_INVALID_ARGUMENT, "slabs %d (0 = automatic, at most %d)", opts->slabs, kMaxSlabs);
  if (!out) return set_error(TT_ERR_INVALID_ARGUMENT, "null plan pointer");
  *out = nullptr;
  CsfView v;
  tt_status s = csf_view(B, &v);
  if (s != TT_OK) return s;
  // MTTKRP of another mode: the plan holds the tensor re-rooted at that mode
  // (levels: mode, then the other modes in increasing order) and runs the same
  // mode-0 walk on it; the host arrays are read here, so they are checked first
  const int mode = opts ? opts->mode : 0;
  taco_tensor_t* rerooted = nullptr;
  struct FreeRerooted {
    taco_tensor_t*& t;
    ~FreeRerooted() { if (t) tt_tensor_free(t); }
  } free_rerooted{rerooted};
  if (mode != 0) {
    if (op != TT_OP_MTTKRP) return set_error(TT_ERR_UNSUPPORTED, "an output mode other than 0 needs an MTTKRP plan");
    if (mode < 0 || mode >= v.order) return set_error(TT_ERR_INVALID_ARGUMENT, "mode %d of an order-%d tensor", mode, v.order);
    if ((s = csf_check(v)) != TT_OK) return s;
    {
      // coordinates in the new level order (host), sorted and built on the GPU
      std::vector<int32_t> co;
      int32_t nd[TT_MAX_ORDER];
      if ((s = csf_rerooted_coords(v, mode, co, nd)) != TT_OK) return s;
      if ((s = tt_csf_from_coo_gpu(v.order, nd, v.nnz, co.data(), v.vals, &rerooted)) != TT_OK) return s;
    }
    if ((s = csf_view(rerooted, &v)) != TT_OK) return s;
    B = rerooted;
  }
  // the root and pos[0] here; the levels on the host only for slab plans (built
  // from the host arrays) and empty tensors, else on the device after upload
  if ((s = csf_check_root(v)) != TT_OK) return s;
  if (op == TT_OP_MTTKRP) {
    if (v.order < 3 || v.order > 5) return set_error(TT_ERR_UNSUPPORTED, "MTTKRP needs order 3, 4 or 5 (got %d)", v.order);
    if (rank < 1 || rank > TT_MAX_RANK) return set_error(TT_ERR_UNSUPPORTED, "rank %d (supported 1..%d)", rank, TT_MAX_RANK);
  } else if (op != TT_OP_TTV) {
    return set_error(TT_ERR_INVALID_ARGUMENT, "op %d", (int)op);
  } else if (prec == TT_PREC_FX16) {
    return set_error(TT_ERR_UNSUPPORTED, "TTV does not take 16-bit fixed-point storage");
  }
  if (prec != TT_PREC_FP32 && prec != TT_PREC_BF16 && prec != TT_PREC_BF16_FACTORS && prec != TT_PREC_FP16 &&
      prec != TT_PREC_FX16)
    return set_error(TT_ERR_INVALID_ARGUMENT, "precision %d", (int)prec);
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    return set_error(TT_ERR_NO_DEVICE, "no CUDA device visible");
  }
  cudaStream_t st = (cudaStream_t)stream;

  auto* p = new tt_plan();
  cudaGetDevice(&p->device);
  p->op = op;
  p->order = v.order;
  for (int i = 0; i < v.order; i++) p->dims[i] = v.dims[i];
  p->nnz = v.nnz;
  p->nroot = v.nroot;
  p->dense_root = v.dense_root;
  p->rank = op == TT_OP_MTTKRP ? rank : 1;
  p->rp = op == TT_OP_MTTKRP ? rank_pad(rank) : 1;
  p->prec = (int)prec;
  p->mode = mode;
  p->stream = st;
  for (int l = 0; l < v.order; l++) p->count[l] = v.count[l];
  p->nfib_last = v.count[v.order - 2];

  auto fail = [&](tt_status st2) { tt_plan_destroy(p); return st2; };

  // leaf-mode slabs: the plan stores the slab-major CSF instead of the original
  SlabCsf sc;
  int S = 1;
  if (op == TT_OP_MTTKRP && v.dense_root && v.nnz > 0) {
    const int req = opts ? opts->slabs : 0;
    S = req > 0 ? req : auto_slabs(v.order, v.dims[v.order - 1], p->rp, (int)prec);
    if (S > kMaxSlabs) return fail(set_error(TT_ERR_INVALID_ARGUMENT, "slabs %d (at most %d)", S, kMaxSlabs));
    if (S > 1 && (s = csf_check(v)) != TT_OK) return fail(s);
    if (S > 1 && (s = build_slabs(v, S, sc)) != TT_OK) return fail(s);
  } else if (opts && opts->slabs > 1) {
    return fail(set_error(TT_ERR_UNSUPPORTED, "slabs need an MTTKRP plan over a dense-root CSF"));
  }
  p->slabs = S;
  {
    const int pol = opts ? opts->l2_policy : 0;
    if (pol < 0 || pol > 2) return fail(set_error(TT_ERR_INVALID_ARGUMENT, "l2_policy %d", pol));
    p->gpol = pol == 1 ? 0 : pol == 2 ? 1 : (S > 1 ? 1 : 0);
  }
  const int L = v.order - 1;
  if (v.nnz == 0 && (s = csf_check(v)) != TT_OK) return fail(s);
  auto upload = [&](int32_t** d, const int32_t* h, int64_t n, size_t alloc, const char* what) -> tt_status {
    tt_status s2 = dev_alloc(p, d, alloc);
    if (s2 != TT_OK) return s2;
    if (alloc > (size_t)n && cudaMemsetAsync(*d + n, 0, (alloc - (size_t)n) * sizeof(int32_t), st) != cudaSuccess)
      return set_error(TT_ERR_CUDA, "clear %s", what);
    if (n > 0 && htod_async(*d, h, sizeof(int32_t) * (size_t)n, st) != cudaSuccess)
      return set_error(TT_ERR_CUDA, "upload %s", what);
    return TT_OK;
  };
  const float* hvals = v.vals;
  int64_t nvals = v.nnz;
  size_t nvals_alloc = (size_t)pad16(v.nnz);
  if (S == 1) {
    // inner pos/crd exact size; nonzero-level crd and vals padded for 128-bit loads
    for (int l = 1; l < v.order; l++) {
      if ((s = upload(&p->d_pos[l], v.pos[l], v.count[l - 1] + 1, (size_t)v.count[l - 1] + 1, "pos")) != TT_OK) return fail(s);
      const bool last = l == L;
      if ((s = upload(&p->d_crd[l], v.crd[l], v.count[l], last ? (size_t)pad16(v.count[l]) : (size_t)v.count[l], "crd")) != TT_OK)
        return fail(s);
    }
    for (int l = 0; l < TT_MAX_ORDER; l++) { p->slab[0].pos[l] = p->d_pos[l]; p->slab[0].crd[l] = p->d_crd[l]; }
    for (int l = 0; l < v.order; l++) p->slab[0].count[l] = v.count[l];
    p->slab[0].nnz = v.nnz;
    p->slab[0].off = 0;
    p->leaf_len = v.nnz;
    if (v.nnz > 0 && (s = device_csf_check(p, v, st)) != TT_OK) return fail(s);
  } else {
    for (int q = 0; q < S; q++) {
      const SlabCsf::Slab& h = sc.slab[q];
      tt_plan::SlabDev& d = p->slab[q];
      for (int l = 1; l <= L; l++)
        if ((s = upload(&d.pos[l], h.pos[l].data(), h.count[l - 1] + 1, (size_t)h.count[l - 1] + 1, "slab pos")) != TT_OK) return fail(s);
      for (int l = 1; l < L; l++)
        if ((s = upload(&d.crd[l], h.crd[l].data(), h.count[l], (size_t)h.count[l], "slab crd")) != TT_OK) return fail(s);
      d.nnz = h.nnz;
      d.off = h.leaf_off;
      for (int l = 0; l < TT_MAX_ORDER; l++) d.count[l] = h.count[l];
    }
    if ((s = upload(&p->d_crd[L], sc.leaf_crd.data(), (int64_t)sc.leaf_crd.size(), sc.leaf_crd.size(), "slab leaf crd")) != TT_OK)
      return fail(s);
    for (int q = 0; q < S; q++) p->slab[q].crd[L] = p->d_crd[L] + p->slab[q].off;
    hvals = sc.leaf_vals.data();
    nvals = (int64_t)sc.leaf_vals.size();
    nvals_alloc = sc.leaf_vals.size();
    p->leaf_len = (int64_t)sc.leaf_vals.size();
  }
  if (!v.dense_root) {
    if ((s = dev_alloc(p, &p->d_crd[0], (size_t)v.nroot)) != TT_OK) return fail(s);
    if (v.nroot > 0 && cudaMemcpyAsync(p->d_crd[0], v.root_crd, sizeof(int32_t) * (size_t)v.nroot,
                                       cudaMemcpyHostToDevice, st) != cudaSuccess)
      return fail(set_error(TT_ERR_CUDA, "upload root crd"));
    p->slab[0].crd[0] = p->d_crd[0];
  }
  if ((s = upload_values(p, hvals, nvals, nvals_alloc, st)) != TT_OK) return fail(s);
  // MTTKRP scratch is sized with the variant; TTV keeps one ticket per block, zeroed once here
  if (op == TT_OP_MTTKRP) {
    if ((s = dev_alloc(p, &p->d_err, 4)) != TT_OK) return fail(s);
    if (cudaMemsetAsync(p->d_err, 0, 4 * sizeof(int32_t), st) != cudaSuccess) return fail(set_error(TT_ERR_CUDA, "clear error word"));
    int id = -1;
    bool placed = false;
    if (select == TT_SELECT_FIXED) {
      if (!variant_valid(variant, p->order, rank, p->prec))
        return fail(set_error(TT_ERR_INVALID_ARGUMENT, "variant %d not valid for order %d rank %d", variant, p->order, rank));
      id = variant;
    } else if (select == TT_SELECT_MODEL) {
      // the network's ranking; a variant that does not fit this tensor is skipped.
      // k > 1: time the k best-ranked variants that run and the fixed heuristic's
      // variant, keep the fastest (automatic: k = 1 inside the model's training
      // range, where its pick is trusted, else kTopkOutside)
      std::vector<int> ranked;
      bool in_range = true;
      const int req_k = opts ? opts->model_topk : 0;
      if (req_k < 0 || req_k > kMaxTopk)
        return fail(set_error(TT_ERR_INVALID_ARGUMENT, "model_topk %d (0..%d)", req_k, kMaxTopk));
      if (selector_rank(p, B, ranked, &in_range) == TT_OK && !ranked.empty()) {
        // slab plans time the candidates too: the network was trained without slabs
        const int k = req_k > 0 ? req_k : (in_range && p->slabs == 1 ? 1 : kTopkOutside);
        if (k > 1) {
          const int dflt = plan_default_variant(p);
          s = time_variants(p, st, ranked, k, dflt);
          // then a local search around the fastest: its neighbours in G, in columns
          // per lane and in register budget (same family), two rounds at most
          for (int round = 0; s == TT_OK && round < 2; round++) {
            const int before = p->variant;
            std::vector<int> nb;
            for (int cand : variant_neighbours(before))
              if (p->sweep_ms[cand] < 0.f && variant_valid(cand, p->order, rank, p->prec)) nb.push_back(cand);
            if (nb.empty()) break;
            s = time_variants(p, st, nb, (int)nb.size(), -1);
            if (p->variant == before) break;
          }
          if (s == TT_OK) {
            id = p->variant;
            placed = true;
            p->selected_by = 3;
          } else if (s != TT_ERR_UNSUPPORTED) {
            return fail(s);
          }
        } else {
          for (int cand : ranked) {
            s = use_variant(p, cand);
            if (s == TT_OK) { id = cand; placed = true; p->selected_by = 1; break; }
            if (s != TT_ERR_UNSUPPORTED) return fail(s);
          }
        }
      }
      clear_error();
      if (!placed) id = plan_default_variant(p);
    } else {
      id = plan_default_variant(p);
    }
    if (id < 0) return fail(set_error(TT_ERR_UNSUPPORTED, "no variant for order %d rank %d", p->order, rank));
    if (!placed && (s = use_variant(p, id)) != TT_OK) return fail(s);
    if (select == TT_SELECT_SWEEP) {
      std::vector<int> all;
      for (int v = 0; v < kNumVariants; v++)
        if (variant_valid(v, p->order, rank, p->prec)) all.push_back(v);
      if ((s = time_variants(p, st, all, kNumVariants, -1)) != TT_OK) return fail(s);
      p->selected_by = 2;
    }
  } else {
    // TTV: one warp per 32 * kTtvNpt nonzeros
    p->tb = 256;
    p->G = kTtvNpt;
    p->P = 32 * kTtvNpt;
    p->nblocks = (int)((p->nnz + p->P - 1) / p->P);
    if ((s = set_ttv_ranges(p)) != TT_OK) return fail(s);
    if ((s = alloc_walk_scratch(p, p->P)) != TT_OK) return fail(s);
    if ((s = prepare_partition(p)) != TT_OK) return fail(s);
  }
  if (cudaStreamSynchronize(st) != cudaSuccess) return fail(set_error(TT_ERR_CUDA, "plan upload: %s", cudaGetErrorString(cudaGetLastError())));
  *out = p;
  return TT_OK;
}

// ---------------------------------------------------------------------------
// plans over sorted COO input (the reference's MATLAB interface,
// tensor_kernels/fmtaco.cpp: TTV 32-115, TTM 117-223, MTTKRP 741-780)
// ---------------------------------------------------------------------------
TT_EXPORT tt_status tt_plan_create_coo(int32_t order, const int32_t* dims, int64_t nnz, const int32_t* coords,
                                       const float* vals, tt_op op, int32_t rank, tt_precision prec,
                                       tt_select select, int32_t variant, void* stream, tt_plan** out) {
  NvtxRange nvtx_range("tt_plan_create_coo");
  clear_error();
  if (!out || !dims || (nnz > 0 && (!coords || !vals)) || nnz < 0)
    return set_error(TT_ERR_INVALID_ARGUMENT, "null argument or negative nonzero count");
  *out = nullptr;
  if (op == TT_OP_MTTKRP) {
    if (order < 3 || order > 5) return set_error(TT_ERR_UNSUPPORTED, "COO MTTKRP needs order 3, 4 or 5 (got %d)", order);
  } else if (op == TT_OP_TTV || op == TT_OP_TTM) {
    if (order != 3) return set_error(TT_ERR_UNSUPPORTED, "COO TTV and TTM take three-mode tensors (got order %d)", order);
  } else {
    return set_error(TT_ERR_INVALID_ARGUMENT, "op %d", (int)op);
  }
  if (op != TT_OP_TTV && (rank < 1 || rank > TT_MAX_RANK))
    return set_error(TT_ERR_UNSUPPORTED, "rank %d (supported 1..%d)", rank, TT_MAX_RANK);
  if (prec < TT_PREC_FP32 || prec > TT_PREC_FX16) return set_error(TT_ERR_INVALID_ARGUMENT, "precision %d", (int)prec);
  if (op == TT_OP_TTM && prec != TT_PREC_FP32) return set_error(TT_ERR_UNSUPPORTED, "COO TTM runs in FP32 storage");
  if (op == TT_OP_TTV && prec == TT_PREC_FX16)
    return set_error(TT_ERR_UNSUPPORTED, "TTV does not take 16-bit fixed-point storage");
  if (nnz >= INT32_MAX) return set_error(TT_ERR_UNSUPPORTED, "%lld nonzeros (at most 2^31 - 2)", (long long)nnz);
  for (int m = 0; m < order; m++)
    if (dims[m] < 1) return set_error(TT_ERR_INVALID_ARGUMENT, "dims[%d] = %d", m, dims[m]);
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    return set_error(TT_ERR_NO_DEVICE, "no CUDA device visible");
  }
  cudaStream_t st = (cudaStream_t)stream;
  auto* p = new tt_plan();
  auto fail = [&](tt_status s2) { tt_plan_destroy(p); return s2; };
  cudaGetDevice(&p->device);
  p->coo = true;
  p->op = op;
  p->order = order;
  for (int m = 0; m < order; m++) p->dims[m] = dims[m];
  p->nnz = nnz;
  p->nroot = dims[0];
  p->dense_root = true;
  p->rank = op == TT_OP_TTV ? 1 : rank;
  p->rp = op == TT_OP_TTV ? 1 : rank_pad(rank);
  p->prec = (int)prec;
  p->stream = st;
  p->slabs = 1;
  p->leaf_len = nnz;
  tt_status s;
  // coordinates and dims on the device, checked there (range and lexicographic order)
  int32_t *dco = nullptr, *ddims = nullptr;
  unsigned long long* derr = nullptr;
  struct Tmp {
    cudaStream_t st;
    std::vector<void*> v;
    ~Tmp() {
      for (void* q : v) pool_free(q, st);
      cudaStreamSynchronize(st);
    }
  } tmp{st, {}};
  auto talloc = [&](void** ptr, size_t bytes) -> tt_status {
    if (pool_alloc(ptr, bytes < 16 ? 16 : bytes, st) != cudaSuccess)
      return set_error(TT_ERR_OUT_OF_MEMORY, "COO staging of %zu bytes", bytes);
    tmp.v.push_back(*ptr);
    return TT_OK;
  };
  if ((s = talloc((void**)&dco, sizeof(int32_t) * (size_t)nnz * order)) != TT_OK) return fail(s);
  if ((s = talloc((void**)&ddims, sizeof(int32_t) * TT_MAX_ORDER)) != TT_OK) return fail(s);
  if ((s = talloc((void**)&derr, sizeof(unsigned long long))) != TT_OK) return fail(s);
  unsigned long long herr = ~0ull;
  if (nnz > 0 && cudaMemcpyAsync(dco, coords, sizeof(int32_t) * (size_t)nnz * order, cudaMemcpyHostToDevice, st) != cudaSuccess)
    return fail(set_error(TT_ERR_CUDA, "upload coordinates"));
  if (cudaMemcpyAsync(ddims, dims, sizeof(int32_t) * order, cudaMemcpyHostToDevice, st) != cudaSuccess ||
      cudaMemcpyAsync(derr, &herr, sizeof(herr), cudaMemcpyHostToDevice, st) != cudaSuccess ||
      launch_coo_check(dco, nnz, order, ddims, derr, st) != cudaSuccess ||
      cudaMemcpyAsync(&herr, derr, sizeof(herr), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess)
    return fail(set_error(TT_ERR_CUDA, "COO check: %s", cudaGetErrorString(cudaGetLastError())));
  if (herr != ~0ull)
    return fail(set_error(TT_ERR_INVALID_ARGUMENT, "COO nonzero %llu: %s", herr >> 3,
                          (herr & 7) == 1 ? "coordinate outside its mode"
                                          : "out of lexicographic order (sort the coordinates)"));
  if ((s = upload_values(p, vals, nnz, (size_t)pad16(nnz), st)) != TT_OK) return fail(s);
  auto column = [&](int col, int32_t** dst) -> tt_status {
    const size_t np = (size_t)pad16(nnz);
    tt_status s2 = dev_alloc(p, dst, np);
    if (s2 != TT_OK) return s2;
    if (cudaMemsetAsync(*dst, 0, sizeof(int32_t) * np, st) != cudaSuccess ||
        launch_coo_column(dco, nnz, order, col, *dst, st) != cudaSuccess)
      return set_error(TT_ERR_CUDA, "COO column %d", col);
    return TT_OK;
  };
  if (op == TT_OP_MTTKRP) {
    // the leaf and upper coordinates are the COO columns; rows are runs of mode 0
    const int L = order - 1;
    if ((s = column(L, &p->d_crd[L])) != TT_OK) return fail(s);
    if ((s = column(1, &p->d_kexp)) != TT_OK) return fail(s);
    if (order >= 4 && (s = column(2, &p->d_kexp2)) != TT_OK) return fail(s);
    if (order == 5 && (s = column(3, &p->d_kexp3)) != TT_OK) return fail(s);
    if ((s = dev_alloc(p, &p->d_rnz, (size_t)dims[0] + 1)) != TT_OK) return fail(s);
    if (launch_coo_row_starts(dco, nnz, order, dims[0], p->d_rnz, st) != cudaSuccess)
      return fail(set_error(TT_ERR_CUDA, "COO rows"));
  } else {
    // fibers: runs of equal (i, j)
    uint32_t *flags = nullptr, *sums = nullptr;
    uint32_t nfib = 0;
    if ((s = talloc((void**)&flags, sizeof(uint32_t) * ((size_t)nnz + 1))) != TT_OK) return fail(s);
    if ((s = talloc((void**)&sums, sizeof(uint32_t) * (size_t)scan_scratch_entries(nnz + 1))) != TT_OK) return fail(s);
    if (launch_coo_fiber_flags(dco, nnz, order, flags, st) != cudaSuccess)
      return fail(set_error(TT_ERR_CUDA, "COO fiber flags"));
    uint32_t* fid = nullptr;
    if ((s = talloc((void**)&fid, sizeof(uint32_t) * ((size_t)nnz + 1))) != TT_OK) return fail(s);
    if (nnz > 0 && device_exclusive_scan(flags, nnz, fid, sums, &nfib, st) != cudaSuccess)
      return fail(set_error(TT_ERR_CUDA, "COO fiber scan"));
    int32_t* fpos = nullptr;
    if ((s = dev_alloc(p, &fpos, (size_t)nfib + 1)) != TT_OK) return fail(s);
    if ((s = dev_alloc(p, &p->d_fcoords, (size_t)nfib * 2)) != TT_OK) return fail(s);
    const int32_t end = (int32_t)nnz;
    if (launch_coo_fibers(dco, nnz, order, flags, fid, fpos, p->d_fcoords, st) != cudaSuccess ||
        cudaMemcpyAsync(fpos + nfib, &end, sizeof(int32_t), cudaMemcpyHostToDevice, st) != cudaSuccess)
      return fail(set_error(TT_ERR_CUDA, "COO fibers"));
    int32_t* leaf = nullptr;
    if ((s = column(2, &leaf)) != TT_OK) return fail(s);
    if (op == TT_OP_TTV) {
      p->d_pos[2] = fpos;
      p->d_crd[2] = leaf;
      p->nfib_last = nfib;
      p->count[1] = nfib;
      p->count[2] = nnz;
    } else {
      // TTM: a two-level walk, the fibers as rows and the leaf coordinates as its
      // one factor's rows
      p->order = 2;
      p->dims[0] = (int32_t)nfib;
      p->dims[1] = dims[2];
      p->nroot = nfib;
      p->d_rnz = fpos;
      p->d_crd[1] = leaf;
      p->count[0] = nfib;
      p->count[1] = nnz;
    }
  }
  for (int l = 0; l < TT_MAX_ORDER; l++) { p->slab[0].pos[l] = p->d_pos[l]; p->slab[0].crd[l] = p->d_crd[l]; }
  p->slab[0].nnz = nnz;
  if (op == TT_OP_TTV) {
    p->tb = 256;
    p->G = kTtvNpt;
    p->P = 32 * kTtvNpt;
    p->nblocks = (int)((p->nnz + p->P - 1) / p->P);
    if ((s = set_ttv_ranges(p)) != TT_OK) return fail(s);
    if ((s = alloc_walk_scratch(p, p->P)) != TT_OK) return fail(s);
    if ((s = prepare_partition(p)) != TT_OK) return fail(s);
  } else {
    if ((s = dev_alloc(p, &p->d_err, 4)) != TT_OK) return fail(s);
    if (cudaMemsetAsync(p->d_err, 0, 4 * sizeof(int32_t), st) != cudaSuccess)
      return fail(set_error(TT_ERR_CUDA, "clear error word"));
    // the strip family only (no CSF levels): the fixed variant, the strip rule, or
    // a sweep over the strip variants (the learned network scores CSF plans)
    int id;
    if (select == TT_SELECT_FIXED) {
      if (!variant_valid(variant, p->order, p->rank, p->prec) || variant_spec(variant).staged != 4)
        return fail(set_error(TT_ERR_INVALID_ARGUMENT, "variant %d is not a strip variant valid here", variant));
      id = variant;
    } else {
      id = strip_default_variant(p->order, p->rank, p->prec);
    }
    if (id < 0) return fail(set_error(TT_ERR_UNSUPPORTED, "no strip variant for order %d rank %d", p->order, p->rank));
    if ((s = use_variant(p, id)) != TT_OK) return fail(s);
    if (select == TT_SELECT_SWEEP) {
      std::vector<int> all;
      for (int v = 4 * kPerFamily; v < kNumVariants; v++)
        if (variant_valid(v, p->order, p->rank, p->prec)) all.push_back(v);
      if ((s = time_variants(p, st, all, kNumVariants, -1)) != TT_OK) return fail(s);
      p->selected_by = 2;
    }
  }
  if (cudaStreamSynchronize(st) != cudaSuccess) return fail(set_error(TT_ERR_CUDA, "COO plan: %s", cudaGetErrorString(cudaGetLastError())));
  *out = p;
  return TT_OK;
}

TT_EXPORT tt_status tt_plan_destroy(tt_plan* p) {
  if (!p) return TT_OK;
  if (p->ev0) cudaEventDestroy(p->ev0);
  if (p->ev1) cudaEventDestroy(p->ev1);
  if (p->evk0) cudaEventDestroy(p->evk0);
  if (p->evk1) cudaEventDestroy(p->evk1);
  if (!p->allocs.empty()) {
    cudaDeviceSynchronize();  // as cudaFree would
    for (void* a : p->allocs) pool_free(a, p->stream);
    cudaStreamSynchronize(p->stream);
  }
  delete p;
  return TT_OK;
}

TT_EXPORT tt_status tt_plan_set_factors(tt_plan* p, const float* const* factors, void* stream) {
  NvtxRange nvtx_range("tt_plan_set_factors");
  clear_error();
  if (!p || !factors) return set_error(TT_ERR_INVALID_ARGUMENT, "null argument");
  if (p->op != TT_OP_MTTKRP && p->op != TT_OP_TTM)
    return set_error(TT_ERR_INVALID_ARGUMENT, "plan is not an MTTKRP or TTM plan");
  if (p->broken) return broken_error();
  cudaStream_t st = stream ? (cudaStream_t)stream : p->stream;
  const int nm = p->order - 1;
  if (p->op == TT_OP_TTM) {
    // U is rank x K row-major (the reference's C, fmtaco.cpp:117-223): the walk
    // gathers its columns as rows of U^T, K x RP, zero padded
    if (!factors[0]) return set_error(TT_ERR_INVALID_ARGUMENT, "U is null");
    tt_status s2;
    if (!p->fac_own[0]) {
      float* d = nullptr;
      if ((s2 = dev_alloc(p, &d, (size_t)p->dims[1] * p->rp)) != TT_OK) return s2;
      p->fac_own[0] = d;
    }
    CK(launch_transpose_pad(factors[0], p->rank, p->dims[1], p->rp, (float*)p->fac_own[0], st));
    p->fac[0] = p->fac_own[0];
    p->d_colscale = nullptr;
    p->factors_set = true;
    return TT_OK;
  }
  for (int m = 0; m < nm; m++)
    if (!factors[m]) return set_error(TT_ERR_INVALID_ARGUMENT, "factor %d is null", m + 1);
  tt_status s;
  if (p->prec == kFP32) {
    for (int m = 0; m < nm; m++) {
      if (p->rank == p->rp) {
        p->fac[m] = factors[m];
      } else {
        const int64_t rows = p->dims[m + 1];
        if (!p->fac_own[m]) {
          float* d = nullptr;
          if ((s = dev_alloc(p, &d, (size_t)rows * p->rp)) != TT_OK) return s;
          p->fac_own[m] = d;
        }
        CK(launch_pad_fp32(factors[m], rows, p->rank, p->rp, (float*)p->fac_own[m], st));
        p->fac[m] = p->fac_own[m];
      }
    }
    p->d_colscale = nullptr;
  } else {
    if (!p->d_scales) {
      if ((s = dev_alloc(p, &p->d_scales, (size_t)(3 * nm + 1) * p->rp)) != TT_OK) return s;
    }
    const float* inv[4] = {nullptr, nullptr, nullptr, nullptr};
    for (int m = 0; m < nm; m++) {
      const int64_t rows = p->dims[m + 1];
      if (p->prec == kFX16 && m < nm - 1) {
        // 16-bit fixed point keeps the upper-level factors in FP32 (small, L2-resident)
        if (p->rank == p->rp) {
          p->fac[m] = factors[m];
        } else {
          if (!p->fac_own[m]) {
            float* d = nullptr;
            if ((s = dev_alloc(p, &d, (size_t)rows * p->rp)) != TT_OK) return s;
            p->fac_own[m] = d;
          }
          CK(launch_pad_fp32(factors[m], rows, p->rank, p->rp, (float*)p->fac_own[m], st));
          p->fac[m] = p->fac_own[m];
        }
        continue;
      }
      float* cmax = p->d_scales + (size_t)(3 * m) * p->rp;
      float* scl = cmax + p->rp;
      float* iv = scl + p->rp;
      CK(cudaMemsetAsync(cmax, 0, sizeof(float) * p->rp, st));
      CK(launch_colmax(factors[m], rows, p->rank, cmax, st));
      if (!p->fac_own[m]) {
        uint16_t* d = nullptr;
        if ((s = dev_alloc(p, &d, (size_t)rows * p->rp)) != TT_OK) return s;
        p->fac_own[m] = d;
      }
      if (p->prec == kFX16) {
        // leaf factor: column scales, then a power of two per row (kept for the
        // values: each nonzero's value is multiplied by its row's inverse power)
        if (!p->d_rowexp && (s = dev_alloc(p, &p->d_rowexp, (size_t)rows)) != TT_OK) return s;
        if (!p->d_vals_fx && (s = dev_alloc(p, &p->d_vals_fx, p->nvals_alloc)) != TT_OK) return s;
        CK(launch_fullrange_scales(cmax, p->rp, scl, iv, st));
        CK(launch_fx16_rows(factors[m], rows, p->rank, p->rp, scl, (uint16_t*)p->fac_own[m], p->d_rowexp, st));
        CK(launch_fx16_values(static_cast<const float*>(p->d_vals), p->d_crd[p->order - 1], p->d_rowexp,
                              (int64_t)p->nvals_alloc, p->d_vals_fx, st));
      } else {
        const bool h16 = fac_kind(p->prec) == kH16;
        CK(launch_pow2_scales(cmax, p->rp, h16 ? 14 : 0, scl, iv, st));
        CK(launch_to_16(factors[m], rows, p->rank, p->rp, scl, h16 ? 2 : 1, (uint16_t*)p->fac_own[m], st));
      }
      p->fac[m] = p->fac_own[m];
      inv[m] = iv;
    }
    p->d_colscale = p->d_scales + (size_t)(3 * nm) * p->rp;
    CK(launch_scale_product(inv, nm, p->rp, val_kind(p->prec) != kF32 ? p->vinv : 1.f, p->d_colscale, st));
  }
  p->factors_set = true;
  return TT_OK;
}

static tt_status timed_begin(tt_plan* p, cudaStream_t st) {
  if (!p->timing) return TT_OK;
  if (!p->ev0) {
    CK(cudaEventCreate(&p->ev0));
    CK(cudaEventCreate(&p->ev1));
    CK(cudaEventCreate(&p->evk0));
    CK(cudaEventCreate(&p->evk1));
  }
  CK(cudaEventRecord(p->ev0, st));
  return TT_OK;
}
static tt_status timed_end(tt_plan* p, cudaStream_t st) {
  if (!p->timing) return TT_OK;
  CK(cudaEventRecord(p->ev1, st));
  p->timed_pending = true;
  p->kernel_timed = p->timing == 1;
  return TT_OK;
}

TT_EXPORT tt_status tt_plan_mttkrp(tt_plan* p, float* A, void* stream) {
  NvtxRange nvtx_range("tt_plan_mttkrp");
  clear_error();
  if (!p || !A) return set_error(TT_ERR_INVALID_ARGUMENT, "null argument");
  if (p->op != TT_OP_MTTKRP) return set_error(TT_ERR_INVALID_ARGUMENT, "plan is not an MTTKRP plan");
  if (p->broken) return broken_error();
  if (!p->factors_set) return set_error(TT_ERR_INVALID_ARGUMENT, "factors not set (tt_plan_set_factors)");
  cudaStream_t st = stream ? (cudaStream_t)stream : p->stream;
  tt_status s;
  if ((s = timed_begin(p, st)) != TT_OK) return s;
  if ((s = run_mttkrp(p, A, st)) != TT_OK) return s;
  return timed_end(p, st);
}

// TTM of a COO plan: Y (nfibers x rank, DEVICE) from the U last set.
TT_EXPORT tt_status tt_plan_ttm(tt_plan* p, float* Y, void* stream) {
  NvtxRange nvtx_range("tt_plan_ttm");
  clear_error();
  if (!p || !Y) return set_error(TT_ERR_INVALID_ARGUMENT, "null argument");
  if (p->op != TT_OP_TTM) return set_error(TT_ERR_INVALID_ARGUMENT, "plan is not a TTM plan");
  if (p->broken) return broken_error();
  if (!p->factors_set) return set_error(TT_ERR_INVALID_ARGUMENT, "U not set (tt_plan_set_factors)");
  cudaStream_t st = stream ? (cudaStream_t)stream : p->stream;
  tt_status s;
  if ((s = timed_begin(p, st)) != TT_OK) return s;
  if ((s = run_mttkrp(p, Y, st)) != TT_OK) return s;
  return timed_end(p, st);
}

// (i, j) of every fiber of a COO TTV or TTM plan, as 2 * nfibers int32 on the host.
TT_EXPORT tt_status tt_plan_coo_fibers(const tt_plan* p, int32_t* ij) {
  clear_error();
  if (!p || !ij) return set_error(TT_ERR_INVALID_ARGUMENT, "null argument");
  if (!p->coo || (p->op != TT_OP_TTV && p->op != TT_OP_TTM))
    return set_error(TT_ERR_INVALID_ARGUMENT, "not a COO TTV or TTM plan");
  const int64_t nf = p->op == TT_OP_TTV ? p->nfib_last : p->nroot;
  if (nf > 0) CK(cudaMemcpy(ij, p->d_fcoords, sizeof(int32_t) * 2 * (size_t)nf, cudaMemcpyDeviceToHost));
  return TT_OK;
}

TT_EXPORT tt_status tt_plan_ttv(tt_plan* p, const float* x, float* y, void* stream) {
  NvtxRange nvtx_range("tt_plan_ttv");
  clear_error();
  if (!p || !x || !y) return set_error(TT_ERR_INVALID_ARGUMENT, "null argument");
  if (p->op != TT_OP_TTV) return set_error(TT_ERR_INVALID_ARGUMENT, "plan is not a TTV plan");
  if (p->broken) return broken_error();
  cudaStream_t st = stream ? (cudaStream_t)stream : p->stream;
  tt_status s;
  if ((s = timed_begin(p, st)) != TT_OK) return s;
  if ((s = run_ttv(p, x, y, st)) != TT_OK) return s;
  return timed_end(p, st);
}

TT_EXPORT tt_status tt_plan_set_timing(tt_plan* p, int32_t enabled) {
  if (!p) return set_error(TT_ERR_INVALID_ARGUMENT, "null plan");
  if (enabled < 0 || enabled > 2) return set_error(TT_ERR_INVALID_ARGUMENT, "timing mode %d (0, 1 or 2)", (int)enabled);
  p->timing = enabled;
  return TT_OK;
}

TT_EXPORT float tt_plan_last_ms(tt_plan* p) {
  if (!p || !p->timed_pending) return -1.f;
  if (cudaEventSynchronize(p->ev1) != cudaSuccess) return -1.f;
  float ms = -1.f;
  cudaEventElapsedTime(&ms, p->ev0, p->ev1);
  return ms;
}

TT_EXPORT int32_t tt_plan_variant(const tt_plan* p) { return p ? p->variant : -1; }
TT_EXPORT int32_t tt_plan_selected_by(const tt_plan* p) { return p ? p->selected_by : -1; }
TT_EXPORT int32_t tt_plan_slabs(const tt_plan* p) { return p ? p->slabs : -1; }
TT_EXPORT int64_t tt_plan_nnz(const tt_plan* p) { return p ? p->nnz : -1; }
TT_EXPORT int64_t tt_plan_num_fibers(const tt_plan* p, int32_t level) {
  if (!p || level < 0 || level >= p->order) return -1;
  return p->count[level];
}
TT_EXPORT int64_t tt_plan_device_bytes(const tt_plan* p) { return p ? p->device_bytes : -1; }
TT_EXPORT int32_t tt_plan_nblocks(const tt_plan* p) { return p ? p->nblocks : -1; }

// Device-side error word of the plan's kernels (0: none), read after the plan's
// stream has finished.
TT_EXPORT int32_t tt_plan_device_error(tt_plan* p) {
  if (!p || !p->d_err) return 0;
  int32_t e = 0;
  if (cudaStreamSynchronize(p->stream) != cudaSuccess) return -1;
  if (cudaMemcpy(&e, p->d_err, sizeof(int32_t), cudaMemcpyDeviceToHost) != cudaSuccess) return -1;
  return e;
}

// Switch an existing plan to another variant (scratch grows as needed).
TT_EXPORT tt_status tt_plan_use_variant(tt_plan* p, int32_t id) {
  clear_error();
  if (!p || p->op != TT_OP_MTTKRP) return set_error(TT_ERR_INVALID_ARGUMENT, "need an MTTKRP plan");
  if (p->broken) return broken_error();
  if (!variant_valid(id, p->order, p->rank, p->prec)) return set_error(TT_ERR_INVALID_ARGUMENT, "variant %d invalid here", id);
  // a COO plan has no CSF levels: only the strip walk (rows through rnz) reads it
  if (p->coo && variant_spec(id).staged != 4)
    return set_error(TT_ERR_INVALID_ARGUMENT, "variant %d: a COO plan runs the strip family only", id);
  return use_variant(p, id);
}

TT_EXPORT tt_status tt_debug_tma_wait(int32_t withhold, int64_t wait_ns) {
  clear_error();
  if (wait_ns < 0 || wait_ns > 1000000000) return set_error(TT_ERR_INVALID_ARGUMENT, "wait_ns %lld", (long long)wait_ns);
  g_tma_wait_ns.store(wait_ns);
  g_tma_withhold.store(withhold ? 1 : 0);
  return TT_OK;
}

TT_EXPORT tt_status tt_debug_fail_pool_alloc(int64_t n) {
  clear_error();
  if (n < 0) return set_error(TT_ERR_INVALID_ARGUMENT, "n %lld", (long long)n);
  g_fail_countdown.store(n);
  return TT_OK;
}

TT_EXPORT int64_t tt_debug_pool_live(void) { return g_pool_live.load(); }

namespace {
// Time variants (3 runs each after one warm-up) with placeholder factors and keep
// the fastest; timing does not depend on factor values.  cands are tried in order
// until max_timed of them have run (a variant that does not fit this tensor is
// skipped); extra (>= 0), if not timed yet, is timed as well.  The times go to
// sweep_ms (untimed variants keep -1).
tt_status time_variants(tt_plan* p, cudaStream_t st, const std::vector<int>& cands, int max_timed, int extra) {
  // the plan's current variant, if already timed, stays the one to beat
  int best = p->variant;
  float best_ms = best >= 0 && best < kNumVariants && p->sweep_ms[best] > 0.f ? p->sweep_ms[best] : 1e30f;
  tt_status s = TT_OK;
  {
    // placeholder factors and output, and the events; on leaving this block, by
    // any path, the temporaries are freed and the plan gets its own factors back
    struct Scratch {
      tt_plan* p;
      cudaStream_t st;
      const void* saved[4];
      float* saved_scale;
      std::vector<void*> tmp;
      cudaEvent_t e0 = nullptr, e1 = nullptr;
      ~Scratch() {
        if (e0) cudaEventDestroy(e0);
        if (e1) cudaEventDestroy(e1);
        cudaStreamSynchronize(st);
        for (void* d : tmp) pool_free(d, st);
        cudaStreamSynchronize(st);
        for (int m = 0; m < 4; m++) p->fac[m] = saved[m];
        p->d_colscale = saved_scale;
      }
    } sc{p, st, {p->fac[0], p->fac[1], p->fac[2], p->fac[3]}, p->d_colscale, {}};
    const int nm = p->order - 1;
    for (int m = 0; m < nm; m++) {
      // bytes per entry of factor m in this plan's storage (16-bit fixed point keeps
      // the upper-level factors in FP32)
      const size_t esz = p->prec == kFP32 || (p->prec == kFX16 && m < nm - 1) ? 4 : 2;
      void* d = nullptr;
      CK(pool_alloc(&d, (size_t)p->dims[m + 1] * p->rp * esz, st));
      sc.tmp.push_back(d);
      CK(cudaMemsetAsync(d, 0, (size_t)p->dims[m + 1] * p->rp * esz, st));
      p->fac[m] = d;
    }
    p->d_colscale = nullptr;
    float* A = nullptr;
    CK(pool_alloc((void**)&A, (size_t)p->dims[0] * p->rank * sizeof(float), st));
    sc.tmp.push_back(A);
    CK(cudaEventCreate(&sc.e0));
    CK(cudaEventCreate(&sc.e1));
    std::vector<int> order;
    order.reserve(cands.size() + 1);
    for (int id : cands) order.push_back(id);
    if (extra >= 0) order.push_back(extra);
    int timed = 0;
    for (size_t i = 0; i < order.size() && s == TT_OK; i++) {
      const int id = order[i];
      const bool is_extra = extra >= 0 && i + 1 == order.size();
      if (is_extra ? p->sweep_ms[id] >= 0.f : timed >= max_timed) continue;
      if (!variant_valid(id, p->order, p->rank, p->prec)) continue;
      if ((s = use_variant(p, id)) != TT_OK) {
        if (s == TT_ERR_UNSUPPORTED) { s = TT_OK; continue; }  // does not fit this tensor's windows
        break;
      }
      if ((s = run_mttkrp(p, A, st)) != TT_OK) {
        if (s == TT_ERR_UNSUPPORTED) { s = TT_OK; clear_error(); continue; }  // e.g. no TMA descriptor
        break;
      }
      float tot = 0.f;
      for (int r = 0; r < 3; r++) {
        cudaEventRecord(sc.e0, st);
        if ((s = run_mttkrp(p, A, st)) != TT_OK) break;
        cudaEventRecord(sc.e1, st);
        cudaEventSynchronize(sc.e1);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, sc.e0, sc.e1);
        tot += ms;
      }
      if (s != TT_OK) break;
      p->sweep_ms[id] = tot / 3.f;
      timed++;
      if (tot / 3.f < best_ms) { best_ms = tot / 3.f; best = id; }
    }
  }
  if (s != TT_OK) return s;
  if (best < 0) return set_error(TT_ERR_UNSUPPORTED, "no candidate variant runs on this tensor");
  return use_variant(p, best);
}
}  // namespace

// Milliseconds of the work-unit partition computed once when the plan's variant was
// set (0 when the plan runs it in every call: slab passes).
TT_EXPORT float tt_plan_partition_ms(const tt_plan* p) { return p && p->part_ready ? p->part_ms : 0.f; }

// Returns the memory the library's pool keeps for reuse (plans alive keep theirs).
TT_EXPORT tt_status tt_release_cached_memory(void) {
  std::lock_guard<std::mutex> lk(g_pool_mu);
  for (int d = 0; d < kMaxDevices; d++)
    if (g_pool[d] && cudaMemPoolTrimTo(g_pool[d], 0) != cudaSuccess)
      return set_error(TT_ERR_CUDA, "trim device %d pool: %s", d, cudaGetErrorString(cudaGetLastError()));
  return TT_OK;
}

// Per-variant mean ms measured at plan creation by TT_SELECT_SWEEP or by the
// network's timed candidates (negative: not timed).
TT_EXPORT tt_status tt_plan_sweep_times(const tt_plan* p, float* ms, int32_t n) {
  if (!p || !ms) return set_error(TT_ERR_INVALID_ARGUMENT, "null argument");
  for (int i = 0; i < n && i < kNumVariants; i++) ms[i] = p->sweep_ms[i];
  return TT_OK;
}

// The library's stream-ordered device memory pool for the other translation units
// (the GPU CSF builder's scratch): the same accounting and failure injection.
namespace tt {
cudaError_t device_pool_alloc(void** ptr, size_t bytes, cudaStream_t st) { return pool_alloc(ptr, bytes, st); }
void device_pool_free(void* ptr, cudaStream_t st) { pool_free(ptr, st); }
}  // namespace tt

// ---------------------------------------------------------------------------
// one-shot host calls
// ---------------------------------------------------------------------------
namespace {

// Page-locked (registered or pinned-allocated) host memory: copies from it are DMA
// and return at once, so a call can queue all of them before its device work.
bool host_pinned(const void* ptr) {
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, ptr) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return at.type == cudaMemoryTypeHost;
}

// Nonzeros per chunk of the leaf coordinates in the overlapped one-shot call: a
// multiple of the work unit, at most 16 chunks, at least 64 units each.
int64_t oneshot_chunk(int64_t nnz, int P) {
  const int64_t c = std::max<int64_t>((int64_t)P * 64, (nnz + 15) / 16);
  return (c + P - 1) / P * P;
}

// The one-shot MTTKRP of a strip-walk variant over page-locked host buffers, with
// the host-to-device copies overlapped with the device work.  The copies bound the
// call (a GB300 moves host data at about 200 GB/s, from one stream as from
// several), so the rest runs under them:
//   copy stream  the fiber structure, the values, the factors, then the leaf
//                coordinates in chunks (starting on 128-byte host boundaries);
//   check stream each chunk's leaf coordinates as the chunk lands;
//   work stream  the structure check (the host waits for its result before
//                anything indexes through pos), kexp / rnz / the partition (the
//                structure alone), the value and factor conversion, then per
//                checked chunk the walk of every unit whose nonzeros have all
//                arrived; the row merge, and A.  (A chunk's check, about 35 us for
//                6M nonzeros, runs beside the previous chunk's walk instead of
//                before it: the walks keep up with the copies.)
// Results are bit-identical to the serial path: the same conversions, the same walk
// of every unit and the same fixed-order merge.  A chunk's check overwrites an
// out-of-range leaf coordinate with 0 before the chunk's walk runs; the call then
// reports the first violation and leaves A untouched.
tt_status oneshot_overlapped(taco_tensor_t* A, const CsfView& v, const taco_tensor_t* const* factors, int prec,
                             int variant, int rank) {
  NvtxRange nvtx_range("tt_mttkrp_host: overlapped");
  tt_status s = csf_check_root(v);
  if (s != TT_OK) return s;
  const int L = v.order - 1, nm = v.order - 1;
  const int64_t nnz = v.nnz;
  cudaStream_t cs = nullptr, xs = nullptr, ks = nullptr;
  std::vector<cudaEvent_t> evs;
  std::vector<float*> dfac(nm, nullptr);
  float *dA = nullptr, *tmp = nullptr;
  uint32_t *starts_up = nullptr, *starts_leaf = nullptr;
  unsigned long long* err = nullptr;
  tt_plan* p = nullptr;
  auto cleanup = [&](tt_status st2) {
    // copies still in flight land in buffers that go back to the pool
    if (xs) cudaStreamSynchronize(xs);
    if (ks) cudaStreamSynchronize(ks);
    if (cs) cudaStreamSynchronize(cs);
    for (float* d : dfac) pool_free(d, cs);
    pool_free(dA, cs);
    pool_free(tmp, cs);
    pool_free(starts_up, cs);
    pool_free(starts_leaf, cs);
    pool_free(err, cs);
    tt_plan_destroy(p);
    if (cs) cudaStreamSynchronize(cs);
    for (cudaEvent_t e : evs) cudaEventDestroy(e);
    if (xs) cudaStreamDestroy(xs);
    if (ks) cudaStreamDestroy(ks);
    if (cs) cudaStreamDestroy(cs);
    return st2;
  };
  auto cuda_fail = [&](cudaError_t e, const char* what) {
    return cleanup(set_error(e == cudaErrorMemoryAllocation ? TT_ERR_OUT_OF_MEMORY : TT_ERR_CUDA, "%s: %s", what,
                             cudaGetErrorString(e)));
  };
  auto event = [&](cudaEvent_t* e, bool timing) {
    const cudaError_t r = cudaEventCreateWithFlags(e, timing ? cudaEventDefault : cudaEventDisableTiming);
    if (r == cudaSuccess) evs.push_back(*e);
    return r;
  };
  cudaError_t e = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&xs, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ks, cudaStreamNonBlocking);
  if (e != cudaSuccess) return cuda_fail(e, "streams");

  p = new tt_plan();
  cudaGetDevice(&p->device);
  p->op = TT_OP_MTTKRP;
  p->order = v.order;
  for (int i = 0; i < v.order; i++) p->dims[i] = v.dims[i];
  p->nnz = nnz;
  p->nroot = v.nroot;
  p->dense_root = true;
  p->rank = rank;
  p->rp = rank_pad(rank);
  p->prec = prec;
  p->stream = cs;
  for (int l = 0; l < v.order; l++) p->count[l] = v.count[l];
  p->nfib_last = v.count[v.order - 2];
  p->slabs = 1;
  p->leaf_len = nnz;

  // device buffers (stream-ordered on the work stream; the copy stream waits)
  for (int l = 1; l <= L; l++) {
    if ((s = dev_alloc(p, &p->d_pos[l], (size_t)v.count[l - 1] + 1)) != TT_OK) return cleanup(s);
    if ((s = dev_alloc(p, &p->d_crd[l], l == L ? (size_t)pad16(nnz) : (size_t)v.count[l])) != TT_OK) return cleanup(s);
  }
  e = cudaMemsetAsync(p->d_crd[L] + nnz, 0, sizeof(int32_t) * (size_t)(pad16(nnz) - nnz), cs);
  for (int l = 0; l < TT_MAX_ORDER; l++) { p->slab[0].pos[l] = p->d_pos[l]; p->slab[0].crd[l] = p->d_crd[l]; }
  for (int l = 0; l < v.order; l++) p->slab[0].count[l] = v.count[l];
  p->slab[0].nnz = nnz;
  p->slab[0].off = 0;
  const bool v16 = val_kind(prec) != kF32;
  p->nvals_alloc = (size_t)pad16(nnz);
  if (v16) {
    uint16_t* d = nullptr;
    if ((s = dev_alloc(p, &d, p->nvals_alloc)) != TT_OK) return cleanup(s);
    p->d_vals = d;
    if (e == cudaSuccess) e = cudaMemsetAsync(d + nnz, 0, (p->nvals_alloc - (size_t)nnz) * 2, cs);
    if (e == cudaSuccess) e = pool_alloc((void**)&tmp, (size_t)nnz * 4 + 64, cs);
  } else {
    float* d = nullptr;
    if ((s = dev_alloc(p, &d, p->nvals_alloc)) != TT_OK) return cleanup(s);
    p->d_vals = d;
    if (e == cudaSuccess) e = cudaMemsetAsync(d + nnz, 0, (p->nvals_alloc - (size_t)nnz) * 4, cs);
  }
  if ((s = dev_alloc(p, &p->d_err, 4)) != TT_OK) return cleanup(s);
  if (e == cudaSuccess) e = cudaMemsetAsync(p->d_err, 0, 4 * sizeof(int32_t), cs);
  for (int m = 0; m < nm && e == cudaSuccess; m++)
    e = pool_alloc((void**)&dfac[m], (size_t)v.dims[m + 1] * rank * sizeof(float), cs);
  const size_t abytes = (size_t)v.dims[0] * rank * sizeof(float);
  if (e == cudaSuccess) e = pool_alloc((void**)&dA, abytes, cs);
  int64_t upmax = 1;
  for (int l = 1; l < L; l++) upmax = std::max<int64_t>(upmax, v.count[l]);
  if (e == cudaSuccess) e = pool_alloc((void**)&starts_up, sizeof(uint32_t) * (size_t)((upmax + 31) / 32 + 1), cs);
  if (e == cudaSuccess) e = pool_alloc((void**)&starts_leaf, sizeof(uint32_t) * (size_t)((nnz + 31) / 32 + 1), cs);
  if (e == cudaSuccess) e = pool_alloc((void**)&err, sizeof(unsigned long long) * 2 * (size_t)L, cs);
  if (e == cudaSuccess) e = cudaMemsetAsync(err, 0xff, sizeof(unsigned long long) * 2 * (size_t)L, cs);
  cudaEvent_t ev_alloc, ev_struct, ev_vals, ev_fac;
  if (e == cudaSuccess) e = event(&ev_alloc, false);
  if (e == cudaSuccess) e = event(&ev_struct, false);
  if (e == cudaSuccess) e = event(&ev_vals, false);
  if (e == cudaSuccess) e = event(&ev_fac, false);
  if (e == cudaSuccess) e = cudaEventRecord(ev_alloc, cs);
  if (e != cudaSuccess) return cuda_fail(e, "one-shot setup");

  // copy stream, first part: the fiber structure, then the values
  e = cudaStreamWaitEvent(xs, ev_alloc, 0);
  for (int l = 1; l <= L && e == cudaSuccess; l++) {
    e = htod_async(p->d_pos[l], v.pos[l], sizeof(int32_t) * (size_t)(v.count[l - 1] + 1), xs);
    if (e == cudaSuccess && l < L)
      e = htod_async(p->d_crd[l], v.crd[l], sizeof(int32_t) * (size_t)v.count[l], xs);
  }
  if (e == cudaSuccess) e = cudaEventRecord(ev_struct, xs);
  if (e == cudaSuccess) e = htod_async(v16 ? (void*)tmp : p->d_vals, v.vals, (size_t)nnz * 4, xs);
  if (e == cudaSuccess) e = cudaEventRecord(ev_vals, xs);
  if (e != cudaSuccess) return cuda_fail(e, "upload");

  // structure check: every pos, the upper levels' crd; the leaf fiber starts are
  // kept for the leaf chunks' checks
  e = cudaStreamWaitEvent(cs, ev_struct, 0);
  for (int l = 1; l <= L && e == cudaSuccess; l++) {
    e = launch_csf_pos_check(p->d_pos[l], v.count[l - 1], l >= 2 ? 1 : 0, v.count[l], l == L ? starts_leaf : starts_up,
                             err + 2 * (l - 1), cs);
    if (e == cudaSuccess && l < L)
      e = launch_csf_crd_check_range(p->d_crd[l], 0, v.count[l], v.dims[l], starts_up, err + 2 * (l - 1) + 1, 0, cs);
  }
  unsigned long long h[2 * TT_MAX_ORDER];
  if (e == cudaSuccess) e = cudaMemcpyAsync(h, err, sizeof(unsigned long long) * 2 * (size_t)L, cudaMemcpyDeviceToHost, cs);
  if (e == cudaSuccess) e = cudaStreamSynchronize(cs);
  if (e != cudaSuccess) return cuda_fail(e, "structure check");
  for (int l = 1; l <= L; l++) {
    s = csf_check_error(l, h[2 * (l - 1)]);
    if (s == TT_OK && l < L) s = csf_check_error(l, h[2 * (l - 1) + 1]);
    if (s != TT_OK) return cleanup(s);
  }
  // the variant: scratch, kexp / rnz, the partition (structure only)
  if ((s = use_variant(p, variant)) != TT_OK) return cleanup(s);

  // copy stream, second part: the factors, then the leaf coordinates in chunks
  // that start on 128-byte host boundaries (the first chunk absorbs the
  // misaligned head); a chunk's walk takes every unit whose nonzeros have arrived
  const int64_t chunk = oneshot_chunk(nnz, p->P);
  const uintptr_t lmis = (uintptr_t)v.crd[L] & 127;
  const int64_t lhead = lmis % 4 == 0 && lmis ? (int64_t)(128 - lmis) / 4 : 0;
  std::vector<int64_t> bounds{0};
  for (int64_t x = lhead + chunk; x < nnz; x += chunk) bounds.push_back(x);
  bounds.push_back(nnz);
  const int K = (int)bounds.size() - 1;
  std::vector<cudaEvent_t> ev_chunk(K), ev_chk(K), ev_w0(K), ev_w1(K);
  e = cudaSuccess;
  for (int i = 0; i < K && e == cudaSuccess; i++) {
    e = event(&ev_chunk[i], false);
    if (e == cudaSuccess) e = event(&ev_chk[i], false);
    if (e == cudaSuccess) e = event(&ev_w0[i], true);
    if (e == cudaSuccess) e = event(&ev_w1[i], true);
  }
  for (int m = 0; m < nm && e == cudaSuccess; m++)
    e = htod_async(dfac[m], factors[m]->vals, (size_t)v.dims[m + 1] * rank * sizeof(float), xs);
  if (e == cudaSuccess) e = cudaEventRecord(ev_fac, xs);
  for (int i = 0; i < K && e == cudaSuccess; i++) {
    const int64_t c0 = bounds[i], c1 = bounds[i + 1];
    e = htod_async(p->d_crd[L] + c0, v.crd[L] + c0, sizeof(int32_t) * (size_t)(c1 - c0), xs);
    if (e == cudaSuccess) e = cudaEventRecord(ev_chunk[i], xs);
  }
  if (e != cudaSuccess) return cuda_fail(e, "upload");
  // check stream: each chunk's leaf coordinates as it lands, in chunk order (a
  // chunk's first position is compared with the previous chunk's last), while the
  // previous chunk is walked; a walk waits for its chunk's check (the clamp of
  // out-of-range coordinates comes before any gather)
  for (int i = 0; i < K && e == cudaSuccess; i++) {
    e = cudaStreamWaitEvent(ks, ev_chunk[i], 0);
    if (e == cudaSuccess)
      e = launch_csf_crd_check_range(p->d_crd[L], bounds[i], bounds[i + 1], v.dims[L], starts_leaf,
                                     err + 2 * (L - 1) + 1, 1, ks);
    if (e == cudaSuccess) e = cudaEventRecord(ev_chk[i], ks);
  }
  if (e != cudaSuccess) return cuda_fail(e, "leaf check");

  // values: one power-of-two scale for 16-bit storage (the factors' output scale
  // needs it on the host)
  e = cudaStreamWaitEvent(cs, ev_vals, 0);
  if (e == cudaSuccess && v16) {
    const bool h16 = prec == kFP16;
    float* cmax = reinterpret_cast<float*>(((uintptr_t)(tmp + nnz) + 15) & ~(uintptr_t)15);
    float vinv = 1.f;
    e = launch_colmax(tmp, nnz, 1, cmax, cs);
    if (e == cudaSuccess) e = launch_pow2_scales(cmax, 1, h16 ? 14 : 0, cmax + 1, cmax + 2, cs);
    if (e == cudaSuccess) e = launch_to_16(tmp, nnz, 1, 1, cmax + 1, h16 ? 2 : 1, (uint16_t*)p->d_vals, cs);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&vinv, cmax + 2, 4, cudaMemcpyDeviceToHost, cs);
    if (e == cudaSuccess) e = cudaStreamSynchronize(cs);
    p->vinv = vinv;
  }
  if (e == cudaSuccess) e = cudaStreamWaitEvent(cs, ev_fac, 0);
  if (e != cudaSuccess) return cuda_fail(e, "value conversion");
  if ((s = tt_plan_set_factors(p, (const float* const*)dfac.data(), cs)) != TT_OK) return cleanup(s);

  // per chunk, once it is checked: walk the units that have arrived
  const size_t smem = variant_smem(variant_spec(p->variant), p->rp, p->prec, p->wcap, p->order);
  WalkArgs a = walk_args(p, dA, 0);
  a.smem_bytes = (int32_t)smem;
  cudaEvent_t ev_m0, ev_m1;
  e = event(&ev_m0, true);
  if (e == cudaSuccess) e = event(&ev_m1, true);
  if (e == cudaSuccess) e = cudaMemsetAsync(dA, 0, abytes, cs);
  int32_t ulo = 0;
  for (int i = 0; i < K && e == cudaSuccess; i++) {
    const int64_t c0 = bounds[i], c1 = bounds[i + 1];
    e = cudaStreamWaitEvent(cs, ev_chk[i], 0);
    const int32_t uhi = i == K - 1 ? a.nblocks : (int32_t)(c1 / p->P);
    if (e == cudaSuccess) e = cudaEventRecord(ev_w0[i], cs);
    if (e == cudaSuccess && uhi > ulo) {
      a.unit_lo = ulo;
      a.unit_hi = uhi;
      e = p->launcher(a, uhi - ulo, p->tb, smem, cs);
      ulo = uhi;
    }
    if (e == cudaSuccess) e = cudaEventRecord(ev_w1[i], cs);
  }
  a.unit_lo = 0;
  a.unit_hi = 0;
  if (e == cudaSuccess) e = cudaEventRecord(ev_m0, cs);
  if (e == cudaSuccess) e = launch_chain_fixup(p->order, a, cs);
  if (e == cudaSuccess) e = cudaEventRecord(ev_m1, cs);
  int32_t derr = 0;
  if (e == cudaSuccess) e = cudaMemcpyAsync(h, err + 2 * (L - 1) + 1, sizeof(unsigned long long), cudaMemcpyDeviceToHost, cs);
  if (e == cudaSuccess) e = cudaMemcpyAsync(&derr, p->d_err, sizeof(int32_t), cudaMemcpyDeviceToHost, cs);
  if (e == cudaSuccess) e = cudaStreamSynchronize(cs);
  if (e != cudaSuccess) return cuda_fail(e, "walk");
  if ((s = csf_check_error(L, h[0])) != TT_OK) return cleanup(s);
  if (derr != 0)
    return cleanup(set_error(derr == 301 ? TT_ERR_DEVICE_WAIT : TT_ERR_CUDA, "device error word %d", (int)derr));
  e = cudaMemcpyAsync(A->vals, dA, abytes, cudaMemcpyDeviceToHost, cs);
  if (e == cudaSuccess) e = cudaStreamSynchronize(cs);
  if (e != cudaSuccess) return cuda_fail(e, "download A");
  // the legacy timer: the walks, the merge and the partition (kernel time, not the copies)
  float ms = 0.f, t = 0.f;
  for (int i = 0; i < K; i++)
    if (cudaEventElapsedTime(&t, ev_w0[i], ev_w1[i]) == cudaSuccess) ms += t;
  if (cudaEventElapsedTime(&t, ev_m0, ev_m1) == cudaSuccess) ms += t;
  g_legacy_ms.store(ms + (p->part_ready ? p->part_ms : 0.f));
  return cleanup(TT_OK);
}

}  // namespace

TT_EXPORT tt_status tt_mttkrp_host(taco_tensor_t* A, const taco_tensor_t* B,
                                   const taco_tensor_t* const* factors, tt_precision prec,
                                   tt_select select, int32_t variant) {
  NvtxRange nvtx_range("tt_mttkrp_host");
  clear_error();
  if (!A || !B || !factors || !A->vals || !A->dimensions || !B->dimensions)
    return set_error(TT_ERR_INVALID_ARGUMENT, "null argument");
  const int order = B->order;
  if (order < 3 || order > 5) return set_error(TT_ERR_UNSUPPORTED, "MTTKRP needs order 3, 4 or 5 (got %d)", order);
  const int rank = A->dimensions[1];
  if (A->dimensions[0] != B->dimensions[0]) return set_error(TT_ERR_INVALID_ARGUMENT, "A rows %d != B dims[0] %d", A->dimensions[0], B->dimensions[0]);
  for (int m = 0; m < order - 1; m++) {
    const taco_tensor_t* F = factors[m];
    if (!F || !F->vals || !F->dimensions) return set_error(TT_ERR_INVALID_ARGUMENT, "factor %d missing", m + 1);
    if (F->dimensions[1] != rank || F->dimensions[0] != B->dimensions[m + 1])
      return set_error(TT_ERR_INVALID_ARGUMENT, "factor %d is %dx%d, expected %dx%d", m + 1, F->dimensions[0], F->dimensions[1], B->dimensions[m + 1], rank);
  }
  // a strip-walk variant over page-locked host buffers: the copies overlapped
  if (select == TT_SELECT_FIXED || select == TT_SELECT_DEFAULT) {
    CsfView v;
    int ndev = 0;
    if (csf_view(B, &v) == TT_OK && v.dense_root && v.nnz > 0 && prec != TT_PREC_FX16 && rank >= 1 && rank <= TT_MAX_RANK &&
        cudaGetDeviceCount(&ndev) == cudaSuccess && ndev > 0) {
      const int id = select == TT_SELECT_FIXED ? variant : default_variant(order, rank, (int)prec, v.nnz);
      bool pinned = variant_valid(id, order, rank, (int)prec) && variant_spec(id).staged == 4 && host_pinned(v.vals);
      for (int l = 1; pinned && l < order; l++) pinned = host_pinned(v.pos[l]) && host_pinned(v.crd[l]);
      for (int m = 0; pinned && m < order - 1; m++) pinned = host_pinned(factors[m]->vals);
      if (pinned) return oneshot_overlapped(A, v, factors, (int)prec, id, rank);
    }
    cudaGetLastError();
    clear_error();
  }
  // one call cannot repay the slab-major layout's one-time host build: no slabs
  tt_plan_options opts{};
  opts.slabs = 1;
  tt_plan* p = nullptr;
  tt_status s = tt_plan_create_ex(B, TT_OP_MTTKRP, rank, prec, select, variant, &opts, nullptr, &p);
  if (s != TT_OK) return s;
  std::vector<float*> dfac(order - 1, nullptr);
  float* dA = nullptr;
  auto cleanup = [&]() {
    for (float* d : dfac) pool_free(d, 0);
    pool_free(dA, 0);
    tt_plan_destroy(p);
  };
  for (int m = 0; m < order - 1; m++) {
    const size_t bytes = (size_t)factors[m]->dimensions[0] * rank * sizeof(float);
    if (pool_alloc((void**)&dfac[m], bytes, 0) != cudaSuccess) { cleanup(); return set_error(TT_ERR_OUT_OF_MEMORY, "factor %d", m + 1); }
    if (htod_async(dfac[m], factors[m]->vals, bytes, 0) != cudaSuccess || cudaStreamSynchronize(0) != cudaSuccess) { cleanup(); return set_error(TT_ERR_CUDA, "upload factor %d", m + 1); }
  }
  const size_t abytes = (size_t)A->dimensions[0] * rank * sizeof(float);
  if (pool_alloc((void**)&dA, abytes, 0) != cudaSuccess) { cleanup(); return set_error(TT_ERR_OUT_OF_MEMORY, "output"); }
  tt_plan_set_timing(p, 2);  // the whole call (no event between the walk and the merge)
  if ((s = tt_plan_set_factors(p, (const float* const*)dfac.data(), nullptr)) != TT_OK) { cleanup(); return s; }
  if ((s = tt_plan_mttkrp(p, dA, nullptr)) != TT_OK) { cleanup(); return s; }
  // the reference times partition + clear + kernel per call; the plan ran its
  // partition once at creation
  g_legacy_ms.store(tt_plan_last_ms(p) + (p->part_ready ? p->part_ms : 0.f));
  if (cudaMemcpy(A->vals, dA, abytes, cudaMemcpyDeviceToHost) != cudaSuccess) {
    tt_status e = set_error(TT_ERR_CUDA, "download A: %s", cudaGetErrorString(cudaGetLastError()));
    cleanup();
    return e;
  }
  // a walk that gave up (a bounded wait that ran out: 301) left A incomplete
  const int32_t derr = tt_plan_device_error(p);
  if (derr != 0) {
    tt_status e = set_error(derr == 301 ? TT_ERR_DEVICE_WAIT : TT_ERR_CUDA, "device error word %d", (int)derr);
    cleanup();
    return e;
  }
  cleanup();
  return TT_OK;
}

TT_EXPORT tt_status tt_ttv_host(taco_tensor_t* y, const taco_tensor_t* B, const taco_tensor_t* x) {
  NvtxRange nvtx_range("tt_ttv_host");
  clear_error();
  if (!y || !B || !x || !y->vals || !x->vals) return set_error(TT_ERR_INVALID_ARGUMENT, "null argument");
  tt_plan* p = nullptr;
  tt_status s = tt_plan_create(B, TT_OP_TTV, 1, TT_PREC_FP32, TT_SELECT_DEFAULT, 0, nullptr, &p);
  if (s != TT_OK) return s;
  const int64_t nx = B->dimensions[B->order - 1];
  const int64_t ny = p->nfib_last;
  if (y->dimensions && y->dimensions[0] < ny) { tt_plan_destroy(p); return set_error(TT_ERR_INVALID_ARGUMENT, "y has %d entries, need %lld", y->dimensions[0], (long long)ny); }
  if (x->dimensions && x->dimensions[0] < nx) { tt_plan_destroy(p); return set_error(TT_ERR_INVALID_ARGUMENT, "x has %d entries, need %lld", x->dimensions[0], (long long)nx); }
  float *dx = nullptr, *dy = nullptr;
  auto cleanup = [&]() {
    pool_free(dx, 0);
    pool_free(dy, 0);
    tt_plan_destroy(p);
  };
  if (pool_alloc((void**)&dx, sizeof(float) * (size_t)std::max<int64_t>(1, nx), 0) != cudaSuccess ||
      pool_alloc((void**)&dy, sizeof(float) * (size_t)std::max<int64_t>(1, ny), 0) != cudaSuccess) {
    cleanup();
    return set_error(TT_ERR_OUT_OF_MEMORY, "ttv buffers");
  }
  if (cudaMemcpy(dx, x->vals, sizeof(float) * (size_t)nx, cudaMemcpyHostToDevice) != cudaSuccess) { cleanup(); return set_error(TT_ERR_CUDA, "upload x"); }
  tt_plan_set_timing(p, 2);  // the whole call (no event between the walk and the merge)
  if ((s = tt_plan_ttv(p, dx, dy, nullptr)) != TT_OK) { cleanup(); return s; }
  g_legacy_ms.store(tt_plan_last_ms(p) + (p->part_ready ? p->part_ms : 0.f));
  if (cudaMemcpy(y->vals, dy, sizeof(float) * (size_t)ny, cudaMemcpyDeviceToHost) != cudaSuccess) { cleanup(); return set_error(TT_ERR_CUDA, "download y"); }
  cleanup();
  return TT_OK;
}

namespace tt {
float legacy_last_ms() { return g_legacy_ms.load(); }
}  // namespace tt

TT_EXPORT const char* tt_last_error_string(void) { return tt::g_last_error_cstr(); }

// ---------------------------------------------------------------------------
// device buffers and timing for callers without CUDA bindings (ctypes, cgo)
// ---------------------------------------------------------------------------
TT_EXPORT tt_status tt_device_malloc(int64_t bytes, void** ptr) {
  clear_error();
  if (!ptr || bytes < 0) return set_error(TT_ERR_INVALID_ARGUMENT, "bad allocation request");
  *ptr = nullptr;
  CK(cudaMalloc(ptr, (size_t)std::max<int64_t>(bytes, 1)));
  return TT_OK;
}
TT_EXPORT tt_status tt_device_free(void* ptr) {
  clear_error();
  CK(cudaFree(ptr));
  return TT_OK;
}
// Page-lock a caller's host buffer so that copies from and to it are direct DMA
// (what a caller keeping its inputs in pinned memory gets); already registered
// memory is accepted.
TT_EXPORT tt_status tt_host_register(void* ptr, int64_t bytes) {
  clear_error();
  if (!ptr || bytes <= 0) return set_error(TT_ERR_INVALID_ARGUMENT, "bad host range");
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
    cudaGetLastError();
    return set_error(TT_ERR_NO_DEVICE, "no CUDA device visible");
  }
  const cudaError_t e = cudaHostRegister(ptr, (size_t)bytes, cudaHostRegisterDefault);
  if (e == cudaErrorHostMemoryAlreadyRegistered) {
    cudaGetLastError();
    return TT_OK;
  }
  if (e != cudaSuccess) return set_error(TT_ERR_CUDA, "host register: %s", cudaGetErrorString(e));
  return TT_OK;
}
TT_EXPORT tt_status tt_host_unregister(void* ptr) {
  clear_error();
  if (!ptr) return set_error(TT_ERR_INVALID_ARGUMENT, "null pointer");
  CK(cudaHostUnregister(ptr));
  return TT_OK;
}
TT_EXPORT tt_status tt_memcpy_htod(void* dst, const void* src, int64_t bytes) {
  clear_error();
  CK(htod_async(dst, src, (size_t)bytes, 0));
  CK(cudaStreamSynchronize(0));
  return TT_OK;
}
TT_EXPORT tt_status tt_memcpy_dtoh(void* dst, const void* src, int64_t bytes) {
  clear_error();
  CK(cudaMemcpy(dst, src, (size_t)bytes, cudaMemcpyDeviceToHost));
  return TT_OK;
}
TT_EXPORT tt_status tt_device_synchronize(void) {
  clear_error();
  CK(cudaDeviceSynchronize());
  return TT_OK;
}
TT_EXPORT int32_t tt_device_count(void) {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess) { cudaGetLastError(); return 0; }
  return n;
}

// Evict L2 between timed steps: write a buffer larger than the 129 MB L2.
TT_EXPORT tt_status tt_l2_flush(void* stream) {
  clear_error();
  static void* buf = nullptr;
  static const size_t bytes = (size_t)512 << 20;
  static std::mutex mu;
  {
    std::lock_guard<std::mutex> g(mu);
    if (!buf) CK(cudaMalloc(&buf, bytes));
  }
  CK(cudaMemsetAsync(buf, 0x5a, bytes, (cudaStream_t)stream));
  return TT_OK;
}

// Milliseconds of the walk kernel alone in the last timed call (no partition, no clear).
TT_EXPORT float tt_plan_last_kernel_ms(tt_plan* p) {
  if (!p || !p->timed_pending || !p->kernel_timed || !p->evk0) return -1.f;
  if (cudaEventSynchronize(p->ev1) != cudaSuccess) return -1.f;
  float ms = -1.f;
  cudaEventElapsedTime(&ms, p->evk0, p->evk1);
  return ms;
}
