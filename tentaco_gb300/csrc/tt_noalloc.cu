// tt_noalloc.cu -- a 3-mode MTTKRP entry point that allocates no device memory.
//
// Some callers cannot call cudaMalloc (or anything that allocates) at the point
// where they need an MTTKRP: code running inside a memory pool or arena they do
// not own, real-time loops that must never hit the driver's allocator (and its
// implicit device synchronisation), or hosts that only hand this library
// pointers into memory they manage themselves.  tt_mttkrp3_noalloc serves them:
// the caller passes the CSF, the factors and the output, all already on the
// device, and the only device memory the call uses beyond them is the fixed
// scratch array below, which every GPU that loads this library holds until the
// process exits.
//
// The scratch holds what the walk kernel needs besides its inputs and outputs:
// the per-block partition, the per-block row metadata, the cross-block carry
// rows and the FP64 partials of the two-level cross-block merge.
#include <cuda_runtime.h>
#include "tt_internal.h"
#include "tt_kernels.h"
#include "tt_mttkrp.cuh"

namespace {

// One fixed variant: 256 threads, 8 lanes per factor row, 64 nonzeros per team,
// so a block covers 32 * 64 = 2048 nonzeros.
constexpr int kTB = 256;
constexpr int kLPR = 8;
constexpr int kG = 64;
constexpr int kP = (kTB / kLPR) * kG;

// Limit of the scratch array (about 4.7 MB): its parts are sized per block of the
// walk, so the nonzero count is what it bounds; the output rows live in the
// caller's A and need no scratch.
constexpr int64_t kMaxBlocks = 8192;     // so nnz <= 8192 * 2048 = 16,777,216
constexpr int kMaxRankPad = 64;
constexpr size_t kMetaBytes = (size_t)kMaxBlocks * 16;
constexpr size_t kPartBytes = (((size_t)(kMaxBlocks + 1) * 2 * 4) + 255) & ~(size_t)255;
constexpr size_t kCarryBytes = (size_t)2 * kMaxBlocks * kMaxRankPad * 4;
constexpr size_t kMaxSegs = (kMaxBlocks + tt::kSeg - 1) / tt::kSeg;
constexpr size_t kSegMetaBytes = kMaxSegs * 16;
constexpr size_t kSegCarryBytes = 2 * kMaxSegs * kMaxRankPad * 8;
constexpr size_t kScratchBytes = kMetaBytes + kPartBytes + kCarryBytes + kSegMetaBytes + kSegCarryBytes;

// Every call writes the parts of it that it reads (partition, metadata, carries).
static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

// Device address of the scratch array on the current device.  In host code the
// array's name is only a host-side stand-in, so the address is looked up with the
// device current; it is looked up on every call (no allocation, and no address
// kept that a device reset would leave stale).
tt_status scratch_address(void** out) {
  void* p = nullptr;
  const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
  if (e != cudaSuccess || !p)
    return tt::set_error(TT_ERR_CUDA, "cudaGetSymbolAddress(scratch): %s", cudaGetErrorString(e));
  *out = p;
  return TT_OK;
}

template <int CPT>
cudaError_t launch_exact(const tt::WalkArgs& a, int grid, size_t smem, cudaStream_t s) {
  tt::mttkrp_walk_kernel<3, tt::kFP32, CPT, kLPR, true><<<grid, kTB, smem, s>>>(a);
  return cudaGetLastError();
}

bool aligned16(const void* p) { return ((uintptr_t)p & 15u) == 0; }

}  // namespace

// See include/tentaco/tentaco.h for the contract.
TT_EXPORT tt_status tt_mttkrp3_noalloc(int32_t nrows, int64_t nnz, int32_t rank,
                                       const int32_t* pos1, const int32_t* crd1,
                                       const int32_t* pos2, const int32_t* crd2,
                                       const float* vals, const float* C, const float* D,
                                       float* A, void* stream) {
  tt::clear_error();
  if (rank != 8 && rank != 16 && rank != 32 && rank != 64)
    return tt::set_error(TT_ERR_UNSUPPORTED, "tt_mttkrp3_noalloc: rank must be 8, 16, 32 or 64 (got %d)", rank);
  if (nrows < 1 || nnz < 0 || !pos1 || !pos2 || !A || (nnz > 0 && (!crd1 || !crd2 || !vals || !C || !D)))
    return tt::set_error(TT_ERR_INVALID_ARGUMENT, "tt_mttkrp3_noalloc: null pointer or negative size");
  const int64_t nblocks = (nnz + kP - 1) / kP;
  if (nblocks > kMaxBlocks)
    return tt::set_error(TT_ERR_INVALID_ARGUMENT,
                         "tt_mttkrp3_noalloc: %lld nonzeros exceed the scratch limit of %lld; use tt_plan_create",
                         (long long)nnz, (long long)(kMaxBlocks * kP));
  if (!aligned16(crd2) || !aligned16(vals) || !aligned16(C) || !aligned16(D) || !aligned16(A))
    return tt::set_error(TT_ERR_INVALID_ARGUMENT,
                         "tt_mttkrp3_noalloc: crd2, vals, C, D and A must be 16-byte aligned");
  void* scratch = nullptr;
  tt_status st = scratch_address(&scratch);
  if (st != TT_OK) return st;
  cudaStream_t s = (cudaStream_t)stream;
  int32_t* meta = static_cast<int32_t*>(scratch);
  int32_t* part = reinterpret_cast<int32_t*>(static_cast<unsigned char*>(scratch) + kMetaBytes);
  float* carry = reinterpret_cast<float*>(static_cast<unsigned char*>(scratch) + kMetaBytes + kPartBytes);
  int32_t* segmeta = reinterpret_cast<int32_t*>(reinterpret_cast<unsigned char*>(carry) + kCarryBytes);
  double* segcarry = reinterpret_cast<double*>(reinterpret_cast<unsigned char*>(segmeta) + kSegMetaBytes);

  cudaError_t e = cudaMemsetAsync(A, 0, sizeof(float) * (size_t)nrows * (size_t)rank, s);
  if (e != cudaSuccess) return tt::set_error(TT_ERR_CUDA, "clear A: %s", cudaGetErrorString(e));
  if (nnz == 0) return TT_OK;

  tt::WalkArgs a{};
  a.pos[1] = pos1;
  a.pos[2] = pos2;
  a.crd[0] = nullptr;
  a.crd[1] = crd1;
  a.crd[2] = crd2;
  a.vals = vals;
  a.fac[0] = C;
  a.fac[1] = D;
  a.colscale = nullptr;
  a.out = A;
  a.part = part;
  a.carry = carry;
  a.meta = meta;
  a.segmeta = segmeta;
  a.segcarry = segcarry;
  a.rp = rank;
  a.nnz = nnz;
  a.nrows = nrows;
  a.R = rank;
  a.ldo = rank;
  a.P = kP;
  a.G = kG;
  a.lgG = 6;  // log2(kG)
  a.nblocks = (int32_t)nblocks;
  e = tt::launch_partition(3, a, s);
  if (e != cudaSuccess) return tt::set_error(TT_ERR_CUDA, "partition: %s", cudaGetErrorString(e));
  const size_t smem = tt::walk_smem_bytes(kP, kTB, rank, 4);
  switch (rank) {
    case 8: e = launch_exact<1>(a, (int)nblocks, smem, s); break;
    case 16: e = launch_exact<2>(a, (int)nblocks, smem, s); break;
    case 32: e = launch_exact<4>(a, (int)nblocks, smem, s); break;
    default: e = launch_exact<8>(a, (int)nblocks, smem, s); break;
  }
  if (e != cudaSuccess) return tt::set_error(TT_ERR_CUDA, "walk kernel: %s", cudaGetErrorString(e));
  e = tt::launch_chain_fixup(3, a, s);
  if (e != cudaSuccess) return tt::set_error(TT_ERR_CUDA, "chain merge: %s", cudaGetErrorString(e));
  return TT_OK;
}
