// tt_coo.cu -- device kernels that prepare COO input for the walk kernels.
//
// The reference's MATLAB interface computes TTV, TTM and MTTKRP over sorted COO
// tensors (tensor_kernels/fmtaco.cpp:32-223, 741-780): fibers are runs of
// consecutive nonzeros with equal (i, j), rows are runs of equal i.  Here the
// coordinate stream itself is the walk's input: a column of the COO array is the
// leaf coordinate (or a per-nonzero upper coordinate) the strip and TTV walks
// stream, and the row or fiber boundaries come from runs, found on the device.
// No CSF is built.
#include <cuda_runtime.h>
#include <cstdint>
#include "tt_kernels.h"

namespace tt {
namespace {
int grid_of(int64_t n) {
  int64_t g = (n + 255) / 256;
  if (g > 152 * 32) g = 152 * 32;
  return (int)(g < 1 ? 1 : g);
}
}  // namespace

__global__ void coo_check_kernel(const int32_t* __restrict__ co, int64_t nnz, int order, const int32_t* __restrict__ dims,
                                 unsigned long long* __restrict__ err) {
  for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < nnz; p += (int64_t)gridDim.x * blockDim.x) {
    const int32_t* c = co + p * order;
    int code = 0;
    for (int m = 0; m < order && !code; m++)
      if (c[m] < 0 || c[m] >= dims[m]) code = 1;
    if (!code && p > 0) {
      const int32_t* b = c - order;
      int cmp = 0;
      for (int m = 0; m < order && cmp == 0; m++) cmp = (b[m] < c[m]) ? -1 : (b[m] > c[m] ? 1 : 0);
      if (cmp > 0) code = 2;
    }
    if (code) atomicMin(err, ((unsigned long long)p << 3) | (unsigned long long)code);
  }
}

cudaError_t launch_coo_check(const int32_t* coords, int64_t nnz, int order, const int32_t* dims,
                             unsigned long long* err, cudaStream_t s) {
  if (nnz > 0) coo_check_kernel<<<grid_of(nnz), 256, 0, s>>>(coords, nnz, order, dims, err);
  return cudaGetLastError();
}

__global__ void coo_column_kernel(const int32_t* __restrict__ co, int64_t nnz, int order, int col,
                                  int32_t* __restrict__ out) {
  for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < nnz; p += (int64_t)gridDim.x * blockDim.x)
    out[p] = co[p * order + col];
}

cudaError_t launch_coo_column(const int32_t* coords, int64_t nnz, int order, int col, int32_t* out, cudaStream_t s) {
  if (nnz > 0) coo_column_kernel<<<grid_of(nnz), 256, 0, s>>>(coords, nnz, order, col, out);
  return cudaGetLastError();
}

// A thread at a run start p (the first nonzero, or one whose row differs from its
// predecessor's) writes rnz for the rows from the previous row + 1 to its own; the
// last nonzero also closes the rows after it.  Sorted input: every rnz entry is
// written exactly once.
__global__ void coo_row_starts_kernel(const int32_t* __restrict__ co, int64_t nnz, int order, int64_t nrows,
                                      int32_t* __restrict__ rnz) {
  for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < nnz; p += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = co[p * order];
    const int64_t prev = p == 0 ? -1 : co[(p - 1) * order];
    for (int64_t r = prev + 1; r <= i; r++) rnz[r] = (int32_t)p;
    if (p == nnz - 1)
      for (int64_t r = i + 1; r <= nrows; r++) rnz[r] = (int32_t)nnz;
  }
}

__global__ void fill_i32_kernel(int32_t* d, int64_t n, int32_t v) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) d[i] = v;
}

cudaError_t launch_coo_row_starts(const int32_t* coords, int64_t nnz, int order, int64_t nrows, int32_t* rnz,
                                  cudaStream_t s) {
  if (nnz == 0) fill_i32_kernel<<<grid_of(nrows + 1), 256, 0, s>>>(rnz, nrows + 1, 0);
  else coo_row_starts_kernel<<<grid_of(nnz), 256, 0, s>>>(coords, nnz, order, nrows, rnz);
  return cudaGetLastError();
}

__global__ void coo_fiber_flags_kernel(const int32_t* __restrict__ co, int64_t nnz, int order,
                                       uint32_t* __restrict__ flags) {
  for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < nnz; p += (int64_t)gridDim.x * blockDim.x)
    flags[p] = (p == 0 || co[p * order] != co[(p - 1) * order] || co[p * order + 1] != co[(p - 1) * order + 1]) ? 1u : 0u;
}

cudaError_t launch_coo_fiber_flags(const int32_t* coords, int64_t nnz, int order, uint32_t* flags, cudaStream_t s) {
  if (nnz > 0) coo_fiber_flags_kernel<<<grid_of(nnz), 256, 0, s>>>(coords, nnz, order, flags);
  return cudaGetLastError();
}

__global__ void coo_fibers_kernel(const int32_t* __restrict__ co, int64_t nnz, int order, const uint32_t* __restrict__ flags,
                                  const uint32_t* __restrict__ fid, int32_t* __restrict__ pos,
                                  int32_t* __restrict__ fcoords) {
  for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < nnz; p += (int64_t)gridDim.x * blockDim.x) {
    if (!flags[p]) continue;
    const uint32_t f = fid[p];
    pos[f] = (int32_t)p;
    fcoords[2 * (int64_t)f] = co[p * order];
    fcoords[2 * (int64_t)f + 1] = co[p * order + 1];
  }
}

cudaError_t launch_coo_fibers(const int32_t* coords, int64_t nnz, int order, const uint32_t* flags,
                              const uint32_t* fid, int32_t* pos, int32_t* fcoords, cudaStream_t s) {
  if (nnz > 0) coo_fibers_kernel<<<grid_of(nnz), 256, 0, s>>>(coords, nnz, order, flags, fid, pos, fcoords);
  return cudaGetLastError();
}

__global__ void transpose_pad_kernel(const float* __restrict__ U, int64_t R, int64_t K, int rp, float* __restrict__ dst) {
  const int64_t n = K * rp;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t k = e / rp;
    const int r = (int)(e - k * rp);
    dst[e] = r < R ? U[r * K + k] : 0.f;
  }
}

cudaError_t launch_transpose_pad(const float* U, int64_t R, int64_t K, int rp, float* dst, cudaStream_t s) {
  if (K > 0) transpose_pad_kernel<<<grid_of(K * rp), 256, 0, s>>>(U, R, K, rp, dst);
  return cudaGetLastError();
}

}  // namespace tt
