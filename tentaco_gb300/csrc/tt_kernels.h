// tt_kernels.h -- launchers of the device kernels (host-callable, no templates).
#pragma once
#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

namespace tt {
struct WalkArgs;

using WalkLauncher = cudaError_t (*)(const WalkArgs& a, int grid, int tb, size_t smem, cudaStream_t s);

// The MTTKRP kernel for (order, precision, columns per lane, lanes per row,
// family), or nullptr if that combination is not compiled.  family 0: register
// walk (factor rows gathered into registers); 1: the block's rows gathered into
// shared memory first; 2: register walk fed by a per-lane cp.async ring.
WalkLauncher walk_launcher(int order, int prec, int cpt, int lpr, int staged);
// Largest window (last-level fibers per block) of a computed partition -> *out (device int).
cudaError_t launch_window_max(int order, const WalkArgs& a, int* out, cudaStream_t s);
WalkLauncher walk_launcher_o3_fp32(int cpt, int lpr, int staged);
WalkLauncher walk_launcher_o3_bf16(int cpt, int lpr, int staged);
WalkLauncher walk_launcher_o3_bf16f(int cpt, int lpr, int staged);
WalkLauncher walk_launcher_o4_fp32(int cpt, int lpr, int staged);
WalkLauncher walk_launcher_o4_bf16(int cpt, int lpr, int staged);
WalkLauncher walk_launcher_o4_bf16f(int cpt, int lpr, int staged);
WalkLauncher walk_launcher_o3_fp16(int cpt, int lpr, int staged);
WalkLauncher walk_launcher_o4_fp16(int cpt, int lpr, int staged);
// strip walk units (family 4; launch families 8 and 9)
WalkLauncher walk_launcher_o3_fp32_strip(int cpt, int lpr, int fam);
WalkLauncher walk_launcher_o3_bf16_strip(int cpt, int lpr, int fam);
WalkLauncher walk_launcher_o3_bf16f_strip(int cpt, int lpr, int fam);
WalkLauncher walk_launcher_o3_fp16_strip(int cpt, int lpr, int fam);
WalkLauncher walk_launcher_o3_fx16_strip(int cpt, int lpr, int fam);
WalkLauncher walk_launcher_o4_fp32_strip(int cpt, int lpr, int fam);
WalkLauncher walk_launcher_o4_bf16_strip(int cpt, int lpr, int fam);
WalkLauncher walk_launcher_o4_bf16f_strip(int cpt, int lpr, int fam);
WalkLauncher walk_launcher_o4_fp16_strip(int cpt, int lpr, int fam);
WalkLauncher walk_launcher_o4_fx16_strip(int cpt, int lpr, int fam);
WalkLauncher walk_launcher_o5_fp32_strip(int cpt, int lpr, int fam);
WalkLauncher walk_launcher_o5_fp16_strip(int cpt, int lpr, int fam);
WalkLauncher walk_launcher_o5_fx16_strip(int cpt, int lpr, int fam);
WalkLauncher walk_launcher_o2_fp32_strip(int cpt, int lpr, int fam);  // TTM: fibers times one matrix
// Strip-walk partition: the row (through a.rnz) of every unit boundary, at stride order - 1.
cudaError_t launch_partition_rows(int order, const WalkArgs& a, cudaStream_t s);
// A(i, j) = sum over slabs k in order of V(k * vstride + i, j) for i < nrows, FP32 with
// Kahan compensation; virtual rows r with rnz[r + 1] == rnz[r] are skipped (slab-major
// strip plans).
// ldv: V's row stride (a multiple of 4, at least R rounded up to 4); lda: A's; S <= 16.
cudaError_t launch_virtual_rows(const float* V, const int32_t* rnz, int S, int64_t nrows, int64_t vstride, int ldv,
                                int lda, int R, float* A, cudaStream_t s);
// scale[j] = 32767 / colmax[j], inv[j] = colmax[j] / 32767 (1 for an empty or non-finite column).
cudaError_t launch_fullrange_scales(const float* colmax, int cols, float* scale, float* inv, cudaStream_t s);
// 16-bit fixed point of a leaf factor (rows x cols FP32 -> rows x rp offset-binary
// int16): column scale `scale`, then a power of two 2^rowexp[r] per row that puts
// the row's largest entry in [16384, 32767].  cols and rp at most 64.
cudaError_t launch_fx16_rows(const float* src, int64_t rows, int cols, int rp, const float* scale, uint16_t* dst,
                             int8_t* rowexp, cudaStream_t s);
// out[p] = vals[p] * 2^-rowexp[leaf[p]] for p < n (exact).
cudaError_t launch_fx16_values(const float* vals, const int32_t* leaf, const int8_t* rowexp, int64_t n, float* out,
                               cudaStream_t s);

cudaError_t launch_partition(int order, const WalkArgs& a, cudaStream_t s);
// Flat walk indexes.  launch_expand: out[p] = per_fiber[f] for every entry p of
// fiber f of one level (p < pos[nf] = n).  launch_row_starts: rnz[i] = off + first
// nonzero of root position i (pos2[pos1[i]], through pos3 for four modes and pos4 for five).
cudaError_t launch_expand(const int32_t* per_fiber, const int32_t* pos, int64_t nf, int64_t n, int32_t* out,
                          cudaStream_t s);
cudaError_t launch_row_starts(const int32_t* pos1, const int32_t* pos2, const int32_t* pos3, int64_t nroot,
                              int32_t* rnz, cudaStream_t s, int64_t off = 0, const int32_t* pos4 = nullptr);
// FP64 merge of the rows the walk left in the carry buffer (after the walk kernel).
cudaError_t launch_chain_fixup(int order, const WalkArgs& a, cudaStream_t s);
// Allocation from the library's stream-ordered device memory pool (usable on `st` at
// once, elsewhere after `st` is synchronised), and its release on `st`.
cudaError_t device_pool_alloc(void** ptr, size_t bytes, cudaStream_t st);
void device_pool_free(void* ptr, cudaStream_t st);
// TTV walk over units of 32 * kTtvNpt nonzeros (a: the 2-level view, see tt_ttv.cuh).
cudaError_t launch_ttv_ranges(const WalkArgs& a, int vals_kind, cudaStream_t s);

// Column max |x| of a rows x cols FP32 row-major matrix into colmax (cols floats, zeroed here).
// Structure check of one CSF level on device copies: pos (nf + 1 fiber starts;
// inner != 0: fibers must not be empty), crd (n coordinates below dim); starts:
// scratch of n / 32 + 1 words; err[0..1]: pos / crd violation words, set to
// UINT64_MAX by the caller (see tt_misc.cu).
cudaError_t launch_csf_check(const int32_t* pos, int64_t nf, int inner, const int32_t* crd, int64_t n, int32_t dim,
                             uint32_t* starts, unsigned long long* err, cudaStream_t s);
// The same check in two parts, for a level whose coordinates arrive in pieces: the
// pos pass (err[0]; marks the fiber starts in `starts`), then the crd pass over
// positions [p0, p1) (err: the crd violation word), in increasing ranges on one
// stream.  clamp != 0: out-of-range coordinates are also overwritten with 0.
cudaError_t launch_csf_pos_check(const int32_t* pos, int64_t nf, int inner, int64_t n, uint32_t* starts,
                                 unsigned long long* err, cudaStream_t s);
cudaError_t launch_csf_crd_check_range(int32_t* crd, int64_t p0, int64_t p1, int32_t dim, const uint32_t* starts,
                                       unsigned long long* err, int clamp, cudaStream_t s);
cudaError_t launch_colmax(const float* x, int64_t rows, int cols, float* colmax, cudaStream_t s);
// scale[j] = 2^(target_exp - floor(log2(colmax[j]))) (1 where colmax is 0 or not finite);
// inv[j] = 1/scale[j].  Both exact powers of two.
cudaError_t launch_pow2_scales(const float* colmax, int cols, int target_exp, float* scale, float* inv,
                               cudaStream_t s);
// dst (rows x rp, 16-bit kind: 1 = BF16, 2 = FP16, round to nearest even) =
// src (rows x cols) * scale[col], zero for cols <= j < rp.
cudaError_t launch_to_16(const float* src, int64_t rows, int cols, int rp, const float* scale, int kind,
                         uint16_t* dst, cudaStream_t s);
// Exclusive scan of n uint32 on the device (out may alias in); *total (host) gets the
// sum; sums: scratch of scan_scratch_entries(n) uint32.  Synchronises st.
int64_t scan_scratch_entries(int64_t n);
cudaError_t device_exclusive_scan(const uint32_t* in, int64_t n, uint32_t* out, uint32_t* sums, uint32_t* total,
                                  cudaStream_t st);
// COO input (tt_coo.cu).  coords: nnz x order int32, row-major, on the device.
// Check: every coordinate inside its mode and the nonzeros in lexicographic
// (non-decreasing) order; *err (device, set to UINT64_MAX by the caller) keeps the
// first violation as (index << 3) | code (1: coordinate out of range, 2: out of order).
cudaError_t launch_coo_check(const int32_t* coords, int64_t nnz, int order, const int32_t* dims,
                             unsigned long long* err, cudaStream_t s);
// out[p] = coords[p * order + col] for p < nnz.
cudaError_t launch_coo_column(const int32_t* coords, int64_t nnz, int order, int col, int32_t* out, cudaStream_t s);
// rnz[r] = first nonzero whose mode-0 coordinate is >= r, r = 0..nrows (rows as runs).
cudaError_t launch_coo_row_starts(const int32_t* coords, int64_t nnz, int order, int64_t nrows, int32_t* rnz,
                                  cudaStream_t s);
// flags[p] = 1 where a fiber (a run of equal (mode 0, mode 1) coordinates) starts.
cudaError_t launch_coo_fiber_flags(const int32_t* coords, int64_t nnz, int order, uint32_t* flags, cudaStream_t s);
// For fiber starts p (flags[p]): pos[fid[p]] = p, fcoords[2 fid[p] + {0, 1}] = (i, j).
cudaError_t launch_coo_fibers(const int32_t* coords, int64_t nnz, int order, const uint32_t* flags,
                              const uint32_t* fid, int32_t* pos, int32_t* fcoords, cudaStream_t s);
// dst (K x rp, FP32, zero padded) = transpose of U (R x K, row-major).
cudaError_t launch_transpose_pad(const float* U, int64_t R, int64_t K, int rp, float* dst, cudaStream_t s);
// dst (rows x rp, FP32) = src (rows x cols), zero padded.
cudaError_t launch_pad_fp32(const float* src, int64_t rows, int cols, int rp, float* dst, cudaStream_t s);
// out[j] = prod_m inv_m[j] * vinv   (nm factor inverse-scale arrays, rp entries each)
cudaError_t launch_scale_product(const float* const* inv, int nm, int rp, float vinv, float* out, cudaStream_t s);
}  // namespace tt
