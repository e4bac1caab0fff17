/*
 * tentaco.h -- C ABI of libtentaco_gb300: sparse MTTKRP (3- to 5-mode, any output mode)
 * and TTV over CSF tensors on one GB300 (sm_103a).
 *
 * Two layers:
 *
 *  1. Plan API (this header).  A plan uploads a CSF tensor once, owns its
 *     device copy and scratch, picks a kernel variant (fixed heuristic,
 *     learned selector, or exhaustive sweep) and runs on an explicit stream.
 *     Every call returns a tt_status; tt_last_error_string() explains the
 *     last failure on the calling thread.  Plans are independent objects
 *     (no process-global device state) and may be used from different host
 *     threads as long as one plan is not used by two threads at once.
 *
 *  2. Reference-named entry points (gpu_kernels.cuh in this directory):
 *     mttkrp_gpu_taco, ttv_csf_gpu_taco, every mttkrp_<R>_eb_{pr,sr}_*
 *     variant name, and get_gpu_timer_result().  They keep the reference's
 *     signatures and host-buffer semantics (gpu_kernels.cuh:4-73 of
 *     zhang677/tenTACO) and are built on the plan API.
 *
 * All pointers in this header are plain host or device pointers; streams are
 * passed as void* (a cudaStream_t, or NULL for the legacy default stream).
 * No CUDA or torch types appear in any signature.
 */
#ifndef TENTACO_TENTACO_H
#define TENTACO_TENTACO_H

#include <stdint.h>
#include "taco_tensor_t.h"

#ifdef __cplusplus
extern "C" {
#endif

#define TT_ABI_VERSION 1
#define TT_MAX_ORDER 5
#define TT_MAX_RANK 64

typedef enum tt_status {
  TT_OK = 0,
  TT_ERR_INVALID_ARGUMENT = 1, /* null pointer, bad rank/order, size mismatch   */
  TT_ERR_INVALID_CSF = 2,      /* pos not monotone, crd out of range, empty inner fiber */
  TT_ERR_UNSUPPORTED = 3,      /* order/rank/precision combination not built    */
  TT_ERR_CUDA = 4,             /* a CUDA runtime call failed (message has it)   */
  TT_ERR_OUT_OF_MEMORY = 5,    /* device allocation failed                      */
  TT_ERR_NO_DEVICE = 6,        /* no CUDA device visible                        */
  TT_ERR_DEVICE_WAIT = 7       /* a bounded device-side wait gave up            */
} tt_status;

typedef enum tt_op {
  TT_OP_MTTKRP = 0, /* A(i,:) = sum B(i,k,l[,m[,n]]) C(k,:) .* D(l,:) [.* E(m,:) [.* F(n,:)]] */
  TT_OP_TTV = 1,    /* y(fiber) = sum_l B(i,j,l) x(l), one output per (i,j) fiber */
  TT_OP_TTM = 2     /* Y(fiber,:) = sum_l B(i,j,l) U(:,l), U rank x dims[2]: COO plans
                       (tt_plan_create_coo), as the reference's MATLAB interface    */
} tt_op;

typedef enum tt_precision {
  TT_PREC_FP32 = 0,        /* values and factors FP32, FP32 accumulation               */
  TT_PREC_BF16 = 1,        /* values and factors stored BF16 with power-of-two
                              per-column scales; FP32 accumulation, FP64 cross-block merge */
  TT_PREC_BF16_FACTORS = 2, /* values FP32, factors BF16 (per-column scales)           */
  TT_PREC_FP16 = 3,         /* values and factors stored FP16 with power-of-two per-column
                               scales (column max in [2^14, 2^15)); FP32 accumulation.
                               Same bytes as BF16 with an 11-bit significand.            */
  TT_PREC_FX16 = 4          /* the last mode's factor stored as 16-bit fixed point (each
                               column's max maps to 32767, then each row is scaled by a
                               power of two so its largest entry lies in [16384, 32767]);
                               values FP32 (each multiplied by its leaf row's power of
                               two, exactly) and the other factors FP32; FP32
                               accumulation.  The leaf rows cost the bytes of FP16 with
                               all 16 bits spent on the significand.  MTTKRP with the
                               strip family only (TT_ERR_UNSUPPORTED for TTV).           */
} tt_precision;

typedef enum tt_select {
  TT_SELECT_DEFAULT = 0, /* fixed heuristic from tensor shape and rank               */
  TT_SELECT_MODEL = 1,   /* learned selector (MLP); heuristic if no model is loaded  */
  TT_SELECT_SWEEP = 2,   /* time every variant on this tensor and keep the fastest   */
  TT_SELECT_FIXED = 3    /* the variant id passed to tt_plan_create                  */
} tt_select;

/* One kernel variant of the MTTKRP walk family. */
typedef struct tt_variant_info {
  int32_t id;
  int32_t threads;       /* threads per block                                  */
  int32_t cols_per_lane; /* factor columns each lane accumulates               */
  int32_t nnz_per_team;  /* nonzeros a team walks serially (EBSR-style "g")    */
  int32_t rank_pad;      /* rank this variant is compiled for (8,16,32,64)     */
  int32_t lanes_per_row; /* rank_pad / cols_per_lane                           */
  int32_t nnz_per_block; /* threads / lanes_per_row * nnz_per_team             */
  int32_t staged;        /* family. 0 lean: factor rows gathered into registers
                            as the team walks a warp's tile; 1 staged: every row
                            of the block's tile gathered into shared memory
                            (cp.async) before the walk; 2 TMA: the nonzero-level
                            rows fetched by TMA gather4 into a per-warp ring of
                            stages; 3 flat: every nonzero gathers all its factor
                            rows from plan-built per-nonzero coordinates, and the
                            walk checks only row ends (no slab plans); 4 strip:
                            the flat family's per-nonzero rows walked warp-
                            synchronously in steps of nonzeros, row ends decided
                            once per step (tensors with long rows); on a slab
                            plan one launch walks all slabs in slab-major order */
  char name[40];
} tt_variant_info;

typedef struct tt_plan tt_plan;

/* ---- plan lifecycle --------------------------------------------------- */

/*
 * Validate B (host CSF, see taco_tensor_t.h), upload it to the current device
 * and choose a variant.  rank: factor columns (1..64) for MTTKRP; ignored for
 * TTV.  variant is used only with TT_SELECT_FIXED.  stream may be NULL.
 */
tt_status tt_plan_create(const taco_tensor_t* B, tt_op op, int32_t rank, tt_precision prec,
                         tt_select select, int32_t variant, void* stream, tt_plan** plan);
tt_status tt_plan_destroy(tt_plan* plan);

/* Plan options (zero-initialise; NULL means all defaults). */
typedef struct tt_plan_options {
  /* MTTKRP over a dense-root CSF: split the last mode's index range into this
   * many slabs, so that one slab's rows of the last factor stay resident in L2
   * while they are gathered.  The strip family walks all slabs in one launch in
   * slab-major order (one output row per slab and row, summed into A in FP32 with Kahan compensation in
   * slab order); the lean, staged and TMA families run one pass per slab, each
   * adding into A; the flat family runs without slabs.  0: automatic (slabs of at
   * most 44 MB of the last factor as stored, when it exceeds 48 MB); 1: no slabs;
   * at most 16.  One-shot calls (tt_mttkrp_host) use no slabs. */
  int32_t slabs;
  /* L2 policy of factor-row gathers in the lean walk: 0 automatic (evict_last
   * without slabs, evict_normal with them), 1 evict_last, 2 evict_normal. */
  int32_t l2_policy;
  /* TT_SELECT_MODEL only: time this many of the network's best-ranked variants
   * (those that run on the tensor) and the fixed heuristic's variant at plan
   * creation, and keep the fastest.  0: automatic -- 1 (the network's first
   * choice, nothing timed) when every feature of the tensor lies inside the range
   * the network was trained on, else 6; 1 to 16 as given. */
  int32_t model_topk;
  /* MTTKRP output mode (0: the root mode, as in the reference).  For mode m > 0
   * the plan re-roots the tensor once, on the host (level order m, then the other
   * modes in increasing order), and computes A_m(j,:) = sum of B over the other
   * coordinates times their factors' rows; tt_plan_set_factors then takes the
   * factors of the other modes in increasing mode order, and A has dims[m] rows. */
  int32_t mode;
  int32_t reserved[4];
} tt_plan_options;

tt_status tt_plan_create_ex(const taco_tensor_t* B, tt_op op, int32_t rank, tt_precision prec,
                            tt_select select, int32_t variant, const tt_plan_options* options,
                            void* stream, tt_plan** plan);
/* Slabs the plan runs (1: none). */
int32_t tt_plan_slabs(const tt_plan* plan);

/*
 * Give the plan its factor matrices: factors[m-1] is the mode-m factor,
 * a DEVICE FP32 row-major array of dims[m] x rank, for m = 1..order-1.
 * FP32 plans with rank in {8,16,32,64} keep the pointers (caller keeps them
 * alive); other plans convert into plan-owned storage (BF16 + scales, or
 * zero-padded FP32 rows).
 */
tt_status tt_plan_set_factors(tt_plan* plan, const float* const* factors, void* stream);

/* MTTKRP with the factors last set: A is DEVICE FP32 dims[0] x rank, overwritten. */
tt_status tt_plan_mttkrp(tt_plan* plan, float* A, void* stream);

/* TTV: x DEVICE FP32 of length dims[order-1]; y DEVICE FP32, one entry per
 * fiber of level order-2 (tt_plan_num_fibers), overwritten. */
tt_status tt_plan_ttv(tt_plan* plan, const float* x, float* y, void* stream);

/*
 * Plans over sorted COO input, for the reference's MATLAB-interface kernels
 * (tensor_kernels/fmtaco.cpp: compute_ttv 32-115, compute_ttm 117-223,
 * compute_mttkrp 741-780).  coords: HOST, nnz x order int32, row-major, in
 * lexicographic (non-decreasing) order -- duplicates are separate nonzeros, as
 * there; vals: HOST FP32.  The plan uploads them once and walks the COO columns
 * directly (no CSF is built): MTTKRP (order 3 to 5; rows are runs of the first
 * coordinate) on the strip walk; TTV and TTM (order 3; fibers are runs of equal
 * (i, j)) on the TTV walk and on the strip walk over the fibers.  Unsorted or
 * out-of-range coordinates: TT_ERR_INVALID_ARGUMENT.  TTM: FP32 storage;
 * tt_plan_set_factors takes U (DEVICE, rank x dims[2] row-major) and tt_plan_ttm
 * writes Y (DEVICE, nfibers x rank); tt_plan_coo_fibers gives every fiber's (i, j)
 * (HOST, 2 x nfibers int32); tt_plan_num_fibers(plan, 1) (TTV) or (plan, 0) (TTM)
 * gives nfibers.  Variants: the strip family (MTTKRP, TTM); TT_SELECT_MODEL takes
 * the strip rule.
 */
tt_status tt_plan_create_coo(int32_t order, const int32_t* dims, int64_t nnz, const int32_t* coords,
                             const float* vals, tt_op op, int32_t rank, tt_precision prec, tt_select select,
                             int32_t variant, void* stream, tt_plan** plan);
tt_status tt_plan_ttm(tt_plan* plan, float* Y, void* stream);
tt_status tt_plan_coo_fibers(const tt_plan* plan, int32_t* ij);

/* Plans and one-shot calls take device memory from a stream-ordered pool per
 * device that keeps freed memory for the next plan; this returns what no live
 * plan holds to the driver. */
tt_status tt_release_cached_memory(void);

/* Time every subsequent call's device work with CUDA events (default 0, off).
 * 1: the whole call and its walk kernel(s) (tt_plan_last_ms, tt_plan_last_kernel_ms);
 * 2: the whole call only.  Mode 1 records an event between the walk and the row
 * merge, which holds back the merge kernels' early (programmatic dependent) launch:
 * on a GB300 a call timed that way takes about 6 us longer than in mode 0 or 2.
 * Other values: TT_ERR_INVALID_ARGUMENT. */
tt_status tt_plan_set_timing(tt_plan* plan, int32_t enabled);
/* Milliseconds of the last timed call (clear + kernels); waits for it.  The
 * work-unit partition of a single-slab plan depends only on the tensor and runs
 * once, when the plan (or its variant) is set up; slab plans run it per pass. */
float tt_plan_last_ms(tt_plan* plan);

/* Milliseconds of the work-unit partition, computed once when the plan's variant
 * was set and reused by every call (0 when calls run it themselves: slab passes).
 * The reference runs its partition inside every timed call
 * (tensor_kernels/mttkrp3_csf_ebpr.h:74-79); this is that time. */
float tt_plan_partition_ms(const tt_plan* plan);
int32_t tt_plan_variant(const tt_plan* plan);
int64_t tt_plan_nnz(const tt_plan* plan);
int64_t tt_plan_num_fibers(const tt_plan* plan, int32_t level);
/* Device bytes the plan holds (CSF copy + factor storage + scratch). */
int64_t tt_plan_device_bytes(const tt_plan* plan);

/* Walk work units of the plan's variant (blocks, or warp tiles for the lean family). */
int32_t tt_plan_nblocks(const tt_plan* plan);
/* Switch an MTTKRP plan to another valid variant (scratch grows as needed).  A
 * switch that fails (TT_ERR_UNSUPPORTED: the variant does not fit this tensor or
 * plan, e.g. the flat family on a slab plan) leaves the plan without a usable
 * variant: tt_plan_mttkrp returns TT_ERR_INVALID_ARGUMENT until a switch succeeds. */
tt_status tt_plan_use_variant(tt_plan* plan, int32_t variant);
/* Per-variant mean ms timed at plan creation by TT_SELECT_SWEEP, or by
 * TT_SELECT_MODEL's top-k candidates (negative: not timed); n entries. */
tt_status tt_plan_sweep_times(const tt_plan* plan, float* ms, int32_t n);
/* Milliseconds of the walk kernel(s) alone in the last timed call (first slab's
 * walk to the last slab's), without partition, clear and row merge; -1 when that
 * call was not timed in mode 1. */
float tt_plan_last_kernel_ms(tt_plan* plan);
/* Device error word of the plan's kernels (0: none; -1: could not be read);
 * waits for the plan's stream. */
int32_t tt_plan_device_error(tt_plan* plan);

/* ---- device memory for callers without CUDA bindings ------------------ */

tt_status tt_device_malloc(int64_t bytes, void** ptr);
tt_status tt_device_free(void* ptr);
/* Page-lock (and release) a caller's host buffer: copies from and to it then run
 * as direct DMA, e.g. the one-shot calls' uploads of a tensor kept in pinned
 * memory.  Registering an already registered range succeeds. */
tt_status tt_host_register(void* ptr, int64_t bytes);
tt_status tt_host_unregister(void* ptr);
tt_status tt_memcpy_htod(void* dst, const void* src, int64_t bytes);
tt_status tt_memcpy_dtoh(void* dst, const void* src, int64_t bytes);
tt_status tt_device_synchronize(void);
int32_t tt_device_count(void);
/* Write 512 MB on the stream (evicts L2 between timed steps). */
tt_status tt_l2_flush(void* stream);

/* ---- one-shot host calls (H2D, run, D2H inside) ------------------------ */

/* A->vals (host, dims[0] x rank) = MTTKRP(B, factors[0..order-2]) (host dense).
 * Returns TT_ERR_DEVICE_WAIT if a walk's bounded wait ran out (A is then
 * incomplete), like any nonzero device error word of the call.
 * With every host array of B and of the factors page-locked (tt_host_register)
 * and a strip-walk variant (TT_SELECT_FIXED with a strip id, or TT_SELECT_DEFAULT
 * where the default is one), the copies to the device overlap the device work:
 * the leaf coordinates arrive in chunks, each checked and walked as it lands.  The
 * results are the same bits as without the overlap; a malformed CSF is reported
 * (TT_ERR_INVALID_CSF) with A left untouched. */
tt_status tt_mttkrp_host(taco_tensor_t* A, const taco_tensor_t* B,
                         const taco_tensor_t* const* factors, tt_precision prec,
                         tt_select select, int32_t variant);
/* y->vals (host) = TTV(B, x) over the last mode. */
tt_status tt_ttv_host(taco_tensor_t* y, const taco_tensor_t* B, const taco_tensor_t* x);

/* ---- allocation-free MTTKRP -------------------------------------------- */

/*
 * 3-mode mode-0 MTTKRP for callers that cannot allocate device memory (code
 * inside a memory pool or arena it does not own, loops that must never enter
 * the driver's allocator).  No counterpart in the reference: its entry points
 * allocate and free device buffers on every call.
 *
 * Everything is a DEVICE pointer the caller owns: a dense-root CSF (pos1 has
 * nrows+1 entries; pos2/crd1 one per level-1 fiber; crd2/vals nnz entries, no
 * padding needed), FP32 factors C (dims[1] x rank) and D (dims[2] x rank), and
 * the FP32 output A (nrows x rank, overwritten).  crd2, vals, C, D and A must
 * be 16-byte aligned; the CSF must be valid (tt_csf_validate on the host copy).
 * rank must be 8, 16, 32 or 64.  Limit: nnz <= 16,777,216 (the scratch holds
 * per-block state for 8192 blocks of 2048 nonzeros); a larger tensor returns
 * TT_ERR_INVALID_ARGUMENT (use the plan API).  The call allocates nothing: its
 * scratch is a fixed 4.7 MB device array that every GPU loading this library
 * holds until the process exits.  Each call looks that array's address up on the
 * current device (make calls outside stream capture).  All calls share the array,
 * so calls whose work overlaps on the GPU (different streams, or several host
 * threads) race and must be serialised by the caller.
 */
tt_status tt_mttkrp3_noalloc(int32_t nrows, int64_t nnz, int32_t rank,
                             const int32_t* pos1, const int32_t* crd1,
                             const int32_t* pos2, const int32_t* crd2,
                             const float* vals, const float* C, const float* D,
                             float* A, void* stream);

/* ---- variants ---------------------------------------------------------- */

int32_t tt_num_variants(void);
tt_status tt_variant_get(int32_t id, tt_variant_info* info);
/* 1 if variant id is compiled and fits shared memory for (order, rank, prec). */
int32_t tt_variant_valid(int32_t id, int32_t order, int32_t rank, tt_precision prec);
/* The variant the fixed heuristic picks for a shape (used by TT_SELECT_DEFAULT). */
int32_t tt_variant_default(int32_t order, int32_t rank, tt_precision prec, int64_t nnz);

/* ---- errors ------------------------------------------------------------ */

const char* tt_last_error_string(void);
const char* tt_status_string(tt_status s);
int32_t tt_abi_version(void);

/* ---- host CSF utilities ------------------------------------------------ */

/*
 * Build the canonical CSF (modes in order 0..order-1, lexicographic,
 * duplicates summed, dense root with compressed-root arrays also filled in
 * indices[0] for reference callers) from COO coordinates (nnz x order,
 * row-major, int32) and FP32 values.  *out is library-owned: free it with
 * tt_tensor_free.
 */
tt_status tt_csf_from_coo(int32_t order, const int32_t* dims, int64_t nnz,
                          const int32_t* coords, const float* vals, taco_tensor_t** out);
/* The same canonical CSF as tt_csf_from_coo, built on the GPU (stable radix
 * sort of packed coordinates, duplicates summed in FP64 in input order, levels
 * from prefix sums); bit-identical to the host builder.  nnz < 2^31; needs a
 * CUDA device (TT_ERR_NO_DEVICE otherwise). */
tt_status tt_csf_from_coo_gpu(int32_t order, const int32_t* dims, int64_t nnz,
                              const int32_t* coords, const float* vals, taco_tensor_t** out);
/* Check monotone pos, in-range crd, sorted distinct children, non-empty inner fibers. */
tt_status tt_csf_validate(const taco_tensor_t* B);
/* The same tensor as a canonical CSF rooted at `mode` (level order: mode, then
 * the other modes in increasing order; dims permuted alike), e.g. for MTTKRP of
 * another mode.  B is validated first.  *out is library-owned (tt_tensor_free). */
tt_status tt_csf_reroot(const taco_tensor_t* B, int32_t mode, taco_tensor_t** out);
void tt_tensor_free(taco_tensor_t* t);

/* ---- Test hooks (process-wide; failure-detection tests, off by default) ----
 * tt_debug_tma_wait: withhold != 0 makes the TMA walk (variant family 2) arm each
 * stage's barrier without issuing the stage's copy, so that its first wait runs out
 * after wait_ns nanoseconds (0: the default 5 ms; at most 10^9).  The call then
 * records device error 301 (tt_plan_device_error; TT_ERR_DEVICE_WAIT from
 * tt_mttkrp_host), leaves A incomplete and the context usable.  Applies to launches
 * made after the call; tt_debug_tma_wait(0, 0) restores normal operation.
 * tt_debug_fail_pool_alloc: the n-th device allocation of the library from now
 * (n >= 1) fails once, as an out-of-memory condition; 0 disarms.  The environment
 * variable TT_FAIL_POOL_ALLOC_AT=n arms the same before the library's first
 * allocation.  A plan whose allocation failed after its creation refuses every later
 * call but tt_plan_destroy (TT_ERR_INVALID_ARGUMENT).
 * tt_debug_pool_live: device allocations the library holds right now (plans, their
 * scratch and one-shot temporaries; not tt_device_malloc buffers). */
tt_status tt_debug_tma_wait(int32_t withhold, int64_t wait_ns);
tt_status tt_debug_fail_pool_alloc(int64_t n);
int64_t tt_debug_pool_live(void);

#ifdef __cplusplus
}
#endif
#endif /* TENTACO_TENTACO_H */
