/*
 * gpu_kernels.cuh -- the reference's exported entry points, served by
 * libtentaco_gb300 (replaces gpu_kernels.cuh:1-74 of zhang677/tenTACO).
 *
 * Same names, signatures and host-buffer semantics as the reference:
 *   - every pointer is host memory owned by the caller;
 *   - A->vals (dims[0] x R, R = A->dimensions[1]) is overwritten with the result;
 *   - B is a 3-mode CSF with int32 indices; level 0 may be the reference's
 *     compressed top level (compress_top_level, ds.h:426-436) or a dense root;
 *   - get_gpu_timer_result() returns the milliseconds of the last call's timed
 *     region (partition + output clear + kernel), like the reference's GPUTimer
 *     (gpu_library.h:949-988).
 * Differences: errors do not exit() the process (the reference's gpuErrchk
 * does, gpu_library.h:22-30); they are printed to stderr and kept for
 * tt_last_error_string().  Each call uploads, runs and downloads on the legacy
 * default stream; nothing persists between calls.
 *
 * These declarations have C linkage.  libtentaco_gb300 additionally exports the
 * same functions with C++ linkage, so objects compiled against the reference's
 * own header (which declares them without extern "C") link unchanged.
 */
#ifndef TENTACO_GPU_KERNELS_CUH
#define TENTACO_GPU_KERNELS_CUH
#include "taco_tensor_t.h"

#ifdef __cplusplus
extern "C" {
#endif

float get_gpu_timer_result(void);
void ttv_csf_gpu_taco(taco_tensor_t* A, taco_tensor_t* B, taco_tensor_t* C);

#define X(name, kind, rank, tb, p1, p2) \
  void name(taco_tensor_t* A, taco_tensor_t* B, taco_tensor_t* C, taco_tensor_t* D);
#include "tt_legacy_names.def"
#undef X

#ifdef __cplusplus
}
#endif
#endif /* TENTACO_GPU_KERNELS_CUH */
