/*
 * Stand-in for the reference's ds.h when compiling its CPU TACO kernels
 * (tensor_kernels/*_cpu_taco.h) as the oracle.  The reference ds.h pulls in
 * SPLATT and Eigen, which are absent; the kernels themselves only need the
 * types below.  Test infrastructure only.
 */
#ifndef TT_ORACLE_SHIM_DS_H
#define TT_ORACLE_SHIM_DS_H
#include <stdint.h>
#include <stdlib.h>
#include <omp.h>
#define restrict __restrict__
/* SPLATT's default index type is 64-bit (the CPU kernels cast indices to it) */
typedef uint64_t splatt_idx_t;
#include "../../include/tentaco/taco_tensor_t.h"
#endif
