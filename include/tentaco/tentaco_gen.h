/*
 * tentaco_gen.h -- seeded synthetic inputs for libtentaco_gb300 (host side).
 *
 * The reference reads FROSTT .tns files through SPLATT (ds.h:351-366) and fills
 * factors with rand() seeded from the wall clock (ds.h:386-410, timers.h:27).
 * Neither the data nor SPLATT is available, so the drivers, tests and benchmark
 * use these generators instead: every output is a pure function of its seed
 * (independent of the thread count), built directly in the canonical CSF
 * layout of tt_csf_from_coo (dense root, lexicographic, no duplicates).
 * Tensors returned here are library-owned: free with tt_tensor_free.
 */
#ifndef TENTACO_TENTACO_GEN_H
#define TENTACO_TENTACO_GEN_H
#include <stdint.h>
#include "tentaco.h"

#ifdef __cplusplus
extern "C" {
#endif

/*
 * nnz distinct coordinates; mode m drawn from a Zipf(zipf_s[m]) law over
 * [0, dims[m]) (zipf_s[m] == 0: uniform) whose ranks are mapped through a
 * seeded permutation, so heavy indices are scattered.  Values U(vlo, vhi).
 * Draws are repeated until nnz distinct coordinates exist or max_rounds
 * top-up rounds have run (saturated Zipf cells can cap the count; the
 * returned tensor's vals_size is the actual nnz).
 */
tt_status tt_gen_zipf(int32_t order, const int32_t* dims, const double* zipf_s, int64_t nnz,
                      float vlo, float vhi, uint64_t seed, int32_t max_rounds,
                      taco_tensor_t** out);

/*
 * 3-mode tensor whose level-1 fibers (i,k) are distinct pairs drawn uniformly
 * from dims[0] x dims[1], with lengths round(lognormal(mu, sigma)) clipped to
 * [1, dims[2]], n_long of them forced to lengths in [long_min, dims[2]]; each
 * fiber holds distinct sorted l values uniform in [0, dims[2]); values
 * U(0,1).  Fibers are added until the total reaches nnz (the last is trimmed).
 */
tt_status tt_gen_lognormal_fibers(const int32_t* dims, int64_t nnz, double mu, double sigma,
                                  int64_t n_long, int64_t long_min, uint64_t seed,
                                  taco_tensor_t** out);

/*
 * Dense row-major rows x cols FP32 matrix into out (host).
 * dist 0: U(0,1).  dist 1: N(0,1) times a per-column factor 2^u, u ~ U(-3,3).
 * dist 2: U(-1,1).
 */
tt_status tt_gen_dense(int64_t rows, int64_t cols, int32_t dist, uint64_t seed, float* out);

/*
 * Read a FROSTT .tns file (one nonzero per line: `order` 1-based coordinates
 * and a value; '#' comment lines) into the canonical CSF of tt_csf_from_coo,
 * with dims[m] = the largest coordinate of mode m.  Replaces the reference's
 * SPLATT loader (ds.h:351-366).  order 0: taken from the first line.
 * Malformed lines return TT_ERR_INVALID_ARGUMENT naming the line.
 */
tt_status tt_read_tns(const char* path, int32_t order, taco_tensor_t** out);

/*
 * Features of a CSF tensor used by the learned variant selector (12 floats):
 * log2 of dims[0..2] (0 for missing modes), log2 nnz, log2 nnz per root row,
 * log2 nnz per last-level fiber, CV of last-level fiber lengths, skewness of
 * log fiber length, log2 max fiber / mean fiber, CV of row nnz, order, log2 rank.
 */
tt_status tt_csf_features(const taco_tensor_t* B, int32_t rank, float* features12);

#ifdef __cplusplus
}
#endif
#endif
