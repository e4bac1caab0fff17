/*
 * tt_oracle.c -- TEST INFRASTRUCTURE ONLY.
 *
 * CPU restatement, in FP64, of the reference's CPU algorithms for the sparse
 * MTTKRP / TTV hot path of zhang677/tenTACO.  Only tests/, the package's smoke
 * check and bench.py's CPU-baseline leg may load this library, and only as the
 * checker (or as the timed stand-in for the reference CPU kernels on a host
 * where the reference sources are absent).  The product (libtentaco_gb300)
 * never links or calls it.
 *
 * Pinning: tests/golden/ holds outputs of the reference's own CPU kernels
 * (tensor_kernels/mttkrp3_csf_cpu_taco.h, mttkrp4_csf_cpu_taco.h,
 * mttkrp5_csf_cpu_taco.h, ttv_csf_cpu_taco.h) compiled unmodified through oracle/shim by oracle/Makefile;
 * tests/test_oracle.py checks every function here against them bit-for-bit.
 *
 * Index arrays are int64 (the reference CPU path reads splatt_idx_t / long),
 * values are double.  Level 0 is a dense root: pos1 has nrows+1 entries.
 * Build with -ffp-contract=off so x86 and Arm hosts round identically.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <math.h>
#include <time.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORACLE_API __attribute__((visibility("default")))

/*
 * MTTKRP, 3 modes, mode 0:  A(i,j) = sum_{k,l} B(i,k,l) * C(k,j) * D(l,j).
 * Follows tensor_kernels/mttkrp3_csf_cpu_taco.h:25-49: zero A, then rows in
 * chunks of 64 (dynamic schedule), per nonzero A[i,j] += (B*C)*D in j order.
 * Each row is owned by one thread, so the result does not depend on threads.
 */
ORACLE_API void oracle_mttkrp3(int64_t nrows, int64_t R,
                               const int64_t* pos1, const int64_t* crd1,
                               const int64_t* pos2, const int64_t* crd2,
                               const double* vals, const double* C,
                               const double* D, double* A) {
  int64_t n = nrows * R;
#pragma omp parallel for schedule(static)
  for (int64_t p = 0; p < n; p++) A[p] = 0.0;
#pragma omp parallel for schedule(dynamic, 1)
  for (int64_t i1 = 0; i1 < (nrows + 63) / 64; i1++) {
    for (int64_t i2 = 0; i2 < 64; i2++) {
      int64_t i = i1 * 64 + i2;
      if (i >= nrows) continue;
      for (int64_t kB = pos1[i]; kB < pos1[i + 1]; kB++) {
        int64_t k = crd1[kB];
        for (int64_t lB = pos2[kB]; lB < pos2[kB + 1]; lB++) {
          int64_t l = crd2[lB];
          for (int64_t j = 0; j < R; j++) {
            A[i * R + j] = A[i * R + j] + (vals[lB] * C[k * R + j]) * D[l * R + j];
          }
        }
      }
    }
  }
}

/*
 * MTTKRP, 4 modes, mode 0:  A(i,j) = sum B(i,k,l,m) C(k,j) D(l,j) E(m,j).
 * Follows tensor_kernels/mttkrp4_csf_cpu_taco.h:31-57 (same schedule as above,
 * product order ((B*C)*D)*E).
 */
ORACLE_API void oracle_mttkrp4(int64_t nrows, int64_t R,
                               const int64_t* pos1, const int64_t* crd1,
                               const int64_t* pos2, const int64_t* crd2,
                               const int64_t* pos3, const int64_t* crd3,
                               const double* vals, const double* C,
                               const double* D, const double* E, double* A) {
  int64_t n = nrows * R;
#pragma omp parallel for schedule(static)
  for (int64_t p = 0; p < n; p++) A[p] = 0.0;
#pragma omp parallel for schedule(dynamic, 1)
  for (int64_t i1 = 0; i1 < (nrows + 63) / 64; i1++) {
    for (int64_t i2 = 0; i2 < 64; i2++) {
      int64_t i = i1 * 64 + i2;
      if (i >= nrows) continue;
      for (int64_t kB = pos1[i]; kB < pos1[i + 1]; kB++) {
        int64_t k = crd1[kB];
        for (int64_t lB = pos2[kB]; lB < pos2[kB + 1]; lB++) {
          int64_t l = crd2[lB];
          for (int64_t mB = pos3[lB]; mB < pos3[lB + 1]; mB++) {
            int64_t m = crd3[mB];
            for (int64_t j = 0; j < R; j++) {
              A[i * R + j] = A[i * R + j] +
                             ((vals[mB] * C[k * R + j]) * D[l * R + j]) * E[m * R + j];
            }
          }
        }
      }
    }
  }
}

/*
 * MTTKRP, 5 modes, mode 0:  A(i,j) = sum B(i,k,l,m,n) C(k,j) D(l,j) E(m,j) F(n,j).
 * Follows tensor_kernels/mttkrp5_csf_cpu_taco.h:35-95, which, unlike the 3- and
 * 4-mode kernels, factors the sum level by level (same schedule as above):
 *   per level-3 fiber (i,k,l,m):  f(j) = sum_n B(..,n) * F(n,j)
 *   per level-2 fiber (i,k,l):    e(j) = sum_m f(j) * E(m,j)
 *   per level-1 fiber (i,k):      d(j) = sum_l e(j) * D(l,j)
 *   then                          A(i,j) += d(j) * C(k,j)
 * each sum taken in CSF order.  The three partial rows are per-thread buffers
 * of R doubles, zeroed where the reference zeroes its per-fiber workspaces.
 */
ORACLE_API void oracle_mttkrp5(int64_t nrows, int64_t R,
                               const int64_t* pos1, const int64_t* crd1,
                               const int64_t* pos2, const int64_t* crd2,
                               const int64_t* pos3, const int64_t* crd3,
                               const int64_t* pos4, const int64_t* crd4,
                               const double* vals, const double* C, const double* D,
                               const double* E, const double* F, double* A) {
  int64_t n = nrows * R;
#pragma omp parallel for schedule(static)
  for (int64_t p = 0; p < n; p++) A[p] = 0.0;
#pragma omp parallel
  {
    double* part = (double*)malloc(sizeof(double) * (size_t)(3 * (R > 0 ? R : 1)));
    double* d = part;          /* level-1 fiber partial */
    double* e = part + R;      /* level-2 fiber partial */
    double* f = part + 2 * R;  /* level-3 fiber partial */
#pragma omp for schedule(dynamic, 1)
    for (int64_t i1 = 0; i1 < (nrows + 63) / 64; i1++) {
      for (int64_t i2 = 0; i2 < 64; i2++) {
        int64_t i = i1 * 64 + i2;
        if (i >= nrows) continue;
        for (int64_t kB = pos1[i]; kB < pos1[i + 1]; kB++) {
          int64_t k = crd1[kB];
          for (int64_t j = 0; j < R; j++) d[j] = 0.0;
          for (int64_t lB = pos2[kB]; lB < pos2[kB + 1]; lB++) {
            int64_t l = crd2[lB];
            for (int64_t j = 0; j < R; j++) e[j] = 0.0;
            for (int64_t mB = pos3[lB]; mB < pos3[lB + 1]; mB++) {
              int64_t m = crd3[mB];
              for (int64_t j = 0; j < R; j++) f[j] = 0.0;
              for (int64_t nB = pos4[mB]; nB < pos4[mB + 1]; nB++) {
                int64_t q = crd4[nB];
                for (int64_t j = 0; j < R; j++) f[j] = f[j] + vals[nB] * F[q * R + j];
              }
              for (int64_t j = 0; j < R; j++) e[j] = e[j] + f[j] * E[m * R + j];
            }
            for (int64_t j = 0; j < R; j++) d[j] = d[j] + e[j] * D[l * R + j];
          }
          for (int64_t j = 0; j < R; j++) A[i * R + j] = A[i * R + j] + d[j] * C[k * R + j];
        }
      }
    }
    free(part);
  }
}

/*
 * Binary search used by the scheduled TTV: the largest index in
 * [arrayStart, arrayEnd] whose value is <= target (ttv_csf_cpu_taco.h:2-22).
 */
static int64_t oracle_search_before(const int64_t* a, int64_t lo, int64_t hi, int64_t target) {
  if (a[hi] <= target) return hi;
  int64_t lower = lo, upper = hi;
  while (upper - lower > 1) {
    int64_t mid = (upper + lower) / 2;
    int64_t v = a[mid];
    if (v < target) lower = mid;
    else if (v > target) upper = mid;
    else return mid;
  }
  return lower;
}

/*
 * TTV over the last mode:  y(f) = sum_{l in fiber f} B(i,j,l) * c(l), one
 * output per level-1 fiber f (the (i,j) pairs of B, in CSF order).
 * Follows tensor_kernels/ttv_csf_cpu_taco.h:24-66: chunks of 8 fibers, a
 * search for the first row of the chunk, per nonzero y[f] += B*c.
 */
ORACLE_API void oracle_ttv(int64_t nrows, const int64_t* pos1, const int64_t* crd1,
                           const int64_t* pos2, const int64_t* crd2,
                           const double* vals, const double* c, double* y) {
  int64_t nf = pos1[nrows];
  (void)crd1;
#pragma omp parallel for schedule(static)
  for (int64_t f = 0; f < nf; f++) y[f] = 0.0;
#pragma omp parallel for schedule(dynamic, 1)
  for (int64_t chunk = 0; chunk < (nf + 7) / 8; chunk++) {
    int64_t i_pos = oracle_search_before(pos1, 0, nrows, chunk * 8);
    for (int64_t q = 0; q < 8; q++) {
      int64_t f = chunk * 8 + q;
      if (f >= nf) continue;
      while (i_pos < nrows && f == pos1[i_pos + 1]) i_pos++;
      for (int64_t kB = pos2[f]; kB < pos2[f + 1]; kB++) {
        y[f] = y[f] + vals[kB] * c[crd2[kB]];
      }
    }
  }
}

/*
 * Same MTTKRP3 in the "workspace" (fiber-factored) order of
 * tensor_kernels/mttkrp3_csf_cpu_taco_workspace.h:27-58:
 * t = sum_l B*D(l,:) per fiber, then A(i,:) += t .* C(k,:).
 */
ORACLE_API void oracle_mttkrp3_workspace(int64_t nrows, int64_t R,
                                         const int64_t* pos1, const int64_t* crd1,
                                         const int64_t* pos2, const int64_t* crd2,
                                         const double* vals, const double* C,
                                         const double* D, double* A) {
  int64_t n = nrows * R;
  for (int64_t p = 0; p < n; p++) A[p] = 0.0;
#pragma omp parallel for schedule(dynamic, 1)
  for (int64_t i1 = 0; i1 < (nrows + 63) / 64; i1++) {
    double* t = (double*)calloc((size_t)R, sizeof(double));
    for (int64_t i2 = 0; i2 < 64; i2++) {
      int64_t i = i1 * 64 + i2;
      if (i >= nrows) continue;
      for (int64_t kB = pos1[i]; kB < pos1[i + 1]; kB++) {
        int64_t k = crd1[kB];
        for (int64_t lB = pos2[kB]; lB < pos2[kB + 1]; lB++) {
          int64_t l = crd2[lB];
          for (int64_t j = 0; j < R; j++) t[j] = t[j] + vals[lB] * D[l * R + j];
        }
        for (int64_t j = 0; j < R; j++) {
          A[i * R + j] = A[i * R + j] + t[j] * C[k * R + j];
          t[j] = 0.0;
        }
      }
    }
    free(t);
  }
}

/*
 * MTTKRP, mode 0, restricted to a list of rows (size-independent parity at
 * full scale: the rows a test samples are recomputed exactly).  Same per-row
 * operation order as oracle_mttkrp3 / oracle_mttkrp4.  order is 3 or 4;
 * for order 3, pos3/crd3/E are ignored.
 */
ORACLE_API void oracle_mttkrp_rows(int32_t order, int64_t R, int64_t nsel, const int64_t* rows,
                                   const int64_t* pos1, const int64_t* crd1,
                                   const int64_t* pos2, const int64_t* crd2,
                                   const int64_t* pos3, const int64_t* crd3,
                                   const double* vals, const double* C, const double* D,
                                   const double* E, double* out) {
#pragma omp parallel for schedule(dynamic, 1)
  for (int64_t s = 0; s < nsel; s++) {
    int64_t i = rows[s];
    double* a = out + s * R;
    for (int64_t j = 0; j < R; j++) a[j] = 0.0;
    for (int64_t kB = pos1[i]; kB < pos1[i + 1]; kB++) {
      int64_t k = crd1[kB];
      for (int64_t lB = pos2[kB]; lB < pos2[kB + 1]; lB++) {
        int64_t l = crd2[lB];
        if (order == 3) {
          for (int64_t j = 0; j < R; j++) a[j] = a[j] + (vals[lB] * C[k * R + j]) * D[l * R + j];
        } else {
          for (int64_t mB = pos3[lB]; mB < pos3[lB + 1]; mB++) {
            int64_t m = crd3[mB];
            for (int64_t j = 0; j < R; j++)
              a[j] = a[j] + ((vals[mB] * C[k * R + j]) * D[l * R + j]) * E[m * R + j];
          }
        }
      }
    }
  }
}

/* ---------------------------------------------------------------------------
 * Comparators of the reference (ds.h).
 * ------------------------------------------------------------------------- */

/* ds.h:551-565 compare_array: max |y/x - 1| over x != 0; +inf if x == 0 and y != 0. */
ORACLE_API double oracle_compare_array(const float* x, const float* y, int64_t n) {
  double ret = 0.0;
  for (int64_t i = 0; i < n; i++) {
    if (x[i] != 0.0f) {
      double d = fabs((double)(y[i] / x[i]) - 1.0);
      if (d > ret) ret = d;
    } else if (y[i] != 0.0f) {
      return INFINITY;
    }
  }
  return ret;
}

/* ds.h:566-580 compare_array_my: count of |x-y| > 1e-3, stopping once the count exceeds 10. */
ORACLE_API double oracle_compare_array_my(const float* x, const float* y, int64_t n) {
  const float thres = 0.001f;
  float count = 0.0f;
  for (int64_t i = 0; i < n; i++) {
    if (fabsf(x[i] - y[i]) > thres) count += 1.0f;
    if (count > 10) break;
  }
  return count;
}

/* ---------------------------------------------------------------------------
 * CSF construction: lexicographic order of the mode coordinates, duplicates
 * summed, dense root.  The reference delegates this to SPLATT (absent), so
 * this is the canonical definition both the library's host and GPU builders
 * are checked against bit-for-bit.
 * ------------------------------------------------------------------------- */
#define ORACLE_MAX_ORDER 5
typedef struct { int64_t key[ORACLE_MAX_ORDER]; double v; int64_t seq; } oracle_entry;
static int oracle_order_g = 3;
static int oracle_cmp(const void* a, const void* b) {
  const oracle_entry* x = (const oracle_entry*)a;
  const oracle_entry* y = (const oracle_entry*)b;
  for (int d = 0; d < oracle_order_g; d++) {
    if (x->key[d] < y->key[d]) return -1;
    if (x->key[d] > y->key[d]) return 1;
  }
  /* stable on input order so that duplicate sums are added in input order */
  return (x->seq < y->seq) ? -1 : (x->seq > y->seq);
}

/*
 * coords: nnz x order (row-major), vals: nnz doubles.
 * Outputs (caller-allocated, sized for the worst case):
 *   pos[1] (dims0+1 entries), pos[l] for l = 2..order-1 ((#level l-1 fibers)+1),
 *   crd[l] for l = 1..order-1, out_vals,
 *   counts[l] = #fibers at level l (counts[0] = dims0, counts[order-1] = nnz').
 * A new level-l fiber starts wherever the coordinate prefix of length l+1
 * changes.  Returns the deduplicated nnz.
 */
ORACLE_API int64_t oracle_build_csf(int32_t order, int64_t dims0, int64_t nnz,
                                    const int64_t* coords, const double* vals,
                                    int64_t** pos, int64_t** crd, double* out_vals,
                                    int64_t* counts) {
  if (order < 2 || order > ORACLE_MAX_ORDER) return -1;
  oracle_entry* e = (oracle_entry*)malloc(sizeof(oracle_entry) * (size_t)(nnz > 0 ? nnz : 1));
  for (int64_t p = 0; p < nnz; p++) {
    for (int d = 0; d < order; d++) e[p].key[d] = coords[p * order + d];
    e[p].v = vals[p];
    e[p].seq = p;
  }
  oracle_order_g = order;
  qsort(e, (size_t)nnz, sizeof(oracle_entry), oracle_cmp);
  int64_t m = 0;
  for (int64_t p = 0; p < nnz; p++) {
    if (m > 0) {
      int same = 1;
      for (int d = 0; d < order; d++) same &= (e[m - 1].key[d] == e[p].key[d]);
      if (same) { e[m - 1].v += e[p].v; continue; }
    }
    e[m++] = e[p];
  }
  counts[0] = dims0;
  for (int l = 1; l < order; l++) counts[l] = 0;
  for (int64_t i = 0; i <= dims0; i++) pos[1][i] = 0;
  for (int64_t p = 0; p < m; p++) {
    int nl = 0;
    if (p > 0) {
      nl = order;
      for (int d = 0; d < order; d++) if (e[p].key[d] != e[p - 1].key[d]) { nl = d; break; }
    }
    for (int l = (nl < 1 ? 1 : nl); l < order; l++) {
      if (l == 1) pos[1][e[p].key[0] + 1]++;
      else if (nl <= l - 1) pos[l][counts[l - 1] - 1] = counts[l];
      crd[l][counts[l]] = e[p].key[l];
      counts[l]++;
    }
    out_vals[p] = e[p].v;
  }
  for (int64_t i = 0; i < dims0; i++) pos[1][i + 1] += pos[1][i];
  for (int l = 2; l < order; l++) pos[l][counts[l - 1]] = counts[l];
  free(e);
  return m;
}

/* ---------------------------------------------------------------------------
 * Wall clock for the CPU-baseline leg.
 * ------------------------------------------------------------------------- */
ORACLE_API double oracle_now_ms(void) {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return ts.tv_sec * 1e3 + ts.tv_nsec * 1e-6;
}

/* Threads of the oracle's parallel loops from now on (the CPU baseline's legs). */
ORACLE_API void oracle_set_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
}

ORACLE_API int oracle_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

/*
 * MTTKRP of any output mode from coordinates:
 *   A(c[mode], j) = sum over nonzeros p of vals[p] * prod_{n != mode} F_n(c[n], j),
 * nonzeros in the given order, the product taken left to right over the other
 * modes in increasing order ((v * F_a) * F_b) [* F_c]), serial, FP64.  The
 * reference computes the root mode only; for mode 0, with nonzeros in CSF order,
 * this is the same arithmetic as oracle_mttkrp3 / oracle_mttkrp4 (which follow
 * tensor_kernels/mttkrp3_csf_cpu_taco.h:45 and mttkrp4_csf_cpu_taco.h:53).
 *   coords: nnz x order (row-major); factors: order pointers (factors[mode]
 *   unused), each dims[n] x R row-major; A: nrows x R, overwritten.
 */
ORACLE_API void oracle_mttkrp_coo(int32_t order, int64_t nnz, const int64_t* coords, const double* vals,
                                  int32_t mode, int64_t R, const double* const* factors, int64_t nrows,
                                  double* A) {
  for (int64_t p = 0; p < nrows * R; p++) A[p] = 0.0;
  for (int64_t p = 0; p < nnz; p++) {
    const int64_t* c = coords + p * order;
    double* a = A + c[mode] * R;
    for (int64_t j = 0; j < R; j++) {
      double t = vals[p];
      for (int32_t n = 0; n < order; n++)
        if (n != mode) t = t * factors[n][c[n] * R + j];
      a[j] = a[j] + t;
    }
  }
}

/* ---------------------------------------------------------------------------
 * COO kernels of the reference's MATLAB interface (tensor_kernels/fmtaco.cpp),
 * restated without MATLAB.  Parity unpinned against fmtaco.cpp itself, which
 * needs MATLAB's mex.h and matrix.h to compile: its MTTKRP (fmtaco.cpp:741-780)
 * is oracle_mttkrp_coo for mode 0 (same order, same association ((v * C) * D));
 * its TTV (fmtaco.cpp:32-115) sums each fiber from 0 in nonzero order, the
 * arithmetic of the pinned CSF TTV (ttv_csf_cpu_taco.h:61-63); its TTM
 * (fmtaco.cpp:117-223) is checked against a dense evaluation.
 *
 * Fibers are runs of consecutive nonzeros with equal (i, j), as in fmtaco.cpp:
 * sorted input gives one run per fiber.  coords: nnz x 3 (row-major).  Outputs
 * are sized by the caller for nnz fibers; the functions return the fiber count.
 * ------------------------------------------------------------------------- */

/* y(f) = sum over the run's nonzeros of v * c[k]; fib[2f], fib[2f+1] = (i, j). */
ORACLE_API int64_t oracle_coo_ttv(int64_t nnz, const int64_t* coords, const double* vals,
                                  const double* c, int64_t* fib, double* y) {
  int64_t nf = 0;
  for (int64_t p = 0; p < nnz;) {
    const int64_t i = coords[3 * p], j = coords[3 * p + 1];
    double t = 0.0;
    int64_t q = p;
    for (; q < nnz && coords[3 * q] == i && coords[3 * q + 1] == j; q++) t = t + vals[q] * c[coords[3 * q + 2]];
    fib[2 * nf] = i;
    fib[2 * nf + 1] = j;
    y[nf++] = t;
    p = q;
  }
  return nf;
}

/* Y(f, r) = sum over the run's nonzeros of v * U(r, k), r = 0..R-1; U is R x K
 * row-major (the reference's C: C0_size x C1_size, C1_size the last mode). */
ORACLE_API int64_t oracle_coo_ttm(int64_t nnz, const int64_t* coords, const double* vals, int64_t R,
                                  int64_t K, const double* U, int64_t* fib, double* Y) {
  int64_t nf = 0;
  for (int64_t p = 0; p < nnz;) {
    const int64_t i = coords[3 * p], j = coords[3 * p + 1];
    int64_t e = p;
    while (e < nnz && coords[3 * e] == i && coords[3 * e + 1] == j) e++;
    for (int64_t r = 0; r < R; r++) {
      double t = 0.0;
      for (int64_t q = p; q < e; q++) t = t + vals[q] * U[r * K + coords[3 * q + 2]];
      Y[nf * R + r] = t;
    }
    fib[2 * nf] = i;
    fib[2 * nf + 1] = j;
    nf++;
    p = e;
  }
  return nf;
}
