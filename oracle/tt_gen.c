/*
 * tt_gen.c -- test infrastructure: a C restatement of libtentaco_gb300's seeded
 * generators (tt_gen_dense, tt_gen_lognormal_fibers in tentaco_gb300/csrc/tt_host.cpp),
 * so that the reference arm of bench.py and the oracle tests build the same
 * synthetic tensors without loading the product library.  tests/test_oracle.py
 * checks that both produce identical arrays.
 *
 * Generator: xoshiro256** seeded through splitmix64 from (seed, stream); uniform
 * doubles from the top 53 bits; normal deviates by Box-Muller.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

typedef struct {
  uint64_t s[4];
} gen_rng;

static uint64_t sm64(uint64_t* x) {
  uint64_t z = (*x += 0x9e3779b97f4a7c15ull);
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}
static gen_rng rng_make(uint64_t seed, uint64_t stream) {
  gen_rng g;
  uint64_t x = seed ^ (stream * 0xd1342543de82ef95ull + 0x2545f4914f6cdd1dull);
  for (int i = 0; i < 4; i++) g.s[i] = sm64(&x);
  return g;
}
static uint64_t rot(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }
static uint64_t rng_next(gen_rng* g) {
  const uint64_t r = rot(g->s[1] * 5, 7) * 9, t = g->s[1] << 17;
  g->s[2] ^= g->s[0];
  g->s[3] ^= g->s[1];
  g->s[1] ^= g->s[2];
  g->s[0] ^= g->s[3];
  g->s[2] ^= t;
  g->s[3] = rot(g->s[3], 45);
  return r;
}
static double rng_uniform(gen_rng* g) { return (double)(rng_next(g) >> 11) * 0x1.0p-53; }
static double rng_normal(gen_rng* g) {
  double u1 = rng_uniform(g), u2 = rng_uniform(g);
  if (u1 < 1e-300) u1 = 1e-300;
  return sqrt(-2.0 * log(u1)) * cos(6.283185307179586 * u2);
}

/* rows x cols row-major: dist 0 U(0,1); 1 N(0,1) times a per-column scale 2^(-3 + 6 U);
 * 2 U(-1,1).  Rows are drawn in chunks of 4096 with their own streams. */
void oracle_gen_dense(int64_t rows, int64_t cols, int dist, uint64_t seed, float* out) {
  double* cs = (double*)malloc(sizeof(double) * (size_t)cols);
  for (int64_t j = 0; j < cols; j++) cs[j] = 1.0;
  if (dist == 1) {
    gen_rng g = rng_make(seed, 0xc0);
    for (int64_t j = 0; j < cols; j++) cs[j] = exp2(-3.0 + 6.0 * rng_uniform(&g));
  }
  const int64_t nch = (rows + 4095) / 4096;
#pragma omp parallel for schedule(static)
  for (int64_t ch = 0; ch < nch; ch++) {
    gen_rng g = rng_make(seed, 0x100000ull + (uint64_t)ch);
    const int64_t r1 = (ch + 1) * 4096 < rows ? (ch + 1) * 4096 : rows;
    for (int64_t r = ch * 4096; r < r1; r++)
      for (int64_t j = 0; j < cols; j++) {
        double v;
        if (dist == 0) v = rng_uniform(&g);
        else if (dist == 1) v = rng_normal(&g) * cs[j];
        else v = 2.0 * rng_uniform(&g) - 1.0;
        out[r * cols + j] = (float)v;
      }
  }
  free(cs);
}

static int cmp_u64(const void* a, const void* b) {
  const uint64_t x = *(const uint64_t*)a, y = *(const uint64_t*)b;
  return x < y ? -1 : x > y;
}
static int cmp_i32(const void* a, const void* b) {
  const int32_t x = *(const int32_t*)a, y = *(const int32_t*)b;
  return x < y ? -1 : x > y;
}
static int64_t unique_u64(uint64_t* a, int64_t n) {
  int64_t m = 0;
  for (int64_t i = 0; i < n; i++)
    if (m == 0 || a[i] != a[m - 1]) a[m++] = a[i];
  return m;
}

/* Fiber lengths: n_long fibers of at least long_min nonzeros, then
 * round(lognormal(mu, sigma)) clipped to [1, dims[2]], until nnz; shuffled. */
static int64_t fiber_lengths(const int32_t* dims, int64_t nnz, double mu, double sigma, int64_t n_long,
                             int64_t long_min, gen_rng* g, int64_t** out) {
  const int64_t L = dims[2];
  if (long_min > L) long_min = L;
  int64_t cap = 1024, nf = 0, total = 0;
  int64_t* len = (int64_t*)malloc(sizeof(int64_t) * (size_t)cap);
  for (int64_t i = 0; i < n_long && total < nnz; i++) {
    int64_t x = long_min + (int64_t)(rng_uniform(g) * (double)(L - long_min + 1));
    const int64_t lim = L < nnz - total ? L : nnz - total;
    if (x > lim) x = lim;
    if (nf == cap) len = (int64_t*)realloc(len, sizeof(int64_t) * (size_t)(cap *= 2));
    len[nf++] = x;
    total += x;
  }
  while (total < nnz) {
    const double v = exp(mu + sigma * rng_normal(g));
    int64_t x = (int64_t)llround(v);
    if (x > L) x = L;
    if (x < 1) x = 1;
    if (x > nnz - total) x = nnz - total;
    if (nf == cap) len = (int64_t*)realloc(len, sizeof(int64_t) * (size_t)(cap *= 2));
    len[nf++] = x;
    total += x;
  }
  for (int64_t i = nf - 1; i > 0; i--) {
    const int64_t j = (int64_t)(rng_next(g) % (uint64_t)(i + 1));
    const int64_t t = len[i];
    len[i] = len[j];
    len[j] = t;
  }
  *out = len;
  return nf;
}

/* Number of level-1 fibers oracle_gen_lognormal will produce. */
int64_t oracle_lognormal_nfibers(const int32_t* dims, int64_t nnz, double mu, double sigma, int64_t n_long,
                                 int64_t long_min, uint64_t seed) {
  gen_rng g = rng_make(seed, 1);
  int64_t* len = NULL;
  const int64_t nf = fiber_lengths(dims, nnz, mu, sigma, n_long, long_min, &g, &len);
  free(len);
  return nf;
}

/* The dense-root 3-mode CSF of tt_gen_lognormal_fibers: distinct (i, k) per fiber
 * from [dims0] x [dims1], distinct sorted leaf coordinates per fiber, values
 * U(0,1).  pos1: dims0 + 1; crd1, pos2: nf and nf + 1; crd2, vals: nnz.
 * Returns 0, or -1 if the distinct fibers could not be drawn. */
int oracle_gen_lognormal(const int32_t* dims, int64_t nnz, double mu, double sigma, int64_t n_long,
                         int64_t long_min, uint64_t seed, int32_t* pos1, int32_t* crd1, int32_t* pos2, int32_t* crd2,
                         float* vals) {
  const int64_t L = dims[2];
  gen_rng g = rng_make(seed, 1);
  int64_t* len = NULL;
  const int64_t nf = fiber_lengths(dims, nnz, mu, sigma, n_long, long_min, &g, &len);
  const uint64_t cells = (uint64_t)dims[0] * (uint64_t)dims[1];
  if ((uint64_t)nf > cells) { free(len); return -1; }
  const int64_t kChunk = 1 << 16;
  uint64_t* ik = NULL;
  int64_t nik = 0;
  for (int round = 0; nik < nf && round < 64; round++) {
    const int64_t need = nf - nik, draw = need + need / 8 + 64;
    const int64_t nch = (draw + kChunk - 1) / kChunk;
    uint64_t* fresh = (uint64_t*)malloc(sizeof(uint64_t) * (size_t)(draw + nik));
#pragma omp parallel for schedule(static)
    for (int64_t ch = 0; ch < nch; ch++) {
      gen_rng h = rng_make(seed, ((uint64_t)(round + 2) << 40) + (uint64_t)ch);
      const int64_t p1 = (ch + 1) * kChunk < draw ? (ch + 1) * kChunk : draw;
      for (int64_t p = ch * kChunk; p < p1; p++) fresh[p] = rng_next(&h) % cells;
    }
    if (nik) memcpy(fresh + draw, ik, sizeof(uint64_t) * (size_t)nik);
    int64_t m = draw + nik;
    qsort(fresh, (size_t)m, sizeof(uint64_t), cmp_u64);
    m = unique_u64(fresh, m);
    if (m > nf) {  /* a seeded random subset of exactly nf, in order */
      gen_rng h = rng_make(seed, 0x1234 + (uint64_t)round);
      int64_t left = m, want = nf, k = 0;
      for (int64_t i = 0; i < m && want > 0; i++, left--)
        if (rng_uniform(&h) * (double)left < (double)want) { fresh[k++] = fresh[i]; want--; }
      m = k;
    }
    free(ik);
    ik = fresh;
    nik = m;
  }
  if (nik != nf) { free(ik); free(len); return -1; }
  memset(pos1, 0, sizeof(int32_t) * (size_t)(dims[0] + 1));
  for (int64_t f = 0; f < nf; f++) {
    const int64_t i = (int64_t)(ik[f] / (uint64_t)dims[1]);
    crd1[f] = (int32_t)(ik[f] % (uint64_t)dims[1]);
    pos1[i + 1]++;
  }
  for (int64_t r = 0; r < dims[0]; r++) pos1[r + 1] += pos1[r];
  pos2[0] = 0;
  for (int64_t f = 0; f < nf; f++) pos2[f + 1] = pos2[f] + (int32_t)len[f];
#pragma omp parallel for schedule(dynamic, 256)
  for (int64_t f = 0; f < nf; f++) {
    gen_rng h = rng_make(seed, 0x7000000000ull + (uint64_t)f);
    const int64_t a = pos2[f], n = len[f];
    int32_t* out_l = crd2 + a;
    if (n * 8 >= L) {  /* selection sampling over all of [0, L) */
      int64_t want = n, left = L, k = 0;
      for (int64_t l = 0; l < L && want > 0; l++, left--)
        if (rng_uniform(&h) * (double)left < (double)want) { out_l[k++] = (int32_t)l; want--; }
    } else {
      int64_t cap = n * 2 + 8, m = 0;
      int32_t* s = (int32_t*)malloc(sizeof(int32_t) * (size_t)cap);
      while (m < n) {
        while (m < n + n / 4 + 4) {
          if (m == cap) s = (int32_t*)realloc(s, sizeof(int32_t) * (size_t)(cap *= 2));
          s[m++] = (int32_t)(rng_next(&h) % (uint64_t)L);
        }
        qsort(s, (size_t)m, sizeof(int32_t), cmp_i32);
        int64_t u = 0;
        for (int64_t i = 0; i < m; i++)
          if (u == 0 || s[i] != s[u - 1]) s[u++] = s[i];
        m = u;
      }
      while (m > n) {  /* drop a random surplus entry */
        const int64_t e = (int64_t)(rng_next(&h) % (uint64_t)m);
        memmove(s + e, s + e + 1, sizeof(int32_t) * (size_t)(m - e - 1));
        m--;
      }
      memcpy(out_l, s, sizeof(int32_t) * (size_t)n);
      free(s);
    }
    float* ov = vals + a;
    for (int64_t p = 0; p < n; p++) ov[p] = (float)rng_uniform(&h);
  }
  free(ik);
  free(len);
  return 0;
}
