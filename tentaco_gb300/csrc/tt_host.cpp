// tt_host.cpp -- host side of libtentaco_gb300: error state, library-owned tensors,
// canonical CSF construction and validation, seeded generators, selector features.
//
// The reference builds CSF inside SPLATT (ds.h:351-384, splatt_csf_load with
// SPLATT_CSF_ONEMODE) and then rewrites level 0 with compress_top_level
// (ds.h:426-436).  This file defines the canonical CSF of this library instead:
// modes in order 0..order-1, coordinates sorted lexicographically, duplicates
// summed (in FP64, in input order), a dense root whose pos has dims[0]+1 entries
// (empty rows allowed), plus the compressed-root arrays {pos=[0,dims0],
// crd=0..dims0-1} in indices[0] for callers that expect compress_top_level.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdarg>
#include <cstring>
#include <numeric>
#include <omp.h>
#include "tt_internal.h"
#include "../../include/tentaco/tentaco_gen.h"

namespace tt {

// ---------------------------------------------------------------------------
// errors
// ---------------------------------------------------------------------------
static thread_local std::string g_last_error;

tt_status set_error(tt_status s, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_last_error = std::string(tt_status_string(s)) + ": " + buf;
  return s;
}
void clear_error() { g_last_error.clear(); }
const char* g_last_error_cstr() { return g_last_error.c_str(); }

// ---------------------------------------------------------------------------
// owned tensors
// ---------------------------------------------------------------------------
OwnedTensor::OwnedTensor() : magic(kMagic) {
  std::memset(&t, 0, sizeof(t));
  std::memset(dims, 0, sizeof(dims));
  std::memset(levels, 0, sizeof(levels));
  std::memset(slots, 0, sizeof(slots));
  for (int i = 0; i < TT_MAX_ORDER; i++) { mode_ordering[i] = i; mode_types[i] = taco_mode_sparse; }
}

void OwnedTensor::publish(int order, const int32_t* d) {
  t.order = order;
  for (int i = 0; i < order; i++) dims[i] = d[i];
  t.dimensions = dims;
  t.csize = 4;
  t.mode_ordering = mode_ordering;
  mode_types[0] = taco_mode_dense;
  t.mode_types = mode_types;
  for (int l = 0; l < order; l++) {
    levels[l] = &slots[2 * l];
    slots[2 * l] = pos[l].empty() ? nullptr : pos[l].data();
    slots[2 * l + 1] = crd[l].empty() ? nullptr : crd[l].data();
  }
  t.indices = levels;
  t.vals = vals.data();
  t.vals_size = (int32_t)std::min<size_t>(vals.size(), 0x7fffffff);
}

// ---------------------------------------------------------------------------
// CSF view / validation
// ---------------------------------------------------------------------------
tt_status csf_view(const taco_tensor_t* B, CsfView* v) {
  if (!B || !B->dimensions || !B->indices) return set_error(TT_ERR_INVALID_ARGUMENT, "null tensor");
  if (B->order < 2 || B->order > TT_MAX_ORDER)
    return set_error(TT_ERR_UNSUPPORTED, "order %d (supported: 2..%d)", B->order, TT_MAX_ORDER);
  v->order = B->order;
  for (int i = 0; i < B->order; i++) {
    v->dims[i] = B->dimensions[i];
    if (v->dims[i] <= 0) return set_error(TT_ERR_INVALID_ARGUMENT, "dimension %d is %d", i, v->dims[i]);
  }
  const bool dense = (B->mode_types && B->mode_types[0] == taco_mode_dense) || !B->indices[0] ||
                     !B->indices[0][0];
  v->dense_root = dense;
  if (dense) {
    v->nroot = v->dims[0];
    v->root_crd = nullptr;
  } else {
    const int32_t* p0 = B->indices[0][0];
    if (p0[0] != 0) return set_error(TT_ERR_INVALID_CSF, "root pos[0] = %d", p0[0]);
    v->nroot = p0[1];
    v->root_crd = B->indices[0][1];
    if (v->nroot > 0 && !v->root_crd) return set_error(TT_ERR_INVALID_CSF, "compressed root without crd");
  }
  v->count[0] = v->nroot;
  for (int l = 1; l < v->order; l++) {
    if (!B->indices[l] || !B->indices[l][0]) return set_error(TT_ERR_INVALID_CSF, "level %d pos missing", l);
    v->pos[l] = B->indices[l][0];
    v->crd[l] = B->indices[l][1];
    v->count[l] = v->pos[l][v->count[l - 1]];
    if (v->count[l] > 0 && !v->crd[l]) return set_error(TT_ERR_INVALID_CSF, "level %d crd missing", l);
  }
  v->nnz = v->count[v->order - 1];
  v->vals = B->vals;
  if (v->nnz > 0 && !v->vals) return set_error(TT_ERR_INVALID_CSF, "vals missing");
  return TT_OK;
}

tt_status csf_check_root(const CsfView& v) {
  if (!v.dense_root) {
    for (int64_t r = 0; r < v.nroot; r++) {
      if (v.root_crd[r] < 0 || v.root_crd[r] >= v.dims[0])
        return set_error(TT_ERR_INVALID_CSF, "root crd[%lld] = %d out of [0,%d)", (long long)r, v.root_crd[r], v.dims[0]);
      if (r > 0 && v.root_crd[r] <= v.root_crd[r - 1])
        return set_error(TT_ERR_INVALID_CSF, "root crd not strictly increasing at %lld", (long long)r);
    }
  }
  if (v.nnz > 0x7fffffffLL) return set_error(TT_ERR_UNSUPPORTED, "nnz %lld exceeds int32 positions", (long long)v.nnz);
  for (int l = 1; l < v.order; l++)
    if (v.pos[l][0] != 0) return set_error(TT_ERR_INVALID_CSF, "level %d pos[0] = %d", l, v.pos[l][0]);
  return TT_OK;
}

tt_status csf_check(const CsfView& v) {
  tt_status s = csf_check_root(v);
  if (s != TT_OK) return s;
  for (int l = 1; l < v.order; l++) {
    const int32_t* pos = v.pos[l];
    const int32_t* crd = v.crd[l];
    const int64_t np = v.count[l - 1];
    if (pos[0] != 0) return set_error(TT_ERR_INVALID_CSF, "level %d pos[0] = %d", l, pos[0]);
    std::atomic<int> bad(0);
    std::atomic<int64_t> where(-1);
#pragma omp parallel for schedule(static)
    for (int64_t f = 0; f < np; f++) {
      const int64_t a = pos[f], b = pos[f + 1];
      int err = 0;
      if (b < a) err = 1;
      else if (l >= 2 && b == a) err = 2;  // empty inner fiber
      else {
        for (int64_t p = a; p < b; p++) {
          if (crd[p] < 0 || crd[p] >= v.dims[l]) { err = 3; break; }
          if (p > a && crd[p] <= crd[p - 1]) { err = 4; break; }
        }
      }
      if (err) { bad.store(err); where.store(f); }
    }
    const char* why[] = {"", "pos decreasing", "empty inner fiber", "crd out of range",
                         "crd not strictly increasing in a fiber"};
    if (bad.load()) return set_error(TT_ERR_INVALID_CSF, "level %d fiber %lld: %s", l, (long long)where.load(), why[bad.load()]);
  }
  return TT_OK;
}

tt_status csf_check_error(int level, uint64_t word) {
  if (word == UINT64_MAX) return TT_OK;
  const int code = (int)(word & 7u);
  const long long at = (long long)(word >> 3);
  const char* why[] = {"", "pos decreasing", "empty inner fiber", "crd out of range",
                       "crd not strictly increasing in a fiber"};
  return set_error(TT_ERR_INVALID_CSF, "level %d %s %lld: %s", level, code <= 2 ? "fiber" : "position", at,
                   why[code >= 1 && code <= 4 ? code : 0]);
}

// ---------------------------------------------------------------------------
// radix sort
// ---------------------------------------------------------------------------
void radix_sort_pairs(std::vector<uint64_t>& keys, std::vector<uint32_t>& payload, int bits) {
  const size_t n = keys.size();
  if (n < 2) return;
  std::vector<uint64_t> k2(n);
  std::vector<uint32_t> p2(n);
  const int nt = std::max(1, std::min(omp_get_max_threads(), (int)(n / 65536) + 1));
  const int DB = 11, NB = 1 << DB;
  std::vector<size_t> hist((size_t)nt * NB);
  for (int shift = 0; shift < bits; shift += DB) {
    std::fill(hist.begin(), hist.end(), 0);
#pragma omp parallel num_threads(nt)
    {
      const int t = omp_get_thread_num();
      const size_t lo = n * t / nt, hi = n * (t + 1) / nt;
      size_t* h = &hist[(size_t)t * NB];
      for (size_t i = lo; i < hi; i++) h[(keys[i] >> shift) & (NB - 1)]++;
    }
    size_t sum = 0;
    for (int d = 0; d < NB; d++)
      for (int t = 0; t < nt; t++) {
        size_t c = hist[(size_t)t * NB + d];
        hist[(size_t)t * NB + d] = sum;
        sum += c;
      }
#pragma omp parallel num_threads(nt)
    {
      const int t = omp_get_thread_num();
      const size_t lo = n * t / nt, hi = n * (t + 1) / nt;
      size_t* h = &hist[(size_t)t * NB];
      for (size_t i = lo; i < hi; i++) {
        size_t d = h[(keys[i] >> shift) & (NB - 1)]++;
        k2[d] = keys[i];
        p2[d] = payload[i];
      }
    }
    keys.swap(k2);
    payload.swap(p2);
  }
}

// ---------------------------------------------------------------------------
// RNG
// ---------------------------------------------------------------------------
static inline uint64_t splitmix64(uint64_t& x) {
  uint64_t z = (x += 0x9e3779b97f4a7c15ull);
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}
Rng::Rng(uint64_t seed, uint64_t stream) {
  uint64_t x = seed ^ (stream * 0xd1342543de82ef95ull + 0x2545f4914f6cdd1dull);
  for (int i = 0; i < 4; i++) s[i] = splitmix64(x);
}
static inline uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }
uint64_t Rng::next() {
  const uint64_t r = rotl(s[1] * 5, 7) * 9;
  const uint64_t t = s[1] << 17;
  s[2] ^= s[0]; s[3] ^= s[1]; s[1] ^= s[2]; s[0] ^= s[3];
  s[2] ^= t; s[3] = rotl(s[3], 45);
  return r;
}
double Rng::uniform() { return (next() >> 11) * 0x1.0p-53; }
double Rng::normal() {
  double u1 = uniform(), u2 = uniform();
  if (u1 < 1e-300) u1 = 1e-300;
  return std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2);
}

}  // namespace tt

using namespace tt;

// ---------------------------------------------------------------------------
// CSF from sorted unique packed keys
// ---------------------------------------------------------------------------
namespace {

struct Packing {
  int order;
  int bits[TT_MAX_ORDER];
  int shift[TT_MAX_ORDER];
  int total;
  bool ok;
  explicit Packing(int o, const int32_t* dims) : order(o), total(0) {
    for (int m = o - 1; m >= 0; m--) {
      int b = 1;
      while ((1ll << b) < dims[m]) b++;
      bits[m] = b;
      shift[m] = total;
      total += b;
    }
    ok = total <= 63;
  }
  inline uint64_t pack(const int32_t* c) const {
    uint64_t k = 0;
    for (int m = 0; m < order; m++) k |= (uint64_t)c[m] << shift[m];
    return k;
  }
  inline int32_t get(uint64_t k, int m) const { return (int32_t)((k >> shift[m]) & ((1ull << bits[m]) - 1)); }
};

// keys: sorted, distinct; vals aligned.  Fills o->pos/crd/vals.
void csf_from_sorted_keys(const Packing& pk, const int32_t* dims, const std::vector<uint64_t>& keys,
                          std::vector<float>&& vals, OwnedTensor* o) {
  const int order = pk.order;
  const int64_t n = (int64_t)keys.size();
  // first level whose coordinate differs from the previous entry
  std::vector<uint8_t> nl((size_t)n);
#pragma omp parallel for schedule(static)
  for (int64_t p = 0; p < n; p++) {
    if (p == 0) { nl[0] = 0; continue; }
    const uint64_t diff = keys[p] ^ keys[p - 1];
    int l = order;
    for (int m = 0; m < order; m++)
      if ((diff >> pk.shift[m]) & ((1ull << pk.bits[m]) - 1)) { l = m; break; }
    nl[p] = (uint8_t)l;
  }
  // per-thread counts of fiber starts per level, then offsets
  const int nt = omp_get_max_threads();
  std::vector<int64_t> cnt((size_t)nt * TT_MAX_ORDER, 0);
#pragma omp parallel num_threads(nt)
  {
    const int t = omp_get_thread_num();
    const int64_t lo = n * t / nt, hi = n * (t + 1) / nt;
    int64_t* c = &cnt[(size_t)t * TT_MAX_ORDER];
    for (int64_t p = lo; p < hi; p++)
      for (int l = std::max<int>(1, nl[p]); l < order; l++) c[l]++;
  }
  int64_t total[TT_MAX_ORDER] = {0, 0, 0, 0};
  for (int t = 0; t < nt; t++)
    for (int l = 1; l < order; l++) {
      int64_t c = cnt[(size_t)t * TT_MAX_ORDER + l];
      cnt[(size_t)t * TT_MAX_ORDER + l] = total[l];
      total[l] += c;
    }
  o->pos[1].assign((size_t)dims[0] + 1, 0);
  for (int l = 1; l < order; l++) {
    o->crd[l].resize((size_t)total[l]);
    if (l >= 2) o->pos[l].resize((size_t)total[l - 1] + 1);
  }
#pragma omp parallel num_threads(nt)
  {
    const int t = omp_get_thread_num();
    const int64_t lo = n * t / nt, hi = n * (t + 1) / nt;
    int64_t c[TT_MAX_ORDER];
    for (int l = 0; l < TT_MAX_ORDER; l++) c[l] = cnt[(size_t)t * TT_MAX_ORDER + l];
    for (int64_t p = lo; p < hi; p++) {
      for (int l = std::max<int>(1, nl[p]); l < order; l++) {
        // a new level-l fiber; if it also opens a new parent, record the parent's first child
        if (l >= 2 && nl[p] <= l - 1) o->pos[l][(size_t)c[l - 1] - 1] = (int32_t)c[l];
        o->crd[l][(size_t)c[l]] = pk.get(keys[p], l);
        c[l]++;
      }
    }
  }
  // dense root: pos1[r] = level-1 fibers in rows below r (their rows are sorted)
  std::vector<int32_t> frow((size_t)total[1]);
#pragma omp parallel num_threads(nt)
  {
    const int t = omp_get_thread_num();
    int64_t c1 = cnt[(size_t)t * TT_MAX_ORDER + 1];
    for (int64_t p = n * t / nt; p < n * (t + 1) / nt; p++)
      if (nl[p] <= 1) frow[(size_t)c1++] = pk.get(keys[p], 0);
  }
#pragma omp parallel for schedule(static)
  for (int64_t r = 0; r <= dims[0]; r++)
    o->pos[1][(size_t)r] = (int32_t)(std::lower_bound(frow.begin(), frow.end(), (int32_t)r) - frow.begin());
  for (int l = 2; l < order; l++) o->pos[l][(size_t)total[l - 1]] = (int32_t)total[l];
  // compressed-root arrays for reference callers (compress_top_level form)
  o->pos[0] = {0, dims[0]};
  o->crd[0].resize((size_t)dims[0]);
  std::iota(o->crd[0].begin(), o->crd[0].end(), 0);
  o->vals = std::move(vals);
  o->publish(order, dims);
}

// Sort packed keys with their values, merge duplicates (FP64 sum in input order).
void sort_dedupe(const Packing& pk, std::vector<uint64_t>& keys, std::vector<float>& vals,
                 std::vector<float>& out_vals) {
  const size_t n = keys.size();
  std::vector<uint32_t> idx(n);
  std::iota(idx.begin(), idx.end(), 0u);
  radix_sort_pairs(keys, idx, pk.total);
  // runs of equal keys, in parallel: a run belongs to the thread whose chunk holds
  // its first entry; its values are summed in FP64 in input order (the sort is stable)
  std::vector<uint8_t> first(n);
#pragma omp parallel for schedule(static)
  for (size_t p = 0; p < n; p++) first[p] = p == 0 || keys[p] != keys[p - 1];
  const int nt = std::max(1, std::min(omp_get_max_threads(), (int)(n / 65536) + 1));
  std::vector<size_t> off((size_t)nt + 1, 0);
#pragma omp parallel num_threads(nt)
  {
    const int t = omp_get_thread_num();
    size_t c = 0;
    for (size_t p = n * t / nt; p < n * (t + 1) / nt; p++) c += first[p];
    off[(size_t)t + 1] = c;
  }
  for (int t = 0; t < nt; t++) off[(size_t)t + 1] += off[(size_t)t];
  const size_t m = off[(size_t)nt];
  std::vector<uint64_t> k2(m);
  out_vals.assign(m, 0.f);
#pragma omp parallel num_threads(nt)
  {
    const int t = omp_get_thread_num();
    size_t r = off[(size_t)t];
    for (size_t p = n * t / nt; p < n * (t + 1) / nt; p++) {
      if (!first[p]) continue;
      double s = 0.0;
      size_t q = p;
      do { s += (double)vals[idx[q]]; q++; } while (q < n && !first[q]);
      k2[r] = keys[p];
      out_vals[r] = (float)s;
      r++;
    }
  }
  keys.swap(k2);
}

}  // namespace

TT_EXPORT tt_status tt_csf_from_coo(int32_t order, const int32_t* dims, int64_t nnz,
                                    const int32_t* coords, const float* vals, taco_tensor_t** out) {
  clear_error();
  if (!out || !dims || (nnz > 0 && (!coords || !vals)))
    return set_error(TT_ERR_INVALID_ARGUMENT, "null argument");
  *out = nullptr;
  if (order < 2 || order > TT_MAX_ORDER) return set_error(TT_ERR_UNSUPPORTED, "order %d", order);
  if (nnz < 0 || nnz > 0xffffffffLL) return set_error(TT_ERR_UNSUPPORTED, "nnz %lld", (long long)nnz);
  for (int m = 0; m < order; m++)
    if (dims[m] <= 0) return set_error(TT_ERR_INVALID_ARGUMENT, "dims[%d] = %d", m, dims[m]);
  Packing pk(order, dims);
  if (!pk.ok) return set_error(TT_ERR_UNSUPPORTED, "coordinates need %d bits (> 63)", pk.total);
  std::vector<uint64_t> keys((size_t)nnz);
  std::atomic<int64_t> bad(-1);
#pragma omp parallel for schedule(static)
  for (int64_t p = 0; p < nnz; p++) {
    const int32_t* c = coords + p * order;
    for (int m = 0; m < order; m++)
      if (c[m] < 0 || c[m] >= dims[m]) bad.store(p);
    keys[(size_t)p] = pk.pack(c);
  }
  if (bad.load() >= 0) return set_error(TT_ERR_INVALID_ARGUMENT, "coordinate %lld out of range", (long long)bad.load());
  std::vector<float> v(vals, vals + nnz), uv;
  sort_dedupe(pk, keys, v, uv);
  auto* o = new OwnedTensor();
  csf_from_sorted_keys(pk, dims, keys, std::move(uv), o);
  *out = &o->t;
  return TT_OK;
}

// Every nonzero's coordinates in the level order of the CSF rooted at `mode`
// (mode, then the other modes in increasing order), at its leaf position:
// co[p * order + k] = coordinate of old mode perm[k]; nd: the permuted dims.
// v must be a validated CSF.
tt_status tt::csf_rerooted_coords(const CsfView& v, int mode, std::vector<int32_t>& co, int32_t* nd) {
  const int order = v.order;
  if (mode < 0 || mode >= order) return set_error(TT_ERR_INVALID_ARGUMENT, "mode %d of an order-%d tensor", mode, order);
  int perm[TT_MAX_ORDER];  // new level k holds old mode perm[k]
  perm[0] = mode;
  for (int m = 0, k = 1; m < order; m++)
    if (m != mode) perm[k++] = m;
  for (int k = 0; k < order; k++) nd[k] = v.dims[perm[k]];
  co.resize((size_t)v.nnz * order);
  // walk every root position depth first; a nonzero's coordinates go to its leaf position
#pragma omp parallel for schedule(dynamic, 64)
  for (int64_t r = 0; r < v.nroot; r++) {
    int32_t c[TT_MAX_ORDER];
    c[0] = v.dense_root ? (int32_t)r : v.root_crd[r];
    int64_t lo[TT_MAX_ORDER], hi[TT_MAX_ORDER];
    lo[1] = v.pos[1][r];
    hi[1] = v.pos[1][r + 1];
    int l = 1;
    while (l >= 1) {
      if (lo[l] >= hi[l]) { l--; if (l >= 1) lo[l]++; continue; }
      c[l] = v.crd[l][lo[l]];
      if (l == order - 1) {
        int32_t* q = co.data() + (size_t)lo[l] * order;
        for (int k = 0; k < order; k++) q[k] = c[perm[k]];
        lo[l]++;
      } else {
        lo[l + 1] = v.pos[l + 1][lo[l]];
        hi[l + 1] = v.pos[l + 1][lo[l] + 1];
        l++;
      }
    }
  }
  return TT_OK;
}

// The same tensor as a CSF rooted at `mode`, built on the host like
// tt_csf_from_coo (packed keys, radix sort, lexicographic, dense root).
tt_status tt::csf_reroot(const CsfView& v, int mode, taco_tensor_t** out) {
  *out = nullptr;
  std::vector<int32_t> co;
  int32_t nd[TT_MAX_ORDER];
  tt_status s = csf_rerooted_coords(v, mode, co, nd);
  if (s != TT_OK) return s;
  return tt_csf_from_coo(v.order, nd, v.nnz, co.data(), v.vals, out);
}

TT_EXPORT tt_status tt_csf_reroot(const taco_tensor_t* B, int32_t mode, taco_tensor_t** out) {
  clear_error();
  if (!out) return set_error(TT_ERR_INVALID_ARGUMENT, "null argument");
  *out = nullptr;
  CsfView v;
  tt_status s = csf_view(B, &v);
  if (s != TT_OK) return s;
  if ((s = csf_check(v)) != TT_OK) return s;
  return csf_reroot(v, mode, out);
}

TT_EXPORT void tt_tensor_free(taco_tensor_t* t) {
  if (!t) return;
  auto* o = reinterpret_cast<OwnedTensor*>(t);
  if (o->magic != OwnedTensor::kMagic) return;  // not ours
  o->magic = 0;
  delete o;
}

TT_EXPORT tt_status tt_csf_validate(const taco_tensor_t* B) {
  clear_error();
  CsfView v;
  tt_status s = csf_view(B, &v);
  if (s != TT_OK) return s;
  return csf_check(v);
}

// ---------------------------------------------------------------------------
// generators
// ---------------------------------------------------------------------------
namespace {

// Inverse-CDF sampler of a Zipf(s) law over ranks [0, n), ranks mapped by a permutation.
struct ZipfMode {
  int32_t n;
  double s;
  std::vector<double> cdf;
  std::vector<int32_t> perm;
  ZipfMode(int32_t n_, double s_, uint64_t seed, int mode) : n(n_), s(s_) {
    if (s > 0) {
      cdf.resize((size_t)n);
      double acc = 0;
      for (int32_t r = 0; r < n; r++) { acc += std::pow((double)(r + 1), -s); cdf[(size_t)r] = acc; }
      for (auto& c : cdf) c /= acc;
      perm.resize((size_t)n);
      std::iota(perm.begin(), perm.end(), 0);
      Rng g(seed, 0x5000 + mode);
      for (int32_t i = n - 1; i > 0; i--) std::swap(perm[(size_t)i], perm[(size_t)(g.next() % (uint64_t)(i + 1))]);
    }
  }
  inline int32_t draw(Rng& g) const {
    if (s <= 0) return (int32_t)(g.next() % (uint64_t)n);
    const double u = g.uniform();
    size_t r = (size_t)(std::upper_bound(cdf.begin(), cdf.end(), u) - cdf.begin());
    if (r >= (size_t)n) r = (size_t)n - 1;
    return perm[r];
  }
};

constexpr int64_t kChunk = 1 << 16;

}  // namespace

TT_EXPORT tt_status tt_gen_zipf(int32_t order, const int32_t* dims, const double* zipf_s, int64_t nnz,
                                float vlo, float vhi, uint64_t seed, int32_t max_rounds,
                                taco_tensor_t** out) {
  clear_error();
  if (!out || !dims || !zipf_s) return set_error(TT_ERR_INVALID_ARGUMENT, "null argument");
  *out = nullptr;
  if (order < 2 || order > TT_MAX_ORDER) return set_error(TT_ERR_UNSUPPORTED, "order %d", order);
  Packing pk(order, dims);
  if (!pk.ok) return set_error(TT_ERR_UNSUPPORTED, "coordinates need %d bits (> 63)", pk.total);
  double cap = 1.0;
  for (int m = 0; m < order; m++) cap *= dims[m];
  if ((double)nnz > cap) return set_error(TT_ERR_INVALID_ARGUMENT, "nnz exceeds the number of cells");
  std::vector<ZipfMode> modes;
  for (int m = 0; m < order; m++) modes.emplace_back(dims[m], zipf_s[m], seed, m);

  std::vector<uint64_t> have;
  for (int round = 0; round < std::max(1, max_rounds) && (int64_t)have.size() < nnz; round++) {
    const int64_t need = nnz - (int64_t)have.size();
    const int64_t draw = need + need / 4 + 1024;
    const int64_t nch = (draw + kChunk - 1) / kChunk;
    std::vector<uint64_t> fresh((size_t)draw);
#pragma omp parallel for schedule(dynamic, 1)
    for (int64_t ch = 0; ch < nch; ch++) {
      Rng g(seed, ((uint64_t)round << 40) + (uint64_t)ch);
      int32_t c[TT_MAX_ORDER];
      for (int64_t p = ch * kChunk; p < std::min(draw, (ch + 1) * kChunk); p++) {
        for (int m = 0; m < order; m++) c[m] = modes[(size_t)m].draw(g);
        fresh[(size_t)p] = pk.pack(c);
      }
    }
    fresh.insert(fresh.end(), have.begin(), have.end());
    std::vector<uint32_t> dummy(fresh.size(), 0);
    radix_sort_pairs(fresh, dummy, pk.total);
    fresh.erase(std::unique(fresh.begin(), fresh.end()), fresh.end());
    have.swap(fresh);
  }
  // exactly nnz (if reachable): drop the surplus by selection sampling
  if ((int64_t)have.size() > nnz) {
    Rng g(seed, 0x77777);
    std::vector<uint64_t> kept;
    kept.reserve((size_t)nnz);
    int64_t left = (int64_t)have.size(), want = nnz;
    for (size_t i = 0; i < have.size() && want > 0; i++, left--) {
      if ((double)(g.next() >> 11) * 0x1.0p-53 * (double)left < (double)want) { kept.push_back(have[i]); want--; }
    }
    have.swap(kept);
  }
  const int64_t m = (int64_t)have.size();
  std::vector<float> vals((size_t)m);
  const int64_t nch = (m + kChunk - 1) / kChunk;
#pragma omp parallel for schedule(static)
  for (int64_t ch = 0; ch < nch; ch++) {
    Rng g(seed, 0x9000000000ull + (uint64_t)ch);
    for (int64_t p = ch * kChunk; p < std::min(m, (ch + 1) * kChunk); p++)
      vals[(size_t)p] = (float)(vlo + (vhi - vlo) * g.uniform());
  }
  auto* o = new OwnedTensor();
  csf_from_sorted_keys(pk, dims, have, std::move(vals), o);
  *out = &o->t;
  return TT_OK;
}

TT_EXPORT tt_status tt_gen_lognormal_fibers(const int32_t* dims, int64_t nnz, double mu, double sigma,
                                            int64_t n_long, int64_t long_min, uint64_t seed,
                                            taco_tensor_t** out) {
  clear_error();
  if (!out || !dims) return set_error(TT_ERR_INVALID_ARGUMENT, "null argument");
  *out = nullptr;
  const int64_t L = dims[2];
  if (long_min > L) long_min = L;
  // fiber lengths
  std::vector<int64_t> len;
  Rng g(seed, 1);
  int64_t total = 0;
  for (int64_t i = 0; i < n_long && total < nnz; i++) {
    int64_t x = long_min + (int64_t)(g.uniform() * (double)(L - long_min + 1));
    x = std::min(x, std::min(L, nnz - total));
    len.push_back(x);
    total += x;
  }
  while (total < nnz) {
    double v = std::exp(mu + sigma * g.normal());
    int64_t x = (int64_t)std::llround(v);
    x = std::max<int64_t>(1, std::min<int64_t>(x, L));
    x = std::min(x, nnz - total);
    len.push_back(x);
    total += x;
  }
  const int64_t nf = (int64_t)len.size();
  // shuffle the lengths so the long fibers land at random (i,k)
  for (int64_t i = nf - 1; i > 0; i--) std::swap(len[(size_t)i], len[(size_t)(g.next() % (uint64_t)(i + 1))]);
  // distinct (i,k) pairs, sorted
  const uint64_t cells = (uint64_t)dims[0] * (uint64_t)dims[1];
  if ((uint64_t)nf > cells) return set_error(TT_ERR_INVALID_ARGUMENT, "more fibers than (i,k) cells");
  std::vector<uint64_t> ik;
  for (int round = 0; (int64_t)ik.size() < nf && round < 64; round++) {
    const int64_t need = nf - (int64_t)ik.size();
    const int64_t draw = need + need / 8 + 64;
    const int64_t nch = (draw + kChunk - 1) / kChunk;
    std::vector<uint64_t> fresh((size_t)draw);
#pragma omp parallel for schedule(static)
    for (int64_t ch = 0; ch < nch; ch++) {
      Rng h(seed, ((uint64_t)(round + 2) << 40) + (uint64_t)ch);
      for (int64_t p = ch * kChunk; p < std::min(draw, (ch + 1) * kChunk); p++) fresh[(size_t)p] = h.next() % cells;
    }
    fresh.insert(fresh.end(), ik.begin(), ik.end());
    std::vector<uint32_t> dummy(fresh.size(), 0);
    int bits = 1;
    while ((1ull << bits) < cells) bits++;
    radix_sort_pairs(fresh, dummy, bits);
    fresh.erase(std::unique(fresh.begin(), fresh.end()), fresh.end());
    if ((int64_t)fresh.size() > nf) {
      // keep a seeded random subset of exactly nf
      Rng h(seed, 0x1234 + round);
      std::vector<uint64_t> kept;
      kept.reserve((size_t)nf);
      int64_t left = (int64_t)fresh.size(), want = nf;
      for (size_t i = 0; i < fresh.size() && want > 0; i++, left--)
        if (h.uniform() * (double)left < (double)want) { kept.push_back(fresh[i]); want--; }
      fresh.swap(kept);
    }
    ik.swap(fresh);
  }
  if ((int64_t)ik.size() != nf) return set_error(TT_ERR_INVALID_ARGUMENT, "could not draw distinct fibers");
  auto* o = new OwnedTensor();
  o->pos[1].assign((size_t)dims[0] + 1, 0);
  o->crd[1].resize((size_t)nf);
  o->pos[2].resize((size_t)nf + 1);
  for (int64_t f = 0; f < nf; f++) {
    const int64_t i = (int64_t)(ik[(size_t)f] / (uint64_t)dims[1]);
    o->crd[1][(size_t)f] = (int32_t)(ik[(size_t)f] % (uint64_t)dims[1]);
    o->pos[1][(size_t)i + 1]++;
  }
  for (int64_t r = 0; r < dims[0]; r++) o->pos[1][(size_t)r + 1] += o->pos[1][(size_t)r];
  o->pos[2][0] = 0;
  for (int64_t f = 0; f < nf; f++) o->pos[2][(size_t)f + 1] = o->pos[2][(size_t)f] + (int32_t)len[(size_t)f];
  o->crd[2].resize((size_t)nnz);
  o->vals.resize((size_t)nnz);
  // per fiber: distinct sorted l values, values U(0,1)
#pragma omp parallel for schedule(dynamic, 256)
  for (int64_t f = 0; f < nf; f++) {
    Rng h(seed, 0x7000000000ull + (uint64_t)f);
    const int64_t a = o->pos[2][(size_t)f], n = len[(size_t)f];
    int32_t* out_l = o->crd[2].data() + a;
    if (n * 8 >= L) {
      // selection sampling over all of [0, L)
      int64_t want = n, left = L, k = 0;
      for (int64_t l = 0; l < L && want > 0; l++, left--)
        if (h.uniform() * (double)left < (double)want) { out_l[k++] = (int32_t)l; want--; }
    } else {
      std::vector<int32_t> s;
      s.reserve((size_t)n * 2);
      while ((int64_t)s.size() < n) {
        while ((int64_t)s.size() < n + n / 4 + 4) s.push_back((int32_t)(h.next() % (uint64_t)L));
        std::sort(s.begin(), s.end());
        s.erase(std::unique(s.begin(), s.end()), s.end());
      }
      // drop random surplus
      while ((int64_t)s.size() > n) s.erase(s.begin() + (ptrdiff_t)(h.next() % s.size()));
      std::copy(s.begin(), s.end(), out_l);
    }
    float* ov = o->vals.data() + a;
    for (int64_t p = 0; p < n; p++) ov[p] = (float)h.uniform();
  }
  o->pos[0] = {0, dims[0]};
  o->crd[0].resize((size_t)dims[0]);
  std::iota(o->crd[0].begin(), o->crd[0].end(), 0);
  o->publish(3, dims);
  *out = &o->t;
  return TT_OK;
}

TT_EXPORT tt_status tt_gen_dense(int64_t rows, int64_t cols, int32_t dist, uint64_t seed, float* out) {
  clear_error();
  if (!out || rows < 0 || cols <= 0) return set_error(TT_ERR_INVALID_ARGUMENT, "bad dense shape");
  std::vector<double> colscale((size_t)cols, 1.0);
  if (dist == 1) {
    Rng g(seed, 0xc0);
    for (auto& c : colscale) c = std::exp2(-3.0 + 6.0 * g.uniform());
  }
  const int64_t nch = (rows + 4095) / 4096;
#pragma omp parallel for schedule(static)
  for (int64_t ch = 0; ch < nch; ch++) {
    Rng g(seed, 0x100000ull + (uint64_t)ch);
    for (int64_t r = ch * 4096; r < std::min(rows, (ch + 1) * 4096); r++)
      for (int64_t j = 0; j < cols; j++) {
        double v;
        if (dist == 0) v = g.uniform();
        else if (dist == 1) v = g.normal() * colscale[(size_t)j];
        else v = 2.0 * g.uniform() - 1.0;
        out[r * cols + j] = (float)v;
      }
  }
  return TT_OK;
}

TT_EXPORT tt_status tt_csf_features(const taco_tensor_t* B, int32_t rank, float* f) {
  clear_error();
  if (!f) return set_error(TT_ERR_INVALID_ARGUMENT, "null features");
  CsfView v;
  tt_status s = csf_view(B, &v);
  if (s != TT_OK) return s;
  const int L = v.order - 1;          // nnz level
  const int64_t nf = v.count[L - 1];  // last-level fibers
  const int32_t* pos = v.pos[L];
  double mean = nf ? (double)v.nnz / (double)nf : 0.0, m2 = 0, lm = 0, lm2 = 0, lm3 = 0, mx = 0;
#pragma omp parallel for reduction(+ : m2, lm, lm2) reduction(max : mx)
  for (int64_t i = 0; i < nf; i++) {
    const double n = pos[i + 1] - pos[i];
    m2 += (n - mean) * (n - mean);
    const double ln = std::log2(std::max(1.0, n));
    lm += ln;
    lm2 += ln * ln;
    mx = std::max(mx, n);
  }
  double lmean = nf ? lm / (double)nf : 0.0;
#pragma omp parallel for reduction(+ : lm3)
  for (int64_t i = 0; i < nf; i++) {
    const double d = std::log2(std::max(1.0, (double)(pos[i + 1] - pos[i]))) - lmean;
    lm3 += d * d * d;
  }
  const double lvar = nf ? std::max(0.0, lm2 / (double)nf - lmean * lmean) : 0.0;
  const double skew = lvar > 1e-12 ? (lm3 / (double)nf) / std::pow(lvar, 1.5) : 0.0;
  // row nnz CV
  double rm = v.nroot ? (double)v.nnz / (double)v.nroot : 0.0, r2 = 0;
#pragma omp parallel for reduction(+ : r2)
  for (int64_t r = 0; r < v.nroot; r++) {
    int64_t a = v.pos[1][r], b = v.pos[1][r + 1];
    for (int l = 2; l <= L; l++) { a = v.pos[l][a]; b = v.pos[l][b]; }
    const double n = (double)(b - a);
    r2 += (n - rm) * (n - rm);
  }
  auto lg = [](double x) { return (float)std::log2(std::max(1.0, x)); };
  f[0] = lg(v.dims[0]);
  f[1] = lg(v.dims[1]);
  f[2] = v.order > 2 ? lg(v.dims[2]) : 0.f;
  f[3] = lg((double)v.nnz);
  f[4] = lg(rm);
  f[5] = lg(mean);
  f[6] = (float)(mean > 0 && nf ? std::sqrt(m2 / (double)nf) / mean : 0.0);
  f[7] = (float)skew;
  f[8] = (float)(mean > 0 ? std::log2(std::max(1.0, mx / mean)) : 0.0);
  f[9] = (float)(rm > 0 && v.nroot ? std::sqrt(r2 / (double)v.nroot) / rm : 0.0);
  f[10] = (float)v.order;
  f[11] = lg((double)rank);
  return TT_OK;
}
