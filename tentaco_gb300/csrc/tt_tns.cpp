// tt_tns.cpp -- FROSTT .tns reader (host side).
//
// The reference loads tensors with SPLATT's splatt_csf_load (ds.h:351-366) from
// FROSTT .tns files: one nonzero per line, `order` 1-based integer coordinates
// followed by the value, whitespace separated; lines starting with '#' are
// comments.  SPLATT is not a dependency of this library, so this reader produces the
// same coordinates and values and hands them to the canonical CSF builder
// (tt_csf_from_coo: modes in file order, lexicographic, duplicates summed).
//
// The file is read whole and parsed in parallel: it is cut into one chunk per
// thread at line boundaries, every chunk is parsed into its own arrays, and
// the chunks are concatenated in file order, so the result does not depend on
// the thread count.
#include <omp.h>
#include <algorithm>
#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>
#include "tt_internal.h"
#include "../../include/tentaco/tentaco_gen.h"

namespace tt {
namespace {

inline bool is_space(char c) { return c == ' ' || c == '\t' || c == '\r' || c == '\v' || c == '\f'; }

struct Chunk {
  std::vector<int64_t> coords;  // order per nonzero, 1-based as read
  std::vector<float> vals;
  int64_t bad_line = -1;        // byte offset of the first malformed line
  int order = 0;                // entries per line seen first (0: none yet)
};

// Parse [b, e) (whole lines).  order_req > 0 fixes the number of coordinates.
void parse_chunk(const char* b, const char* e, int order_req, Chunk& out, const char* base) {
  const char* p = b;
  std::vector<double> tok;
  while (p < e) {
    const char* line = p;
    const char* nl = static_cast<const char*>(std::memchr(p, '\n', (size_t)(e - p)));
    const char* le = nl ? nl : e;
    p = nl ? nl + 1 : e;
    const char* q = line;
    while (q < le && is_space(*q)) q++;
    if (q == le || *q == '#' || *q == '%') continue;  // blank or comment
    tok.clear();
    bool ok = true;
    while (q < le) {
      char* end = nullptr;
      errno = 0;
      const double v = std::strtod(q, &end);
      if (end == q || end > le || errno == ERANGE) { ok = false; break; }
      tok.push_back(v);
      q = end;
      while (q < le && is_space(*q)) q++;
    }
    const int ord = (int)tok.size() - 1;
    if (ok) {
      if (out.order == 0) out.order = order_req > 0 ? order_req : ord;
      ok = ord == out.order && ord >= 1 && ord <= TT_MAX_ORDER;
    }
    for (int m = 0; ok && m < ord; m++) {
      const double c = tok[(size_t)m];
      ok = c >= 1.0 && c <= 2147483647.0 && c == std::floor(c);
    }
    if (!ok) {
      if (out.bad_line < 0) out.bad_line = (int64_t)(line - base);
      continue;
    }
    for (int m = 0; m < ord; m++) out.coords.push_back((int64_t)tok[(size_t)m]);
    out.vals.push_back((float)tok[(size_t)ord]);
  }
}

}  // namespace
}  // namespace tt

using namespace tt;

TT_EXPORT tt_status tt_read_tns(const char* path, int32_t order, taco_tensor_t** out) {
  clear_error();
  if (!path || !out) return set_error(TT_ERR_INVALID_ARGUMENT, "null argument");
  *out = nullptr;
  if (order < 0 || order > TT_MAX_ORDER) return set_error(TT_ERR_INVALID_ARGUMENT, "order %d", order);
  FILE* f = std::fopen(path, "rb");
  if (!f) return set_error(TT_ERR_INVALID_ARGUMENT, "cannot open %s", path);
  std::fseek(f, 0, SEEK_END);
  const long sz = std::ftell(f);
  std::fseek(f, 0, SEEK_SET);
  std::vector<char> buf(sz > 0 ? (size_t)sz : 0);
  const bool read_ok = sz <= 0 || std::fread(buf.data(), 1, (size_t)sz, f) == (size_t)sz;
  std::fclose(f);
  if (!read_ok) return set_error(TT_ERR_INVALID_ARGUMENT, "cannot read %s", path);
  const char* base = buf.data();
  const char* end = base + buf.size();
  // chunk boundaries at line starts
  const int nt = std::max(1, std::min(omp_get_max_threads(), (int)(buf.size() / (1 << 20)) + 1));
  std::vector<const char*> cut((size_t)nt + 1);
  cut[0] = base;
  cut[(size_t)nt] = end;
  for (int t = 1; t < nt; t++) {
    const char* c = base + (buf.size() * (size_t)t) / (size_t)nt;
    c = std::max(c, cut[(size_t)t - 1]);
    const char* nl = c < end ? static_cast<const char*>(std::memchr(c, '\n', (size_t)(end - c))) : nullptr;
    cut[(size_t)t] = nl ? nl + 1 : end;
  }
  std::vector<Chunk> ch((size_t)nt);
#pragma omp parallel for schedule(static, 1) num_threads(nt)
  for (int t = 0; t < nt; t++) parse_chunk(cut[(size_t)t], cut[(size_t)t + 1], order, ch[(size_t)t], base);
  int ord = order;
  int64_t bad = -1, nnz = 0;
  for (size_t t = 0; t < ch.size(); t++) {
    const Chunk& c = ch[t];
    if (c.bad_line >= 0 && bad < 0) bad = c.bad_line;
    if (c.order > 0) {
      if (ord == 0) ord = c.order;
      else if (c.order != ord && bad < 0) bad = (int64_t)(cut[t] - base);
    }
    nnz += (int64_t)c.vals.size();
  }
  if (bad >= 0) {
    // report the line number of the first malformed line
    const int64_t line = 1 + std::count(base, base + bad, '\n');
    return set_error(TT_ERR_INVALID_ARGUMENT, "%s:%lld: expected %d positive integer coordinates and a value",
                     path, (long long)line, ord);
  }
  if (ord == 0) return set_error(TT_ERR_INVALID_ARGUMENT, "%s: no nonzeros and no order given", path);
  // 0-based coordinates in file order; dims = largest coordinate per mode
  std::vector<int32_t> coords((size_t)nnz * (size_t)ord);
  std::vector<float> vals((size_t)nnz);
  std::vector<int64_t> off(ch.size() + 1, 0);
  for (size_t t = 0; t < ch.size(); t++) off[t + 1] = off[t] + (int64_t)ch[t].vals.size();
  int32_t dims[TT_MAX_ORDER] = {1, 1, 1, 1};
  std::vector<int32_t> dmax(ch.size() * TT_MAX_ORDER, 0);
#pragma omp parallel for schedule(static, 1) num_threads(nt)
  for (int t = 0; t < nt; t++) {
    const Chunk& c = ch[(size_t)t];
    const int64_t n = (int64_t)c.vals.size();
    for (int64_t i = 0; i < n; i++) {
      for (int m = 0; m < ord; m++) {
        const int32_t x = (int32_t)(c.coords[(size_t)(i * ord + m)] - 1);
        coords[(size_t)((off[(size_t)t] + i) * ord + m)] = x;
        dmax[(size_t)t * TT_MAX_ORDER + m] = std::max(dmax[(size_t)t * TT_MAX_ORDER + m], x + 1);
      }
      vals[(size_t)(off[(size_t)t] + i)] = c.vals[(size_t)i];
    }
  }
  for (size_t t = 0; t < ch.size(); t++)
    for (int m = 0; m < ord; m++) dims[m] = std::max(dims[m], dmax[t * TT_MAX_ORDER + m]);
  return tt_csf_from_coo(ord, dims, nnz, coords.data(), vals.data(), out);
}
