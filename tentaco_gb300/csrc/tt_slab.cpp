// tt_slab.cpp -- split a dense-root CSF into leaf-mode slabs (host side).
//
// The walk kernels gather one leaf-level factor row per nonzero at random.
// When that factor is larger than what stays resident in L2, most gathers go
// to DRAM as 64-byte random reads, which run far below the streaming rate.
// Splitting the leaf mode's index range into S slabs and running one pass per
// slab keeps each pass's factor rows (dims[leaf] / S of them) L2-resident.
//
// Inside a leaf fiber the coordinates are sorted, so the nonzeros of one slab
// are a contiguous run of the fiber: slab s of the tensor is the CSF of those
// runs, with every fiber (and, for order 4, every level-1 fiber) that keeps at
// least one nonzero.  The root stays dense, so every slab has the same rows and
// a pass adds its partial rows into the output.
#include <algorithm>
#include <cstring>
#include <omp.h>
#include "tt_internal.h"

namespace tt {

namespace {
int64_t pad_entries(int64_t n) { return ((n + 15) / 16) * 16 + 16; }
}  // namespace

tt_status build_slabs(const CsfView& v, int S, SlabCsf& out) {
  if (!v.dense_root || (v.order != 3 && v.order != 4) || S < 2 || S > kMaxSlabs)
    return set_error(TT_ERR_UNSUPPORTED, "slabs need a dense-root order-3/4 CSF and 2..%d slabs", kMaxSlabs);
  const int L = v.order - 1;  // leaf level
  const int64_t width = ((int64_t)v.dims[L] + S - 1) / S;
  const int64_t nrows = v.nroot;
  out = SlabCsf();
  out.S = S;
  out.order = v.order;
  out.width = width;
  // run of leaf fiber f inside slab s
  auto run = [&](int64_t f, int s, int64_t& a, int64_t& b) {
    const int32_t* c = v.crd[L];
    const int64_t lo = v.pos[L][f], hi = v.pos[L][f + 1];
    a = std::lower_bound(c + lo, c + hi, (int32_t)std::min<int64_t>(s * width, INT32_MAX)) - c;
    b = std::lower_bound(c + a, c + hi, (int32_t)std::min<int64_t>((s + 1) * width, INT32_MAX)) - c;
  };
  std::vector<int64_t> cnt((size_t)(nrows + 1) * 3);  // per row: level-1, level-2 entries, leaf nonzeros
  int64_t leaf_total = 0;
  for (int s = 0; s < S; s++) {
    // pass 1: what each row keeps
#pragma omp parallel for schedule(dynamic, 256)
    for (int64_t i = 0; i < nrows; i++) {
      int64_t n1 = 0, n2 = 0, nz = 0;
      for (int64_t f1 = v.pos[1][i]; f1 < v.pos[1][i + 1]; f1++) {
        if (L == 2) {
          int64_t a, b;
          run(f1, s, a, b);
          if (b > a) { n1++; nz += b - a; }
        } else {
          int64_t kept = 0;
          for (int64_t f2 = v.pos[2][f1]; f2 < v.pos[2][f1 + 1]; f2++) {
            int64_t a, b;
            run(f2, s, a, b);
            if (b > a) { kept++; nz += b - a; }
          }
          if (kept) { n1++; n2 += kept; }
        }
      }
      cnt[(size_t)i * 3] = n1;
      cnt[(size_t)i * 3 + 1] = n2;
      cnt[(size_t)i * 3 + 2] = nz;
    }
    // exclusive prefix sums (serial: one pass over the rows)
    std::vector<int64_t> o1((size_t)nrows + 1), o2((size_t)nrows + 1), oz((size_t)nrows + 1);
    for (int64_t i = 0; i < nrows; i++) {
      o1[(size_t)i + 1] = o1[(size_t)i] + cnt[(size_t)i * 3];
      o2[(size_t)i + 1] = o2[(size_t)i] + cnt[(size_t)i * 3 + 1];
      oz[(size_t)i + 1] = oz[(size_t)i] + cnt[(size_t)i * 3 + 2];
    }
    SlabCsf::Slab& sl = out.slab[s];
    sl.nnz = oz[(size_t)nrows];
    if (sl.nnz > INT32_MAX) return set_error(TT_ERR_UNSUPPORTED, "slab of %lld nonzeros", (long long)sl.nnz);
    sl.count[0] = nrows;
    sl.count[1] = o1[(size_t)nrows];
    sl.count[2] = L == 2 ? sl.nnz : o2[(size_t)nrows];
    if (L == 3) sl.count[3] = sl.nnz;
    sl.leaf_off = leaf_total;
    sl.pos[1].resize((size_t)nrows + 1);
    sl.crd[1].resize((size_t)sl.count[1]);
    sl.pos[2].resize((size_t)sl.count[1] + 1);
    if (L == 3) {
      sl.crd[2].resize((size_t)sl.count[2]);
      sl.pos[3].resize((size_t)sl.count[2] + 1);
    }
    leaf_total += pad_entries(sl.nnz);
    out.leaf_crd.resize((size_t)leaf_total, 0);
    out.leaf_vals.resize((size_t)leaf_total, 0.f);
    int32_t* lc = out.leaf_crd.data() + sl.leaf_off;
    float* lv = out.leaf_vals.data() + sl.leaf_off;
    // pass 2: fill (row i writes only its own ranges)
#pragma omp parallel for schedule(dynamic, 256)
    for (int64_t i = 0; i < nrows; i++) {
      int64_t k1 = o1[(size_t)i], k2 = o2[(size_t)i], z = oz[(size_t)i];
      sl.pos[1][(size_t)i] = (int32_t)k1;
      for (int64_t f1 = v.pos[1][i]; f1 < v.pos[1][i + 1]; f1++) {
        if (L == 2) {
          int64_t a, b;
          run(f1, s, a, b);
          if (b > a) {
            sl.crd[1][(size_t)k1] = v.crd[1][f1];
            sl.pos[2][(size_t)k1] = (int32_t)z;
            std::memcpy(lc + z, v.crd[2] + a, sizeof(int32_t) * (size_t)(b - a));
            std::memcpy(lv + z, v.vals + a, sizeof(float) * (size_t)(b - a));
            z += b - a;
            k1++;
          }
        } else {
          const int64_t k2start = k2;
          for (int64_t f2 = v.pos[2][f1]; f2 < v.pos[2][f1 + 1]; f2++) {
            int64_t a, b;
            run(f2, s, a, b);
            if (b > a) {
              sl.crd[2][(size_t)k2] = v.crd[2][f2];
              sl.pos[3][(size_t)k2] = (int32_t)z;
              std::memcpy(lc + z, v.crd[3] + a, sizeof(int32_t) * (size_t)(b - a));
              std::memcpy(lv + z, v.vals + a, sizeof(float) * (size_t)(b - a));
              z += b - a;
              k2++;
            }
          }
          if (k2 > k2start) {
            sl.crd[1][(size_t)k1] = v.crd[1][f1];
            sl.pos[2][(size_t)k1] = (int32_t)k2start;
            k1++;
          }
        }
      }
    }
    sl.pos[1][(size_t)nrows] = (int32_t)sl.count[1];
    sl.pos[2][(size_t)sl.count[1]] = (int32_t)(L == 2 ? sl.nnz : sl.count[2]);
    if (L == 3) sl.pos[3][(size_t)sl.count[2]] = (int32_t)sl.nnz;
  }
  return TT_OK;
}

}  // namespace tt
