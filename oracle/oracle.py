"""Test infrastructure only: numpy bindings of the CPU oracle.

Two libraries sit behind this module:

* ``_build/libtt_oracle.so`` -- the FP64 restatement in ``tt_oracle.c`` of the
  reference's CPU TACO kernels (always built by ``make -C oracle``);
* ``_ref/libtaco_ref.so`` -- the reference's own CPU kernels
  (``tensor_kernels/*_cpu_taco.h``) compiled unmodified through ``shim/``; built
  only where the reference sources exist.

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg
import this module.  The product library never does.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from dataclasses import dataclass, field

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_ORACLE_SO = os.path.join(HERE, "_build", "libtt_oracle.so")
_REF_SO = os.path.join(HERE, "_ref", "libtaco_ref.so")

_P = ctypes.c_void_p
_I = ctypes.c_int64


def build(ref: bool = True) -> None:
    """Compile the oracle (and, where the reference sources exist, _ref)."""
    target = "all" if ref else "oracle"
    subprocess.run(["make", "-s", "-C", HERE, target], check=True)


def _ptr(a: np.ndarray | None):
    return None if a is None else a.ctypes.data_as(_P)


_lib = None
_ref = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_ORACLE_SO):
            build(ref=False)
        _lib = ctypes.CDLL(_ORACLE_SO)
        _lib.oracle_compare_array.restype = ctypes.c_double
        _lib.oracle_compare_array_my.restype = ctypes.c_double
        _lib.oracle_build_csf.restype = ctypes.c_int64
        _lib.oracle_now_ms.restype = ctypes.c_double
        _lib.oracle_max_threads.restype = ctypes.c_int
        _lib.oracle_mlp_num_params.restype = ctypes.c_int64
        _lib.oracle_mlp_num_params.argtypes = [ctypes.c_int]
        _lib.oracle_mlp_forward.argtypes = [_P, ctypes.c_int, _P, ctypes.c_int, _P]
        _lib.oracle_mlp_grad.argtypes = [_P, ctypes.c_int, _P, ctypes.c_int, _P, _P, _P, _P]
    return _lib


def ref_lib():
    """The reference's own kernels, or None where they could not be built."""
    global _ref
    if _ref is None:
        if not os.path.exists(_REF_SO):
            try:
                build(ref=True)
            except Exception:
                return None
        if not os.path.exists(_REF_SO):
            return None
        _ref = ctypes.CDLL(_REF_SO)
        _ref.ref_last_kernel_ms.restype = ctypes.c_double
        _ref.ref_flush_cache.restype = ctypes.c_double
    return _ref


@dataclass
class Csf:
    """A CSF tensor with a dense root, as int64 index arrays and float64 values.

    ``pos[l]``/``crd[l]`` for levels l = 1..order-1 (index 0 unused);
    ``pos[1]`` has dims[0]+1 entries.
    """

    order: int
    dims: tuple
    pos: list
    crd: list
    vals: np.ndarray
    extra: dict = field(default_factory=dict)

    @property
    def nnz(self) -> int:
        return int(self.vals.shape[0])

    def nfibers(self, level: int) -> int:
        return int(self.crd[level].shape[0])


def _c64(a):
    return np.ascontiguousarray(a, dtype=np.int64)


def _cf(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def build_csf(dims, coords: np.ndarray, vals: np.ndarray) -> Csf:
    """Canonical CSF: lexicographic coordinate order, duplicates summed, dense root."""
    coords = _c64(coords)
    vals = _cf(vals)
    nnz, order = coords.shape
    pos = [None] * order
    crd = [None] * order
    pos[1] = np.zeros(int(dims[0]) + 1, dtype=np.int64)
    for l in range(1, order):
        crd[l] = np.zeros(max(nnz, 1), dtype=np.int64)
        if l >= 2:
            pos[l] = np.zeros(max(nnz, 1) + 1, dtype=np.int64)
    out_vals = np.zeros(max(nnz, 1), dtype=np.float64)
    counts = np.zeros(order, dtype=np.int64)
    pos_ptrs = (_P * order)(*[None if p is None else p.ctypes.data for p in pos])
    crd_ptrs = (_P * order)(*[None if c is None else c.ctypes.data for c in crd])
    m = lib().oracle_build_csf(ctypes.c_int32(order), _I(int(dims[0])), _I(nnz), _ptr(coords),
                               _ptr(vals), pos_ptrs, crd_ptrs, _ptr(out_vals), _ptr(counts))
    for l in range(1, order):
        crd[l] = crd[l][: counts[l]].copy()
        if l >= 2:
            pos[l] = pos[l][: counts[l - 1] + 1].copy()
    return Csf(order, tuple(int(d) for d in dims), pos, crd, out_vals[:m].copy())


def mttkrp(csf: Csf, factors: list, rows: np.ndarray | None = None) -> np.ndarray:
    """Mode-0 MTTKRP in FP64; factors[m-1] is the mode-m factor (dims[m] x R)."""
    fs = [_cf(f) for f in factors]
    R = fs[0].shape[1]
    L = lib()
    p = [None] + [_c64(x) for x in csf.pos[1:]]
    c = [None] + [_c64(x) for x in csf.crd[1:]]
    v = _cf(csf.vals)
    if rows is not None:
        if csf.order not in (3, 4):
            raise ValueError("row-sampled oracle MTTKRP supports orders 3 and 4")
        rows = _c64(rows)
        out = np.zeros((rows.shape[0], R))
        E = fs[2] if csf.order == 4 else None
        L.oracle_mttkrp_rows(ctypes.c_int32(csf.order), _I(R), _I(rows.shape[0]), _ptr(rows),
                             _ptr(p[1]), _ptr(c[1]), _ptr(p[2]), _ptr(c[2]),
                             _ptr(p[3]) if csf.order == 4 else None,
                             _ptr(c[3]) if csf.order == 4 else None,
                             _ptr(v), _ptr(fs[0]), _ptr(fs[1]), _ptr(E), _ptr(out))
        return out
    A = np.zeros((csf.dims[0], R))
    if csf.order == 3:
        L.oracle_mttkrp3(_I(csf.dims[0]), _I(R), _ptr(p[1]), _ptr(c[1]), _ptr(p[2]), _ptr(c[2]),
                         _ptr(v), _ptr(fs[0]), _ptr(fs[1]), _ptr(A))
    elif csf.order == 4:
        L.oracle_mttkrp4(_I(csf.dims[0]), _I(R), _ptr(p[1]), _ptr(c[1]), _ptr(p[2]), _ptr(c[2]),
                         _ptr(p[3]), _ptr(c[3]), _ptr(v), _ptr(fs[0]), _ptr(fs[1]), _ptr(fs[2]),
                         _ptr(A))
    elif csf.order == 5:
        L.oracle_mttkrp5(_I(csf.dims[0]), _I(R), _ptr(p[1]), _ptr(c[1]), _ptr(p[2]), _ptr(c[2]),
                         _ptr(p[3]), _ptr(c[3]), _ptr(p[4]), _ptr(c[4]), _ptr(v),
                         _ptr(fs[0]), _ptr(fs[1]), _ptr(fs[2]), _ptr(fs[3]), _ptr(A))
    else:
        raise ValueError("oracle MTTKRP supports orders 3, 4 and 5")
    return A


def coords_of(csf: Csf) -> np.ndarray:
    """Every nonzero's coordinates (nnz x order, int64), in CSF order."""
    n = csf.nnz
    out = np.empty((n, csf.order), dtype=np.int64)
    # the leaf level: its own crd; upper levels: expand each fiber's coordinate
    # over the nonzeros below it
    out[:, csf.order - 1] = csf.crd[csf.order - 1]
    span = np.arange(n + 1, dtype=np.int64)  # level-L position p covers nonzeros [p, p+1)
    for l in range(csf.order - 1, 0, -1):
        pos = np.asarray(csf.pos[l], dtype=np.int64)
        starts = span[pos[:-1]]
        ends = span[pos[1:]]
        ids = np.asarray(csf.crd[l - 1], dtype=np.int64) if l >= 2 else np.arange(csf.dims[0], dtype=np.int64)
        out[:, l - 1] = np.repeat(ids, ends - starts)
        span = span[pos]
    return out


def mttkrp_coo(coords: np.ndarray, vals: np.ndarray, factors: list, mode: int, nrows: int) -> np.ndarray:
    """MTTKRP of output mode `mode` in FP64 from coordinates (oracle_mttkrp_coo):
    factors[n] is the mode-n factor (factors[mode] is ignored)."""
    order = coords.shape[1]
    co = np.ascontiguousarray(coords, dtype=np.int64)
    v = _cf(vals)
    R = next(f for n, f in enumerate(factors) if n != mode).shape[1]
    fs = [_cf(f) if (n != mode and f is not None) else np.zeros((1, R)) for n, f in enumerate(factors)]
    arr = (_P * order)(*[f.ctypes.data for f in fs])
    A = np.zeros((nrows, R))
    lib().oracle_mttkrp_coo(ctypes.c_int32(order), _I(co.shape[0]), _ptr(co), _ptr(v), ctypes.c_int32(mode),
                            _I(R), arr, _I(nrows), _ptr(A))
    return A


def coo_ttv(coords: np.ndarray, vals: np.ndarray, c: np.ndarray):
    """COO TTV of the reference's MATLAB interface (oracle_coo_ttv): fibers are runs
    of equal (i, j); returns (fibers x 2 coordinates, y)."""
    co = np.ascontiguousarray(coords, dtype=np.int64)
    n = co.shape[0]
    fib = np.zeros((max(n, 1), 2), dtype=np.int64)
    y = np.zeros(max(n, 1))
    L = lib()
    L.oracle_coo_ttv.restype = ctypes.c_int64
    nf = L.oracle_coo_ttv(_I(n), _ptr(co), _ptr(_cf(vals)), _ptr(_cf(c)), _ptr(fib), _ptr(y))
    return fib[:nf].copy(), y[:nf].copy()


def coo_ttm(coords: np.ndarray, vals: np.ndarray, U: np.ndarray):
    """COO TTM of the reference's MATLAB interface (oracle_coo_ttm): Y(f, r) =
    sum v * U(r, k) over fiber f's nonzeros; U is R x K.  Returns (fibers x 2, Y)."""
    co = np.ascontiguousarray(coords, dtype=np.int64)
    U = _cf(U)
    n = co.shape[0]
    R, K = U.shape
    fib = np.zeros((max(n, 1), 2), dtype=np.int64)
    Y = np.zeros((max(n, 1), R))
    L = lib()
    L.oracle_coo_ttm.restype = ctypes.c_int64
    nf = L.oracle_coo_ttm(_I(n), _ptr(co), _ptr(_cf(vals)), _I(R), _I(K), _ptr(U), _ptr(fib), _ptr(Y))
    return fib[:nf].copy(), Y[:nf].copy()


def mttkrp3_workspace(csf: Csf, C, D) -> np.ndarray:
    C, D = _cf(C), _cf(D)
    R = C.shape[1]
    A = np.zeros((csf.dims[0], R))
    p1, c1, p2, c2 = (_c64(x) for x in (csf.pos[1], csf.crd[1], csf.pos[2], csf.crd[2]))
    lib().oracle_mttkrp3_workspace(_I(csf.dims[0]), _I(R), _ptr(p1), _ptr(c1), _ptr(p2), _ptr(c2),
                                   _ptr(_cf(csf.vals)), _ptr(C), _ptr(D), _ptr(A))
    return A


def ttv(csf: Csf, c: np.ndarray) -> np.ndarray:
    """TTV over the last mode of a 3-mode CSF: one output per level-1 fiber."""
    c = _cf(c)
    y = np.zeros(csf.nfibers(1))
    p1, c1, p2, c2 = (_c64(x) for x in (csf.pos[1], csf.crd[1], csf.pos[2], csf.crd[2]))
    lib().oracle_ttv(_I(csf.dims[0]), _ptr(p1), _ptr(c1), _ptr(p2), _ptr(c2),
                     _ptr(_cf(csf.vals)), _ptr(c), _ptr(y))
    return y


def compare_array(x: np.ndarray, y: np.ndarray) -> float:
    """Reference ds.h compare_array: max |y/x - 1| (inf if x == 0 != y)."""
    x = np.ascontiguousarray(x, dtype=np.float32).ravel()
    y = np.ascontiguousarray(y, dtype=np.float32).ravel()
    return lib().oracle_compare_array(_ptr(x), _ptr(y), _I(x.size))


def compare_array_my(x: np.ndarray, y: np.ndarray) -> float:
    """Reference ds.h compare_array_my: count of |x-y| > 1e-3 (stops after 10)."""
    x = np.ascontiguousarray(x, dtype=np.float32).ravel()
    y = np.ascontiguousarray(y, dtype=np.float32).ravel()
    return lib().oracle_compare_array_my(_ptr(x), _ptr(y), _I(x.size))


def gen_dense(rows: int, cols: int, dist: int, seed: int) -> np.ndarray:
    """The library's seeded dense generator (tt_gen_dense), restated in tt_gen.c."""
    out = np.empty((rows, cols), dtype=np.float32)
    lib().oracle_gen_dense(_I(rows), _I(cols), ctypes.c_int(dist), ctypes.c_uint64(seed), _ptr(out))
    return out


def gen_lognormal(dims, nnz: int, mu: float, sigma: float, n_long: int, long_min: int, seed: int) -> Csf:
    """The library's lognormal-fiber 3-mode tensor (tt_gen_lognormal_fibers), restated
    in tt_gen.c, as an oracle CSF with int64 indices and FP64 values."""
    L = lib()
    d = np.ascontiguousarray(dims, dtype=np.int32)
    args = (_I(nnz), ctypes.c_double(mu), ctypes.c_double(sigma), _I(n_long), _I(long_min), ctypes.c_uint64(seed))
    L.oracle_lognormal_nfibers.restype = ctypes.c_int64
    nf = int(L.oracle_lognormal_nfibers(_ptr(d), *args))
    pos1 = np.empty(int(d[0]) + 1, np.int32)
    crd1 = np.empty(nf, np.int32)
    pos2 = np.empty(nf + 1, np.int32)
    crd2 = np.empty(nnz, np.int32)
    vals = np.empty(nnz, np.float32)
    rc = L.oracle_gen_lognormal(_ptr(d), *args, _ptr(pos1), _ptr(crd1), _ptr(pos2), _ptr(crd2), _ptr(vals))
    if rc != 0:
        raise ValueError("could not draw distinct fibers")
    return Csf(3, tuple(int(x) for x in d), [None, pos1.astype(np.int64), pos2.astype(np.int64)],
               [None, crd1.astype(np.int64), crd2.astype(np.int64)], vals.astype(np.float64))


def now_ms() -> float:
    return lib().oracle_now_ms()


def set_threads(n: int) -> None:
    """Threads the oracle's OpenMP loops use from now on."""
    lib().oracle_set_threads(ctypes.c_int(int(n)))


def max_threads() -> int:
    return lib().oracle_max_threads()


# ---------------------------------------------------------------------------
# The reference's own kernels (where available)
# ---------------------------------------------------------------------------

def ref_mttkrp(csf: Csf, factors: list, workspace: bool = False) -> np.ndarray:
    r = ref_lib()
    if r is None:
        raise RuntimeError("reference kernels unavailable (sources absent)")
    fs = [_cf(f) for f in factors]
    R = fs[0].shape[1]
    A = np.zeros((csf.dims[0], R))
    p = [None] + [_c64(x) for x in csf.pos[1:]]
    c = [None] + [_c64(x) for x in csf.crd[1:]]
    v = _cf(csf.vals)
    if csf.order == 3:
        r.ref_mttkrp3(_I(csf.dims[0]), _I(csf.dims[1]), _I(csf.dims[2]), _I(R),
                      _ptr(p[1]), _ptr(c[1]), _ptr(p[2]), _ptr(c[2]), _ptr(v),
                      _ptr(fs[0]), _ptr(fs[1]), _ptr(A), ctypes.c_int(1 if workspace else 0))
    elif csf.order == 4:
        r.ref_mttkrp4(_I(csf.dims[0]), _I(csf.dims[1]), _I(csf.dims[2]), _I(csf.dims[3]), _I(R),
                      _ptr(p[1]), _ptr(c[1]), _ptr(p[2]), _ptr(c[2]), _ptr(p[3]), _ptr(c[3]),
                      _ptr(v), _ptr(fs[0]), _ptr(fs[1]), _ptr(fs[2]), _ptr(A))
    else:
        dims = _c64(csf.dims)
        parr = (_P * 5)(None, *[x.ctypes.data for x in p[1:]])
        carr = (_P * 5)(None, *[x.ctypes.data for x in c[1:]])
        farr = (_P * 4)(*[f.ctypes.data for f in fs])
        r.ref_mttkrp5(_ptr(dims), _I(R), parr, carr, _ptr(v), farr, _ptr(A))
    return A


def ref_ttv(csf: Csf, c: np.ndarray) -> np.ndarray:
    r = ref_lib()
    if r is None:
        raise RuntimeError("reference kernels unavailable (sources absent)")
    c = _cf(c)
    y = np.zeros(csf.nfibers(1))
    p1, c1, p2, c2 = (_c64(x) for x in (csf.pos[1], csf.crd[1], csf.pos[2], csf.crd[2]))
    r.ref_ttv(_I(csf.dims[0]), _I(csf.dims[1]), _I(csf.dims[2]), _ptr(p1), _ptr(c1), _ptr(p2),
              _ptr(c2), _ptr(_cf(csf.vals)), _ptr(c), _ptr(y))
    return y


# ---------------------------------------------------------------------------
# selector network (FP64): forward and masked-MSE gradient
# ---------------------------------------------------------------------------
def mlp_num_params(nout: int) -> int:
    return int(lib().oracle_mlp_num_params(nout))


def mlp_forward(params: np.ndarray, nout: int, X: np.ndarray) -> np.ndarray:
    p = _cf(params)
    x = _cf(X)
    out = np.zeros((x.shape[0], nout), dtype=np.float64)
    lib().oracle_mlp_forward(_ptr(p), nout, _ptr(x), x.shape[0], _ptr(out))
    return out


def mlp_grad(params: np.ndarray, nout: int, X: np.ndarray, T: np.ndarray, M: np.ndarray):
    """(loss, grads) of sum M (net(X) - T)^2 / sum M."""
    p = _cf(params)
    x, t, m = _cf(X), _cf(T), _cf(M)
    g = np.zeros_like(p)
    loss = np.zeros(1, dtype=np.float64)
    lib().oracle_mlp_grad(_ptr(p), nout, _ptr(x), x.shape[0], _ptr(t), _ptr(m), _ptr(g), _ptr(loss))
    return float(loss[0]), g
