"""tentaco_gb300 -- Python bindings of libtentaco_gb300 (sparse MTTKRP / TTV on GB300).

The library is C/C++/CUDA; this module only wraps its C ABI
(``include/tentaco/tentaco.h``, ``gpu_kernels.cuh``, ``tentaco_gen.h``) with
ctypes and numpy.  It never computes anything itself: if the compiled library
is missing, importing the binding raises instead of falling back to another
implementation.  Build it with ``python -m tentaco_gb300.build``.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "libtentaco_gb300.so")

TT_OK = 0
TT_ERR_INVALID_ARGUMENT = 1
TT_ERR_INVALID_CSF = 2
TT_ERR_UNSUPPORTED = 3
TT_ERR_CUDA = 4
TT_ERR_OUT_OF_MEMORY = 5
TT_ERR_NO_DEVICE = 6
TT_ERR_DEVICE_WAIT = 7

OP_MTTKRP, OP_TTV, OP_TTM = 0, 1, 2
PREC_FP32, PREC_BF16, PREC_BF16_FACTORS, PREC_FP16, PREC_FX16 = 0, 1, 2, 3, 4
SELECT_DEFAULT, SELECT_MODEL, SELECT_SWEEP, SELECT_FIXED = 0, 1, 2, 3
PRECISIONS = {"fp32": PREC_FP32, "bf16": PREC_BF16, "bf16f": PREC_BF16_FACTORS, "fp16": PREC_FP16, "fx16": PREC_FX16}


class TacoTensor(C.Structure):
    """Same layout as taco_tensor_t (taco_tensor_t.h:6-15 of the reference)."""

    _fields_ = [
        ("order", C.c_int32),
        ("dimensions", C.POINTER(C.c_int32)),
        ("csize", C.c_int32),
        ("mode_ordering", C.POINTER(C.c_int32)),
        ("mode_types", C.POINTER(C.c_int)),
        ("indices", C.POINTER(C.POINTER(C.POINTER(C.c_int32)))),
        ("vals", C.POINTER(C.c_float)),
        ("vals_size", C.c_int32),
    ]


class VariantInfo(C.Structure):
    _fields_ = [(n, C.c_int32) for n in ("id", "threads", "cols_per_lane", "nnz_per_team", "rank_pad",
                                         "lanes_per_row", "nnz_per_block", "staged")] + [("name", C.c_char * 40)]


class TTError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(msg)
        self.status = status


_lib = None
_P = C.c_void_p
_TP = C.POINTER(TacoTensor)


def lib():
    """The loaded C library (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError(f"{LIB_PATH} is not built; run `python -m tentaco_gb300.build`")
    L = C.CDLL(LIB_PATH)
    S = C.c_int
    sig = {
        "tt_abi_version": (C.c_int32, []),
        "tt_last_error_string": (C.c_char_p, []),
        "tt_status_string": (C.c_char_p, [S]),
        "tt_num_variants": (C.c_int32, []),
        "tt_variant_get": (S, [C.c_int32, C.POINTER(VariantInfo)]),
        "tt_variant_default": (C.c_int32, [C.c_int32, C.c_int32, S, C.c_int64]),
        "tt_variant_valid": (C.c_int32, [C.c_int32, C.c_int32, C.c_int32, S]),
        "tt_plan_create": (S, [_TP, S, C.c_int32, S, S, C.c_int32, _P, C.POINTER(_P)]),
        "tt_plan_create_ex": (S, [_TP, S, C.c_int32, S, S, C.c_int32, _P, _P, C.POINTER(_P)]),
        "tt_plan_slabs": (C.c_int32, [_P]),
        "tt_plan_destroy": (S, [_P]),
        "tt_plan_set_factors": (S, [_P, C.POINTER(_P), _P]),
        "tt_plan_mttkrp": (S, [_P, _P, _P]),
        "tt_plan_ttv": (S, [_P, _P, _P, _P]),
        "tt_plan_ttm": (S, [_P, _P, _P]),
        "tt_plan_coo_fibers": (S, [_P, _P]),
        "tt_plan_create_coo": (S, [C.c_int32, _P, C.c_int64, _P, _P, S, C.c_int32, S, S, C.c_int32, _P,
                                   C.POINTER(_P)]),
        "tt_plan_set_timing": (S, [_P, C.c_int32]),
        "tt_plan_last_ms": (C.c_float, [_P]),
        "tt_plan_last_kernel_ms": (C.c_float, [_P]),
        "tt_plan_partition_ms": (C.c_float, [_P]),
        "tt_plan_variant": (C.c_int32, [_P]),
        "tt_plan_selected_by": (C.c_int32, [_P]),
        "tt_plan_nnz": (C.c_int64, [_P]),
        "tt_plan_num_fibers": (C.c_int64, [_P, C.c_int32]),
        "tt_plan_device_bytes": (C.c_int64, [_P]),
        "tt_plan_nblocks": (C.c_int32, [_P]),
        "tt_plan_device_error": (C.c_int32, [_P]),
        "tt_plan_use_variant": (S, [_P, C.c_int32]),
        "tt_plan_sweep_times": (S, [_P, C.POINTER(C.c_float), C.c_int32]),
        "tt_debug_tma_wait": (S, [C.c_int32, C.c_int64]),
        "tt_debug_fail_pool_alloc": (S, [C.c_int64]),
        "tt_debug_pool_live": (C.c_int64, []),
        "tt_mttkrp_host": (S, [_TP, _TP, C.POINTER(_TP), S, S, C.c_int32]),
        "tt_ttv_host": (S, [_TP, _TP, _TP]),
        "tt_csf_from_coo": (S, [C.c_int32, C.POINTER(C.c_int32), C.c_int64, _P, _P, C.POINTER(_TP)]),
        "tt_csf_reroot": (S, [_TP, C.c_int32, C.POINTER(_TP)]),
        "tt_csf_from_coo_gpu": (S, [C.c_int32, C.POINTER(C.c_int32), C.c_int64, _P, _P, C.POINTER(_TP)]),
        "tt_csf_validate": (S, [_TP]),
        "tt_tensor_free": (None, [_TP]),
        "tt_gen_zipf": (S, [C.c_int32, C.POINTER(C.c_int32), C.POINTER(C.c_double), C.c_int64, C.c_float,
                            C.c_float, C.c_uint64, C.c_int32, C.POINTER(_TP)]),
        "tt_gen_lognormal_fibers": (S, [C.POINTER(C.c_int32), C.c_int64, C.c_double, C.c_double, C.c_int64,
                                        C.c_int64, C.c_uint64, C.POINTER(_TP)]),
        "tt_gen_dense": (S, [C.c_int64, C.c_int64, C.c_int32, C.c_uint64, _P]),
        "tt_csf_features": (S, [_TP, C.c_int32, C.POINTER(C.c_float)]),
        "tt_read_tns": (S, [C.c_char_p, C.c_int32, C.POINTER(_TP)]),
        "tt_device_malloc": (S, [C.c_int64, C.POINTER(_P)]),
        "tt_device_free": (S, [_P]),
        "tt_host_register": (S, [_P, C.c_int64]),
        "tt_host_unregister": (S, [_P]),
        "tt_memcpy_htod": (S, [_P, _P, C.c_int64]),
        "tt_memcpy_dtoh": (S, [_P, _P, C.c_int64]),
        "tt_device_synchronize": (S, []),
        "tt_device_count": (C.c_int32, []),
        "tt_l2_flush": (S, [_P]),
        "get_gpu_timer_result": (C.c_float, []),
        "tt_mlp_num_params": (C.c_int64, [C.c_int32]),
        "tt_mlp_scratch_floats": (C.c_int64, [C.c_int32, C.c_int32]),
        "tt_mlp_forward": (S, [_P, C.c_int32, _P, C.c_int32, _P, _P, _P]),
        "tt_mlp_grad": (S, [_P, C.c_int32, _P, C.c_int32, _P, _P, _P, _P, _P, _P]),
        "tt_mlp_adam": (S, [_P, _P, _P, _P, C.c_int64, C.c_float, C.c_float, C.c_float, C.c_float, C.c_float,
                            C.c_int32, _P]),
        "tt_selector_load": (S, [C.c_char_p]),
        "tt_release_cached_memory": (S, []),
        "tt_selector_models": (C.c_int32, []),
        "tt_selector_models_for_order": (C.c_int32, [C.c_int32]),
        "tt_selector_scores": (S, [_TP, C.c_int32, S, C.POINTER(C.c_float), C.c_int32]),
        "ttv_csf_gpu_taco": (None, [_TP, _TP, _TP]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def check(status: int) -> None:
    if status != TT_OK:
        raise TTError(status, lib().tt_last_error_string().decode())


def legacy_entry(name: str):
    """A reference-named entry point (e.g. 'mttkrp_32_eb_sr_512_4_1') from the library."""
    f = getattr(lib(), name)
    f.restype = None
    f.argtypes = [_TP, _TP, _TP, _TP]
    return f


def legacy_names() -> list:
    path = os.path.join(os.path.dirname(PKG), "include", "tentaco", "tt_legacy_names.def")
    out = []
    with open(path) as fh:
        for line in fh:
            if line.startswith("X("):
                out.append(line[2:].split(",")[0].strip())
    return out


# ---------------------------------------------------------------------------
# tensors
# ---------------------------------------------------------------------------

def _i32p(a):
    return a.ctypes.data_as(C.POINTER(C.c_int32))


class Tensor:
    """A CSF tensor owned by the library (from a generator or tt_csf_from_coo)."""

    def __init__(self, ptr):
        self.ptr = ptr
        t = ptr.contents
        self.order = int(t.order)
        self.dims = tuple(int(t.dimensions[i]) for i in range(self.order))

    def __del__(self):
        if getattr(self, "ptr", None) and _lib is not None:
            _lib.tt_tensor_free(self.ptr)
            self.ptr = None

    def count(self, level: int) -> int:
        if level == 0:
            return self.dims[0]
        return int(self.pos(level)[-1])

    @property
    def nnz(self) -> int:
        return self.count(self.order - 1)

    def pos(self, level: int) -> np.ndarray:
        n = (self.dims[0] if level == 1 else self.count(level - 1)) + 1
        if level == 0:
            n = 2
        p = self.ptr.contents.indices[level][0]
        return np.ctypeslib.as_array(p, shape=(n,))

    def crd(self, level: int) -> np.ndarray:
        n = self.dims[0] if level == 0 else self.count(level)
        if n == 0:
            return np.zeros(0, dtype=np.int32)
        return np.ctypeslib.as_array(self.ptr.contents.indices[level][1], shape=(n,))

    @property
    def vals(self) -> np.ndarray:
        n = self.nnz
        if n == 0:
            return np.zeros(0, dtype=np.float32)
        return np.ctypeslib.as_array(self.ptr.contents.vals, shape=(n,))

    def host_arrays(self) -> list:
        """The tensor's host arrays (every level's pos and crd, and the values)."""
        out = [self.pos(l) for l in range(1, self.order)] + [self.crd(l) for l in range(1, self.order)]
        return [a for a in out + [self.vals] if a.size]

    def features(self, rank: int) -> np.ndarray:
        f = np.zeros(12, dtype=np.float32)
        check(lib().tt_csf_features(self.ptr, rank, f.ctypes.data_as(C.POINTER(C.c_float))))
        return f


def csf_from_coo_gpu(dims, coords: np.ndarray, vals: np.ndarray) -> "Tensor":
    """csf_from_coo built on the GPU (bit-identical result)."""
    coords = np.ascontiguousarray(coords, dtype=np.int32)
    vals = np.ascontiguousarray(vals, dtype=np.float32)
    d = np.ascontiguousarray(dims, dtype=np.int32)
    out = _TP()
    check(lib().tt_csf_from_coo_gpu(len(d), _i32p(d), coords.shape[0], coords.ctypes.data, vals.ctypes.data,
                                    C.byref(out)))
    return Tensor(out)


def csf_reroot(B, mode: int) -> "Tensor":
    """B as the canonical CSF rooted at `mode` (other modes after it in increasing order)."""
    out = _TP()
    check(lib().tt_csf_reroot(_tensor_ptr(B), int(mode), C.byref(out)))
    return Tensor(out)


def csf_from_coo(dims, coords: np.ndarray, vals: np.ndarray) -> Tensor:
    coords = np.ascontiguousarray(coords, dtype=np.int32)
    vals = np.ascontiguousarray(vals, dtype=np.float32)
    d = np.ascontiguousarray(dims, dtype=np.int32)
    out = _TP()
    check(lib().tt_csf_from_coo(len(d), _i32p(d), coords.shape[0], coords.ctypes.data, vals.ctypes.data,
                                C.byref(out)))
    return Tensor(out)


def gen_zipf(dims, zipf_s, nnz: int, seed: int, vlo=0.0, vhi=1.0, max_rounds=8) -> Tensor:
    d = np.ascontiguousarray(dims, dtype=np.int32)
    s = np.ascontiguousarray(zipf_s, dtype=np.float64)
    out = _TP()
    check(lib().tt_gen_zipf(len(d), _i32p(d), s.ctypes.data_as(C.POINTER(C.c_double)), nnz, vlo, vhi, seed,
                            max_rounds, C.byref(out)))
    return Tensor(out)


def read_tns(path, order: int = 0) -> Tensor:
    """A FROSTT .tns file (1-based coordinates and a value per line) as a canonical CSF."""
    out = _TP()
    check(lib().tt_read_tns(os.fsencode(path), order, C.byref(out)))
    return Tensor(out)


def gen_lognormal_fibers(dims, nnz: int, mu: float, sigma: float, n_long: int, long_min: int,
                         seed: int) -> Tensor:
    d = np.ascontiguousarray(dims, dtype=np.int32)
    out = _TP()
    check(lib().tt_gen_lognormal_fibers(_i32p(d), nnz, mu, sigma, n_long, long_min, seed, C.byref(out)))
    return Tensor(out)


def gen_dense(rows: int, cols: int, dist: int, seed: int) -> np.ndarray:
    out = np.empty((rows, cols), dtype=np.float32)
    check(lib().tt_gen_dense(rows, cols, dist, seed, out.ctypes.data))
    return out


class HostTaco:
    """A taco_tensor_t over numpy arrays (dense matrices/vectors or a CSF given as arrays)."""

    def __init__(self, dims, vals=None, levels=None, dense_root=True, order=None):
        self._keep = []
        self.dims = np.ascontiguousarray(dims, dtype=np.int32)
        self.t = TacoTensor()
        self.t.order = int(order if order is not None else len(self.dims))
        self.t.dimensions = _i32p(self.dims)
        self._keep.append(self.dims)
        self.t.csize = 4
        if levels is not None:
            n = len(levels)
            arr = (C.POINTER(C.POINTER(C.c_int32)) * n)()
            for l, lv in enumerate(levels):
                pair = (C.POINTER(C.c_int32) * 2)()
                if lv is not None:
                    p, c = (np.ascontiguousarray(x, dtype=np.int32) for x in lv)
                    self._keep += [p, c]
                    pair[0] = _i32p(p)
                    pair[1] = _i32p(c)
                self._keep.append(pair)
                arr[l] = C.cast(pair, C.POINTER(C.POINTER(C.c_int32)))
            self._keep.append(arr)
            self.t.indices = C.cast(arr, C.POINTER(C.POINTER(C.POINTER(C.c_int32))))
            mt = np.array([0 if dense_root else 1] + [1] * (n - 1), dtype=np.int32)
            self._keep.append(mt)
            self.t.mode_types = mt.ctypes.data_as(C.POINTER(C.c_int))
        if vals is not None:
            self.vals = np.ascontiguousarray(vals, dtype=np.float32)
            self._keep.append(self.vals)
            self.t.vals = self.vals.ctypes.data_as(C.POINTER(C.c_float))
            self.t.vals_size = int(self.vals.size)

    @property
    def ptr(self):
        return C.pointer(self.t)


def dense(mat: np.ndarray) -> HostTaco:
    mat = np.ascontiguousarray(mat, dtype=np.float32)
    dims = mat.shape if mat.ndim == 2 else (mat.shape[0],)
    return HostTaco(dims, vals=mat)


def _tensor_ptr(B):
    return B.ptr


def pin(arrays) -> None:
    """Page-lock host arrays (tt_host_register): copies from and to them become DMA."""
    for a in arrays:
        if a.size:
            check(lib().tt_host_register(a.ctypes.data, a.nbytes))


def unpin(arrays) -> None:
    for a in arrays:
        if a.size:
            check(lib().tt_host_unregister(a.ctypes.data))


def mttkrp_host(B, factors, prec="fp32", select=SELECT_DEFAULT, variant=0, out=None) -> np.ndarray:
    """One-shot MTTKRP through tt_mttkrp_host: host in, host out (into `out`, a
    C-contiguous FP32 dims[0] x R array, when given)."""
    R = factors[0].shape[1]
    if out is not None:
        assert out.dtype == np.float32 and out.shape == (B.dims[0], R) and out.flags.c_contiguous
        A = out
    else:
        A = np.zeros((B.dims[0], R), dtype=np.float32)
    Ah = dense(A)
    Fh = [dense(f) for f in factors]
    arr = (_TP * len(Fh))(*[f.ptr for f in Fh])
    check(lib().tt_mttkrp_host(Ah.ptr, _tensor_ptr(B), arr, PRECISIONS.get(prec, prec), select, variant))
    return Ah.vals.reshape(A.shape)


def ttv_host(B, x: np.ndarray, nfib: int) -> np.ndarray:
    y = dense(np.zeros(nfib, dtype=np.float32))
    xh = dense(np.ascontiguousarray(x, dtype=np.float32))
    check(lib().tt_ttv_host(y.ptr, _tensor_ptr(B), xh.ptr))
    return y.vals


def gpu_timer_ms() -> float:
    return float(lib().get_gpu_timer_result())


# ---------------------------------------------------------------------------
# device buffers and plans
# ---------------------------------------------------------------------------

class DeviceBuffer:
    def __init__(self, nbytes: int):
        self.nbytes = int(nbytes)
        self.ptr = _P()
        check(lib().tt_device_malloc(self.nbytes, C.byref(self.ptr)))

    @classmethod
    def from_array(cls, a: np.ndarray) -> "DeviceBuffer":
        a = np.ascontiguousarray(a)
        b = cls(a.nbytes)
        check(lib().tt_memcpy_htod(b.ptr, a.ctypes.data, a.nbytes))
        return b

    def to_array(self, shape, dtype=np.float32) -> np.ndarray:
        out = np.empty(shape, dtype=dtype)
        check(lib().tt_memcpy_dtoh(out.ctypes.data, self.ptr, out.nbytes))
        return out

    def upload(self, a: np.ndarray) -> None:
        a = np.ascontiguousarray(a)
        check(lib().tt_memcpy_htod(self.ptr, a.ctypes.data, a.nbytes))

    def __del__(self):
        if getattr(self, "ptr", None) and self.ptr.value and _lib is not None:
            _lib.tt_device_free(self.ptr)
            self.ptr = _P()


class PlanOptions(C.Structure):
    _fields_ = [("slabs", C.c_int32), ("l2_policy", C.c_int32), ("model_topk", C.c_int32),
                ("mode", C.c_int32), ("reserved", C.c_int32 * 4)]


class Plan:
    """slabs: leaf-mode slabs for MTTKRP (None/0 automatic, 1 none, up to 16).
    model_topk: with SELECT_MODEL, how many of the network's best-ranked variants
    to time at creation (0 automatic: 1 inside the training range, else 6).
    mode: MTTKRP output mode; for mode m > 0 the plan re-roots the tensor at m and
    set_factors takes the other modes' factors in increasing mode order."""

    def __init__(self, B, op=OP_MTTKRP, rank=32, prec="fp32", select=SELECT_DEFAULT, variant=0, stream=None,
                 slabs=None, l2_policy=0, model_topk=0, mode=0):
        self.ptr = _P()
        self.op = op
        self.rank = rank
        self.dims = B.dims
        opts = PlanOptions()
        opts.slabs = int(slabs or 0)
        opts.l2_policy = int(l2_policy)
        opts.model_topk = int(model_topk)
        opts.mode = int(mode)
        self.mode = int(mode)
        check(lib().tt_plan_create_ex(_tensor_ptr(B), op, rank, PRECISIONS.get(prec, prec), select, variant,
                                      C.byref(opts), stream, C.byref(self.ptr)))

    @classmethod
    def from_coo(cls, dims, coords, vals, op=OP_MTTKRP, rank=32, prec="fp32", select=SELECT_DEFAULT, variant=0,
                 stream=None):
        """A plan over sorted COO input (tt_plan_create_coo): coords nnz x order int32
        (lexicographically sorted), vals FP32.  MTTKRP (orders 3..5), TTV or TTM
        (order 3; fibers are runs of equal (i, j))."""
        self = cls.__new__(cls)
        self.ptr = _P()
        self.op = op
        self.rank = rank
        self.dims = tuple(int(x) for x in dims)
        self.mode = 0
        d = np.ascontiguousarray(dims, dtype=np.int32)
        co = np.ascontiguousarray(coords, dtype=np.int32)
        v = np.ascontiguousarray(vals, dtype=np.float32)
        self._keep = (d, co, v)
        check(lib().tt_plan_create_coo(len(d), d.ctypes.data, co.shape[0], co.ctypes.data, v.ctypes.data, op, rank,
                                       PRECISIONS.get(prec, prec), select, variant, stream, C.byref(self.ptr)))
        return self

    def ttm(self, Y: "DeviceBuffer", stream=None) -> None:
        check(lib().tt_plan_ttm(self.ptr, Y.ptr, stream))

    def coo_fibers(self) -> np.ndarray:
        """(i, j) of every fiber of a COO TTV or TTM plan (nfibers x 2)."""
        n = self.num_fibers(1 if self.op == OP_TTV else 0)
        out = np.empty((max(n, 0), 2), dtype=np.int32)
        if n > 0:
            check(lib().tt_plan_coo_fibers(self.ptr, out.ctypes.data))
        return out

    @property
    def slabs(self) -> int:
        return int(lib().tt_plan_slabs(self.ptr))

    def __del__(self):
        if getattr(self, "ptr", None) and self.ptr.value and _lib is not None:
            _lib.tt_plan_destroy(self.ptr)
            self.ptr = _P()

    def set_factors(self, bufs) -> None:
        arr = (_P * len(bufs))(*[b.ptr.value for b in bufs])
        check(lib().tt_plan_set_factors(self.ptr, arr, None))
        # FP32 plans of rank 8/16/32/64 read the caller's buffers at every call
        self._factors = list(bufs)

    def mttkrp(self, A: DeviceBuffer, stream=None) -> None:
        check(lib().tt_plan_mttkrp(self.ptr, A.ptr, stream))

    def ttv(self, x: DeviceBuffer, y: DeviceBuffer, stream=None) -> None:
        check(lib().tt_plan_ttv(self.ptr, x.ptr, y.ptr, stream))

    def set_timing(self, on) -> None:
        """False/0: off; True/1: the call and its walk kernels; 2: the call only (no event between the
        walk and the merge kernels, which would hold back their dependent launch)."""
        check(lib().tt_plan_set_timing(self.ptr, int(on)))

    def last_ms(self) -> float:
        return float(lib().tt_plan_last_ms(self.ptr))

    def last_kernel_ms(self) -> float:
        return float(lib().tt_plan_last_kernel_ms(self.ptr))

    def partition_ms(self) -> float:
        return float(lib().tt_plan_partition_ms(self.ptr))

    @property
    def variant(self) -> int:
        return int(lib().tt_plan_variant(self.ptr))

    @property
    def selected_by(self) -> int:
        return int(lib().tt_plan_selected_by(self.ptr))

    def device_error(self) -> int:
        return int(lib().tt_plan_device_error(self.ptr))

    @property
    def nblocks(self) -> int:
        return int(lib().tt_plan_nblocks(self.ptr))

    def num_fibers(self, level: int) -> int:
        return int(lib().tt_plan_num_fibers(self.ptr, level))

    def device_bytes(self) -> int:
        return int(lib().tt_plan_device_bytes(self.ptr))

    def use_variant(self, vid: int) -> None:
        check(lib().tt_plan_use_variant(self.ptr, vid))

    def sweep_times(self) -> np.ndarray:
        n = num_variants()
        out = np.zeros(n, dtype=np.float32)
        check(lib().tt_plan_sweep_times(self.ptr, out.ctypes.data_as(C.POINTER(C.c_float)), n))
        return out


def num_variants() -> int:
    return int(lib().tt_num_variants())


def variant_info(vid: int) -> dict:
    v = VariantInfo()
    check(lib().tt_variant_get(vid, C.byref(v)))
    return {f: getattr(v, f) for f, _ in VariantInfo._fields_ if f != "name"} | {"name": v.name.decode()}


def variant_valid(vid: int, order: int, rank: int, prec="fp32") -> bool:
    return bool(lib().tt_variant_valid(vid, order, rank, PRECISIONS.get(prec, prec)))


def default_variant(order: int, rank: int, prec="fp32", nnz: int = 0) -> int:
    return int(lib().tt_variant_default(order, rank, PRECISIONS.get(prec, prec), nnz))


def device_count() -> int:
    return int(lib().tt_device_count())


def synchronize() -> None:
    check(lib().tt_device_synchronize())


def l2_flush(stream=None) -> None:
    check(lib().tt_l2_flush(stream))


# ---------------------------------------------------------------------------
# learned selector: the network's kernels and the model file
# ---------------------------------------------------------------------------
def mlp_num_params(nout: int) -> int:
    return int(lib().tt_mlp_num_params(nout))


class Mlp:
    """The selector network (12 -> 64 -> 64 -> 64 -> nout) on the device, driven
    through the library's forward / gradient / Adam kernels.  batch: rows per call."""

    def __init__(self, nout: int, batch: int):
        self.nout, self.batch = int(nout), int(batch)
        self.np = mlp_num_params(nout)
        f = 4
        self.params = DeviceBuffer(self.np * f)
        self.grads = DeviceBuffer(self.np * f)
        self.m = DeviceBuffer(self.np * f)
        self.v = DeviceBuffer(self.np * f)
        self.X = DeviceBuffer(self.batch * 12 * f)
        self.T = DeviceBuffer(self.batch * nout * f)
        self.M = DeviceBuffer(self.batch * nout * f)
        self.out = DeviceBuffer(self.batch * nout * f)
        self.loss = DeviceBuffer(f)
        self.scratch = DeviceBuffer(int(lib().tt_mlp_scratch_floats(self.batch, nout)) * f)

    def _rows(self, X):
        X = np.ascontiguousarray(X, dtype=np.float32)
        if X.ndim != 2 or X.shape[1] != 12 or X.shape[0] > self.batch:
            raise ValueError(f"X must be (<= {self.batch}) x 12")
        return X

    def forward(self, params: np.ndarray, X: np.ndarray) -> np.ndarray:
        X = self._rows(X)
        self.params.upload(np.ascontiguousarray(params, dtype=np.float32))
        self.X.upload(X)
        check(lib().tt_mlp_forward(self.params.ptr, self.nout, self.X.ptr, X.shape[0], self.scratch.ptr,
                                   self.out.ptr, None))
        return self.out.to_array((X.shape[0], self.nout))

    def grad(self, params, X, T, M):
        """(loss, gradient) of the masked mean squared error."""
        X = self._rows(X)
        self.params.upload(np.ascontiguousarray(params, dtype=np.float32))
        self.X.upload(X)
        self.T.upload(np.ascontiguousarray(T, dtype=np.float32))
        self.M.upload(np.ascontiguousarray(M, dtype=np.float32))
        check(lib().tt_mlp_grad(self.params.ptr, self.nout, self.X.ptr, X.shape[0], self.T.ptr, self.M.ptr,
                                self.scratch.ptr, self.grads.ptr, self.loss.ptr, None))
        return float(self.loss.to_array((1,))[0]), self.grads.to_array((self.np,))

    def train(self, params, X, T, M, steps: int, lr: float, beta1=0.9, beta2=0.999, eps=1e-8,
              weight_decay=0.0, log_every: int = 100):
        """Full-batch Adam on the device; returns (final parameters, losses every log_every steps)."""
        X = self._rows(X)
        self.params.upload(np.ascontiguousarray(params, dtype=np.float32))
        zeros = np.zeros(self.np, dtype=np.float32)
        self.m.upload(zeros)
        self.v.upload(zeros)
        self.X.upload(X)
        self.T.upload(np.ascontiguousarray(T, dtype=np.float32))
        self.M.upload(np.ascontiguousarray(M, dtype=np.float32))
        L = lib()
        losses = []
        for step in range(1, steps + 1):
            check(L.tt_mlp_grad(self.params.ptr, self.nout, self.X.ptr, X.shape[0], self.T.ptr, self.M.ptr,
                                self.scratch.ptr, self.grads.ptr, self.loss.ptr, None))
            if step == 1 or step % log_every == 0 or step == steps:
                losses.append(float(self.loss.to_array((1,))[0]))
            check(L.tt_mlp_adam(self.params.ptr, self.grads.ptr, self.m.ptr, self.v.ptr, self.np, lr, beta1,
                                beta2, eps, weight_decay, step, None))
        return self.params.to_array((self.np,)), losses


def release_cached_memory() -> None:
    """Return the device memory the library's pool keeps for later plans."""
    check(lib().tt_release_cached_memory())


def selector_load(path=None) -> None:
    check(lib().tt_selector_load(None if path is None else os.fsencode(path)))


def selector_models(order: int = 3) -> int:
    """Models loaded for tensors of this order (3 or 4)."""
    return int(lib().tt_selector_models_for_order(order))


def selector_scores(B, rank: int, prec="fp32") -> np.ndarray:
    """The network's score for every variant on tensor B (device inference); +inf = not valid."""
    n = num_variants()
    out = np.zeros(n, dtype=np.float32)
    check(lib().tt_selector_scores(_tensor_ptr(B), rank, PRECISIONS[prec], out.ctypes.data_as(C.POINTER(C.c_float)), n))
    return out
