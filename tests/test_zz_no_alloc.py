"""tt_mttkrp3_noalloc: the MTTKRP entry point for callers that cannot allocate.

Callers inside a memory pool they do not own, or in loops that must never enter
the allocator, pass device inputs and outputs and the call uses only a fixed
scratch array compiled into the library.  This file checks it through the C ABI
against the FP64 oracle and against the plan API's result (the existing entry
point), both within the FP32 tolerance of the other parity tests
(max|x-y| <= 2e-5 max|y|, ||x-y||_F <= 1e-5 ||y||_F), on two calls in a row: the
scratch keeps the previous call's contents, so the second call shows it is
cleared where it must be.  It runs last in the suite and also alone in a fresh
process.
"""
import ctypes as C

import numpy as np
import pytest

import tentaco_gb300 as tt
from helpers import to_oracle
from oracle import oracle as O

pytestmark = pytest.mark.gpu

FP32_MAX, FP32_FRO = 2e-5, 1e-5


def noalloc():
    f = tt.lib().tt_mttkrp3_noalloc
    f.restype = C.c_int
    f.argtypes = [C.c_int32, C.c_int64, C.c_int32] + [C.c_void_p] * 9
    return f


def close(got, ref):
    got = got.astype(np.float64)
    assert np.abs(got - ref).max() <= FP32_MAX * np.abs(ref).max()
    assert np.linalg.norm(got - ref) <= FP32_FRO * np.linalg.norm(ref)


def dev(a):
    return tt.DeviceBuffer.from_array(np.ascontiguousarray(a))


@pytest.mark.parametrize("R,nnz,rows", [(32, 400_003, 4000), (16, 150_001, 4000), (8, 50_001, 4000),
                                        (64, 120_000, 4000), (16, 1_333, 40), (32, 2_047, 7)])
def test_noalloc_matches_oracle_and_plan_twice(R, nnz, rows):
    B = tt.gen_zipf((rows, 1500, 3000), (1.1, 0.6, 0.0), nnz, seed=100 + R + nnz % 97)
    Cf = tt.gen_dense(1500, R, 1, 7)
    Df = tt.gen_dense(3000, R, 1, 8)
    ref = O.mttkrp(to_oracle(B), [Cf, Df])
    # the existing entry point (plan API)
    plan = tt.Plan(B, rank=R)
    fb = [dev(Cf), dev(Df)]
    plan.set_factors(fb)
    Ab = tt.DeviceBuffer(rows * R * 4)
    plan.mttkrp(Ab)
    from_plan = Ab.to_array((rows, R))
    close(from_plan, ref)
    # exact-length device copies of the CSF (no padding)
    arrs = [dev(B.pos(1)), dev(B.crd(1)), dev(B.pos(2)), dev(B.crd(2)), dev(B.vals)]
    out = tt.DeviceBuffer(rows * R * 4)
    f = noalloc()
    for _ in range(2):
        out.upload(np.full((rows, R), np.nan, np.float32))
        st = f(rows, B.nnz, R, *[a.ptr for a in arrs], fb[0].ptr, fb[1].ptr, out.ptr, None)
        assert st == tt.TT_OK, tt.lib().tt_last_error_string()
        tt.synchronize()
        got = out.to_array((rows, R))
        close(got, ref)
        close(got, from_plan.astype(np.float64))


def test_noalloc_rejects_sizes_beyond_its_scratch():
    f = noalloc()
    dummy = tt.DeviceBuffer(1024)
    p = dummy.ptr
    st = f(100, 20_000_000, 32, p, p, p, p, p, p, p, p, None)
    assert st == tt.TT_ERR_INVALID_ARGUMENT
    assert b"scratch limit" in tt.lib().tt_last_error_string()
    st = f(100, 10, 24, p, p, p, p, p, p, p, p, None)
    assert st == tt.TT_ERR_UNSUPPORTED
