"""GPU parity of the COO plans (the reference's MATLAB-interface kernels,
tensor_kernels/fmtaco.cpp: TTV 32-115, TTM 117-223, MTTKRP 741-780) against the
oracle's restatements of them (oracle_coo_ttv, oracle_coo_ttm, oracle_mttkrp_coo).

Inputs are sorted COO tensors with duplicate coordinates (separate nonzeros, as in
fmtaco.cpp's runs).  Tolerances as for the CSF plans (FP32: max|x-y| <= 2e-5
max|y|, ||x-y||_F <= 1e-5 ||y||_F; FP16: 3e-3 and 1e-3; FX16: 5e-4 and 2e-4);
fiber coordinates are exact.
"""
import numpy as np
import pytest

import tentaco_gb300 as tt
from helpers import rel_errors, to_oracle
from oracle import oracle as O

pytestmark = pytest.mark.gpu

TOL = {"fp32": (2e-5, 1e-5), "fp16": (3e-3, 1e-3), "fx16": (5e-4, 2e-4)}


def close(got, ref, prec="fp32"):
    mx, fr = TOL[prec]
    got = np.asarray(got, np.float64)
    e = rel_errors(got, ref)
    assert np.abs(got - ref).max() <= mx * np.abs(ref).max() + 1e-30, e
    assert e["fro"] <= fr, e


def sorted_coo(dims, zipf, nnz, seed, dup=0.1):
    """Sorted coordinates of a Zipf tensor plus duplicated nonzeros (separate entries)."""
    B = tt.gen_zipf(dims, zipf, nnz, seed=seed)
    co = O.coords_of(to_oracle(B)).astype(np.int64)
    v = B.vals.astype(np.float64)
    rng = np.random.default_rng(seed)
    k = rng.choice(co.shape[0], int(dup * co.shape[0]), replace=False)
    co = np.concatenate([co, co[k]])
    v = np.concatenate([v, rng.random(k.size)])
    order = np.lexsort(co.T[::-1])
    return co[order], v[order].astype(np.float32).astype(np.float64)


@pytest.mark.parametrize("order,prec", [(3, "fp32"), (3, "fp16"), (3, "fx16"), (4, "fp32"), (4, "fx16"),
                                        (5, "fp32"), (5, "fp16")])
def test_coo_mttkrp(order, prec):
    dims = {3: (3000, 800, 5000), 4: (900, 200, 100, 4000), 5: (300, 40, 30, 20, 2000)}[order]
    zipf = (1.2,) + (0.5,) * (order - 2) + (0.8,)
    co, v = sorted_coo(dims, zipf, 300_000, seed=order)
    facs = [tt.gen_dense(d, 32, 1, 40 + m) for m, d in enumerate(dims[1:])]
    ref = O.mttkrp_coo(co, v, [None] + [f.astype(np.float64) for f in facs], 0, dims[0])
    for select in (tt.SELECT_DEFAULT, tt.SELECT_SWEEP):
        plan = tt.Plan.from_coo(dims, co, v, op=tt.OP_MTTKRP, rank=32, prec=prec, select=select)
        assert tt.variant_info(plan.variant)["staged"] == 4
        plan.set_factors([tt.DeviceBuffer.from_array(f) for f in facs])
        A = tt.DeviceBuffer(dims[0] * 32 * 4)
        for _ in range(2):
            plan.mttkrp(A)
            close(A.to_array((dims[0], 32)), ref, prec)
        assert plan.device_error() == 0


def test_coo_ttv():
    dims = (4000, 3000, 20_000)
    co, v = sorted_coo(dims, (1.1, 1.1, 0.0), 400_000, seed=11)
    x = tt.gen_dense(dims[2], 1, 2, 5)[:, 0].copy()
    fib, yref = O.coo_ttv(co, v, x.astype(np.float64))
    plan = tt.Plan.from_coo(dims, co, v, op=tt.OP_TTV)
    nf = plan.num_fibers(1)
    assert nf == fib.shape[0]
    assert np.array_equal(plan.coo_fibers(), fib.astype(np.int32))
    y = tt.DeviceBuffer(nf * 4)
    plan.ttv(tt.DeviceBuffer.from_array(x), y)
    close(y.to_array((nf,)), yref)


@pytest.mark.parametrize("R", [8, 16, 32, 50])
def test_coo_ttm(R):
    dims = (3000, 2000, 8000)
    co, v = sorted_coo(dims, (1.2, 1.0, 0.5), 300_000, seed=20 + R)
    U = tt.gen_dense(R, dims[2], 1, 7)  # R x K, the reference's layout
    fib, Yref = O.coo_ttm(co, v, U.astype(np.float64))
    plan = tt.Plan.from_coo(dims, co, v, op=tt.OP_TTM, rank=R)
    nf = plan.num_fibers(0)
    assert nf == fib.shape[0]
    assert np.array_equal(plan.coo_fibers(), fib.astype(np.int32))
    plan.set_factors([tt.DeviceBuffer.from_array(U)])
    Y = tt.DeviceBuffer(nf * R * 4)
    plan.ttm(Y)
    close(Y.to_array((nf, R)), Yref)


def test_coo_rejects_unsorted_and_out_of_range():
    dims = (10, 10, 10)
    co = np.array([[0, 1, 2], [0, 1, 1]], np.int32)  # out of order
    with pytest.raises(tt.TTError) as e:
        tt.Plan.from_coo(dims, co, np.ones(2, np.float32))
    assert e.value.status == tt.TT_ERR_INVALID_ARGUMENT and "order" in str(e.value)
    co = np.array([[0, 1, 2], [0, 1, 10]], np.int32)  # coordinate 10 in a mode of 10
    with pytest.raises(tt.TTError) as e:
        tt.Plan.from_coo(dims, co, np.ones(2, np.float32))
    assert e.value.status == tt.TT_ERR_INVALID_ARGUMENT and "outside" in str(e.value)


def test_coo_empty_and_single():
    dims = (5, 4, 3)
    plan = tt.Plan.from_coo(dims, np.zeros((0, 3), np.int32), np.zeros(0, np.float32), rank=8)
    plan.set_factors([tt.DeviceBuffer.from_array(np.ones((d, 8), np.float32)) for d in dims[1:]])
    A = tt.DeviceBuffer(5 * 8 * 4)
    A.upload(np.full((5, 8), np.nan, np.float32))
    plan.mttkrp(A)
    assert np.array_equal(A.to_array((5, 8)), np.zeros((5, 8), np.float32))
    co = np.array([[3, 2, 1]], np.int32)
    plan = tt.Plan.from_coo(dims, co, np.array([2.0], np.float32), rank=8)
    C, D = tt.gen_dense(4, 8, 1, 1), tt.gen_dense(3, 8, 1, 2)
    plan.set_factors([tt.DeviceBuffer.from_array(C), tt.DeviceBuffer.from_array(D)])
    plan.mttkrp(A)
    ref = np.zeros((5, 8))
    ref[3] = 2.0 * C[2].astype(np.float64) * D[1]
    close(A.to_array((5, 8)), ref)
