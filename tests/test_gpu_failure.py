"""Failure detection without a GPU fault (the library's test hooks).

* A bounded device wait made to run out: with tt_debug_tma_wait(1, ns) the TMA walk
  (variant family 2) arms each stage's mbarrier with its expected bytes but issues no
  copy, so nothing is in flight and the first wait gives up after `ns`.  The call
  records error word 301 (TT_ERR_DEVICE_WAIT from the one-shot entry point), the
  row merge skips, and the next call on the same plan runs normally: the error word
  is cleared per call and the context stays usable.
* Injected allocation failures: tt_debug_fail_pool_alloc(n) fails the n-th device
  allocation from now.  Every n up to the sequence's last allocation is tried: the
  failing call returns a status, a plan whose allocation failed after its creation
  refuses later calls, and once the plan is gone the library holds no allocation
  more than before (tt_debug_pool_live).
"""
import gc

import numpy as np
import pytest

import tentaco_gb300 as tt
from helpers import rel_errors, to_oracle
from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(autouse=True)
def hooks_off():
    yield
    L = tt.lib()
    L.tt_debug_tma_wait(0, 0)
    L.tt_debug_fail_pool_alloc(0)


def close(got, ref):
    e = rel_errors(got, ref)
    assert np.abs(got.astype(np.float64) - ref).max() <= 2e-5 * np.abs(ref).max(), e
    assert e["fro"] <= 1e-5, e


def tma_variant(order, rank, prec):
    ids = [v for v in range(tt.num_variants())
           if tt.variant_info(v)["staged"] == 2 and tt.variant_valid(v, order, rank, prec)]
    assert ids, "no TMA variant"
    return ids[len(ids) // 2]


def case3(nnz=200_000, seed=3):
    B = tt.gen_zipf((2000, 500, 3000), (1.1, 0.6, 0.8), nnz, seed=seed)
    facs = [tt.gen_dense(500, 32, 1, 1), tt.gen_dense(3000, 32, 1, 2)]
    return B, facs, O.mttkrp(to_oracle(B), facs)


@pytest.mark.parametrize("wait_ns", [20_000, 1_000_000])
def test_tma_wait_runs_out_then_plan_recovers(wait_ns):
    B, facs, ref = case3()
    vid = tma_variant(3, 32, "fp32")
    plan = tt.Plan(B, rank=32, prec="fp32", select=tt.SELECT_FIXED, variant=vid)
    assert plan.variant == vid
    plan.set_factors([tt.DeviceBuffer.from_array(f) for f in facs])
    A = tt.DeviceBuffer(B.dims[0] * 32 * 4)
    tt.check(tt.lib().tt_debug_tma_wait(1, wait_ns))
    plan.mttkrp(A)  # asynchronous: the status is the error word
    assert plan.device_error() == 301
    tt.check(tt.lib().tt_debug_tma_wait(0, 0))
    plan.mttkrp(A)
    assert plan.device_error() == 0  # cleared by the call itself
    close(A.to_array((B.dims[0], 32)), ref)


def test_tma_wait_one_shot_reports_device_wait():
    B, facs, ref = case3(nnz=50_000, seed=4)
    vid = tma_variant(3, 32, "fp32")
    tt.check(tt.lib().tt_debug_tma_wait(1, 20_000))
    with pytest.raises(tt.TTError) as e:
        tt.mttkrp_host(B, facs, select=tt.SELECT_FIXED, variant=vid)
    assert e.value.status == tt.TT_ERR_DEVICE_WAIT and "301" in str(e.value)
    tt.check(tt.lib().tt_debug_tma_wait(0, 0))
    close(tt.mttkrp_host(B, facs, select=tt.SELECT_FIXED, variant=vid), ref)


def test_tma_wait_hook_rejects_bad_bounds():
    with pytest.raises(tt.TTError):
        tt.check(tt.lib().tt_debug_tma_wait(1, -1))
    with pytest.raises(tt.TTError):
        tt.check(tt.lib().tt_debug_tma_wait(1, 2_000_000_000))


def sweep_failures(sequence, limit=400):
    """Run `sequence(state)` with the n-th allocation failing, n = 1, 2, ... until it
    completes; returns how many failures were injected."""
    L = tt.lib()
    tt.synchronize()
    base = L.tt_debug_pool_live()
    for n in range(1, limit):
        state = {}
        tt.check(L.tt_debug_fail_pool_alloc(n))
        failed = None
        try:
            sequence(state)
        except tt.TTError as e:
            failed = e.status
        if failed is None:
            tt.check(L.tt_debug_fail_pool_alloc(0))
        else:
            assert failed in (tt.TT_ERR_OUT_OF_MEMORY, tt.TT_ERR_CUDA), (n, failed)
            if "plan" in state:
                # created, then an allocation failed: every later call is refused
                refused = None
                try:
                    state["retry"]()
                except tt.TTError as e:
                    refused = (e.status, str(e))
                assert refused and refused[0] == tt.TT_ERR_INVALID_ARGUMENT and "unusable" in refused[1], (n, refused)
        state.clear()
        gc.collect()
        tt.synchronize()
        assert L.tt_debug_pool_live() == base, n
        if failed is None:
            return n - 1
    raise AssertionError("the sequence never completed")


def test_allocation_failures_csf_plans():
    B, facs, ref = case3(nnz=30_000, seed=5)
    out = {}

    def seq(state, prec, slabs):
        plan = tt.Plan(B, rank=32, prec=prec, slabs=slabs)
        state["plan"] = plan
        bufs = [tt.DeviceBuffer.from_array(f) for f in facs]
        A = tt.DeviceBuffer(B.dims[0] * 32 * 4)
        state["retry"] = lambda: plan.mttkrp(A)
        plan.set_factors(bufs)
        plan.use_variant(plan.variant)
        plan.mttkrp(A)
        out["A"] = A.to_array((B.dims[0], 32))

    for prec, slabs in (("fp32", 1), ("fp16", 3), ("fx16", 1)):
        n = sweep_failures(lambda st: seq(st, prec, slabs))
        assert n >= 5, (prec, n)
        e = rel_errors(out["A"], ref)
        assert e["fro"] <= (1e-5 if prec == "fp32" else 1e-3), (prec, e)


def test_allocation_failures_coo_and_one_shot():
    B, facs, ref = case3(nnz=30_000, seed=6)
    co = O.coords_of(to_oracle(B))
    v = B.vals.astype(np.float64)
    out = {}

    def coo(state):
        plan = tt.Plan.from_coo(B.dims, co, v, rank=32)
        state["plan"] = plan
        A = tt.DeviceBuffer(B.dims[0] * 32 * 4)
        state["retry"] = lambda: plan.mttkrp(A)
        plan.set_factors([tt.DeviceBuffer.from_array(f) for f in facs])
        plan.mttkrp(A)
        out["A"] = A.to_array((B.dims[0], 32))

    assert sweep_failures(coo) >= 5
    close(out["A"], ref)

    def ttm(state):
        U = facs[1][:, :16].T.copy()  # 16 x K
        plan = tt.Plan.from_coo(B.dims, co, v, op=tt.OP_TTM, rank=16)
        state["plan"] = plan
        Y = tt.DeviceBuffer(plan.num_fibers(0) * 16 * 4)
        state["retry"] = lambda: plan.ttm(Y)
        plan.set_factors([tt.DeviceBuffer.from_array(U)])
        plan.ttm(Y)

    assert sweep_failures(ttm) >= 3

    def one_shot(state):
        out["A"] = tt.mttkrp_host(B, facs)

    assert sweep_failures(one_shot) >= 3
    close(out["A"], ref)
