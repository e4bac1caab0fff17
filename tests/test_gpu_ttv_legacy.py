"""GPU parity of TTV and of the reference-named entry points.

TTV tolerance (FP32 storage, FP64 oracle): max|x-y| <= 2e-5 * max|y| and
||x-y||_F <= 1e-5 ||y||_F; BF16 values: ||x-y||_F <= 8e-3 ||y||_F.
"""
import numpy as np
import pytest

import tentaco_gb300 as tt
from helpers import golden_csf, golden_files, host_taco, rel_errors, to_oracle
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def close(got, ref, mx=2e-5, fr=1e-5):
    err = np.abs(got.astype(np.float64) - ref).max() if ref.size else 0.0
    assert err <= mx * max(np.abs(ref).max() if ref.size else 0.0, 1e-30) + 1e-30, err
    e = rel_errors(got, ref)
    assert e["fro"] <= fr or np.linalg.norm(ref) == 0, e
    return e


def run_ttv(B, x, prec="fp32"):
    plan = tt.Plan(B, op=tt.OP_TTV, prec=prec)
    nf = plan.num_fibers(len(B.dims) - 2)
    xb = tt.DeviceBuffer.from_array(x.astype(np.float32))
    yb = tt.DeviceBuffer(max(nf, 1) * 4)
    plan.ttv(xb, yb)
    return yb.to_array((nf,))


@pytest.mark.parametrize("path", golden_files("ttv"), ids=lambda p: p.split("/")[-1])
def test_ttv_golden(path):
    z = np.load(path)
    csf = golden_csf(z)
    B = host_taco(csf)
    got = run_ttv(B, z["x"])
    close(got, z["y"])
    got2 = tt.ttv_host(B, z["x"].astype(np.float32), csf.nfibers(1))
    assert np.array_equal(got, got2)


@pytest.fixture(scope="module")
def c2_small():
    """The 50M-nonzero TTV tensor's shape family scaled to 3M nonzeros: Zipf(1.1) on modes 0 and 1, U(-1,1)."""
    B = tt.gen_zipf((50000, 40000, 30000), (1.1, 1.1, 0), 3_000_000, seed=2, vlo=-1, vhi=1)
    x = tt.gen_dense(30000, 1, 2, 22).ravel()
    return B, x, O.ttv(to_oracle(B), x)


def test_ttv_c2_small(c2_small):
    B, x, ref = c2_small
    got = run_ttv(B, x)
    close(got, ref)
    got2 = run_ttv(B, x)
    assert np.array_equal(got, got2)
    e = close(run_ttv(B, x, prec="bf16"), ref, mx=2e-2, fr=8e-3)
    print("ttv bf16", e)
    e = close(run_ttv(B, x, prec="fp16"), ref, mx=3e-3, fr=1e-3)
    print("ttv fp16", e)


def test_ttv_long_fiber():
    L = 100_000
    co = np.array([[0, 0, l] for l in range(L)] + [[1, 2, 3], [1, 3, 4]], np.int32)
    B = tt.csf_from_coo((2, 4, L), co, np.random.default_rng(1).random(len(co)).astype(np.float32))
    x = tt.gen_dense(L, 1, 2, 3).ravel()
    close(run_ttv(B, x), O.ttv(to_oracle(B), x))


@pytest.mark.parametrize("nnz,mu", [(100_003, 0.0), (262_151, 1.0), (513, 0.5), (17, 0.0)])
def test_ttv_short_fibers_ragged_units(nnz, mu):
    """Many fibers of one or two nonzeros per lane, fibers crossing lanes and
    units, and a last unit whose count is not a multiple of 16."""
    B = tt.gen_lognormal_fibers((300, 200, 5000), nnz, mu, 1.2, 1 if nnz > 10_000 else 0, 3000, 11)
    x = tt.gen_dense(5000, 1, 2, 5).ravel()
    ref = O.ttv(to_oracle(B), x)
    got = run_ttv(B, x)
    close(got, ref)
    assert np.array_equal(got, run_ttv(B, x))
    close(run_ttv(B, x, prec="fp16"), ref, mx=3e-3, fr=1e-3)


@pytest.fixture(scope="module")
def legacy_case():
    B = tt.gen_zipf((600, 500, 700), (0.8, 0.5, 0), 60_000, seed=9)
    Oc = to_oracle(B)
    C = tt.gen_dense(500, 32, 0, 1)
    D = tt.gen_dense(700, 32, 0, 2)
    ref = O.mttkrp(Oc, [C, D])
    # the reference prepares level 0 with compress_top_level before every GPU call
    Bc = host_taco(Oc, compressed_root=True)
    return Bc, C, D, ref


def test_every_reference_entry_point(legacy_case):
    Bc, C, D, ref = legacy_case
    Ch, Dh = tt.dense(C), tt.dense(D)
    for name in tt.legacy_names():
        A = tt.dense(np.full((600, 32), np.nan, np.float32))
        tt.legacy_entry(name)(A.ptr, Bc.ptr, Ch.ptr, Dh.ptr)
        got = A.vals.reshape(600, 32)
        close(got, ref)
        assert tt.gpu_timer_ms() > 0


def test_reference_ttv_entry_point():
    z = np.load(golden_files("ttv")[0])
    csf = golden_csf(z)
    B = host_taco(csf)
    y = tt.dense(np.zeros(csf.nfibers(1), np.float32))
    x = tt.dense(z["x"].astype(np.float32))
    tt.lib().ttv_csf_gpu_taco(y.ptr, B.ptr, x.ptr)
    close(y.vals, z["y"])
    assert tt.gpu_timer_ms() > 0


@pytest.mark.parametrize("leaf,long_min", [(40_000, 30_000), (1_000_000, 400_000)])
def test_ttv_ranges_with_fibers_across_ranges(leaf, long_min):
    """12M nonzeros: ranges of several units each, with fibers longer than a range
    (crossing several ranges) among short ones; x in shared memory (40,000 entries)
    and in global memory (1,000,000 entries)."""
    B = tt.gen_lognormal_fibers((3000, 2000, leaf), 12_000_000, 2.5, 1.5, 6, long_min, 31)
    x = tt.gen_dense(leaf, 1, 2, 6).ravel()
    ref = O.ttv(to_oracle(B), x)
    got = run_ttv(B, x)
    close(got, ref)
    assert np.array_equal(got, run_ttv(B, x))
    close(run_ttv(B, x, prec="bf16"), ref, mx=2e-2, fr=8e-3)
