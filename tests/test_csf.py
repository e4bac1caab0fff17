"""Host CSF construction, validation and the seeded generators (CPU only).

The library's canonical CSF (lexicographic, duplicates summed in FP64 in input
order, dense root) must equal the oracle's definition bit-for-bit.
"""
import numpy as np
import pytest

import tentaco_gb300 as tt
from helpers import to_oracle
from oracle import oracle as O


def same(B, Oc):
    for l in range(1, B.order):
        assert np.array_equal(B.pos(l), Oc.pos[l]), f"pos{l}"
        assert np.array_equal(B.crd(l), Oc.crd[l]), f"crd{l}"
    assert np.array_equal(B.vals, Oc.vals.astype(np.float32))


@pytest.mark.parametrize("dims,nnz", [((50, 40, 30), 5000), ((7, 5, 6, 9), 300), ((3, 1000, 1000), 2000),
                                       ((1, 4, 4), 10), ((1000, 3, 3), 20), ((6, 5, 4, 7, 9), 2000)])
def test_builder_matches_oracle(dims, nnz):
    rng = np.random.default_rng(nnz)
    co = np.stack([rng.integers(0, d, nnz) for d in dims], 1)
    v = rng.random(nnz).astype(np.float32)
    B = tt.csf_from_coo(dims, co, v)
    same(B, O.build_csf(dims, co, v.astype(np.float64)))
    assert tt.lib().tt_csf_validate(B.ptr) == 0


def test_builder_duplicates_sum_in_input_order():
    co = np.array([[1, 2, 3]] * 5 + [[0, 0, 0]], dtype=np.int32)
    v = np.array([1e8, 1.0, -1e8, 1.0, 0.5, 2.0], dtype=np.float32)
    B = tt.csf_from_coo((2, 3, 4), co, v)
    assert B.nnz == 2
    assert np.array_equal(B.vals, np.array([2.0, np.float32(1e8 + 1.0 - 1e8 + 1.0 + 0.5)], np.float32))


def test_builder_empty_and_bad_input():
    B = tt.csf_from_coo((4, 4, 4), np.zeros((0, 3), np.int32), np.zeros(0, np.float32))
    assert B.nnz == 0 and np.array_equal(B.pos(1), np.zeros(5, np.int32))
    with pytest.raises(tt.TTError):
        tt.csf_from_coo((4, 4, 4), np.array([[0, 4, 0]], np.int32), np.ones(1, np.float32))


def _bad(levels, dims=(2, 3, 3)):
    B = tt.HostTaco(dims, vals=np.ones(8, np.float32), levels=levels)
    return tt.lib().tt_csf_validate(B.ptr)


def test_validator_rejects_malformed_csf():
    ok = [None, (np.array([0, 1, 2]), np.array([0, 2])), (np.array([0, 2, 3]), np.array([0, 1, 2]))]
    assert _bad(ok) == 0
    dec = [None, (np.array([0, 2, 1]), np.array([0, 2])), (np.array([0, 2, 3]), np.array([0, 1, 2]))]
    assert _bad(dec) == tt.TT_ERR_INVALID_CSF
    rng_ = [None, (np.array([0, 1, 2]), np.array([0, 3])), (np.array([0, 2, 3]), np.array([0, 1, 2]))]
    assert _bad(rng_) == tt.TT_ERR_INVALID_CSF
    empty_inner = [None, (np.array([0, 1, 2]), np.array([0, 2])), (np.array([0, 0, 3]), np.array([0, 1, 2]))]
    assert _bad(empty_inner) == tt.TT_ERR_INVALID_CSF
    unsorted = [None, (np.array([0, 1, 2]), np.array([0, 2])), (np.array([0, 2, 3]), np.array([1, 0, 2]))]
    assert _bad(unsorted) == tt.TT_ERR_INVALID_CSF


def test_zipf_generator_deterministic_and_valid():
    a = tt.gen_zipf((500, 400, 300), (1.1, 1.1, 0), 20000, seed=2, vlo=-1, vhi=1)
    b = tt.gen_zipf((500, 400, 300), (1.1, 1.1, 0), 20000, seed=2, vlo=-1, vhi=1)
    c = tt.gen_zipf((500, 400, 300), (1.1, 1.1, 0), 20000, seed=3, vlo=-1, vhi=1)
    assert a.nnz == 20000
    for l in (1, 2):
        assert np.array_equal(a.pos(l), b.pos(l)) and np.array_equal(a.crd(l), b.crd(l))
    assert np.array_equal(a.vals, b.vals) and not np.array_equal(a.vals, c.vals)
    assert a.vals.min() >= -1 and a.vals.max() <= 1
    assert tt.lib().tt_csf_validate(a.ptr) == 0
    # the generated CSF is canonical: rebuilding it from its own COO changes nothing
    Oc = to_oracle(a)
    rows = np.repeat(np.arange(500), np.diff(Oc.pos[1]))
    ks = np.repeat(Oc.crd[1], np.diff(Oc.pos[2]))
    co = np.stack([np.repeat(rows, np.diff(Oc.pos[2])), ks, Oc.crd[2]], 1)
    same(a, O.build_csf((500, 400, 300), co, Oc.vals))


def test_lognormal_generator_has_long_fibers():
    B = tt.gen_lognormal_fibers((2000, 1000, 50000), 400000, 1.5, 1.8, 3, 20000, seed=3)
    assert B.nnz == 400000
    lens = np.diff(B.pos(2))
    assert (lens >= 20000).sum() >= 3
    assert tt.lib().tt_csf_validate(B.ptr) == 0
    f = B.features(32)
    assert f.shape == (12,) and np.all(np.isfinite(f))


def test_dense_generator():
    a = tt.gen_dense(100, 8, 1, 7)
    b = tt.gen_dense(100, 8, 1, 7)
    assert np.array_equal(a, b) and a.std() > 0
    u = tt.gen_dense(1000, 4, 0, 1)
    assert u.min() >= 0 and u.max() < 1


@pytest.mark.parametrize("order", [3, 4, 5])
def test_reroot_matches_builder_on_permuted_coordinates(order):
    """tt_csf_reroot(B, m) is bit-identical to building the canonical CSF from B's
    coordinates permuted to (m, then the other modes in increasing order)."""
    dims = {3: (40, 30, 50), 4: (20, 15, 12, 30), 5: (9, 8, 7, 6, 11)}[order]
    B = tt.gen_zipf(dims, (0.8,) * order, 4000, 11 + order)
    co = O.coords_of(to_oracle(B)).astype(np.int32)
    for m in range(order):
        perm = [m] + [n for n in range(order) if n != m]
        rr = tt.csf_reroot(B, m)
        ref = tt.csf_from_coo(tuple(dims[n] for n in perm), co[:, perm], B.vals)
        assert rr.dims == ref.dims and rr.nnz == B.nnz
        for l in range(1, order):
            assert np.array_equal(rr.pos(l), ref.pos(l)) and np.array_equal(rr.crd(l), ref.crd(l)), (m, l)
        assert np.array_equal(rr.vals, ref.vals)
    with pytest.raises(tt.TTError):
        tt.csf_reroot(B, order)
