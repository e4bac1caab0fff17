"""GPU CSF builder (tt_csf_from_coo_gpu) against the host builder: the same
canonical CSF bit for bit (pos, crd, values), for unsorted coordinates with
duplicates (summed in FP64 in input order), orders 2 to 4, empty rows, and a
large case."""
import numpy as np
import pytest

import tentaco_gb300 as tt

pytestmark = pytest.mark.gpu


def same(a, b):
    assert a.dims == b.dims and a.nnz == b.nnz
    for l in range(1, a.order):
        assert np.array_equal(a.pos(l), b.pos(l)), ("pos", l)
        assert np.array_equal(a.crd(l), b.crd(l)), ("crd", l)
    assert np.array_equal(a.vals.view(np.uint32), b.vals.view(np.uint32))


@pytest.mark.parametrize("dims,nnz", [((7, 9), 40), ((50, 40, 30), 20_000), ((300, 200, 5000), 3_000_000),
                                      ((12, 10, 9, 40), 30_000), ((3, 2, 2), 1), ((1000, 5, 5), 10),
                                      ((8, 7, 6, 5, 40), 20_000)])
def test_gpu_builder_matches_host(dims, nnz):
    rng = np.random.default_rng(len(dims) * 7 + nnz % 97)
    co = np.stack([rng.integers(0, d, nnz) for d in dims], axis=1).astype(np.int32)
    if nnz > 4:
        co[nnz // 2:nnz // 2 + nnz // 5] = co[: nnz // 5]  # duplicates, out of order
    vals = rng.standard_normal(nnz).astype(np.float32)
    same(tt.csf_from_coo_gpu(dims, co, vals), tt.csf_from_coo(dims, co, vals))


def test_gpu_builder_empty_and_bad_input():
    e = tt.csf_from_coo_gpu((4, 4, 4), np.zeros((0, 3), np.int32), np.zeros(0, np.float32))
    assert e.nnz == 0 and np.array_equal(e.pos(1), np.zeros(5, np.int32))
    with pytest.raises(tt.TTError):
        tt.csf_from_coo_gpu((4, 4, 4), np.array([[0, 4, 0]], np.int32), np.ones(1, np.float32))
