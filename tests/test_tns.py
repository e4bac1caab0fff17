"""FROSTT .tns reader: 1-based coordinates, comments, dims from the data,
duplicates summed like tt_csf_from_coo, malformed lines rejected."""
import numpy as np
import pytest

import tentaco_gb300 as tt


def _same(a, b):
    assert a.dims == b.dims and a.order == b.order
    for l in range(1, a.order):
        assert np.array_equal(a.pos(l), b.pos(l))
    for l in range(a.order):
        assert np.array_equal(a.crd(l), b.crd(l))
    assert np.array_equal(a.vals, b.vals)


@pytest.mark.parametrize("order", [3, 4])
def test_read_matches_coo_builder(tmp_path, order):
    rng = np.random.default_rng(order)
    n = 5000
    dims = [37, 11, 53, 7][:order]
    co = np.stack([rng.integers(0, d, n) for d in dims], 1).astype(np.int32)
    vals = rng.random(n).astype(np.float32)
    path = tmp_path / "t.tns"
    with open(path, "w") as f:
        f.write("# a comment\n\n")
        for c, v in zip(co, vals):
            f.write(" ".join(str(int(x) + 1) for x in c) + f"\t{float(v)!r}\n")
    B = tt.read_tns(str(path))
    ref_dims = [int(co[:, m].max()) + 1 for m in range(order)]
    _same(B, tt.csf_from_coo(ref_dims, co, vals))


def test_large_file_parallel_chunks(tmp_path):
    rng = np.random.default_rng(7)
    n = 400_000
    co = np.stack([rng.integers(0, 500, n), rng.integers(0, 400, n), rng.integers(0, 300, n)], 1).astype(np.int32)
    vals = rng.random(n).astype(np.float32)
    lines = "\n".join(f"{a + 1} {b + 1} {c + 1} {float(v)!r}" for (a, b, c), v in zip(co, vals))
    path = tmp_path / "big.tns"
    path.write_text(lines + "\n")
    B = tt.read_tns(str(path), 3)
    dims = [int(co[:, m].max()) + 1 for m in range(3)]
    _same(B, tt.csf_from_coo(dims, co, vals))


@pytest.mark.parametrize("text", ["1 2 3 0.5\n0 1 1 1.0\n", "1 2 3 0.5\n1 2 1.0\n", "1 2 x 0.5\n", "1.5 2 3 1\n"])
def test_malformed(tmp_path, text):
    path = tmp_path / "bad.tns"
    path.write_text(text)
    with pytest.raises(tt.TTError) as e:
        tt.read_tns(str(path))
    assert e.value.status == tt.TT_ERR_INVALID_ARGUMENT


def test_missing_file(tmp_path):
    with pytest.raises(tt.TTError):
        tt.read_tns(str(tmp_path / "nope.tns"))
