"""The oracle restatement is pinned against the reference's own CPU kernels.

tests/golden/*.npz were produced by the reference's tensor_kernels/*_cpu_taco.h
compiled unmodified (tests/golden/make_golden.py); the restatement must
reproduce them bit-for-bit.  Where the reference sources are present, the
compiled reference is also compared directly on fresh random inputs.
"""
import numpy as np
import pytest

from helpers import golden_csf, golden_files
from oracle import oracle as O


@pytest.mark.parametrize("path", golden_files("mttkrp"), ids=lambda p: p.split("/")[-1])
def test_mttkrp_golden_bitexact(path):
    z = np.load(path)
    csf = golden_csf(z)
    facs = [z[f"F{m}"] for m in range(1, int(z["order"]))]
    A = O.mttkrp(csf, facs)
    assert np.array_equal(A, z["A"])
    if "A_workspace" in z:
        assert np.array_equal(O.mttkrp3_workspace(csf, *facs), z["A_workspace"])


@pytest.mark.parametrize("path", golden_files("ttv"), ids=lambda p: p.split("/")[-1])
def test_ttv_golden_bitexact(path):
    z = np.load(path)
    assert np.array_equal(O.ttv(golden_csf(z), z["x"]), z["y"])


def test_hand_case():
    z = np.load(golden_files("mttkrp")[0].replace(golden_files("mttkrp")[0].split("/")[-1], "mttkrp3_hand.npz"))
    assert np.array_equal(z["A"], np.array([[59.0, 104.0], [84.0, 128.0]]))
    assert np.array_equal(O.mttkrp(golden_csf(z), [z["F1"], z["F2"]]), z["A"])


def test_all_ones_counts_row_nonzeros():
    # With B, C and D all ones (what the reference's mttkrp_ref effectively checks,
    # tensor_experiments/mttkrp_csf_gpu.h:42) every output entry is the row's nnz.
    rng = np.random.default_rng(5)
    dims = (30, 20, 25)
    co = np.stack([rng.integers(0, d, 800) for d in dims], 1)
    csf = O.build_csf(dims, co, np.ones(800))
    csf.vals[:] = 1.0
    A = O.mttkrp(csf, [np.ones((20, 4)), np.ones((25, 4))])
    per_row = np.array([csf.pos[2][csf.pos[1][i + 1]] - csf.pos[2][csf.pos[1][i]] for i in range(30)])
    assert np.array_equal(A, np.repeat(per_row[:, None], 4, axis=1).astype(float))


def test_rows_subset_matches_full():
    z = np.load([p for p in golden_files("mttkrp") if "zipf_r20" in p][0])
    csf = golden_csf(z)
    facs = [z["F1"], z["F2"]]
    rows = np.array([0, 5, 17, 299])
    assert np.array_equal(O.mttkrp(csf, facs, rows=rows), z["A"][rows])
    z4 = np.load([p for p in golden_files("mttkrp") if "mttkrp4" in p][0])
    c4 = golden_csf(z4)
    f4 = [z4["F1"], z4["F2"], z4["F3"]]
    assert np.array_equal(O.mttkrp(c4, f4, rows=np.array([1, 2, 39])), z4["A"][[1, 2, 39]])


def test_csf_builder_dense_reconstruction():
    rng = np.random.default_rng(9)
    dims = (6, 5, 7, 4)
    co = np.stack([rng.integers(0, d, 150) for d in dims], 1)
    v = rng.random(150)
    csf = O.build_csf(dims, co, v)
    T = np.zeros(dims)
    for c, x in zip(co, v):
        T[tuple(c)] += x
    facs = [rng.random((d, 3)) for d in dims[1:]]
    A = np.einsum("iklm,kr,lr,mr->ir", T, *facs)
    assert np.allclose(O.mttkrp(csf, facs), A, rtol=1e-12, atol=1e-12)


def test_reference_comparators():
    x = np.array([1.0, 2.0, 0.0], dtype=np.float32)
    assert O.compare_array(x, np.array([1.0, 2.2, 0.0], dtype=np.float32)) == pytest.approx(0.1, rel=1e-5)
    assert O.compare_array(x, np.array([1.0, 2.0, 1.0], dtype=np.float32)) == np.inf
    assert O.compare_array_my(x, x + np.float32(0.01)) == 3
    big = np.zeros(100, dtype=np.float32)
    assert O.compare_array_my(big, big + 1) == 11  # the reference stops counting after 10


@pytest.mark.skipif(O.ref_lib() is None, reason="reference sources absent on this host")
def test_reference_matches_restatement_random():
    rng = np.random.default_rng(77)
    for dims, R in (((40, 30, 50), 16), ((12, 9, 8, 20), 8), ((8, 6, 5, 4, 20), 8)):
        co = np.stack([rng.integers(0, d, 2000) for d in dims], 1)
        csf = O.build_csf(dims, co, rng.random(2000))
        facs = [rng.standard_normal((d, R)) for d in dims[1:]]
        assert np.array_equal(O.mttkrp(csf, facs), O.ref_mttkrp(csf, facs))
    dims = (40, 30, 50)
    co = np.stack([rng.integers(0, d, 3000) for d in dims], 1)
    csf = O.build_csf(dims, co, rng.random(3000))
    x = rng.uniform(-1, 1, 50)
    assert np.array_equal(O.ttv(csf, x), O.ref_ttv(csf, x))


@pytest.mark.parametrize("path", golden_files("mttkrp5"), ids=lambda p: p.split("/")[-1])
def test_mttkrp5_golden_bitexact(path):
    """Five modes (oracle only; the library's kernels cover three and four): the
    restatement of the reference's level-by-level factored loop reproduces its
    output bit-for-bit, and both agree with a dense einsum."""
    z = np.load(path)
    csf = golden_csf(z)
    facs = [z[f"F{m}"] for m in range(1, 5)]
    A = O.mttkrp(csf, facs)
    assert np.array_equal(A, z["A"])
    dense = np.zeros(csf.dims)
    dense[tuple(O.coords_of(csf).T)] = csf.vals
    ref = np.einsum("abcde,br,cr,dr,er->ar", dense, *facs, optimize=True)
    assert np.allclose(A, ref, rtol=1e-10, atol=1e-10 * np.abs(ref).max())


@pytest.mark.parametrize("order", [3, 4, 5])
def test_any_mode_oracle(order):
    """The any-mode oracle (oracle_mttkrp_coo) equals the reference-pinned CSF
    oracle bit-for-bit for mode 0 with three or four modes (same nonzero order and
    product association; the five-mode kernel factors its sums level by level, so
    there the two agree to rounding) and a dense einsum for every mode."""
    rng = np.random.default_rng(5 + order)
    dims = {3: (12, 9, 11), 4: (7, 6, 5, 8), 5: (5, 4, 3, 4, 6)}[order]
    co = np.array(sorted({tuple(int(rng.integers(0, d)) for d in dims) for _ in range(300)}), dtype=np.int64)
    vals = rng.random(len(co))
    csf = O.build_csf(dims, co, vals)
    coords = O.coords_of(csf)
    assert np.array_equal(coords, co)
    F = [rng.random((d, 6)) for d in dims]
    got0, csf0 = O.mttkrp_coo(coords, csf.vals, F, 0, dims[0]), O.mttkrp(csf, F[1:])
    if order < 5:
        assert np.array_equal(got0, csf0)
    else:
        assert np.allclose(got0, csf0, rtol=1e-12, atol=1e-12)
    dense = np.zeros(dims)
    dense[tuple(co.T)] = vals
    letters = "abcde"[:order]
    for m in range(order):
        others = [n for n in range(order) if n != m]
        eq = letters + "," + ",".join(letters[n] + "r" for n in others) + "->" + letters[m] + "r"
        ref = np.einsum(eq, dense, *[F[n] for n in others])
        got = O.mttkrp_coo(coords, csf.vals, F, m, dims[m])
        assert np.allclose(got, ref, rtol=1e-12, atol=1e-12), m


def test_coo_kernels_of_the_matlab_interface():
    """COO TTV / TTM / MTTKRP as in the reference's MATLAB interface (fmtaco.cpp,
    which needs MATLAB to compile, so parity is anchored here): over the canonical
    nonzero order, COO TTV reproduces the reference's CSF TTV output bit-for-bit and
    COO MTTKRP the CSF MTTKRP; TTM agrees with a dense evaluation."""
    z = np.load(golden_files("ttv")[0])
    csf = golden_csf(z)
    co = O.coords_of(csf)
    fib, y = O.coo_ttv(co, csf.vals, z["x"])
    assert np.array_equal(y, z["y"])
    assert fib.shape[0] == csf.nfibers(1)
    assert np.array_equal(fib[:, 1], csf.crd[1])
    zm = np.load([p for p in golden_files("mttkrp") if "zipf_r20" in p][0])
    cm = golden_csf(zm)
    F = [None, zm["F1"], zm["F2"]]
    assert np.array_equal(O.mttkrp_coo(O.coords_of(cm), cm.vals, F, 0, cm.dims[0]), zm["A"])
    rng = np.random.default_rng(31)
    U = rng.standard_normal((7, csf.dims[2]))
    fib2, Y = O.coo_ttm(co, csf.vals, U)
    assert np.array_equal(fib2, fib)
    dense = np.zeros(csf.dims)
    dense[tuple(co.T)] = csf.vals
    ref = np.einsum("ijk,rk->ijr", dense, U)[fib[:, 0], fib[:, 1]]
    assert np.allclose(Y, ref, rtol=1e-12, atol=1e-12 * np.abs(ref).max())
    # runs, not sorting: an unsorted stream splits a fiber wherever (i, j) changes
    fib3, y3 = O.coo_ttv(co[::-1], csf.vals[::-1], z["x"])
    assert fib3.shape[0] == fib.shape[0] and np.allclose(y3[::-1], y, rtol=1e-12, atol=1e-12)


@pytest.mark.skipif(O.ref_lib() is None, reason="reference sources absent on this host")
def test_golden_fixtures_regenerate_identically(tmp_path):
    """The committed fixtures are exactly what tests/golden/make_golden.py makes from
    the compiled reference kernels."""
    import importlib.util
    import os
    here = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
    spec = importlib.util.spec_from_file_location("make_golden", os.path.join(here, "make_golden.py"))
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    mg.main(str(tmp_path))
    made = sorted(p.name for p in tmp_path.glob("*.npz"))
    assert made == sorted(f for f in os.listdir(here) if f.endswith(".npz"))
    for name in made:
        a, b = np.load(tmp_path / name), np.load(os.path.join(here, name))
        assert sorted(a.files) == sorted(b.files), name
        for k in a.files:
            assert np.array_equal(a[k], b[k]), (name, k)


@pytest.mark.parametrize("seed", [3, 11])
def test_generator_restatement_matches_library(seed):
    """The oracle's C restatement of the seeded generators (used by the bench's
    reference arm, which must not load the product library) yields the library's
    tensors and factors bit for bit."""
    import tentaco_gb300 as tt

    dims = (300, 200, 5000)
    B = tt.gen_lognormal_fibers(dims, 200_000, 1.5, 1.8, 2, 2000, seed)
    G = O.gen_lognormal(dims, 200_000, 1.5, 1.8, 2, 2000, seed)
    for lvl in (1, 2):
        assert np.array_equal(B.pos(lvl).astype(np.int64), G.pos[lvl])
        assert np.array_equal(B.crd(lvl).astype(np.int64), G.crd[lvl])
    assert np.array_equal(B.vals.astype(np.float64), G.vals)
    for dist in (0, 1, 2):
        assert np.array_equal(tt.gen_dense(5000, 32, dist, seed), O.gen_dense(5000, 32, dist, seed))
