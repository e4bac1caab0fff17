"""The one-shot MTTKRP (tt_mttkrp_host) over page-locked host buffers.

With a strip-walk variant and page-locked inputs the call queues every
host-to-device copy first and runs the device work under them: the structure
check, kexp / rnz / the partition, the conversions, then per chunk of leaf
coordinates (whole work units, at most 16 chunks of at least 64 units) the
chunk's check and the walk of the units that have arrived.  These tests check:

  * bit-identical results to the same call over pageable buffers (the serial
    path: the same conversions, walk and fixed-order merge), for every strip
    variant and storage precision of three modes, and for four and five modes;
  * the FP64 oracle within the tolerances of the other MTTKRP tests
    (FP32: max|x-y| <= 2e-5 max|y|, ||x-y||_F <= 1e-5 ||y||_F; FP16: 3e-3 / 1e-3;
    BF16: 2e-2 / 8e-3);
  * one chunk, two chunks with a ragged end, a tensor smaller than one unit, and
    16 chunks of 1.25M nonzeros;
  * a leaf coordinate out of range, or out of order, in a late chunk: the call
    reports TT_ERR_INVALID_CSF and leaves the output untouched, and the next call
    is correct.
"""
import numpy as np
import pytest

import tentaco_gb300 as tt
from helpers import to_oracle
from oracle import oracle as O

pytestmark = pytest.mark.gpu

TOL = {"fp32": (2e-5, 1e-5), "fp16": (3e-3, 1e-3), "bf16": (2e-2, 8e-3), "bf16f": (2e-2, 8e-3)}
PREC_ID = {"fp32": 0, "bf16": 1, "bf16f": 2, "fp16": 3}


def close(got, ref, prec):
    mx, fr = TOL[prec]
    got = got.astype(np.float64)
    assert np.abs(got - ref).max() <= mx * np.abs(ref).max()
    assert np.linalg.norm(got - ref) <= fr * np.linalg.norm(ref)


def one_shot(B, facs, prec, variant, pinned, select=tt.SELECT_FIXED):
    R = facs[0].shape[1]
    A = np.full((B.dims[0], R), np.nan, np.float32)
    arrays = B.host_arrays() + list(facs) + [A]
    if pinned:
        tt.pin(arrays)
    try:
        tt.mttkrp_host(B, facs, prec=PREC_ID[prec], select=select, variant=variant, out=A)
    finally:
        if pinned:
            tt.unpin(arrays)
    return A


def strip_variants(order, R, prec):
    return [v for v in range(tt.num_variants()) if tt.variant_info(v)["staged"] == 4
            and tt.variant_valid(v, order, R, prec)]


@pytest.fixture(scope="module")
def t3():
    """600,003 nonzeros over 4,000 Zipf rows: 7 to 10 leaf chunks, a ragged last one."""
    B = tt.gen_zipf((4000, 1500, 3000), (1.1, 0.6, 0.0), 600_003, seed=31)
    C = tt.gen_dense(1500, 32, 1, 3)
    D = tt.gen_dense(3000, 32, 1, 4)
    return B, [C, D], O.mttkrp(to_oracle(B), [C, D])


@pytest.mark.parametrize("prec", ["fp32", "fp16", "bf16", "bf16f"])
def test_every_strip_variant_three_modes(t3, prec):
    B, facs, ref = t3
    vs = strip_variants(3, 32, prec)
    assert vs
    for v in vs:
        got = one_shot(B, facs, prec, v, pinned=True)
        serial = one_shot(B, facs, prec, v, pinned=False)
        assert np.array_equal(got, serial), tt.variant_info(v)["name"]
        close(got, ref, prec)


@pytest.mark.parametrize("order,prec", [(4, "fp32"), (4, "fp16"), (5, "fp32"), (5, "fp16")])
def test_four_and_five_modes_default_variant(order, prec):
    dims = (300, 40, 30, 500) if order == 4 else (200, 20, 15, 10, 400)
    zipf = (1.0, 0.4, 0.2, 0.0) if order == 4 else (1.0, 0.3, 0.3, 0.2, 0.0)
    B = tt.gen_zipf(dims, zipf, 300_001, seed=40 + order)
    facs = [tt.gen_dense(d, 32, 1, 50 + m) for m, d in enumerate(dims[1:])]
    ref = O.mttkrp(to_oracle(B), facs)
    # SELECT_DEFAULT picks the strip walk for four and five modes
    assert tt.variant_info(tt.default_variant(order, 32, prec))["staged"] == 4
    got = one_shot(B, facs, prec, 0, pinned=True, select=tt.SELECT_DEFAULT)
    serial = one_shot(B, facs, prec, 0, pinned=False, select=tt.SELECT_DEFAULT)
    assert np.array_equal(got, serial)
    close(got, ref, prec)


@pytest.mark.parametrize("nnz,rows", [(1_333, 40), (70_001, 300), (65_536, 200)])
def test_chunk_edges(nnz, rows):
    """Below one unit (one chunk, one ragged unit); just over one minimum chunk of
    64 units of 1,024 nonzeros (two chunks, the second holding one ragged unit);
    exactly one minimum chunk."""
    B = tt.gen_zipf((rows, 700, 900), (1.1, 0.5, 0.0), nnz, seed=nnz % 1009)
    facs = [tt.gen_dense(700, 32, 1, 5), tt.gen_dense(900, 32, 1, 6)]
    ref = O.mttkrp(to_oracle(B), facs)
    v = tt.default_variant(3, 32, "fp16", nnz)
    vs = [x for x in strip_variants(3, 32, "fp16") if tt.variant_info(x)["nnz_per_team"] == 128][:1] + [v]
    for vid in vs:
        if tt.variant_info(vid)["staged"] != 4:
            continue
        got = one_shot(B, facs, "fp16", vid, pinned=True)
        assert np.array_equal(got, one_shot(B, facs, "fp16", vid, pinned=False))
        close(got, ref, "fp16")


def test_sixteen_chunks_20m_nonzeros():
    """20,000,003 nonzeros: 16 leaf chunks of 1.25M nonzeros, each checked and
    walked as it lands, the last one ragged."""
    B = tt.gen_zipf((20_000, 3_000, 400_000), (1.1, 0.6, 0.0), 20_000_003, seed=91)
    facs = [tt.gen_dense(3_000, 32, 1, 9), tt.gen_dense(400_000, 32, 1, 10)]
    ref = O.mttkrp(to_oracle(B), facs)
    v = tt.default_variant(3, 32, "fp16", B.nnz)
    if tt.variant_info(v)["staged"] != 4:
        v = strip_variants(3, 32, "fp16")[0]
    got = one_shot(B, facs, "fp16", v, pinned=True)
    assert np.array_equal(got, one_shot(B, facs, "fp16", v, pinned=False))
    close(got, ref, "fp16")


@pytest.mark.parametrize("bad", ["range", "order"])
def test_bad_leaf_coordinate_in_a_late_chunk(bad):
    B = tt.gen_zipf((2000, 800, 1200), (1.1, 0.5, 0.0), 500_000, seed=77)
    facs = [tt.gen_dense(800, 32, 1, 7), tt.gen_dense(1200, 32, 1, 8)]
    vid = [x for x in strip_variants(3, 32, "fp32") if tt.variant_info(x)["nnz_per_team"] == 128][0]
    good = one_shot(B, facs, "fp32", vid, pinned=True)
    crd = B.crd(2)  # the library-owned leaf coordinates, changed in place
    pos2 = B.pos(2)
    # a position late in the tensor that does not start a fiber
    starts = np.zeros(B.nnz + 1, bool)
    starts[pos2] = True
    p = int(np.nonzero(~starts[:B.nnz])[0][-10])
    old = int(crd[p])
    crd[p] = 1_000_000 if bad == "range" else crd[p - 1]
    R = 32
    A = np.full((B.dims[0], R), 7.0, np.float32)
    arrays = B.host_arrays() + facs + [A]
    tt.pin(arrays)
    try:
        with pytest.raises(tt.TTError) as ei:
            tt.mttkrp_host(B, facs, prec=0, select=tt.SELECT_FIXED, variant=vid, out=A)
        assert ei.value.status == tt.TT_ERR_INVALID_CSF
        assert str(p) in str(ei.value)
        assert np.all(A == 7.0)
    finally:
        tt.unpin(arrays)
        crd[p] = old
    assert np.array_equal(one_shot(B, facs, "fp32", vid, pinned=True), good)
