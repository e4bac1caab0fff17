"""GPU parity of MTTKRP (3- and 4-mode) against the FP64 oracle and the golden vectors.

Tolerances (stated per precision, against the FP64 oracle on the same
FP32-representable inputs):
  FP32 storage:  max|x-y| <= 2e-5 * max|y|  and  ||x-y||_F <= 1e-5 * ||y||_F
  BF16 storage (values and/or factors rounded to 8-bit significands):
                 ||x-y||_F <= 8e-3 * ||y||_F   and  max|x-y| <= 2e-2 * max|y|
  FP16 storage with power-of-two column scales (11-bit significands):
                 ||x-y||_F <= 1e-3 * ||y||_F   and  max|x-y| <= 3e-3 * max|y|
Index work (CSF, partition, row placement) is exact: an error there shows up
as whole wrong rows, far outside these bounds.
"""
import numpy as np
import pytest

import tentaco_gb300 as tt
from helpers import golden_csf, golden_files, host_taco, rel_errors, to_oracle
from oracle import oracle as O

pytestmark = pytest.mark.gpu

FP32_MAX, FP32_FRO = 2e-5, 1e-5
BF16_MAX, BF16_FRO = 2e-2, 8e-3
FP16_MAX, FP16_FRO = 3e-3, 1e-3


def close(got, ref, prec="fp32"):
    mx, fr = {"fp32": (FP32_MAX, FP32_FRO), "fp16": (FP16_MAX, FP16_FRO)}.get(prec, (BF16_MAX, BF16_FRO))
    amax = np.abs(ref).max() if ref.size else 0.0
    err = np.abs(got.astype(np.float64) - ref).max() if ref.size else 0.0
    e = rel_errors(got, ref)
    assert err <= mx * max(amax, 1e-30) + 1e-30, (err, amax, e)
    assert e["fro"] <= fr or np.linalg.norm(ref) == 0, e
    return e


def run_plan(B, factors, prec="fp32", select=tt.SELECT_DEFAULT, variant=0, reps=1, slabs=None):
    R = factors[0].shape[1]
    plan = tt.Plan(B, rank=R, prec=prec, select=select, variant=variant, slabs=slabs)
    bufs = [tt.DeviceBuffer.from_array(f.astype(np.float32)) for f in factors]
    plan.set_factors(bufs)
    A = tt.DeviceBuffer(B.dims[0] * R * 4)
    outs = []
    for _ in range(reps):
        plan.mttkrp(A)
        outs.append(A.to_array((B.dims[0], R)))
    assert plan.device_error() == 0
    return outs if reps > 1 else outs[0], plan


@pytest.mark.parametrize("path", golden_files("mttkrp"), ids=lambda p: p.split("/")[-1])
def test_golden_vectors(path):
    z = np.load(path)
    csf = golden_csf(z)
    facs = [z[f"F{m}"].astype(np.float32) for m in range(1, int(z["order"]))]
    B = host_taco(csf)
    got, _ = run_plan(B, facs)
    close(got, z["A"])
    got2 = tt.mttkrp_host(B, facs)
    close(got2, z["A"])
    assert np.array_equal(got, got2)


@pytest.fixture(scope="module")
def c1():
    """Uniform 1024^3 tensor: 1,000,000 distinct uniform coordinates, U(0,1), R=32 U(0,1)."""
    B = tt.gen_zipf((1024, 1024, 1024), (0, 0, 0), 1_000_000, seed=1)
    C = tt.gen_dense(1024, 32, 0, 11)
    D = tt.gen_dense(1024, 32, 0, 12)
    ref = O.mttkrp(to_oracle(B), [C, D])
    return B, [C, D], ref


def test_c1_every_variant(c1):
    B, facs, ref = c1
    nvalid = 0
    for v in range(tt.num_variants()):
        if not tt.variant_valid(v, 3, 32, "fp32"):
            continue
        print("variant", v, tt.variant_info(v)["name"], flush=True)
        try:
            got, plan = run_plan(B, facs, select=tt.SELECT_FIXED, variant=v)
        except tt.TTError as e:
            # staged variants whose largest fiber window does not fit shared memory
            assert e.status == tt.TT_ERR_UNSUPPORTED and tt.variant_info(v)["staged"] == 1
            continue
        nvalid += 1
        assert plan.variant == v
        close(got, ref)
    assert nvalid >= 50


def test_c1_deterministic_repeated_calls(c1):
    B, facs, ref = c1
    outs, _ = run_plan(B, facs, reps=4)
    for o in outs[1:]:
        assert np.array_equal(o, outs[0])
    close(outs[-1], ref)


@pytest.mark.parametrize("prec", ["bf16", "bf16f", "fp16"])
def test_c1_16bit_storage(c1, prec):
    B, facs, ref = c1
    got, _ = run_plan(B, facs, prec=prec)
    e = close(got, ref, prec)
    print(prec, e)


@pytest.fixture(scope="module")
def skewed():
    """Zipf rows and fibers with empty slices; N(0,1) factors with per-column scales."""
    B = tt.gen_zipf((3000, 2000, 5000), (1.2, 1.1, 0), 300_000, seed=21)
    return B, to_oracle(B)


@pytest.mark.parametrize("R", [1, 8, 10, 16, 20, 32, 40, 64])
def test_ranks(skewed, R):
    B, Oc = skewed
    facs = [tt.gen_dense(2000, R, 1, 30 + R), tt.gen_dense(5000, R, 1, 60 + R)]
    ref = O.mttkrp(Oc, facs)
    for v in {tt.default_variant(3, R, "fp32"), tt.variant_valid(39, 3, R) and 39 or 0}:
        if tt.variant_valid(v, 3, R):
            got, _ = run_plan(B, facs, select=tt.SELECT_FIXED, variant=v)
            close(got, ref)
    for prec in ("bf16", "fp16"):
        got, _ = run_plan(B, facs, prec=prec)
        close(got, ref, prec)


def test_long_fiber_spans_many_blocks():
    # one fiber of 200k nonzeros (hundreds of blocks) between short rows
    L = 200_000
    rng = np.random.default_rng(4)
    co = [np.array([[5, 3, l] for l in range(L)])]
    co.append(np.stack([rng.integers(0, 20, 500), rng.integers(0, 10, 500), rng.integers(0, L, 500)], 1))
    co = np.concatenate(co).astype(np.int32)
    B = tt.csf_from_coo((20, 10, L), co, rng.random(len(co)).astype(np.float32))
    facs = [tt.gen_dense(10, 32, 1, 1), tt.gen_dense(L, 32, 1, 2)]
    ref = O.mttkrp(to_oracle(B), facs)
    for v in (0, 17, 39, 41, 57, 65):
        if tt.variant_valid(v, 3, 32):
            got, _ = run_plan(B, facs, select=tt.SELECT_FIXED, variant=v)
            close(got, ref)


def test_edge_cases():
    facs = [np.ones((4, 8), np.float32), np.ones((4, 8), np.float32)]
    # empty tensor: all-zero output
    B0 = tt.csf_from_coo((6, 4, 4), np.zeros((0, 3), np.int32), np.zeros(0, np.float32))
    got, _ = run_plan(B0, facs)
    assert np.array_equal(got, np.zeros((6, 8), np.float32))
    # one nonzero in the last row
    B1 = tt.csf_from_coo((6, 4, 4), np.array([[5, 2, 3]], np.int32), np.array([2.5], np.float32))
    got, _ = run_plan(B1, facs)
    exp = np.zeros((6, 8), np.float32)
    exp[5] = 2.5
    assert np.array_equal(got, exp)
    # a single row holding everything, and empty leading/trailing rows
    rng = np.random.default_rng(8)
    co = np.stack([np.full(3000, 7), rng.integers(0, 50, 3000), rng.integers(0, 60, 3000)], 1).astype(np.int32)
    B2 = tt.csf_from_coo((15, 50, 60), co, rng.random(3000).astype(np.float32))
    f2 = [tt.gen_dense(50, 16, 0, 3), tt.gen_dense(60, 16, 0, 4)]
    got, _ = run_plan(B2, f2)
    close(got, O.mttkrp(to_oracle(B2), f2))


def test_compressed_root_with_gaps():
    # root listed as {pos=[0,3], crd=[2,5,9]} of 12 rows: unlisted rows stay zero
    rng = np.random.default_rng(12)
    dims = (12, 30, 40)
    co = np.stack([rng.choice([2, 5, 9], 900), rng.integers(0, 30, 900), rng.integers(0, 40, 900)], 1)
    Oc = O.build_csf(dims, co, rng.random(900))
    facs = [tt.gen_dense(30, 32, 0, 5), tt.gen_dense(40, 32, 0, 6)]
    ref = O.mttkrp(Oc, facs)
    rows = np.array([2, 5, 9], np.int32)
    p1 = np.concatenate([[0], np.cumsum(np.diff(Oc.pos[1])[rows])]).astype(np.int32)
    lv = [(np.array([0, 3], np.int32), rows), (p1, Oc.crd[1].astype(np.int32)),
          (Oc.pos[2].astype(np.int32), Oc.crd[2].astype(np.int32))]
    B = tt.HostTaco(dims, vals=Oc.vals.astype(np.float32), levels=lv, dense_root=False)
    got, _ = run_plan(B, facs)
    close(got, ref)


@pytest.fixture(scope="module")
def c5_small():
    """The 80M-nonzero 4-mode family scaled to 2M nonzeros: 4-mode, Zipf(1.2) on modes 0 and 3."""
    B = tt.gen_zipf((5000, 3000, 2000, 100000), (1.2, 0, 0, 1.2), 2_000_000, seed=5)
    facs = [tt.gen_dense(d, 32, 1, 50 + m) for m, d in enumerate((3000, 2000, 100000))]
    return B, facs, O.mttkrp(to_oracle(B), facs)


def test_mttkrp4_variants(c5_small):
    B, facs, ref = c5_small
    for v in range(tt.num_variants()):
        if tt.variant_valid(v, 4, 32, "fp32") and v % 3 == 0:
            try:
                got, _ = run_plan(B, facs, select=tt.SELECT_FIXED, variant=v)
            except tt.TTError as e:
                assert e.status == tt.TT_ERR_UNSUPPORTED
                continue
            close(got, ref)
    got, _ = run_plan(B, facs)
    close(got, ref)
    for prec in ("bf16", "bf16f", "fp16"):
        got, _ = run_plan(B, facs, prec=prec)
        print(prec, close(got, ref, prec))


def test_sweep_selects_a_timed_variant(c1):
    B, facs, ref = c1
    got, plan = run_plan(B, facs, select=tt.SELECT_SWEEP)
    times = plan.sweep_times()
    assert plan.selected_by == 2
    timed = times[times > 0]
    assert len(timed) >= 50 and times[plan.variant] == timed.min()
    close(got, ref)


@pytest.mark.parametrize("slabs", [2, 3, 16])
def test_slabs_parity(skewed, slabs):
    """Leaf-mode slabs: one pass per slab adding into A, for every family."""
    B, Oc = skewed
    facs = [tt.gen_dense(2000, 32, 1, 71), tt.gen_dense(5000, 32, 1, 72)]
    ref = O.mttkrp(Oc, facs)
    for prec in ("fp32", "fp16"):
        got, plan = run_plan(B, facs, prec=prec, slabs=slabs)
        assert plan.slabs == slabs
        close(got, ref, prec)
        for v in (8, 13, 18, 49, 54, 97):
            if tt.variant_valid(v, 3, 32, prec):
                try:
                    outs, _ = run_plan(B, facs, prec=prec, select=tt.SELECT_FIXED, variant=v, slabs=slabs, reps=2)
                except tt.TTError as e:
                    assert e.status == tt.TT_ERR_UNSUPPORTED
                    continue
                assert np.array_equal(outs[0], outs[1])  # passes add in a fixed order
                close(outs[0], ref, prec)


def test_timing_modes(skewed):
    """Timing mode 1 times the call and its walk kernel, mode 2 the call only (no event between the walk
    and the merge kernels); the results are the same bits in every mode."""
    B, Oc = skewed
    facs = [tt.gen_dense(2000, 32, 1, 81), tt.gen_dense(5000, 32, 1, 82)]
    ref = O.mttkrp(Oc, facs)
    v = next(v for v in range(tt.num_variants())
             if tt.variant_valid(v, 3, 32, "fp16") and tt.variant_info(v)["staged"] == 4)
    plan = tt.Plan(B, rank=32, prec="fp16", select=tt.SELECT_FIXED, variant=v, slabs=3)
    plan.set_factors([tt.DeviceBuffer.from_array(f) for f in facs])
    A = tt.DeviceBuffer(B.dims[0] * 32 * 4)
    outs = []
    for mode in (0, 1, 2, 1):
        plan.set_timing(mode)
        plan.mttkrp(A)
        outs.append(A.to_array((B.dims[0], 32)))
        if mode == 1:
            assert 0 < plan.last_kernel_ms() <= plan.last_ms()
        if mode == 2:
            assert plan.last_ms() > 0 and plan.last_kernel_ms() == -1
    for o in outs[1:]:
        assert np.array_equal(o, outs[0])
    close(outs[0], ref, "fp16")
    with pytest.raises(tt.TTError) as e:
        plan.set_timing(3)
    assert e.value.status == tt.TT_ERR_INVALID_ARGUMENT


def test_failed_variant_switch_blocks_calls(skewed):
    """A failed switch (the flat family on a slab plan) leaves the plan without a
    variant: a call reports an error instead of launching, until a switch succeeds."""
    B, Oc = skewed
    facs = [tt.gen_dense(2000, 32, 1, 71), tt.gen_dense(5000, 32, 1, 72)]
    ref = O.mttkrp(Oc, facs)
    plan = tt.Plan(B, rank=32, prec="fp32", slabs=2)
    good = plan.variant
    bufs = [tt.DeviceBuffer.from_array(f.astype(np.float32)) for f in facs]
    plan.set_factors(bufs)
    A = tt.DeviceBuffer(B.dims[0] * 32 * 4)
    flat = [v for v in range(tt.num_variants())
            if tt.variant_info(v)["staged"] == 3 and tt.variant_valid(v, 3, 32, "fp32")]
    assert flat
    with pytest.raises(tt.TTError) as e:
        plan.use_variant(flat[0])
    assert e.value.status == tt.TT_ERR_UNSUPPORTED
    with pytest.raises(tt.TTError) as e:
        plan.mttkrp(A)
    assert e.value.status == tt.TT_ERR_INVALID_ARGUMENT
    plan.use_variant(good)
    plan.mttkrp(A)
    close(A.to_array((B.dims[0], 32)), ref)
    assert plan.device_error() == 0


def test_slabs_long_fiber_and_order4(c5_small):
    # a fiber crossing every slab, rows spanning many warp tiles
    L = 200_000
    rng = np.random.default_rng(9)
    co = np.concatenate([np.array([[5, 3, l] for l in range(0, L, 2)]),
                         np.stack([rng.integers(0, 20, 800), rng.integers(0, 10, 800), rng.integers(0, L, 800)], 1)])
    B = tt.csf_from_coo((20, 10, L), co.astype(np.int32), rng.random(len(co)).astype(np.float32))
    facs = [tt.gen_dense(10, 32, 1, 1), tt.gen_dense(L, 32, 1, 2)]
    ref = O.mttkrp(to_oracle(B), facs)
    for slabs in (4, 7):
        got, _ = run_plan(B, facs, slabs=slabs)
        close(got, ref)
    B4, facs4, ref4 = c5_small
    for slabs in (2, 5):
        for prec in ("fp32", "fp16"):
            got, plan = run_plan(B4, facs4, prec=prec, slabs=slabs)
            assert plan.slabs == slabs
            close(got, ref4, prec)


def test_slabs_over_large_leaf_factor():
    # leaf factor 2M x 32 FP32 = 256 MB: automatic slabs of at most 44 MB (6), then
    # explicit counts (8 slabs: 32 MB of FP32, 16 MB of FP16)
    B = tt.gen_zipf((1000, 800, 2_000_000), (0.5, 0, 0), 300_000, seed=31)
    facs = [tt.gen_dense(800, 32, 1, 3), tt.gen_dense(2_000_000, 32, 1, 4)]
    ref = O.mttkrp(to_oracle(B), facs)
    got, plan = run_plan(B, facs)
    assert plan.slabs == 6  # automatic: slabs of at most 44 MB of the leaf factor
    close(got, ref)
    got, plan = run_plan(B, facs, slabs=1)
    assert plan.slabs == 1
    close(got, ref)
    got, plan = run_plan(B, facs, slabs=8)
    assert plan.slabs == 8
    close(got, ref)
    got, plan = run_plan(B, facs, prec="fp16", slabs=8)
    close(got, ref, "fp16")


def test_plan_rejects_malformed_csf_on_device():
    """The plan's structure check runs on the device copies after upload: each
    malformed level is reported as TT_ERR_INVALID_CSF, for MTTKRP and TTV plans
    alike, and a well-formed tensor of the same shape passes."""
    def taco(levels, dims=(2, 3, 3)):
        lv = [None] + [(np.asarray(p, np.int32), np.asarray(c, np.int32)) for p, c in levels]
        return tt.HostTaco(dims, vals=np.ones(8, np.float32), levels=lv)
    ok = [([0, 1, 2], [0, 2]), ([0, 2, 3], [0, 1, 2])]
    bad = {
        "pos decreasing": [([0, 2, 1], [0, 2]), ([0, 2, 3], [0, 1, 2])],
        "crd out of range": [([0, 1, 2], [0, 3]), ([0, 2, 3], [0, 1, 2])],
        "empty inner fiber": [([0, 1, 2], [0, 2]), ([0, 0, 3], [0, 1, 2])],
        "leaf crd unsorted": [([0, 1, 2], [0, 2]), ([0, 2, 3], [1, 0, 2])],
        "leaf crd out of range": [([0, 1, 2], [0, 2]), ([0, 2, 3], [0, 1, 3])],
        "inner crd unsorted": [([0, 2, 2], [2, 0]), ([0, 1, 2], [0, 1])],
    }
    for op in (tt.OP_MTTKRP, tt.OP_TTV):
        tt.Plan(taco(ok), op=op, rank=8)
        for name, lv in bad.items():
            assert tt.lib().tt_csf_validate(taco(lv).ptr) == tt.TT_ERR_INVALID_CSF, name
            with pytest.raises(tt.TTError) as e:
                tt.Plan(taco(lv), op=op, rank=8)
            assert e.value.status == tt.TT_ERR_INVALID_CSF, (name, e.value)
    # a long valid tensor passes the device check and still computes the oracle's result
    B = tt.gen_zipf((300, 200, 5000), (0.7, 0.7, 0.3), 200_000, 3)
    C = tt.gen_dense(200, 8, 0, 1)
    D = tt.gen_dense(5000, 8, 0, 2)
    close(run_plan(B, [C, D])[0], O.mttkrp(to_oracle(B), [C, D]))


@pytest.mark.parametrize("order,prec", [(3, "fp32"), (3, "fp16"), (4, "fp32"), (4, "bf16")])
def test_other_output_modes(order, prec):
    """MTTKRP of every non-root mode (plan option `mode`: the tensor re-rooted at
    the mode, the other modes' factors in increasing mode order) against the
    any-mode FP64 oracle."""
    dims = (300, 200, 500) if order == 3 else (40, 30, 20, 500)
    zipf = (0.9, 0.6, 0.3) if order == 3 else (0.9, 0.5, 0.5, 0.3)
    B = tt.gen_zipf(dims, zipf, 200_000 if order == 3 else 150_000, 21 + order)
    Oc = to_oracle(B)
    co = O.coords_of(Oc)
    R = 16
    F = [tt.gen_dense(d, R, 0, 40 + n) for n, d in enumerate(dims)]
    for m in range(1, order):
        ref = O.mttkrp_coo(co, Oc.vals, F, m, dims[m])
        plan = tt.Plan(B, rank=R, prec=prec, mode=m)
        bufs = [tt.DeviceBuffer.from_array(F[n].astype(np.float32)) for n in range(order) if n != m]
        plan.set_factors(bufs)
        A = tt.DeviceBuffer(dims[m] * R * 4)
        plan.mttkrp(A)
        close(A.to_array((dims[m], R)), ref, prec)
        assert plan.device_error() == 0
    with pytest.raises(tt.TTError):
        tt.Plan(B, rank=R, mode=order)
    with pytest.raises(tt.TTError):
        tt.Plan(B, op=tt.OP_TTV, mode=1)


def test_one_shot_from_pinned_memory():
    """The one-shot call with the tensor, factors and output page-locked
    (tt_host_register): same result as from pageable memory."""
    B = tt.gen_zipf((3000, 800, 5000), (1.1, 0.5, 0.8), 400_000, seed=12)
    C, D = tt.gen_dense(800, 32, 1, 1), tt.gen_dense(5000, 32, 1, 2)
    ref = tt.mttkrp_host(B, [C, D])
    A = np.zeros((3000, 32), np.float32)
    arrays = B.host_arrays() + [C, D, A]
    tt.pin(arrays)
    tt.pin(arrays)  # registering twice is accepted
    try:
        got = tt.mttkrp_host(B, [C, D], out=A)
        assert got is A or np.shares_memory(got, A)
        assert np.array_equal(A, ref)
    finally:
        tt.unpin(arrays)
    close(A, O.mttkrp(to_oracle(B), [C, D]))
