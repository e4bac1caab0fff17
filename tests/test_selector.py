"""Learned variant selector: the network's training kernels against the FP64
oracle, the committed model file, and what the model gains over the heuristic.

CPU tests check the oracle gradient by finite differences and the committed
corpus/model files; GPU tests check the library's forward/backward/Adam
kernels against the oracle and the product's inference path (TT_SELECT_MODEL)
against the committed sweep timings of the held-out tensors.
"""
import json
import os

import numpy as np
import pytest

import tentaco_gb300 as tt
from oracle import oracle as orc

HERE = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.dirname(tt.__file__)
CORPUS = os.path.join(PKG, "selector_corpus.jsonl")
MODEL = os.path.join(PKG, "selector_model.bin")
NOUT = tt.num_variants()  # one network output per variant of the table


def _model_nout():
    """Outputs of the committed model: the variants its corpus was swept over."""
    with open(CORPUS) as fh:
        return len(json.loads(fh.readline())["ms"])


def _rand_problem(seed, B=24, nout=NOUT):
    rng = np.random.default_rng(seed)
    n = orc.mlp_num_params(nout)
    params = rng.normal(0, 0.2, n)
    X = rng.normal(0, 1, (B, 12))
    T = rng.normal(0, 1, (B, nout))
    M = (rng.random((B, nout)) < 0.7).astype(np.float64)
    return params, X, T, M


def test_oracle_grad_matches_finite_differences():
    params, X, T, M = _rand_problem(1, B=6, nout=10)
    loss, g = orc.mlp_grad(params, 10, X, T, M)
    rng = np.random.default_rng(2)
    idx = rng.choice(params.size, 40, replace=False)
    h = 1e-6
    for i in idx:
        p1 = params.copy(); p1[i] += h
        p0 = params.copy(); p0[i] -= h
        fd = (orc.mlp_grad(p1, 10, X, T, M)[0] - orc.mlp_grad(p0, 10, X, T, M)[0]) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 + 1e-5 * abs(fd), (i, fd, g[i])
    out = orc.mlp_forward(params, 10, X)
    assert abs(loss - float(((out - T) ** 2 * M).sum() / M.sum())) < 1e-12


def test_param_count_agrees():
    assert tt.mlp_num_params(NOUT) == orc.mlp_num_params(NOUT) == 12 * 64 + 64 + 2 * (64 * 64 + 64) + 64 * NOUT + NOUT


def _corpus():
    if not os.path.exists(CORPUS):
        pytest.skip("no committed selector corpus")
    with open(CORPUS) as f:
        return [json.loads(l) for l in f if l.strip()]


def test_corpus_and_model_files():
    recs = _corpus()
    assert len(recs) >= 300
    for r in recs[:20]:
        assert len(r["features"]) == 12 and len(r["ms"]) == _model_nout() <= NOUT
        assert r["best"] == int(np.argmin([t if t > 0 else np.inf for t in r["ms"]]))
    assert os.path.exists(MODEL)
    from tentaco_gb300 import selector
    models = selector.read_model(MODEL)
    assert {m["storage"] for m in models} == {0, 1}
    for m in models:
        assert m["params"].size == orc.mlp_num_params(_model_nout())


def test_model_beats_heuristic_on_held_out():
    """Regret of the committed model on the held-out tensors (FP64 oracle forward,
    same weights the library loads) vs the fixed heuristic, from the committed
    sweep timings."""
    from tentaco_gb300 import selector
    recs = _corpus()
    models = {m["storage"]: m for m in selector.read_model(MODEL)}
    nout = _model_nout()
    rep = selector.evaluate(recs, models, forward=lambda p, X: orc.mlp_forward(p, nout, X), split="test")
    for storage, r in rep.items():
        assert r["n"] >= 20
        assert r["model_mean_regret"] <= 0.10, r
        assert r["model_mean_regret"] < r["heuristic_mean_regret"], r


def test_model_file_ranges_and_versions(tmp_path):
    """The committed model records the training feature range (version 2), a
    version-1 file reads as unbounded, and the library loads both."""
    from tentaco_gb300 import selector
    recs = _corpus()
    models = selector.read_model(MODEL)
    for m in models:
        lo, hi = selector.feature_range(recs, m["storage"])
        assert np.array_equal(m["lo"], lo) and np.array_equal(m["hi"], hi)
        assert np.all(np.isfinite(m["lo"])) and np.all(m["lo"] <= m["hi"])
    train = [r for r in recs if selector.split_of(r["t"]) == "train"]
    assert all(selector.in_range(models[0], r["features"]) for r in train[:50])
    # a 100M-nonzero tensor with a 2M-long leaf mode lies outside the corpus
    far = np.array(train[0]["features"], dtype=np.float32)
    far[2], far[3] = 20.93, 26.58
    assert not selector.in_range(models[0], far)
    v1 = tmp_path / "v1.bin"
    raw = open(MODEL, "rb").read()
    import struct
    ver, nin, hid, nout, nm = struct.unpack_from("<5i", raw, 8)
    assert ver == 2
    out = bytearray(raw[:8] + struct.pack("<5i", 1, nin, hid, nout, nm))
    off = 28
    np_ = orc.mlp_num_params(nout)
    for _ in range(nm):
        out += raw[off:off + 4 + 8 * nin]          # storage, mean, sd
        off += 4 + 16 * nin                         # skip lo, hi
        out += raw[off:off + 4 * np_]
        off += 4 * np_
    assert off == len(raw)
    v1.write_bytes(bytes(out))
    old = selector.read_model(str(v1))
    assert all(np.all(np.isinf(m["lo"])) for m in old)
    assert all(np.array_equal(a["params"], b["params"]) for a, b in zip(old, models))
    tt.selector_load(str(v1))
    assert tt.selector_models() == 2
    tt.selector_load(MODEL)
    assert tt.selector_models() == 2
    bad = tmp_path / "bad.bin"
    bad.write_bytes(raw[:-4])
    with pytest.raises(tt.TTError):
        tt.selector_load(str(bad))


@pytest.mark.gpu
def test_gpu_grad_matches_oracle():
    params, X, T, M = _rand_problem(3)
    B = X.shape[0]
    loss_ref, g_ref = orc.mlp_grad(params, NOUT, X, T, M)
    net = tt.Mlp(NOUT, B)
    loss, g = net.grad(params.astype(np.float32), X.astype(np.float32), T.astype(np.float32), M.astype(np.float32))
    assert abs(loss - loss_ref) <= 1e-5 * abs(loss_ref) + 1e-7
    err = np.linalg.norm(g - g_ref) / np.linalg.norm(g_ref)
    assert err < 1e-5, err
    out = net.forward(params.astype(np.float32), X.astype(np.float32))
    ref = orc.mlp_forward(params, NOUT, X)
    assert np.abs(out - ref).max() <= 1e-5 * (1 + np.abs(ref).max())


@pytest.mark.gpu
def test_gpu_training_is_deterministic_and_learns():
    params, X, T, M = _rand_problem(4, B=64)
    runs = []
    for _ in range(2):
        net = tt.Mlp(NOUT, X.shape[0])
        p, losses = net.train(params.astype(np.float32), X.astype(np.float32), T.astype(np.float32),
                              M.astype(np.float32), steps=200, lr=3e-3)
        runs.append((p, losses))
    assert np.array_equal(runs[0][0], runs[1][0])
    assert runs[0][1][-1] < 0.5 * runs[0][1][0]


def _library_vs_offline(model_path, recs):
    """For each record: the library's pick (device inference, FP32) and the offline
    pick (FP64 oracle forward of the same weights), both the best-scored variant
    that runs on the tensor, as a plan picks it; and the heuristic's variant."""
    from tentaco_gb300 import selector
    tt.selector_load(model_path)
    models = {m["storage"]: m for m in selector.read_model(model_path)}
    out = []
    for r in recs:
        B = selector.corpus_tensor(r)
        ms = np.array(r["ms"])
        lib_pick = selector.pick(tt.selector_scores(B, r["rank"], r["prec"]), ms)
        m = models[selector.storage_of(r["prec"])]
        x = (np.array(r["features"]) - m["mean"].astype(np.float64)) / m["sd"].astype(np.float64)
        off = orc.mlp_forward(m["params"].astype(np.float64), len(ms), x[None, :])[0]
        out.append((r, ms, lib_pick, selector.pick(off, ms), selector.heuristic_pick(r)))
    return out


def _check_product(rows, bound):
    agree = sum(lib == off for _, _, lib, off, _ in rows)
    # FP32 device inference may order near-ties differently from the FP64 oracle
    assert agree >= 0.9 * len(rows), (agree, len(rows))
    reg_m = [ms[lib] / ms[r["best"]] - 1 for r, ms, lib, _, _ in rows if ms[lib] > 0]
    reg_h = [ms[d] / ms[r["best"]] - 1 for r, ms, _, _, d in rows if ms[d] > 0]
    assert len(reg_m) >= 0.75 * len(rows)
    assert np.mean(reg_m) <= bound, np.mean(reg_m)
    assert np.mean(reg_m) < np.mean(reg_h)


@pytest.mark.gpu
def test_product_selector_regret_on_held_out():
    """TT_SELECT_MODEL's inference through the library on the 40 smallest
    regenerated held-out tensors: its picks are the offline model's (the 10% bound
    over every held-out tensor is test_model_beats_heuristic_on_held_out), and
    their regret beats the heuristic's.  These tensors run in tens of microseconds,
    where the sweep's timings are noisiest: regret measured 10.5% on them against
    8.7% / 8.6% over the whole held-out set, so the bound here is 12%."""
    from tentaco_gb300 import selector
    recs = [r for r in _corpus() if selector.split_of(r["t"]) == "test"]
    _check_product(_library_vs_offline(MODEL, sorted(recs, key=lambda r: r["nnz"])[:40]), 0.12)


@pytest.mark.gpu
def test_model_topk_times_candidates():
    """model_topk > 1 times the network's best-ranked variants (and the fixed
    heuristic's, then neighbours of the fastest) at plan creation and keeps the
    fastest; automatic selection
    trusts the network inside its training range and times candidates outside it."""
    from tentaco_gb300 import selector
    tt.selector_load(MODEL)
    recs = [r for r in _corpus() if selector.split_of(r["t"]) == "test"]
    r = sorted(recs, key=lambda r: r["nnz"])[5]
    B = selector.corpus_tensor(r)
    auto = tt.Plan(B, rank=r["rank"], prec=r["prec"], select=tt.SELECT_MODEL)
    assert auto.selected_by == 1
    assert np.all(auto.sweep_times() < 0)
    plan = tt.Plan(B, rank=r["rank"], prec=r["prec"], select=tt.SELECT_MODEL, model_topk=4)
    assert plan.selected_by == 3
    ms = plan.sweep_times()
    timed = np.flatnonzero(ms > 0)
    assert 4 <= timed.size <= 5 + 10  # 4 candidates, the heuristic's, two rounds of 5 neighbours
    assert plan.variant == timed[np.argmin(ms[timed])]
    assert auto.variant in timed  # the network's first runnable choice is a candidate
    # mode sizes of 100 are below the corpus's 10^3: outside the training range
    small = tt.gen_zipf((100, 120, 140), (0.5, 0.5, 0.5), 20_000, 7)
    far = tt.Plan(small, rank=32, prec="fp16", select=tt.SELECT_MODEL)
    assert far.selected_by == 3
    assert np.count_nonzero(far.sweep_times() > 0) >= 6
    with pytest.raises(tt.TTError):
        tt.Plan(small, rank=32, prec="fp16", select=tt.SELECT_MODEL, model_topk=17)


@pytest.mark.parametrize("order", [3, 4])
def test_features_match_a_numpy_restatement(order):
    """The 12 selector features (tt_csf_features) from the CSF arrays, restated in
    numpy: mode sizes, nnz, nnz per row and per last-level fiber, the spread and
    skew of fiber lengths, and the spread of row nnz."""
    dims = (300, 200, 500) if order == 3 else (60, 40, 30, 200)
    B = tt.gen_zipf(dims, (1.2, 1.0) + (0,) * (order - 2), 40_000, seed=12)
    L = order - 1
    lens = np.diff(B.pos(L).astype(np.int64)).astype(np.float64)
    rows = B.pos(1).astype(np.int64)
    for l in range(2, L + 1):
        rows = B.pos(l).astype(np.int64)[rows]
    rnz = np.diff(rows).astype(np.float64)
    nnz = float(B.nnz)
    lg = lambda x: np.log2(max(1.0, x))  # noqa: E731
    mean, rm = nnz / lens.size, nnz / rnz.size
    ll = np.log2(np.maximum(1.0, lens))
    lvar = max(0.0, (ll * ll).mean() - ll.mean() ** 2)
    skew = ((ll - ll.mean()) ** 3).mean() / lvar ** 1.5 if lvar > 1e-12 else 0.0
    want = np.array([lg(dims[0]), lg(dims[1]), lg(dims[2]), lg(nnz), lg(rm), lg(mean),
                     np.sqrt(((lens - mean) ** 2).mean()) / mean, skew, lg(lens.max() / mean),
                     np.sqrt(((rnz - rm) ** 2).mean()) / rm, order, lg(32)])
    got = B.features(32).astype(np.float64)
    assert np.allclose(got, want, rtol=1e-5, atol=1e-5), (got, want)


# ---------------------------------------------------------------------------
# four modes: a model of its own (version-3 file recording the order), trained on
# a corpus of seeded four-mode tensors swept over every variant of the table
# ---------------------------------------------------------------------------
CORPUS_O4 = os.path.join(PKG, "selector_corpus_o4.jsonl")
MODEL_O4 = os.path.join(PKG, "selector_model_o4.bin")
# held-out mean regret bound of the four-mode model (measured 7.7% FP32 and 9.6%
# 16-bit storage over all 60 held-out tensors of each class, against 64% and 96%
# for the fixed heuristic)
O4_MEAN_REGRET = 0.10


def _corpus_o4():
    if not os.path.exists(CORPUS_O4):
        pytest.skip("no committed four-mode selector corpus")
    with open(CORPUS_O4) as f:
        return [json.loads(l) for l in f if l.strip()]


def test_o4_corpus_and_model_files():
    from tentaco_gb300 import selector
    recs = _corpus_o4()
    assert len(recs) >= 500
    for r in recs[:20]:
        assert r["order"] == 4 and len(r["dims"]) == 4
        assert len(r["features"]) == 12 and r["features"][10] == 4.0
        assert len(r["ms"]) == NOUT
        assert r["best"] == int(np.argmin([t if t > 0 else np.inf for t in r["ms"]]))
    models = selector.read_model(MODEL_O4)
    assert {m["storage"] for m in models} == {0, 1}
    for m in models:
        assert m["order"] == 4 and m["params"].size == orc.mlp_num_params(NOUT)
        lo, hi = selector.feature_range(recs, m["storage"])
        assert np.array_equal(m["lo"], lo) and np.array_equal(m["hi"], hi)


def test_o4_model_beats_heuristic_on_held_out():
    """Regret of the four-mode model on its held-out tensors (FP64 oracle forward
    of the committed weights) against the fixed heuristic (the strip rule), from
    the committed sweep timings."""
    from tentaco_gb300 import selector
    recs = _corpus_o4()
    models = {m["storage"]: m for m in selector.read_model(MODEL_O4)}
    rep = selector.evaluate(recs, models, forward=lambda p, X: orc.mlp_forward(p, NOUT, X), split="test")
    assert set(rep) == {0, 1}
    for storage, r in rep.items():
        assert r["n"] >= 50
        assert r["model_mean_regret"] <= O4_MEAN_REGRET, r
        assert r["model_mean_regret"] < r["heuristic_mean_regret"], r


def test_o4_model_loads_beside_the_three_mode_one():
    """A version-3 file replaces only its order's models."""
    tt.selector_load(MODEL)
    tt.selector_load(MODEL_O4)
    assert tt.selector_models(3) == 2 and tt.selector_models(4) == 2
    tt.selector_load(MODEL)
    assert tt.selector_models(3) == 2 and tt.selector_models(4) == 2


@pytest.mark.gpu
def test_product_selector_four_modes():
    """TT_SELECT_MODEL on regenerated held-out four-mode tensors: the library's
    device inference picks variants whose recorded sweep time is close to the best
    on average, better than the heuristic, and a plan made with it runs and uses
    the network's choice.  The pick is the best-scored variant that runs on the
    tensor, as a plan makes it: a staged variant whose fiber window does not fit in
    shared memory is valid for the shape but refused by the tensor (the sweep could
    not time it either), and the plan moves on to the next."""
    from tentaco_gb300 import selector
    recs = [r for r in _corpus_o4() if selector.split_of(r["t"]) == "test"]
    small = sorted(recs, key=lambda r: r["nnz"])[:40]
    _check_product(_library_vs_offline(MODEL_O4, small), 0.12)
    tt.selector_load(MODEL_O4)
    r = small[5]
    B = selector.corpus_tensor(r)
    plan = tt.Plan(B, rank=r["rank"], prec=r["prec"], select=tt.SELECT_MODEL)
    assert plan.selected_by in (1, 3)
