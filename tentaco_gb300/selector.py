"""Learned variant selector: corpus sweep, training and evaluation.

The reference tunes its kernels by generating every variant
(generated_kernels/codegen.py:44-247), timing them with *_tune.sh and letting a
person pick.  Here the same exhaustive sweep (TT_SELECT_SWEEP) times every
variant of the walk table on a corpus of seeded synthetic tensors, and a small
network (tentaco_select.h: 12 features -> 3 x 64 -> one score per variant) is
trained on those timings with the library's own CUDA forward/backward/Adam
kernels.  Plans created with TT_SELECT_MODEL then run the variant the network
ranks first; regret against the sweep's best is measured on held-out tensors.

Corpus: 400 3-mode tensors; tensor t uses seed 4000 + t for its parameters
and its generator: mode sizes log-uniform in [1e3, 1e6], nnz log-uniform in
[1e5, 5e7], per-mode Zipf exponent U(0, 1.5), values U(0, 1), rank in
{8, 16, 32, 64}.  Tensors with t % 5 == 4 are held out (80/20 split by seed).

Targets: y_v = log2(ms_v / ms_best) for every variant timed on the tensor
(masked mean squared error; untimed variants are masked out).

The model file also records each feature's range over the training tensors; a
plan whose tensor falls outside it times the network's best few variants instead
of trusting its first choice (tt_plan_options::model_topk).

Usage (needs a GPU):
    python -m tentaco_gb300.selector corpus --out tentaco_gb300/selector_corpus.jsonl
    python -m tentaco_gb300.selector train --corpus ... --out tentaco_gb300/selector_model.bin
"""
from __future__ import annotations

import argparse
import json
import os
import struct
import sys
import time

import numpy as np

NIN = 12
HIDDEN = 64
MAGIC = b"TTSEL001"
CORPUS_SEED = 4000
CORPUS_SEED_O4 = 5000  # four-mode corpus: tensor t uses seed 5000 + t
PRECS = ("fp16", "fp32")  # storage classes 1 and 0


def storage_of(prec: str) -> int:
    return 0 if prec == "fp32" else 1


def split_of(t: int) -> str:
    return "test" if t % 5 == 4 else "train"


def corpus_params(t: int) -> dict:
    """Parameters of corpus tensor t (a pure function of t)."""
    rng = np.random.default_rng(CORPUS_SEED + t)
    dims = [int(round(10 ** rng.uniform(3, 6))) for _ in range(3)]
    nnz = int(round(10 ** rng.uniform(5, np.log10(5e7))))
    zipf = [float(rng.uniform(0, 1.5)) for _ in range(3)]
    rank = int(rng.choice([8, 16, 32, 64]))
    cap = dims[0] * dims[1] * dims[2] // 4  # keep the tensor well below full
    return {"t": t, "seed": CORPUS_SEED + t, "dims": dims, "nnz_target": min(nnz, cap), "zipf": zipf, "rank": rank}


def corpus_params_o4(t: int) -> dict:
    """Parameters of four-mode corpus tensor t (config 5's family: four modes of
    10^3-10^5, Zipf skew per mode, rank 8-64; at most 2*10^7 nonzeros so that a
    sweep of every variant stays short)."""
    rng = np.random.default_rng(CORPUS_SEED_O4 + t)
    # the CSF builder packs a nonzero's coordinates into one 64-bit key: mode sizes
    # are redrawn until their bits fit in 62 (config 5's 5,000 x 3,000 x 2,000 x
    # 100,000 needs 53)
    while True:
        dims = [int(round(10 ** rng.uniform(3, 5))) for _ in range(4)]
        if sum(int(np.ceil(np.log2(d))) for d in dims) <= 62:
            break
    nnz = int(round(10 ** rng.uniform(5, np.log10(2e7))))
    zipf = [float(rng.uniform(0, 1.5)) for _ in range(4)]
    rank = int(rng.choice([8, 16, 32, 64]))
    cap = dims[0] * dims[1] * dims[2] * dims[3] // 4
    return {"t": t, "seed": CORPUS_SEED_O4 + t, "dims": dims, "nnz_target": min(nnz, cap), "zipf": zipf,
            "rank": rank, "order": 4}


def params_for(t: int, order: int) -> dict:
    return corpus_params(t) if order == 3 else corpus_params_o4(t)


def corpus_tensor(r: dict):
    import tentaco_gb300 as tt
    return tt.gen_zipf(r["dims"], r["zipf"], r["nnz_target"], r["seed"], 0.0, 1.0, 8)


def run_corpus(out_path: str, n: int = 400, start: int = 0, precs=PRECS, log=sys.stdout, order: int = 3) -> None:
    """Sweep every variant on corpus tensors start..n-1 (three or four modes); one
    JSON line per (tensor, precision)."""
    import tentaco_gb300 as tt
    done = set()
    if os.path.exists(out_path):
        with open(out_path) as f:
            for line in f:
                if line.strip():
                    r = json.loads(line)
                    done.add((r["t"], r["prec"]))
    with open(out_path, "a") as f:
        for t in range(start, n):
            if all((t, p) in done for p in precs):
                continue
            r0 = params_for(t, order)
            t0 = time.time()
            B = corpus_tensor(r0)
            feats = B.features(r0["rank"])
            for prec in precs:
                if (t, prec) in done:
                    continue
                plan = tt.Plan(B, rank=r0["rank"], prec=prec, select=tt.SELECT_SWEEP)
                ms = [float(x) for x in plan.sweep_times()]
                valid = [m if m > 0 else np.inf for m in ms]
                rec = dict(r0, nnz=int(B.nnz), prec=prec, features=[float(x) for x in feats], ms=ms,
                           best=int(np.argmin(valid)),
                           default=int(tt.default_variant(order, r0["rank"], prec, int(B.nnz))))
                del plan
                f.write(json.dumps(rec) + "\n")
                f.flush()
            print(f"tensor {t} nnz {B.nnz} {time.time() - t0:.1f}s", file=log, flush=True)
            del B


# ---------------------------------------------------------------------------
# dataset, model file
# ---------------------------------------------------------------------------
def dataset(recs: list, storage: int, split: str | None):
    rs = [r for r in recs if storage_of(r["prec"]) == storage and (split is None or split_of(r["t"]) == split)]
    X = np.array([r["features"] for r in rs], dtype=np.float64)
    ms = np.array([r["ms"] for r in rs], dtype=np.float64)
    valid = ms > 0
    best = np.where(valid, ms, np.inf).min(axis=1, keepdims=True)
    T = np.where(valid, np.log2(np.where(valid, ms, 1.0) / best), 0.0)
    return rs, X, T, valid.astype(np.float64)


def write_model(path: str, models: list, order: int = 3) -> None:
    """Version 2 (three modes) or 3 (the tensor order recorded after the model
    count): per model storage, mean, sd, lo, hi (training feature range), params."""
    with open(path, "wb") as f:
        f.write(MAGIC)
        if order == 3:
            f.write(struct.pack("<5i", 2, NIN, HIDDEN, models[0]["nout"], len(models)))
        else:
            f.write(struct.pack("<6i", 3, NIN, HIDDEN, models[0]["nout"], len(models), order))
        for m in models:
            f.write(struct.pack("<i", m["storage"]))
            for key in ("mean", "sd", "lo", "hi"):
                f.write(np.asarray(m[key], dtype="<f4").tobytes())
            f.write(np.asarray(m["params"], dtype="<f4").tobytes())


def read_model(path: str) -> list:
    with open(path, "rb") as f:
        data = f.read()
    assert data[:8] == MAGIC, "not a selector model file"
    ver, nin, hid, nout, nm = struct.unpack_from("<5i", data, 8)
    assert ver in (1, 2, 3) and nin == NIN and hid == HIDDEN
    np_ = NIN * HIDDEN + HIDDEN + 2 * (HIDDEN * HIDDEN + HIDDEN) + HIDDEN * nout + nout
    off = 28
    order = 3
    if ver == 3:
        (order,) = struct.unpack_from("<i", data, off)
        off += 4
    out = []
    for _ in range(nm):
        (storage,) = struct.unpack_from("<i", data, off)
        off += 4
        mean = np.frombuffer(data, "<f4", NIN, off); off += 4 * NIN
        sd = np.frombuffer(data, "<f4", NIN, off); off += 4 * NIN
        if ver >= 2:
            lo = np.frombuffer(data, "<f4", NIN, off).copy(); off += 4 * NIN
            hi = np.frombuffer(data, "<f4", NIN, off).copy(); off += 4 * NIN
        else:  # no recorded range: every tensor counts as inside it
            lo = np.full(NIN, -np.inf, np.float32)
            hi = np.full(NIN, np.inf, np.float32)
        params = np.frombuffer(data, "<f4", np_, off); off += 4 * np_
        out.append({"storage": storage, "nout": nout, "mean": mean.copy(), "sd": sd.copy(), "lo": lo, "hi": hi,
                    "params": params.copy(), "order": order})
    assert off == len(data)
    return out


# ---------------------------------------------------------------------------
# training (library kernels) and evaluation
# ---------------------------------------------------------------------------
def feature_range(recs: list, storage: int):
    """Per-feature min and max over the training tensors of a storage class (FP32)."""
    _, X, _, _ = dataset(recs, storage, "train")
    return X.min(axis=0).astype(np.float32), X.max(axis=0).astype(np.float32)


def in_range(m: dict, feats) -> bool:
    f = np.asarray(feats, dtype=np.float32)
    return bool(np.all(f >= m["lo"]) and np.all(f <= m["hi"]))


def init_params(nout: int, seed: int) -> np.ndarray:
    """He-normal weights, zero biases, in the library's flat layout."""
    rng = np.random.default_rng(seed)
    dims = [(NIN, HIDDEN), (HIDDEN, HIDDEN), (HIDDEN, HIDDEN), (HIDDEN, nout)]
    parts = []
    for k, n in dims:
        parts.append(rng.normal(0, np.sqrt(2.0 / k), k * n))
        parts.append(np.zeros(n))
    return np.concatenate(parts).astype(np.float32)


def train(recs: list, storage: int, nout: int, steps: int = 3000, lr: float = 3e-4, wd: float = 3e-3,
          seed: int = 0, log=sys.stdout) -> dict:
    import tentaco_gb300 as tt
    _, X, T, M = dataset(recs, storage, "train")
    mean = X.mean(axis=0)
    sd = X.std(axis=0)
    sd[sd < 1e-6] = 1.0
    Xn = ((X - mean) / sd).astype(np.float32)
    net = tt.Mlp(nout, Xn.shape[0])
    params, losses = net.train(init_params(nout, seed), Xn, T.astype(np.float32), M.astype(np.float32),
                               steps=steps, lr=lr, weight_decay=wd)
    print(f"storage {storage}: {Xn.shape[0]} tensors, loss {losses[0]:.4f} -> {losses[-1]:.4f}", file=log)
    lo, hi = feature_range(recs, storage)
    return {"storage": storage, "nout": nout, "mean": mean.astype(np.float32), "sd": sd.astype(np.float32),
            "lo": lo, "hi": hi, "params": params}


def pick(scores: np.ndarray, ms: np.ndarray) -> int:
    """The first variant in score order that the sweep could time on this tensor
    (what a plan does: a staged variant that does not fit is skipped)."""
    for v in np.argsort(scores, kind="stable"):
        if np.isfinite(scores[v]) and ms[v] > 0:
            return int(v)
    return -1


def heuristic_pick(r: dict) -> int:
    """The fixed heuristic's variant for a corpus record (the library's current rule)."""
    try:
        import tentaco_gb300 as tt
        return int(tt.default_variant(r.get("order", 3), r["rank"], r["prec"], r["nnz"]))
    except Exception:  # library not built: the rule recorded with the sweep
        return int(r["default"])


def evaluate(recs: list, models: dict, forward, split: str = "test") -> dict:
    """Per storage class: mean/max regret of the model's pick and of the heuristic."""
    out = {}
    for storage, m in models.items():
        rs, X, _, M = dataset(recs, storage, split)
        if not rs:
            continue
        Xn = (X - m["mean"].astype(np.float64)) / m["sd"].astype(np.float64)
        S = forward(m["params"].astype(np.float64), Xn)
        reg, regh, within = [], [], 0
        for i, r in enumerate(rs):
            ms = np.array(r["ms"])
            best = ms[ms > 0].min()
            sc = np.where(M[i] > 0, S[i], np.inf)
            v = pick(sc, ms)
            reg.append(ms[v] / best - 1.0)
            within += ms[v] <= 1.10 * best
            d = heuristic_pick(r)
            regh.append((ms[d] if ms[d] > 0 else np.nan) / best - 1.0)
        reg = np.array(reg)
        regh = np.array(regh)
        out[storage] = {"n": len(rs), "model_mean_regret": float(reg.mean()), "model_max_regret": float(reg.max()),
                        "model_within_10pct": float(within / len(rs)),
                        "heuristic_mean_regret": float(np.nanmean(regh)),
                        "heuristic_max_regret": float(np.nanmax(regh))}
    return out


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(prog="python -m tentaco_gb300.selector")
    sub = ap.add_subparsers(dest="cmd", required=True)
    c = sub.add_parser("corpus")
    c.add_argument("--out", required=True)
    c.add_argument("--n", type=int, default=400)
    c.add_argument("--start", type=int, default=0)
    c.add_argument("--order", type=int, default=3, choices=[3, 4])
    t = sub.add_parser("train")
    t.add_argument("--corpus", required=True)
    t.add_argument("--out", required=True)
    t.add_argument("--steps", type=int, default=3000)
    t.add_argument("--lr", type=float, default=3e-4)
    t.add_argument("--wd", type=float, default=3e-3, help="decoupled weight decay")
    t.add_argument("--seed", type=int, default=0, help="seed of the initial weights")
    t.add_argument("--report", default=None, help="write the held-out regret report (JSON) here")
    t.add_argument("--order", type=int, default=3, choices=[3, 4], help="tensor order of the corpus")
    a = ap.parse_args(argv)
    if a.cmd == "corpus":
        run_corpus(a.out, a.n, a.start, order=a.order)
        return 0
    import tentaco_gb300 as tt
    with open(a.corpus) as f:
        recs = [json.loads(l) for l in f if l.strip()]
    nout = len(recs[0]["ms"])
    models = [train(recs, s, nout, steps=a.steps, lr=a.lr, wd=a.wd, seed=a.seed) for s in (0, 1)]
    write_model(a.out, models, order=a.order)
    net = tt.Mlp(nout, 1024)
    rep = evaluate(recs, {m["storage"]: m for m in models},
                   forward=lambda p, X: net.forward(p.astype(np.float32), X.astype(np.float32)).astype(np.float64))
    print(json.dumps(rep, indent=1))
    if a.report:
        with open(a.report, "w") as f:
            json.dump(rep, f, indent=1)
    return 0


if __name__ == "__main__":
    sys.exit(main())
