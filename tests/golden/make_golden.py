"""Generate tests/golden/*.npz from the reference's own CPU kernels.

Runs where the reference sources exist: ``make -C oracle`` compiles
tensor_kernels/mttkrp3_csf_cpu_taco.h, mttkrp3_csf_cpu_taco_workspace.h,
mttkrp4_csf_cpu_taco.h, mttkrp5_csf_cpu_taco.h and ttv_csf_cpu_taco.h unmodified into
oracle/_ref/libtaco_ref.so, and this script feeds them small seeded inputs.
Each fixture stores the inputs (canonical CSF as int64 arrays, float32-exact
values and factors) and the reference's FP64 outputs, so the oracle
restatement and the GPU kernels can be checked on hosts without the reference.

Usage:  python tests/golden/make_golden.py [--out DIR]   (default: this directory)
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
OUT = HERE

from oracle import oracle as O  # noqa: E402


def f32exact(a):
    return np.asarray(a, dtype=np.float32).astype(np.float64)


def coo(rng, dims, nnz, zipf=None):
    cols = []
    for m, d in enumerate(dims):
        if zipf and zipf[m] > 0:
            w = 1.0 / np.arange(1, d + 1) ** zipf[m]
            cols.append(rng.permutation(d)[rng.choice(d, size=nnz, p=w / w.sum())])
        else:
            cols.append(rng.integers(0, d, nnz))
    return np.stack(cols, 1)


def save_mttkrp(name, dims, coords, vals, R, rng, dist="uniform", factors=None):
    csf = O.build_csf(dims, coords, f32exact(vals))
    if factors is not None:
        facs = [f32exact(f) for f in factors]
    elif dist == "normal":
        facs = [f32exact(rng.standard_normal((d, R))) for d in dims[1:]]
    else:
        facs = [f32exact(rng.random((d, R))) for d in dims[1:]]
    A = O.ref_mttkrp(csf, facs)
    # five modes have the oracle only (no library kernel yet): their own kind keeps
    # them out of the library's golden tests
    kind = "mttkrp5" if len(dims) == 5 else "mttkrp"
    out = dict(kind=kind, order=len(dims), dims=np.array(dims), R=R, vals=csf.vals, A=A)
    for l in range(1, len(dims)):
        out[f"pos{l}"] = csf.pos[l]
        out[f"crd{l}"] = csf.crd[l]
    for m, f in enumerate(facs):
        out[f"F{m + 1}"] = f
    if len(dims) == 3:
        out["A_workspace"] = O.ref_mttkrp(csf, facs, workspace=True)
    np.savez_compressed(os.path.join(OUT, f"{name}.npz"), **out)
    return csf


def save_ttv(name, dims, coords, vals, rng):
    csf = O.build_csf(dims, coords, f32exact(vals))
    x = f32exact(rng.uniform(-1, 1, dims[2]))
    y = O.ref_ttv(csf, x)
    np.savez_compressed(os.path.join(OUT, f"{name}.npz"), kind="ttv", order=3, dims=np.array(dims),
                        pos1=csf.pos[1], crd1=csf.crd[1], pos2=csf.pos[2], crd2=csf.crd[2], vals=csf.vals,
                        x=x, y=y)


def main(out: str = HERE):
    global OUT
    OUT = out
    if O.ref_lib() is None:
        raise SystemExit("reference kernels could not be built (sources absent)")
    rng = np.random.default_rng(20261203)
    # hand case from the reference probe: A = [[59,104],[84,128]]
    save_mttkrp("mttkrp3_hand", (2, 2, 2), np.array([[0, 0, 1], [0, 1, 0], [1, 1, 1]]),
                np.array([2.0, 3.0, 4.0]), 2, rng,
                factors=[np.array([[1.0, 2.0], [3.0, 4.0]]), np.array([[5.0, 6.0], [7.0, 8.0]])])
    # uniform 3-mode (the 1024^3 uniform family, scaled down), ranks 8 and 32
    d = (96, 64, 80)
    save_mttkrp("mttkrp3_uniform_r32", d, coo(rng, d, 6000), rng.random(6000), 32, rng)
    save_mttkrp("mttkrp3_uniform_r8", d, coo(rng, d, 3000), rng.random(3000), 8, rng)
    # skewed rows with empty slices (Zipf on modes 0 and 1), N(0,1) factors, odd rank
    d = (300, 200, 500)
    save_mttkrp("mttkrp3_zipf_r20", d, coo(rng, d, 8000, zipf=(1.2, 1.1, 0)), rng.random(8000), 20, rng,
                dist="normal")
    # one long fiber spanning many blocks plus a few short ones
    L = 5000
    coords = [(3, 7, l) for l in range(L)] + [(0, 1, 5), (0, 2, 9), (5, 0, 1), (9, 9, 9)]
    save_mttkrp("mttkrp3_longfiber_r16", (10, 10, L), np.array(coords), rng.random(len(coords)), 16, rng)
    # 4-mode (the 80M-nonzero 4-mode family, scaled down)
    d = (40, 30, 20, 100)
    save_mttkrp("mttkrp4_zipf_r32", d, coo(rng, d, 7000, zipf=(1.2, 0, 0, 1.2)), rng.random(7000), 32, rng,
                dist="normal")
    # TTV (the 50M-nonzero TTV family, scaled down)
    d = (200, 150, 120)
    save_ttv("ttv_zipf", d, coo(rng, d, 9000, zipf=(1.1, 1.1, 0)), rng.uniform(-1, 1, 9000), rng)
    # 5-mode (the reference's mttkrp5_csf_cpu_taco.h; oracle only), Zipf on modes 0 and 4
    d = (30, 12, 10, 8, 60)
    save_mttkrp("mttkrp5_zipf_r16", d, coo(rng, d, 5000, zipf=(1.1, 0, 0, 0, 1.1)), rng.random(5000), 16, rng,
                dist="normal")
    print("wrote", sorted(f for f in os.listdir(OUT) if f.endswith(".npz")))


if __name__ == "__main__":
    main(sys.argv[sys.argv.index("--out") + 1] if "--out" in sys.argv else HERE)
