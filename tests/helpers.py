"""Shared test helpers: fixture loading, conversions to the oracle, error norms.

The oracle (oracle/oracle.py) gives the expected results; the library under test is
always called through its C ABI (tentaco_gb300 wraps it with ctypes).
"""
from __future__ import annotations

import glob
import os

import numpy as np

import tentaco_gb300 as tt
from oracle import oracle as O

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def golden_files(kind=None):
    out = []
    for f in sorted(glob.glob(os.path.join(GOLDEN, "*.npz"))):
        z = np.load(f)
        if kind is None or str(z["kind"]) == kind:
            out.append(f)
    return out


def golden_csf(z) -> O.Csf:
    order = int(z["order"])
    pos = [None] + [z[f"pos{l}"] for l in range(1, order)]
    crd = [None] + [z[f"crd{l}"] for l in range(1, order)]
    return O.Csf(order, tuple(int(d) for d in z["dims"]), pos, crd, z["vals"])


def host_taco(csf: O.Csf, compressed_root: bool = False) -> tt.HostTaco:
    """taco_tensor_t (int32 indices, float32 values) over an oracle CSF."""
    levels = [None]
    if compressed_root:
        levels[0] = (np.array([0, csf.dims[0]], dtype=np.int32), np.arange(csf.dims[0], dtype=np.int32))
    for l in range(1, csf.order):
        levels.append((csf.pos[l].astype(np.int32), csf.crd[l].astype(np.int32)))
    return tt.HostTaco(csf.dims, vals=csf.vals.astype(np.float32), levels=levels,
                       dense_root=not compressed_root)


def to_oracle(B: tt.Tensor) -> O.Csf:
    pos = [None] + [B.pos(l).astype(np.int64) for l in range(1, B.order)]
    crd = [None] + [B.crd(l).astype(np.int64) for l in range(1, B.order)]
    return O.Csf(B.order, B.dims, pos, crd, B.vals.astype(np.float64))


def rel_errors(got: np.ndarray, ref: np.ndarray) -> dict:
    """Error of got against an FP64 reference.

    elem: max |x-y| / max(|y|, tau) with tau = 1e-6 * max|y| (elementwise, floored)
    elem_mean: the same, averaged
    row: max over rows of ||x_i - y_i||_2 / ||y_i||_2 (rows with ||y_i|| > tau)
    fro: ||x - y||_F / ||y||_F
    """
    got = np.asarray(got, dtype=np.float64)
    ref = np.asarray(ref, dtype=np.float64)
    amax = float(np.abs(ref).max()) if ref.size else 0.0
    tau = max(1e-6 * amax, 1e-300)
    e = np.abs(got - ref) / np.maximum(np.abs(ref), tau)
    out = {"elem": float(e.max()) if e.size else 0.0, "elem_mean": float(e.mean()) if e.size else 0.0}
    if ref.ndim == 2 and ref.size:
        rn = np.linalg.norm(ref, axis=1)
        dn = np.linalg.norm(got - ref, axis=1)
        m = rn > tau
        out["row"] = float((dn[m] / rn[m]).max()) if m.any() else 0.0
    fr = np.linalg.norm(ref)
    out["fro"] = float(np.linalg.norm(got - ref) / fr) if fr > 0 else float(np.linalg.norm(got))
    return out
