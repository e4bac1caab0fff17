"""tensor-eval-gpu: the reference's driver surface (argv, .tns input, CSV log).

CPU tests cover argument and input handling (they stop before any device work);
the GPU test runs the reference's all-ones check and the plan experiment."""
import csv
import os
import subprocess

import numpy as np
import pytest

import tentaco_gb300 as tt

BIN = os.path.join(os.path.dirname(tt.__file__), "bin", "tensor-eval-gpu")


def run(args, cwd):
    return subprocess.run([BIN] + [str(a) for a in args], cwd=cwd, capture_output=True, text=True, timeout=600)


def test_binary_built():
    assert os.access(BIN, os.X_OK)


def test_bad_arguments(tmp_path):
    r = run([tmp_path, "synthetic-10x10x10-50", "mttkrp_csf_gpu", tmp_path, "gb300", 0], tmp_path)
    assert r.returncode == 2 and "feature_dim" in r.stderr
    r = run([tmp_path, "no_such_tensor", "mttkrp_csf_gpu", tmp_path, "gb300", 32], tmp_path)
    assert r.returncode == 2 and "no tensor file" in r.stderr
    r = run([tmp_path, "synthetic-10x10x10-50", "no_such_experiment", tmp_path, "gb300", 32], tmp_path)
    assert r.returncode == 2 and "unknown experiment" in r.stderr
    r = run([tmp_path, "synthetic-10x10x10-50", "mttkrp_csf_gpu_plan", tmp_path, "gb300", 32, "fp8"], tmp_path)
    assert r.returncode == 2 and "precision" in r.stderr


def test_malformed_tns_is_reported(tmp_path):
    (tmp_path / "bad.tns").write_text("1 2 3 0.5\n1 2 x 1\n")
    r = run([tmp_path, "bad", "mttkrp_csf_gpu", tmp_path, "gb300", 32], tmp_path)
    assert r.returncode == 1 and "bad.tns:2" in r.stderr


@pytest.mark.gpu
def test_verify_and_plan_experiments(tmp_path):
    # a .tns file with duplicates and a synthetic tensor
    rng = np.random.default_rng(3)
    co = np.stack([rng.integers(1, 300, 20000), rng.integers(1, 200, 20000), rng.integers(1, 500, 20000)], 1)
    with open(tmp_path / "t.tns", "w") as f:
        for c in co:
            f.write(f"{c[0]} {c[1]} {c[2]} {rng.random():.6f}\n")
    for name in ("t", "synthetic-3000x2000x5000-300000-5"):
        r = run([tmp_path, name, "mttkrp_csf_gpu_verify", tmp_path, "gb300", 32], tmp_path)
        assert r.returncode == 0, r.stdout + r.stderr
        assert r.stdout.count(": ok 0") == 32
        r = run([tmp_path, name, "mttkrp_csf_gpu_plan", tmp_path, "gb300", 16], tmp_path)
        assert r.returncode == 0, r.stderr
    rows = list(csv.reader(open(tmp_path / "mttkrp_csf_gpu_plan_16_gb300.csv")))
    assert len(rows) == 50 and all(float(r[5]) > 0 for r in rows)
