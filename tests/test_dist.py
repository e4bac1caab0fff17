"""The multi-process (N > 1) path on CPU: world_size-2 runs over gloo at
127.0.0.1, launched the way the bench is launched for N GPUs.  Each GPU rank
runs an independent replica (no data-path collective); what N > 1 adds is the
barrier around the timed region, the max over ranks and rank 0 reporting,
which these tests cover without a GPU."""
import json
import os
import re
import socket
import subprocess
import sys

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _torchrun(args, timeout=600):
    pytest.importorskip("torch.distributed")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(_free_port())] + args
    env = dict(os.environ, OMP_NUM_THREADS="2")
    return subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=timeout, env=env)


def test_barrier_and_max_over_two_ranks():
    r = _torchrun([os.path.join(HERE, "dist_worker.py")])
    assert r.returncode == 0, r.stderr[-2000:]
    # the two ranks write concurrently: read every flat JSON object in the stream
    lines = [json.loads(m) for m in re.findall(r"\{[^{}]*\}", r.stdout)]
    assert sorted(x["rank"] for x in lines) == [0, 1]
    assert all(x["world"] == 2 and x["max"] == 2.5 for x in lines)


def test_reference_arm_two_ranks_rank0_reports():
    r = _torchrun([os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2", "--steps", "1",
                   "--warmup", "0", "--nnz", "200000"])
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [json.loads(l) for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, r.stdout
    out = lines[0]
    assert out["impl"] == "reference" and out["n_gpus"] == 2 and out["value"] > 0
    assert out["cpu_baseline"]["kind"] == "port" and out["e2e"]["h2d_bytes_per_step"] == 0
    # the same metric and workload as the GPU arm's line, so the two arms compare
    sys.path.insert(0, ROOT)
    import bench
    assert out["metric"] == bench.METRIC and out["config"]["workload"] == bench.WORKLOAD
    assert out["unit"] == "GFLOP/s" and out["higher_is_better"] is True
    for k in ("steps", "warmup", "ms_per_step", "scaling", "vs_baseline", "dtype", "data"):
        assert k in out, k


def test_reference_arm_loads_no_product_code():
    """The reference arm builds its tensor with the oracle's generators: after a run,
    no module of the product package is loaded in the process, and its config has
    exactly the GPU arm's keys (the workload, not how an arm runs it)."""
    code = ("import sys, json, argparse; sys.path.insert(0, %r); import bench;"
            "a = argparse.Namespace(nnz=200000, steps=1, warmup=0);"
            "out = bench.run_reference_arm(a, 0, 1);"
            "print(json.dumps({'mods': sorted(m for m in sys.modules if m.startswith('tentaco_gb300')),"
            " 'keys': sorted(out['config']), 'want': sorted(bench.workload_config(1, 1, 1))}))" % ROOT)
    r = subprocess.run([sys.executable, "-c", code], cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    res = json.loads(r.stdout.strip().splitlines()[-1])
    assert res["mods"] == []
    assert res["keys"] == res["want"]


def test_each_rank_computes_on_its_own_gpu():
    """Under torchrun every replica sees one GPU: its LOCAL_RANK-th (of the list the
    launcher set, if any), chosen before CUDA starts; a single process keeps the
    environment as it is.  The clock sampler reads the same physical GPU."""
    sys.path.insert(0, ROOT)
    import bench

    assert bench.rank_visible_devices({"WORLD_SIZE": "1"}) is None
    assert bench.rank_visible_devices({"WORLD_SIZE": "4", "LOCAL_RANK": "3"}) == "3"
    assert bench.rank_visible_devices({"WORLD_SIZE": "2", "LOCAL_RANK": "1", "CUDA_VISIBLE_DEVICES": "4,6"}) == "6"
    assert bench.rank_visible_devices({"WORLD_SIZE": "2", "RANK": "1"}) == "1"
    old = os.environ.get("CUDA_VISIBLE_DEVICES")
    try:
        os.environ["CUDA_VISIBLE_DEVICES"] = "6"
        assert bench.physical_gpu_index() == 6
        os.environ["CUDA_VISIBLE_DEVICES"] = "GPU-1234"
        assert bench.physical_gpu_index() == 0
    finally:
        if old is None:
            os.environ.pop("CUDA_VISIBLE_DEVICES", None)
        else:
            os.environ["CUDA_VISIBLE_DEVICES"] = old
