"""Benchmark: mode-0 MTTKRP over the skewed 100M-nonzero 3-mode CSF tensor, rank 32.

Workload (the configuration the headline metric is quoted on): dims 200,000 x
100,000 x 2,000,000, 100M nonzeros, fiber lengths round(lognormal(1.5, 1.8))
clipped to [1, 2M] with 3 fibers forced above 1M nonzeros, values U(0,1), factors
N(0,1) with per-column scales, rank 32.  Seeded synthetic data (seed 3); the
reference's FROSTT tensors are not available.

One step = one MTTKRP call on device-resident inputs: the walk kernel, the row
merge and (slab plans) the sum of the slabs' rows; the plan's partition was
computed once at plan creation and is reported as ``partition_ms``.  L2 is flushed
(512 MB write) between timed steps, outside the per-step CUDA events.  ``value`` is
GFLOP/s with the reference's flop count (3 * nnz * R); ``e2e`` is the same metric
through the one-shot host API (tt_mttkrp_host: host buffers in, host result out,
every copy inside the timed region).  ``roofline`` relates the walk kernel's
compulsory HBM bytes to its CUDA-event duration and the measured copy bandwidth.
Every result carries its error against the FP64 oracle over all output rows.

``--impl reference`` times the reference's CPU TACO MTTKRP3 algorithm
(tensor_kernels/mttkrp3_csf_cpu_taco.h, as restated in oracle/tt_oracle.c) on the
host cores, on a bounded row sample of the same tensor, built by the oracle's own
restatement of the generators (no product code runs in that arm).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

DIMS = (200_000, 100_000, 2_000_000)
NNZ = 100_000_000
RANK = 32
SEED = 3
WORKLOAD = "mttkrp3_skewed_100M_r32"
# the same metric for both arms; the arithmetic of each arm is in its "dtype" and "plan"
METRIC = f"MTTKRP3 GFLOP/s (3*nnz*R), {WORKLOAD}"
L2_NOTE = "flushed between steps (GPU arm: 512 MB device write; CPU arm: 80 MB host stream)"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--prec", default="fp16", choices=["fp32", "bf16", "bf16f", "fp16", "fx16"],
                    help="storage precision of the headline run")
    ap.add_argument("--compare", default="fp32,fx16",
                    help="other storage precisions timed on the same tensor (comma list, '' for none)")
    ap.add_argument("--select", default="model", choices=["default", "model", "sweep"])
    ap.add_argument("--variant", type=int, default=-1, help="run this variant id (overrides --select)")
    ap.add_argument("--nnz", type=int, default=NNZ, help="smaller nonzero count for quick checks")
    ap.add_argument("--slabs", type=int, default=0, help="leaf-mode slabs (0: the plan's automatic choice)")
    ap.add_argument("--clocks-csv", default=None, help="write the sampled SM clocks to this CSV")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-errors", action="store_true")
    ap.add_argument("--no-secondary", action="store_true",
                    help="skip TTV, MTTKRP4, other modes and other ranks")
    ap.add_argument("--only", default=None, choices=["ttv", "mttkrp4", "modes", "ranks"],
                    help="run only this secondary measurement and print its JSON (for profiling)")
    return ap.parse_args()


def physical_gpu_index() -> int:
    """NVML's index of the GPU this process computes on (NVML ignores
    CUDA_VISIBLE_DEVICES): its first entry when numeric, else 0."""
    first = os.environ.get("CUDA_VISIBLE_DEVICES", "0").split(",")[0].strip()
    return int(first) if first.isdigit() else 0


def rank_visible_devices(env) -> str | None:
    """CUDA_VISIBLE_DEVICES for this rank of a multi-process run (one GPU per rank):
    the LOCAL_RANK-th entry of a list the launcher set, else the LOCAL_RANK-th GPU;
    None for a single process."""
    if int(env.get("WORLD_SIZE", "1")) <= 1:
        return None
    local = int(env.get("LOCAL_RANK", env.get("RANK", "0")))
    given = [d for d in env.get("CUDA_VISIBLE_DEVICES", "").split(",") if d.strip()]
    if given:
        return given[local % len(given)].strip()
    return str(local)


def dist_setup(n):
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    # each replica on its own GPU: the library works on the current device, so the
    # rank sees only its GPU (set before anything initialises CUDA in this process)
    vis = rank_visible_devices(os.environ)
    if vis is not None:
        os.environ["CUDA_VISIBLE_DEVICES"] = vis
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("gloo")
        return rank, world, dist
    return rank, world, None


def barrier(d):
    if d is not None:
        d.barrier()


def allmax(d, v: float) -> float:
    if d is None:
        return v
    import torch

    t = torch.tensor([v], dtype=torch.float64)
    d.all_reduce(t, op=d.ReduceOp.MAX)
    return float(t.item())


def make_workload(nnz, rank=RANK):
    import tentaco_gb300 as tt

    B = tt.gen_lognormal_fibers(DIMS, nnz, 1.5, 1.8, 3, 1_000_000, SEED)
    C = tt.gen_dense(DIMS[1], rank, 1, SEED * 10 + 1)
    D = tt.gen_dense(DIMS[2], rank, 1, SEED * 10 + 2)
    return B, C, D


def workload_config(nnz, fibers, world):
    """Identical in both arms: the workload, not how an arm runs it."""
    return {"workload": WORKLOAD, "dims": list(DIMS), "nnz": int(nnz), "fibers": int(fibers), "rank": RANK,
            "seed": SEED, "l2": L2_NOTE, "parallelism": f"replicas{world}"}


def prec_bytes(prec):
    """(value bytes, upper-factor bytes, leaf-factor bytes) of a storage precision."""
    return {"fp32": (4, 4, 4), "bf16": (2, 2, 2), "bf16f": (4, 2, 2), "fp16": (2, 2, 2), "fx16": (4, 4, 2)}[prec]


def compulsory_bytes(B, prec, rank=RANK):
    """Compulsory HBM bytes of one MTTKRP3 call in the stored format: int32 indices,
    values, each distinct factor row once (16-bit fixed point adds one exponent byte
    per leaf row), the output written once."""
    s_v, s_u, s_l = prec_bytes(prec)
    nnz = B.nnz
    F = B.count(1)
    I = B.dims[0]
    U1 = int(np.count_nonzero(np.bincount(B.crd(1), minlength=B.dims[1])))
    U2 = int(np.count_nonzero(np.bincount(B.crd(2), minlength=B.dims[2])))
    leaf_row = rank * s_l + (1 if prec == "fx16" else 0)
    return nnz * (4 + s_v) + F * 8 + (I + 1) * 4 + U1 * rank * s_u + U2 * leaf_row + I * rank * 4, U1, U2


class Clocks:
    """SM clocks and throttle reasons sampled during the timed region only
    (start() / stop() around it): in-process NVML queries every 2 ms through the
    driver's libnvidia-ml (read-only), else nvidia-smi every 200 ms.  The samples
    are kept in memory (and written to a CSV only when a path is given)."""

    # nvmlClocksEventReason* bits (nvml.h)
    REASONS = {0x4: "sw_power_cap", 0x8: "hw_slowdown", 0x20: "sw_thermal_slowdown", 0x40: "hw_thermal_slowdown"}

    def __init__(self, path=None, period_s=0.002):
        self.path = path
        self.period = period_s
        self.rows = []  # (sm_mhz, max_mhz, reason bits)
        self.proc = None
        self.thread = None
        self.nvml = None
        self.smi_lines = []

    def _nvml_open(self):
        import ctypes
        lib = ctypes.CDLL("libnvidia-ml.so.1")
        if lib.nvmlInit_v2() != 0:
            return None
        h = ctypes.c_void_p()
        # the process's own GPU; index 0 when NVML numbers the GPUs differently (a
        # container that shows one GPU under a host index)
        if lib.nvmlDeviceGetHandleByIndex_v2(physical_gpu_index(), ctypes.byref(h)) != 0 and \
                lib.nvmlDeviceGetHandleByIndex_v2(0, ctypes.byref(h)) != 0:
            return None
        mx = ctypes.c_uint()
        lib.nvmlDeviceGetMaxClockInfo(h, 1, ctypes.byref(mx))  # NVML_CLOCK_SM
        reasons = getattr(lib, "nvmlDeviceGetCurrentClocksEventReasons", None) or \
            getattr(lib, "nvmlDeviceGetCurrentClocksThrottleReasons")
        return lib, h, mx.value, reasons

    def start(self):
        import threading
        self.rows = []
        try:
            self.nvml = self._nvml_open()
        except Exception:
            self.nvml = None
        if self.nvml:
            import ctypes
            lib, h, mx, reasons = self.nvml
            self.stop_flag = threading.Event()

            def loop():
                c = ctypes.c_uint()
                r = ctypes.c_ulonglong()
                while not self.stop_flag.is_set():
                    if lib.nvmlDeviceGetClockInfo(h, 1, ctypes.byref(c)) == 0:
                        bits = r.value if reasons(h, ctypes.byref(r)) == 0 else 0
                        self.rows.append((float(c.value), float(mx), int(bits)))
                    self.stop_flag.wait(self.period)

            self.thread = threading.Thread(target=loop, daemon=True)
            self.thread.start()
            return
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            n = subprocess.run(["nvidia-smi", "-L"], capture_output=True, text=True).stdout.count("GPU ")
            idx = physical_gpu_index() if physical_gpu_index() < n else 0
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(idx), f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None

    def stop(self):
        if self.thread:
            self.stop_flag.set()
            self.thread.join()
            self.thread = None
        if self.proc:
            self.proc.terminate()
            out, _ = self.proc.communicate()
            self.proc = None
            names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
            bitof = {v: k for k, v in self.REASONS.items()}
            for line in (out or "").splitlines():
                r = [x.strip() for x in line.split(",")]
                if len(r) < 9:
                    continue
                try:
                    bits = sum(bitof[nm] for nm, v in zip(names, r[5:9]) if v.lower().startswith("active"))
                    self.rows.append((float(r[1]), float(r[2]), bits))
                except ValueError:
                    pass
        if self.path:
            try:
                with open(self.path, "w") as fh:
                    fh.write("sm_mhz,max_sm_mhz,reason_bits\n")
                    for sm, mx, bits in self.rows:
                        fh.write(f"{sm:.0f},{mx:.0f},{bits:#x}\n")
            except OSError:
                pass

    def summary(self):
        out = {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": len(self.rows),
               "source": "nvml 2 ms" if self.nvml else "nvidia-smi 200 ms"}
        if self.rows:
            out["sm_mhz"] = statistics.median(r[0] for r in self.rows)
            out["sm_max_mhz"] = max(r[1] for r in self.rows)
            bits = 0
            for r in self.rows:
                bits |= r[2]
            out["reasons"] = sorted(nm for b, nm in self.REASONS.items() if bits & b)
        return out


def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as fh:
            p = json.load(fh)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def ncu_profile(prec, variant, slabs):
    """The committed ncu summary of the walk kernel for this workload, precision,
    variant and slab count (None when there is none): DRAM bytes per launch and the
    L2 hit rate."""
    path = os.path.join(ROOT, "profiles", f"walk_kernel_{WORKLOAD}_{prec}.json")
    try:
        with open(path) as fh:
            p = json.load(fh)
        if p.get("variant") == variant and p.get("slabs", 1) == slabs:
            return p
    except Exception:
        pass
    return None


def errors(got, ref):
    """Error of got against the FP64 oracle over every output row, in every norm:
    normwise max|x-y|/max|y|; row-normwise ||x_i-y_i||/||y_i|| (max and mean over
    rows with ||y_i|| > tau); Frobenius; elementwise |x-y|/max(|y|, tau) (max and
    mean), tau = 1e-6 max|y|; and the reference's comparators (ds.h:551-580)."""
    from oracle import oracle as O

    got64 = np.asarray(got, dtype=np.float64)
    ref = np.asarray(ref, dtype=np.float64)
    d = got64 - ref
    amax = float(np.abs(ref).max()) if ref.size else 0.0
    tau = max(1e-6 * amax, 1e-300)
    e = np.abs(d) / np.maximum(np.abs(ref), tau)
    out = {"rows_checked": int(ref.shape[0]) if ref.ndim else int(ref.size),
           "normwise_max": float(np.abs(d).max() / amax) if amax > 0 else 0.0,
           "fro": float(np.linalg.norm(d) / max(np.linalg.norm(ref), 1e-300)),
           "elem_max": float(e.max()) if e.size else 0.0, "elem_mean": float(e.mean()) if e.size else 0.0}
    if ref.ndim == 2:
        rn = np.linalg.norm(ref, axis=1)
        m = rn > tau
        rw = np.linalg.norm(d, axis=1)[m] / rn[m]
        out["row_max"] = float(rw.max()) if rw.size else 0.0
        out["row_mean"] = float(rw.mean()) if rw.size else 0.0
    out["ref_compare_array"] = float(O.compare_array(np.asarray(got, np.float32), ref.astype(np.float32)))
    out["ref_compare_array_my"] = float(O.compare_array_my(np.asarray(got, np.float32), ref.astype(np.float32)))
    return out


def oracle_csf(B):
    from oracle import oracle as O

    return O.Csf(B.order, B.dims, [None] + [B.pos(l).astype(np.int64) for l in range(1, B.order)],
                 [None] + [B.crd(l).astype(np.int64) for l in range(1, B.order)], B.vals.astype(np.float64))


def _call_and_kernel_ms(tt, call, plan, steps, warmup, clk=None):
    """Per-call ms of `steps` timed calls (the L2 flushed before each; CUDA events around each whole call on
    the plan's stream), then the walk kernel's own ms over a second pass of `steps` calls with events around
    the walk.  The first pass records no event between the walk and the merge kernels: one there holds back
    the merge's programmatic dependent launch (about 6 us per call on a GB300)."""
    plan.set_timing(2)
    for _ in range(warmup):
        tt.l2_flush()
        call()
    tt.synchronize()
    step_ms, kern_ms = [], []
    if clk:
        clk.start()
    for _ in range(steps):
        tt.l2_flush()
        call()
        step_ms.append(plan.last_ms())
    tt.synchronize()
    if clk:
        clk.stop()
    plan.set_timing(1)
    for _ in range(steps):
        tt.l2_flush()
        call()
        kern_ms.append(plan.last_kernel_ms())
    tt.synchronize()
    return step_ms, kern_ms


def timed_plan(tt, B, facs, prec, select, args, clk=None, variant=0, rank=RANK, steps=None, mode=0):
    """A plan on device-resident inputs: setup timed on the host; W warm-up calls,
    then K timed calls with the L2 flushed before each (CUDA events)."""
    steps = args.steps if steps is None else steps
    t0 = time.perf_counter()
    plan = tt.Plan(B, rank=rank, prec=prec, select=select, variant=variant, slabs=args.slabs, mode=mode)
    setup_s = time.perf_counter() - t0
    bufs = [tt.DeviceBuffer.from_array(f) for f in facs]
    plan.set_factors(bufs)
    rows = B.dims[mode]
    A = tt.DeviceBuffer(rows * rank * 4)
    step_ms, kern_ms = _call_and_kernel_ms(tt, lambda: plan.mttkrp(A), plan, steps, args.warmup, clk)
    assert plan.device_error() == 0
    info = {"ms_per_step": float(np.mean(step_ms)), "kernel_ms": float(np.mean(kern_ms)),
            "ms_median": round(float(np.median(step_ms)), 4), "ms_min": round(float(np.min(step_ms)), 4),
            "variant": plan.variant, "variant_name": tt.variant_info(plan.variant)["name"], "slabs": plan.slabs,
            "selected_by": "fixed" if select == tt.SELECT_FIXED else
            ["heuristic", "model", "sweep", "model top-k timed"][plan.selected_by],
            "plan_setup_s": round(setup_s, 2), "partition_ms": round(plan.partition_ms(), 4)}
    if plan.selected_by == 3:
        info["candidates_ms"] = {tt.variant_info(v)["name"]: round(float(t), 4)
                                 for v, t in enumerate(plan.sweep_times()) if t > 0}
    return plan, A.to_array((rows, rank)), info


def run_gpu_arm(args, rank, world, d):
    import tentaco_gb300 as tt
    from oracle import oracle as O

    t0 = time.time()
    B, C, D = make_workload(args.nnz)
    gen_s = time.time() - t0
    sel = {"default": tt.SELECT_DEFAULT, "model": tt.SELECT_MODEL, "sweep": tt.SELECT_SWEEP}[args.select]
    if args.variant >= 0:
        sel = tt.SELECT_FIXED
    flops = 3.0 * B.nnz * RANK

    clk = Clocks(args.clocks_csv)
    barrier(d)
    plan, Ah, info = timed_plan(tt, B, [C, D], args.prec, sel, args, clk=clk, variant=max(args.variant, 0))
    barrier(d)
    clocks = clk.summary()
    ms = info["ms_per_step"]
    ms_max = allmax(d, ms)
    kern = info["kernel_ms"]
    value = world * flops / (ms_max * 1e-3) / 1e9
    variant, slabs = plan.variant, plan.slabs
    del plan

    # other storage precisions on the same tensor (plain FP32 gives the 16-bit speed-ups)
    # only rank 0 reports: the other replicas skip what is not timed across ranks
    # (the other storage modes, the FP64 error checks, the secondary workloads)
    lead = rank == 0
    others = {}
    for prec in [x for x in args.compare.split(",") if x and x != args.prec and lead]:
        po, Ao, oi = timed_plan(tt, B, [C, D], prec, tt.SELECT_SWEEP if args.select != "default" else
                                tt.SELECT_DEFAULT, args)
        oi["gflops"] = flops / (oi["ms_per_step"] * 1e-3) / 1e9
        cb, _, _ = compulsory_bytes(B, prec)
        oi["gbs_compulsory"] = round(cb / (oi["ms_per_step"] * 1e-3) / 1e9, 1)
        oi["gbs_fp32_equivalent"] = round(compulsory_bytes(B, "fp32")[0] / (oi["ms_per_step"] * 1e-3) / 1e9, 1)
        oi["_A"] = Ao
        others[prec] = oi
        del po

    cbytes, U1, U2 = compulsory_bytes(B, args.prec)
    peak, peak_kind = peaks()
    achieved = cbytes / (kern * 1e-3) / 1e9
    prof = ncu_profile(args.prec, variant, slabs) if args.nnz == NNZ else None

    out = {
        "metric": METRIC,
        "value": round(value, 2), "unit": "GFLOP/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms_max, 4), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": args.prec,
        "data": "synthetic (seeded lognormal-fiber tensor; FROSTT data absent)",
        "config": workload_config(B.nnz, B.count(1), world),
        "plan": dict(info, precision=args.prec, select=args.select, gen_s=round(gen_s, 1)),
        "gbs_compulsory": round(cbytes / (ms * 1e-3) / 1e9, 1),
        # the same work counted in FP32 bytes (the 16-bit speed-ups on equal work)
        "gbs_fp32_equivalent": round(compulsory_bytes(B, "fp32")[0] / (ms * 1e-3) / 1e9, 1),
        "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                     "frac": round(achieved / peak, 4), "traffic": prof.get("dram_bytes_per_launch") if prof else None,
                     "l2_hit_rate_pct": prof.get("l2_hit_rate_pct") if prof else None,
                     "peak_source": f"{peak_kind} hbm_gbs", "kernel_ms": round(kern, 4),
                     "compulsory_bytes": int(cbytes), "U1": U1, "U2": U2},
        "clocks": clocks,
        # our kernels per step: walk, segment fold, segment chain, and for a slab plan
        # of the strip walk the slabs' row sum (one pass); slab passes of the other
        # families run walk, fold, chain and the partition per slab
        "gpu_launches": args.steps * (4 if (slabs > 1 and tt.variant_info(variant)["staged"] == 4)
                                      else slabs * (3 if slabs == 1 else 4)),
    }
    for prec, o in others.items():
        o["speedup_vs_fp32"] = None
    if "fp32" in others:
        out["speedup_vs_fp32"] = round(others["fp32"]["ms_per_step"] / ms, 3)
        for prec, o in others.items():
            if prec != "fp32":
                o["speedup_vs_fp32"] = round(others["fp32"]["ms_per_step"] / o["ms_per_step"], 3)
    if not args.no_errors and lead:
        ref = O.mttkrp(oracle_csf(B), [C.astype(np.float64), D.astype(np.float64)])
        out["error_vs_fp64"] = errors(Ah, ref)
        for o in others.values():
            o["error_vs_fp64"] = errors(o["_A"], ref)
        del ref
    for o in others.values():
        o.pop("_A", None)
    out["compare"] = others
    if not args.no_errors and others:
        # the fastest mode whose row-normwise error over all rows meets 1e-3
        cands = [(out["ms_per_step"], args.prec, out["error_vs_fp64"]["row_max"])] + \
                [(o["ms_per_step"], p, o["error_vs_fp64"]["row_max"]) for p, o in others.items()]
        ok = sorted(c for c in cands if c[2] <= 1e-3)
        out["tradeoff"] = {"fastest": min(cands)[1],
                           "fastest_row_normwise_le_1e-3": ok[0][1] if ok else None,
                           "row_max_by_precision": {c[1]: c[2] for c in cands},
                           "ms_by_precision": {c[1]: round(c[0], 4) for c in cands}}

    if not args.no_e2e:
        # every replica at once (a barrier first); the job's throughput over the
        # slowest rank's mean call
        barrier(d)
        prec_map = {"fp32": 0, "bf16": 1, "bf16f": 2, "fp16": 3, "fx16": 4}
        e2e_ms = []
        # the inputs and the output live in pinned (page-locked) host memory, as a
        # caller streaming tensors through the GPU keeps them; pinning is not timed
        Ahost = np.zeros((B.dims[0], C.shape[1]), dtype=np.float32)
        pinned = B.host_arrays() + [C, D, Ahost]
        tt.pin(pinned)
        # warm-up calls like the device leg's (the first one also grows the
        # library's device memory pool), then min(steps, 5) timed calls
        n_e2e = max(1, min(args.steps, 5))
        for i in range(args.warmup + n_e2e):
            t = time.perf_counter()
            tt.mttkrp_host(B, [C, D], prec=prec_map[args.prec], select=tt.SELECT_FIXED, variant=variant, out=Ahost)
            if i >= args.warmup:
                e2e_ms.append((time.perf_counter() - t) * 1e3)
        tt.unpin(pinned)
        h2d = B.nnz * 8 + (B.dims[0] + 1 + 2 * B.count(1) + 1) * 4 + (C.size + D.size) * 4
        e2e_mean = allmax(d, float(np.mean(e2e_ms)))
        out["e2e"] = {"value": round(world * flops / (e2e_mean * 1e-3) / 1e9, 2), "unit": "GFLOP/s",
                      "ms_per_step": round(e2e_mean, 2), "h2d_bytes_per_step": int(h2d),
                      "d2h_bytes_per_step": int(Ahost.nbytes),
                      "host_memory": "pinned (tt_host_register)",
                      "api": "tt_mttkrp_host (plan create + upload + factor conversion + run + download, "
                             "the uploads overlapped with the device work; no slabs: one call cannot repay "
                             "the slab layout's host build)"}

    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        out["cpu_baseline"] = cpu_baseline(oracle_csf(B), C, D, budget_s=12.0)
    if not args.no_secondary and lead:
        del B, C, D, Ah
        import gc
        import tentaco_gb300 as tt

        def fresh(leg):
            # each leg starts from the state a fresh process has: the library's
            # device memory pool keeps every buffer freed by the legs before
            gc.collect()
            tt.synchronize()
            tt.release_cached_memory()
            return leg(args)

        out["secondary"] = {"ttv_50M": fresh(secondary_ttv), "mttkrp4_80M": fresh(secondary_mttkrp4),
                            "mttkrp3_other_modes": fresh(secondary_other_modes),
                            "mttkrp3_ranks": fresh(secondary_ranks)}
    return out


def _timed(call, plan, steps, warmup):
    """Mean ms of a plan call and of its walk kernel over `steps` calls each (L2 flushed before each call),
    CUDA events."""
    import tentaco_gb300 as tt

    step_ms, kern_ms = _call_and_kernel_ms(tt, call, plan, steps, warmup)
    return float(np.mean(step_ms)), float(np.mean(kern_ms))


def secondary_ttv(args):
    """TTV on the 50M-nonzero tensor: 50,000 x 40,000 x 30,000, 50M nonzeros, Zipf(1.1) on modes 0 and 1,
    uniform mode 2, values and vector U(-1,1); every output checked against the FP64 oracle."""
    import tentaco_gb300 as tt
    from oracle import oracle as O

    B = tt.gen_zipf((50_000, 40_000, 30_000), (1.1, 1.1, 0.0), 50_000_000, seed=2, vlo=-1.0, vhi=1.0)
    x = tt.gen_dense(30_000, 1, 2, 21)[:, 0].copy()
    plan = tt.Plan(B, op=tt.OP_TTV)
    nfib = B.count(1)
    dx = tt.DeviceBuffer.from_array(x)
    dy = tt.DeviceBuffer(nfib * 4)
    ms, kern = _timed(lambda: plan.ttv(dx, dy), plan, max(3, args.steps), args.warmup)
    y = dy.to_array((nfib,))
    ref = O.ttv(oracle_csf(B), x.astype(np.float64))
    U = int(np.count_nonzero(np.bincount(B.crd(2), minlength=B.dims[2])))
    cbytes = B.nnz * 8 + nfib * 12 + (B.dims[0] + 1) * 4 + U * 4
    peak, _ = peaks()
    return {"nnz": B.nnz, "fibers": nfib, "ms_per_step": round(ms, 4), "kernel_ms": round(kern, 4),
            "partition_ms": round(plan.partition_ms(), 4),
            "gflops": round(2.0 * B.nnz / (ms * 1e-3) / 1e9, 2),
            "gbs_compulsory": round(cbytes / (ms * 1e-3) / 1e9, 1),
        # the same work counted in FP32 bytes (the 16-bit speed-ups on equal work)
        "gbs_fp32_equivalent": round(compulsory_bytes(B, "fp32")[0] / (ms * 1e-3) / 1e9, 1),
            "roofline_frac": round(cbytes / (ms * 1e-3) / 1e9 / peak, 4),
            "error_vs_fp64": errors(y, ref)}


def secondary_mttkrp4(args):
    """MTTKRP on the 80M-nonzero 4-mode tensor: 5,000 x 3,000 x 2,000 x 100,000, 80M nonzeros, Zipf(1.2) on
    modes 0 and 3, rank 32 N(0,1) factors; 16-bit storage against plain FP32, each on the fastest variant of
    an exhaustive sweep, and FP16 with the learned selector's four-mode model (``fp16_model``: its regret
    against the sweep's pick); every output row checked against the FP64 oracle."""
    import tentaco_gb300 as tt
    from oracle import oracle as O

    dims = (5_000, 3_000, 2_000, 100_000)
    B = tt.gen_zipf(dims, (1.2, 0.0, 0.0, 1.2), 80_000_000, seed=5)
    facs = [tt.gen_dense(d, RANK, 1, 50 + m) for m, d in enumerate(dims[1:])]
    ref = O.mttkrp(oracle_csf(B), [f.astype(np.float64) for f in facs])
    peak, _ = peaks()
    res = {"nnz": B.nnz}
    sub = argparse.Namespace(**vars(args))
    sub.steps = max(3, args.steps // 2)
    sweep_ms = None
    for prec in ("fp16", "fx16", "fp32"):
        plan, A, info = timed_plan(tt, B, facs, prec, tt.SELECT_SWEEP, sub)
        if prec == "fp16":
            sweep_ms = plan.sweep_times()
        info["gflops"] = round(4.0 * B.nnz * RANK / (info["ms_per_step"] * 1e-3) / 1e9, 2)
        s_v, s_u, s_l = prec_bytes(prec)
        U = [int(np.count_nonzero(np.bincount(B.crd(l), minlength=dims[l]))) for l in (1, 2, 3)]
        cb = B.nnz * (4 + s_v) + (B.count(2) + B.count(1)) * 8 + (dims[0] + 1) * 4 + \
            (U[0] + U[1]) * RANK * s_u + U[2] * RANK * s_l + dims[0] * RANK * 4
        info["roofline_frac"] = round(cb / (info["kernel_ms"] * 1e-3) / 1e9 / peak, 4)
        info["error_vs_fp64"] = errors(A, ref)
        res[prec] = info
        del plan
    for prec in ("fp16", "fx16"):
        res[f"speedup_{prec}_vs_fp32"] = round(res["fp32"]["ms_per_step"] / res[prec]["ms_per_step"], 3)
    # the learned selector (the four-mode model) on the same tensor, FP16: its pick
    # against the sweep's, and the speed-up over plain FP32
    plan, A, info = timed_plan(tt, B, facs, "fp16", tt.SELECT_MODEL, sub)
    info["gflops"] = round(4.0 * B.nnz * RANK / (info["ms_per_step"] * 1e-3) / 1e9, 2)
    info["error_vs_fp64"] = errors(A, ref)
    # regret from the sweep's own timings of both picks (one timing context)
    info["same_variant_as_sweep"] = info["variant"] == res["fp16"]["variant"]
    mv, sv = float(sweep_ms[info["variant"]]), float(sweep_ms[res["fp16"]["variant"]])
    info["regret_vs_sweep"] = round(mv / sv - 1.0, 4) if mv > 0 and sv > 0 else None
    info["speedup_vs_fp32"] = round(res["fp32"]["ms_per_step"] / info["ms_per_step"], 3)
    res["fp16_model"] = info
    del plan
    return res


def secondary_other_modes(args):
    """MTTKRP of modes 1 and 2 of the headline tensor (FP16 storage, rank 32, the
    learned selector): the plan re-roots the tensor at the mode once (timed as plan
    setup), calls are timed like the headline's, every output row is checked
    against the FP64 oracle on the re-rooted tensor."""
    import tentaco_gb300 as tt
    from oracle import oracle as O

    B, C, D = make_workload(args.nnz)
    facs = {0: tt.gen_dense(DIMS[0], RANK, 1, SEED * 10), 1: C, 2: D}
    res = {"nnz": B.nnz}
    sub = argparse.Namespace(**vars(args))
    sub.steps = max(3, args.steps // 2)
    for m in (1, 2):
        others = [facs[n] for n in range(3) if n != m]
        plan, A, info = timed_plan(tt, B, others, "fp16", tt.SELECT_MODEL, sub, mode=m)
        info["gflops"] = round(3.0 * B.nnz * RANK / (info["ms_per_step"] * 1e-3) / 1e9, 2)
        Bm = tt.csf_reroot(B, m)
        ref = O.mttkrp(oracle_csf(Bm), [f.astype(np.float64) for f in others])
        info["rows"] = DIMS[m]
        info["error_vs_fp64"] = errors(A, ref)
        res[f"mode{m}"] = info
        del plan, Bm, ref
    return res


def secondary_ranks(args):
    """The headline tensor at ranks 16 and 64 (the other ranks of the configuration):
    FP16 and FX16 storage against plain FP32, each selected like the headline, every
    output row checked against the FP64 oracle."""
    import tentaco_gb300 as tt
    from oracle import oracle as O

    res = {}
    peak, _ = peaks()
    sub = argparse.Namespace(**vars(args))
    sub.steps = max(3, args.steps // 2)
    for R in (16, 64):
        B, C, D = make_workload(args.nnz, rank=R)
        ref = O.mttkrp(oracle_csf(B), [C.astype(np.float64), D.astype(np.float64)])
        r = {}
        for prec in ("fp16", "fx16", "fp32"):
            plan, A, info = timed_plan(tt, B, [C, D], prec, tt.SELECT_MODEL, sub, rank=R)
            info["gflops"] = round(3.0 * B.nnz * R / (info["ms_per_step"] * 1e-3) / 1e9, 2)
            cb, _, _ = compulsory_bytes(B, prec, rank=R)
            info["roofline_frac"] = round(cb / (info["kernel_ms"] * 1e-3) / 1e9 / peak, 4)
            info["error_vs_fp64"] = errors(A, ref)
            r[prec] = info
            del plan
        for prec in ("fp16", "fx16"):
            r[f"speedup_{prec}_vs_fp32"] = round(r["fp32"]["ms_per_step"] / r[prec]["ms_per_step"], 3)
        res[f"r{R}"] = r
        del B, C, D, ref
    return res


def cpu_rows_sample(pos1, pos2, nnz, budget_nnz):
    """A contiguous row range holding about budget_nnz nonzeros (all rows if that covers the tensor)."""
    row_nnz_end = pos2[pos1]
    nrows = len(pos1) - 1
    if budget_nnz >= nnz:
        return 0, nrows, int(nnz)
    start = int(np.searchsorted(row_nnz_end, nnz // 3))
    end = int(np.searchsorted(row_nnz_end, row_nnz_end[start] + budget_nnz))
    end = max(min(end, nrows), start + 1)
    return start, end, int(row_nnz_end[end] - row_nnz_end[start])


def _subtensor(Oc, s, e):
    from oracle import oracle as O

    pos1, pos2 = Oc.pos[1], Oc.pos[2]
    f0, f1 = int(pos1[s]), int(pos1[e])
    n0, n1 = int(pos2[f0]), int(pos2[f1])
    return O.Csf(3, (e - s, Oc.dims[1], Oc.dims[2]), [None, pos1[s:e + 1] - f0, pos2[f0:f1 + 1] - n0],
                 [None, Oc.crd[1][f0:f1], Oc.crd[2][n0:n1]], Oc.vals[n0:n1])


def _flush_host_cache(buf):
    """Stream 80 MB through the host caches (the reference's TIME_COLD, timers.h:62-75)."""
    buf += 1.0
    return float(buf[::4096].sum())


def cpu_baseline(Oc, C, D, budget_s=12.0, steps=1, threads=None):
    """The reference CPU algorithm (oracle port of mttkrp3_csf_cpu_taco) on a bounded
    row range, with all host cores and with 4 threads (the reference's
    run_gpu.sh:9)."""
    from oracle import oracle as O

    Cd, Dd = C.astype(np.float64), D.astype(np.float64)
    all_cores = O.max_threads()
    flush = np.zeros(80 * 1024 * 1024 // 8)
    legs = {}
    for nthreads in (all_cores, 4):
        O.set_threads(nthreads)
        s, e, nz = cpu_rows_sample(Oc.pos[1], Oc.pos[2], Oc.nnz, 2_000_000)
        sub = _subtensor(Oc, s, e)
        t = O.now_ms()
        O.mttkrp(sub, [Cd, Dd])
        per_nnz = (O.now_ms() - t) * 1e-3 / max(nz, 1)
        target = int(min(Oc.nnz, max(nz, budget_s / 2 / max(per_nnz, 1e-12) / max(steps, 1))))
        if target >= 0.8 * Oc.nnz:
            target = Oc.nnz
        s, e, nz = cpu_rows_sample(Oc.pos[1], Oc.pos[2], Oc.nnz, target)
        sub = _subtensor(Oc, s, e)
        times = []
        for _ in range(steps):
            _flush_host_cache(flush)
            t = O.now_ms()
            O.mttkrp(sub, [Cd, Dd])
            times.append((O.now_ms() - t) * 1e-3)
        sec = float(np.mean(times))
        legs[nthreads] = {"value": round(3.0 * nz * RANK / sec / 1e9, 3), "unit": "GFLOP/s", "cores": nthreads,
                          "seconds": round(sec, 3), "rows": [s, e], "nnz": nz,
                          "sample": f"rows {s}..{e} ({nz} nonzeros, {100.0 * nz / Oc.nnz:.1f}% of the tensor), "
                                    f"FP64, reference loop order and OpenMP schedule, {nthreads} threads"}
    O.set_threads(all_cores)
    main = legs[all_cores]
    return dict(main, kind="port", threads_4=legs[4])


def run_reference_arm(args, rank, world):
    if rank != 0:
        return None
    # the tensor from the oracle's restatement of the generators: no product code here
    from oracle import oracle as O

    Oc = O.gen_lognormal(DIMS, args.nnz, 1.5, 1.8, 3, 1_000_000, SEED)
    C = O.gen_dense(DIMS[1], RANK, 1, SEED * 10 + 1)
    D = O.gen_dense(DIMS[2], RANK, 1, SEED * 10 + 2)
    base = cpu_baseline(Oc, C, D, budget_s=8.0, steps=1)
    s, e = base["rows"]
    sub = _subtensor(Oc, s, e)
    Cd, Dd = C.astype(np.float64), D.astype(np.float64)
    flush = np.zeros(80 * 1024 * 1024 // 8)
    for _ in range(args.warmup):
        O.mttkrp(sub, [Cd, Dd])
    times = []
    for _ in range(args.steps):
        _flush_host_cache(flush)
        t = O.now_ms()
        O.mttkrp(sub, [Cd, Dd])
        times.append((O.now_ms() - t) * 1e-3)
    sec = float(np.mean(times))
    val = 3.0 * sub.nnz * RANK / sec / 1e9
    return {"metric": METRIC,
            "impl": "reference", "value": round(val, 3), "unit": "GFLOP/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(sec * 1e3, 2),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded lognormal-fiber tensor; FROSTT data absent)",
            "config": workload_config(Oc.nnz, len(Oc.crd[1]), world),
            "plan": {"precision": "fp64 (the reference's CPU kernel on FP32-exact inputs)",
                     "rows": [s, e], "sample_nnz": int(sub.nnz)},
            "cpu_baseline": {"value": round(val, 3), "unit": "GFLOP/s", "cores": base["cores"], "kind": "port",
                             "sample": base["sample"], "threads_4": base["threads_4"]},
            "e2e": {"value": round(val, 3), "unit": "GFLOP/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def main():
    args = parse()
    if args.only:
        print(json.dumps({"ttv": secondary_ttv, "mttkrp4": secondary_mttkrp4,
                          "modes": secondary_other_modes, "ranks": secondary_ranks}[args.only](args)))
        return
    rank, world, d = dist_setup(args.gpus)
    if args.impl == "reference":
        out = run_reference_arm(args, rank, world)
    else:
        out = run_gpu_arm(args, rank, world, d)
    if rank == 0 and out is not None:
        print(json.dumps(out))
    if d is not None:
        d.destroy_process_group()


if __name__ == "__main__":
    main()
