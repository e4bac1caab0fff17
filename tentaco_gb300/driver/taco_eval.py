#!/usr/bin/env python3
"""Run tensor-eval-gpu over a list of tensors and collect one CSV per experiment.

Same arguments as the reference's taco-eval.py (taco-eval.py:7-12):
    taco_eval.py <tensors_dir> <experiment> <results_dir> <hardware> <feature_dim> <names_file>
names_file holds comma-separated tensor names (like the reference's 3mode.txt); each
tensor is read from <tensors_dir>/<name>/<name>.tns, or generated when the name is
synthetic-<I>x<J>x<K>-<nnz>[-<seed>].  The log gets the reference's header line,
kernel,platform,format,library,tensor,time, then one line per trial.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
BINARY = os.path.join(os.path.dirname(HERE), "bin", "tensor-eval-gpu")


def main(argv):
    tensors_dir = argv[1] if len(argv) > 1 else "."
    experiment = argv[2] if len(argv) > 2 else "mttkrp_csf_gpu"
    results_dir = argv[3] if len(argv) > 3 else "."
    hardware = argv[4] if len(argv) > 4 else "gb300"
    feature = argv[5] if len(argv) > 5 else "32"
    names_file = argv[6] if len(argv) > 6 else None
    if names_file:
        with open(names_file) as f:
            names = sorted(n.strip() for n in f.readline().split(",") if n.strip())
    else:
        names = sorted(os.listdir(tensors_dir))
    os.makedirs(results_dir, exist_ok=True)
    log_path = os.path.join(results_dir, f"{experiment}_{feature}_{hardware}.csv")
    with open(log_path, "w") as log:
        log.write("kernel,platform,format,library,tensor,time\n")
    rc = 0
    for name in names:
        cmd = [BINARY, os.path.join(tensors_dir, name), name, experiment, results_dir, hardware, feature]
        print(" ".join(cmd), flush=True)
        rc = subprocess.run(cmd).returncode or rc
    return rc


if __name__ == "__main__":
    sys.exit(main(sys.argv))
