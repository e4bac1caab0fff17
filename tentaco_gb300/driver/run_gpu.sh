#!/bin/bash
# run_gpu.sh <gpu> <hardware> <feature_dim> -- the reference's run_gpu.sh on this library.
# Environment overrides: MATRICES_DIR (tensors, one directory per tensor holding <name>.tns),
# TENSOR_NAME (file with comma-separated names), RESULTS_DIR, EXPERIMENT.
HERE="$(cd "$(dirname "$0")" && pwd)"
MATRICES_DIR=${MATRICES_DIR:-./tensors}
TENSOR_NAME=${TENSOR_NAME:-$HERE/3mode.txt}
RESULTS_DIR=${RESULTS_DIR:-./tensor_result}
EXPERIMENT=${EXPERIMENT:-mttkrp_csf_gpu}
CUDA_VISIBLE_DEVICES=${1:-0} OMP_NUM_THREADS=4 python3 "$HERE/taco_eval.py" "$MATRICES_DIR" "$EXPERIMENT" \
  "$RESULTS_DIR" "${2:-gb300}" "${3:-32}" "$TENSOR_NAME"
