"""The drop-in boundary as a C or C++ caller sees it: programs compiled against
the public headers link to libtentaco_gb300 and run.

* A C99 program includes every public header (tentaco.h, tentaco_gen.h,
  tentaco_select.h and the reference-named gpu_kernels.cuh), builds a CSF on the
  host and creates a plan (TT_ERR_NO_DEVICE where no GPU is visible).
* A C++ program declares the reference's entry points the way the reference's
  own gpu_kernels.cuh does (C++ linkage, no extern "C") and links to the
  library's C++-linkage exports unchanged.

Without a GPU nothing reaches the device; on a GPU host the plan is created (its
setup kernels run on the 3-nonzero tensor) and destroyed, and no walk runs.
"""
import os
import shutil
import subprocess

import pytest

import tentaco_gb300 as tt

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INC = os.path.join(ROOT, "include")
LIBDIR = os.path.dirname(tt.LIB_PATH)

C_SRC = r"""
#include <stdio.h>
#include <stdint.h>
#include "tentaco/tentaco.h"
#include "tentaco/tentaco_gen.h"
#include "tentaco/tentaco_select.h"
#include "tentaco/gpu_kernels.cuh"

int main(void) {
  const int32_t dims[3] = {2, 2, 2};
  const int32_t coords[9] = {0, 0, 1, 0, 1, 0, 1, 1, 1};
  const float vals[3] = {2.0f, 3.0f, 4.0f};
  taco_tensor_t* B = NULL;
  tt_plan* plan = NULL;
  tt_status s = tt_csf_from_coo(3, dims, 3, coords, vals, &B);
  if (s != TT_OK) { printf("coo %d %s\n", (int)s, tt_last_error_string()); return 1; }
  if (tt_csf_validate(B) != TT_OK) return 2;
  s = tt_plan_create(B, TT_OP_MTTKRP, 8, TT_PREC_FP32, TT_SELECT_DEFAULT, 0, NULL, &plan);
  if (s == TT_OK) tt_plan_destroy(plan);
  else if (s != TT_ERR_NO_DEVICE) { printf("plan %d %s\n", (int)s, tt_last_error_string()); return 3; }
  tt_tensor_free(B);
  /* the reference-named entry points resolve (their addresses are taken, not called) */
  void (*f)(taco_tensor_t*, taco_tensor_t*, taco_tensor_t*, taco_tensor_t*) = mttkrp_32_eb_sr_512_4_1;
  float (*g)(void) = get_gpu_timer_result;
  printf("abi %d variants %d plan %d linked %d\n", (int)tt_abi_version(), (int)tt_num_variants(), (int)s,
         f != NULL && g != NULL);
  return 0;
}
"""

CXX_SRC = r"""
#include <cstdio>
#include <cstdint>
#include "tentaco/taco_tensor_t.h"

// declared as in the reference's gpu_kernels.cuh: C++ linkage
void mttkrp_gpu_taco(taco_tensor_t* A, taco_tensor_t* B, taco_tensor_t* C, taco_tensor_t* D);
void mttkrp_32_eb_pr_256_64_32_manual(taco_tensor_t* A, taco_tensor_t* B, taco_tensor_t* C, taco_tensor_t* D);
void ttv_csf_gpu_taco(taco_tensor_t* A, taco_tensor_t* B, taco_tensor_t* C);
float get_gpu_timer_result();

int main() {
  void (*f)(taco_tensor_t*, taco_tensor_t*, taco_tensor_t*, taco_tensor_t*) = mttkrp_gpu_taco;
  void (*h)(taco_tensor_t*, taco_tensor_t*, taco_tensor_t*, taco_tensor_t*) = mttkrp_32_eb_pr_256_64_32_manual;
  void (*t)(taco_tensor_t*, taco_tensor_t*, taco_tensor_t*) = ttv_csf_gpu_taco;
  float (*g)() = get_gpu_timer_result;
  std::printf("linked %d\n", f != nullptr && h != nullptr && t != nullptr && g != nullptr);
  return 0;
}
"""


def _build_and_run(tmp_path, compiler, std, name, src):
    if shutil.which(compiler) is None:
        pytest.skip(f"{compiler} not found")
    path = tmp_path / name
    path.write_text(src)
    exe = tmp_path / (name + ".bin")
    cmd = [compiler, std, "-Wall", "-Werror", "-I" + INC, str(path), "-o", str(exe),
           "-L" + LIBDIR, "-ltentaco_gb300", "-Wl,-rpath," + LIBDIR]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return subprocess.run([str(exe)], check=True, capture_output=True, text=True, timeout=120).stdout


def test_c_program_links_and_runs(tmp_path):
    out = _build_and_run(tmp_path, "gcc", "-std=c99", "caller.c", C_SRC)
    expected_plan = tt.TT_OK if tt.device_count() > 0 else tt.TT_ERR_NO_DEVICE
    assert out.strip() == f"abi 1 variants {tt.num_variants()} plan {expected_plan} linked 1", out


def test_reference_style_cxx_caller_links(tmp_path):
    out = _build_and_run(tmp_path, "g++", "-std=c++17", "caller.cpp", CXX_SRC)
    assert out.strip() == "linked 1", out
