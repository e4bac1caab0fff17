"""The C-ABI library loads and exports every symbol its headers declare.

No compute calls here: this runs on hosts without a GPU.
"""
import os
import re
import subprocess

import numpy as np
import pytest

import tentaco_gb300 as tt

INC = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "tentaco")


def declared_functions():
    names = set()
    for h in ("tentaco.h", "tentaco_gen.h"):
        src = open(os.path.join(INC, h)).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        names |= set(re.findall(r"\b(tt_[a-z0-9_]+)\s*\(", src))
    names |= {"get_gpu_timer_result", "ttv_csf_gpu_taco"}
    names |= set(tt.legacy_names())
    return sorted(names)


def exported():
    out = subprocess.run(["nm", "-D", "--defined-only", tt.LIB_PATH], capture_output=True, text=True, check=True)
    return {line.split()[-1] for line in out.stdout.splitlines() if " T " in line}


def test_library_loads():
    assert tt.lib().tt_abi_version() == 1


def test_every_declared_symbol_is_exported():
    syms = exported()
    missing = [n for n in declared_functions() if n not in syms]
    assert not missing, missing


def test_reference_cxx_linkage_names_are_exported():
    # objects compiled against the reference's gpu_kernels.cuh link to mangled names
    syms = exported()
    for name in ["mttkrp_gpu_taco", "mttkrp_32_eb_sr_512_4_1", "mttkrp_32_eb_pr_256_64_32_manual"]:
        mangled = f"_Z{len(name)}{name}P13taco_tensor_tS0_S0_S0_"
        assert mangled in syms, mangled
    assert "_Z16ttv_csf_gpu_tacoP13taco_tensor_tS0_S0_" in syms
    assert "_Z20get_gpu_timer_resultv" in syms


def test_legacy_names_cover_reference_header():
    # every unique entry point of gpu_kernels.cuh:4-73 (67 MTTKRP names)
    names = tt.legacy_names()
    assert len(names) == len(set(names)) == 67
    assert "mttkrp_gpu_taco" in names and "mttkrp_64_eb_pr_256_32_32" in names


def test_status_strings():
    L = tt.lib()
    assert L.tt_status_string(0) == b"TT_OK"
    assert L.tt_status_string(2) == b"TT_ERR_INVALID_CSF"


def test_variant_table():
    assert tt.num_variants() == 200
    for order in (3, 4):
        for rank in (1, 8, 10, 16, 20, 32, 40, 64):
            for prec in ("fp32", "bf16", "bf16f", "fp16"):
                v = tt.default_variant(order, rank, prec)
                assert v >= 0 and tt.variant_valid(v, order, rank, prec)
            # 16-bit fixed point runs on the strip family (ids 160..199) only
            assert not any(tt.variant_valid(x, order, rank, "fx16") for x in range(160))
            assert any(tt.variant_valid(x, order, rank, "fx16") for x in range(160, 200))
    # five modes: the strip family, FP32, FP16 and 16-bit fixed point
    for rank in (1, 8, 16, 32, 64):
        for prec in ("fp32", "fp16", "fx16"):
            v = tt.default_variant(5, rank, prec)
            assert tt.variant_info(v)["staged"] == 4 and tt.variant_valid(v, 5, rank, prec)
            assert not any(tt.variant_valid(x, 5, rank, prec) for x in range(160))
        assert not any(tt.variant_valid(x, 5, rank, "bf16") for x in range(200))
    # the fixed heuristic: flat family for three modes, strip for four
    info = tt.variant_info(tt.default_variant(3, 32, "fp32"))
    assert info["threads"] == 256 and info["cols_per_lane"] == 4 and info["staged"] == 3
    assert info["name"] == "flat_b2_g64_c4"
    assert tt.variant_info(tt.default_variant(3, 32, "fp16"))["name"] == "flat_b2_g32_c8"
    assert tt.variant_info(tt.default_variant(4, 32, "fp16"))["name"] == "strip_b2_g128_c8"
    assert tt.variant_info(tt.default_variant(4, 32, "fp32"))["name"] == "strip_b2_g128_c4"
    assert tt.variant_info(tt.default_variant(3, 32, "fx16"))["name"] == "strip_b2_g128_c4"
    assert tt.variant_info(3)["staged"] == 0 and tt.variant_info(43)["name"].startswith("stage")
    # the flat family (ids 120..159)
    assert tt.variant_info(134)["name"] == "flat_b3_g128_c2"
    assert tt.variant_valid(134, 3, 32, "fp16") and tt.variant_valid(134, 4, 32, "fp16")


def test_invalid_csf_rejected():
    # pos not monotone: the host validator rejects it; a plan rejects it too (its
    # structure check runs on the device copies, so without a GPU the plan stops
    # at "no device" first; tests/test_gpu_mttkrp.py covers the device check)
    lv = [None, (np.array([0, 2, 1], np.int32), np.array([0, 1], np.int32)),
          (np.array([0, 1, 2], np.int32), np.array([0, 1], np.int32))]
    B = tt.HostTaco((2, 2, 2), vals=np.ones(2, np.float32), levels=lv)
    assert tt.lib().tt_csf_validate(B.ptr) == tt.TT_ERR_INVALID_CSF
    with pytest.raises(tt.TTError) as e:
        tt.Plan(B, rank=8)
    expected = tt.TT_ERR_INVALID_CSF if tt.device_count() > 0 else tt.TT_ERR_NO_DEVICE
    assert e.value.status == expected


@pytest.mark.skipif(tt.device_count() > 0, reason="host has a GPU")
def test_no_device_is_an_error_not_a_fallback():
    lv = [None, (np.array([0, 1, 1], np.int32), np.array([0], np.int32)),
          (np.array([0, 1], np.int32), np.array([1], np.int32))]
    B = tt.HostTaco((2, 2, 2), vals=np.ones(1, np.float32), levels=lv)
    with pytest.raises(tt.TTError) as e:
        tt.Plan(B, rank=8)
    assert e.value.status == tt.TT_ERR_NO_DEVICE
    A = np.zeros((2, 8), np.float32)
    with pytest.raises(tt.TTError):
        tt.mttkrp_host(B, [np.ones((2, 8), np.float32), np.ones((2, 8), np.float32)])


def test_host_call_rejects_unsupported_orders_first():
    """tt_mttkrp_host refuses an order it has no kernels for before it reads the
    tensor's levels or the factor array (which has order - 1 entries)."""
    lv = [None, (np.array([0, 1, 1], np.int32), np.array([0], np.int32)),
          (np.array([0, 1], np.int32), np.array([1], np.int32))]
    for order in (2, 6):
        B = tt.HostTaco((2, 2, 2), vals=np.ones(1, np.float32), levels=lv, order=order)
        with pytest.raises(tt.TTError) as e:
            tt.mttkrp_host(B, [np.ones((2, 8), np.float32), np.ones((2, 8), np.float32)])
        assert e.value.status == tt.TT_ERR_UNSUPPORTED


def test_last_error_is_per_thread():
    """tt_last_error_string() reports the calling thread's last failure: threads
    validating different malformed tensors at once each read their own message."""
    import threading

    def bad(t):
        # t + 1 fibers of one nonzero each; fiber t's coordinate is outside the last mode
        n = t + 1
        lv = [None, (np.array([0, n], np.int32), np.arange(n, dtype=np.int32)),
              (np.arange(n + 1, dtype=np.int32), np.array([0] * t + [4], np.int32))]
        return tt.HostTaco((1, n, 4), vals=np.ones(n, np.float32), levels=lv)

    tensors = [bad(t) for t in range(8)]
    errors = []

    def work(t):
        L = tt.lib()
        for _ in range(300):
            if L.tt_csf_validate(tensors[t].ptr) != tt.TT_ERR_INVALID_CSF:
                errors.append((t, "status"))
                return
            msg = L.tt_last_error_string().decode()
            if f"fiber {t}:" not in msg:
                errors.append((t, msg))
                return

    threads = [threading.Thread(target=work, args=(t,)) for t in range(8)]
    for th in threads:
        th.start()
    for th in threads:
        th.join()
    assert not errors, errors


def test_coo_plan_argument_checks_before_the_device():
    """COO plans refuse what they have no kernels for before touching a device."""
    d = np.array([4, 4, 4, 4, 4, 4], np.int32)
    co = np.zeros((1, 6), np.int32)
    for order, op in ((2, tt.OP_MTTKRP), (6, tt.OP_MTTKRP), (4, tt.OP_TTV), (4, tt.OP_TTM)):
        with pytest.raises(tt.TTError) as e:
            tt.Plan.from_coo(d[:order], co[:, :order], np.ones(1, np.float32), op=op)
        assert e.value.status == tt.TT_ERR_UNSUPPORTED
    with pytest.raises(tt.TTError) as e:
        tt.Plan.from_coo(d[:3], co[:, :3], np.ones(1, np.float32), op=tt.OP_TTM, prec="fp16")
    assert e.value.status == tt.TT_ERR_UNSUPPORTED


def test_debug_hooks_check_arguments_without_a_device():
    L = tt.lib()
    assert L.tt_debug_tma_wait(1, -5) == tt.TT_ERR_INVALID_ARGUMENT
    assert L.tt_debug_tma_wait(0, 0) == tt.TT_OK
    assert L.tt_debug_fail_pool_alloc(-1) == tt.TT_ERR_INVALID_ARGUMENT
    assert L.tt_debug_fail_pool_alloc(0) == tt.TT_OK
    if tt.device_count() == 0:
        assert L.tt_debug_pool_live() == 0
