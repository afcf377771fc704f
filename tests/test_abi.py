"""The C ABI library loads and exports every function include/bg.h declares (no GPU needed)."""
import ctypes
import os
import re

import pytest

from conftest import ROOT


def declared_functions():
    src = open(os.path.join(ROOT, "include", "bg.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(bg_[a-z0-9_]+)\s*\(", src)))


def test_header_matches_binding():
    import bendg
    assert sorted(bendg.EXPORTS) == declared_functions()


def test_library_exports(built_lib):
    lib = ctypes.CDLL(built_lib)
    missing = [name for name in declared_functions() if not hasattr(lib, name)]
    assert not missing, missing


def test_status_strings(built_lib):
    import bendg
    L = bendg.lib()
    for st in range(7):
        assert L.bg_strerror(st)
    assert L.bg_msm_window_bits(1 << 20, 0) >= L.bg_msm_window_bits(1 << 10, 0)
    assert L.bg_msm_table_window_bits(1 << 18, 1) >= L.bg_msm_table_window_bits(1 << 10, 1)
    assert 3 <= L.bg_msm_proof_window_bits(1 << 18, 1) <= 20


def test_argument_errors_carry_a_message(built_lib):
    """a rejected argument returns BG_E_ARG and bg_last_error names the entry point and the
    failed condition; these checks run before any device work, so no GPU is needed"""
    import bendg
    L = bendg.lib()
    out = (ctypes.c_uint32 * 48)()
    assert L.bg_msm_g1(None, None, None, 4, out) == bendg.BG_E_ARG
    msg = L.bg_last_error(None).decode()
    assert msg.startswith("bg_msm_g1: invalid argument") and "!ctx" in msg
    assert L.bg_qap_h(None, None, None, None, 30, None) == bendg.BG_E_ARG
    assert L.bg_last_error(None).decode().startswith("bg_qap_h: invalid argument")
    assert L.bg_msm_g1_noalloc(None, None, 4, None, out) == bendg.BG_E_ARG
    assert L.bg_last_error(None).decode().startswith("bg_msm_g1_noalloc: invalid argument")
    assert L.bg_proof_format(None, None, 0) == bendg.BG_E_ARG
    assert L.bg_last_error(None).decode().startswith("bg_proof_format: invalid argument")


def test_misaligned_device_pointers_are_refused(built_lib):
    """the _dev entry points and bg_msm_g1_noalloc read and write device buffers in 16-byte
    vectors: a pointer off that boundary is refused on the host, before any device work (the
    pointer values here are never dereferenced, so no GPU is needed)"""
    import bendg
    L = bendg.lib()
    out = (ctypes.c_uint32 * 48)()
    bad, good = 0x10004, 0x10000
    cases = [
        ("bg_msm_g1_dev", lambda: L.bg_msm_g1_dev(None, bad, good, 4, out)),
        ("bg_msm_g1_dev", lambda: L.bg_msm_g1_dev(None, good, bad, 4, out)),
        ("bg_msm_g2_dev", lambda: L.bg_msm_g2_dev(None, bad, good, 4, out)),
        ("bg_ntt_dev", lambda: L.bg_ntt_dev(None, bad, 10, 0)),
        ("bg_repack_to_packed_dev", lambda: L.bg_repack_to_packed_dev(None, good, bad, 4)),
        ("bg_repack_to_wire_dev", lambda: L.bg_repack_to_wire_dev(None, bad, good, 4)),
    ]
    for name, call in cases:
        assert call() == bendg.BG_E_ARG, name
        msg = L.bg_last_error(None).decode()
        assert msg.startswith(name + ": invalid argument") and "misaligned16" in msg, msg
    assert L.bg_msm_g1_noalloc(good, bad, 4, None, out) == bendg.BG_E_ARG
    assert "16-byte aligned" in L.bg_last_error(None).decode()
    # aligned pointers pass the alignment check and stop at the missing context instead
    assert L.bg_msm_g1_dev(None, good, good, 4, out) == bendg.BG_E_ARG
    assert "!ctx" in L.bg_last_error(None).decode()


def test_no_device_fails_loudly(built_lib):
    """without a usable GPU, creating a context fails with BG_E_DEVICE and the CUDA reason:
    there is no CPU fallback behind the C ABI"""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    import bendg
    with pytest.raises(bendg.BgError) as e:
        bendg.Context(0)
    assert e.value.status == bendg.BG_E_DEVICE
    assert "bg_ctx_create" in str(e.value) or "cuda" in str(e.value).lower()
