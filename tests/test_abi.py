"""The C ABI library loads and exports every function include/bg.h declares (no GPU needed)."""
import ctypes
import os
import re

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
