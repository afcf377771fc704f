"""Host logic of bench.py (no GPU): the shifted SquareChain witnesses used for the 64-proof
batch satisfy the circuit, the instance generator's witness layout is what they assume, the
NTT roofline's two bounds and the accumulation kernel's HBM view."""
import ctypes
import os

import numpy as np

import bench
import bn254_ref as o
import oracle_c
import oracle_io


def test_shifted_witness_satisfies_square_chain(tmp_path):
    L = oracle_c.lib()
    L.bgo_synth_square_chain.argtypes = [ctypes.c_uint32, ctypes.c_uint64, ctypes.c_char_p, ctypes.c_int]
    assert L.bgo_synth_square_chain(5, 11, str(tmp_path).encode(), 2) == 0
    z_words = np.fromfile(os.path.join(tmp_path, "witness.bin"), dtype="<u4").astype(np.uint32)
    n = 1 << 5
    for m in (1, 2, 7):
        w = bench.shifted_witness(z_words, m)
        z = oracle_io.fes(w.astype("<u4").tobytes(), n + 2, o.P_FR)
        assert z[0] == 1
        xs = z[2:]
        assert all(xs[i + 1] == xs[i] * xs[i] % o.P_FR for i in range(n - 1))
        assert z[1] == xs[-1] * xs[-1] % o.P_FR  # x_N' = x_{N-1}'^2 (the last constraint)
        z0 = oracle_io.fes(z_words.astype("<u4").tobytes(), n + 2, o.P_FR)
        assert xs[0] == pow(z0[2], 2 ** m, o.P_FR)  # x_0' = x_m of the original chain


def test_batch_weights():
    assert abs(sum(bench.BATCH_WEIGHTS) - 1.0) < 1e-12 and len(bench.BATCH_KS) == 5


def test_ntt_roofline_bounds():
    """the NTT roofline reports both bounds; the multiply-add bound binds for a 2^20 transform"""
    r = bench.ntt_roofline(20, 0.36, 13.1e12)
    n = 1 << 20
    assert r["imad"]["work"] == (n // 2) * 20 * 232
    assert r["hbm"]["min_bytes"] == 64 * n
    assert r["bound"] == "imad"
    assert abs(r["imad"]["frac"] - r["imad"]["bound_ms"] / 0.36) < 1e-3
    if r["hbm"]["bound_ms"] is not None:
        assert r["hbm"]["bound_ms"] < r["imad"]["bound_ms"]


def test_accumulation_hbm_view():
    """G1 MSM 2^20 at c = 15 (W = 17): 64 MiB of points, 71 MB of entry codes, 35.7 MB of
    buckets; at the measured 3.82 ms per launch that is a few percent of the copy bandwidth"""
    n = 1 << 20
    r = bench.acc_hbm_view(n, 15, 17, 3.82, traffic=489983744)
    assert r["algorithmic_bytes"] == n * 64 + n * 17 * 4 + 17 * (1 << 14) * 128
    assert r["bound"] == "hbm" and r["unit"] == "GB/s" and r["traffic"] == 489983744
    assert abs(r["achieved"] - r["algorithmic_bytes"] / 3.82e-3 / 1e9) < 0.1
    if r["peak"]:
        assert 0 < r["frac"] < 0.05
