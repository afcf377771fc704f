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


def test_bucket_counts_match_the_device_digits(tmp_path):
    """bench.bucket_counts (the exact work count of the roofline) gives each scalar the buckets
    the device's signed-digit recoding gives it (msm.cu's digits section, compiled for the host)"""
    import device_emul
    lib = ctypes.CDLL(device_emul.build_digits(str(tmp_path)))
    rng = np.random.default_rng(5)
    n = 300
    sc = rng.integers(0, 1 << 32, size=(n, 8), dtype=np.uint64).astype(np.uint32)
    sc[:, 7] &= 0x0FFFFFFF
    sc[:3] = 0
    sc[1, 0] = 1
    sc[2] = np.array([(o.P_FR - 1) >> (32 * i) & 0xFFFFFFFF for i in range(8)], dtype=np.uint32)
    for c in (3, 9, 15, 17):
        W = 254 // c + 1
        nb = 1 << (c - 1)
        want = np.zeros(W * nb, dtype=np.int64)
        mags = (ctypes.c_uint32 * W)()
        negs = (ctypes.c_uint8 * W)()
        for i in range(n):
            s = (ctypes.c_uint32 * 8)(*[int(v) for v in sc[i]])
            assert lib.digits(s, W, mags, negs) == 0
            for w in range(W):
                if mags[w]:
                    want[w * nb + mags[w] - 1] += 1
        assert np.array_equal(bench.bucket_counts(sc, c), want), c


def test_pair_round_additions():
    counts = np.array([0, 1, 2, 3, 7, 64])
    # round 0: 0+0+1+1+3+32 = 37 sums, leaving 0,1,1,2,4,32; round 1: 0+0+0+1+2+16 = 19
    assert bench.pair_round_additions(counts, 2) == [37, 19]
    assert bench.pair_round_additions(counts, 0) == []



def test_proof_imad_model(built_lib):
    """the batch roofline's per-proof work at SquareChain(2^18): 42.0 G (G1 entries) + 20.2 G (G2)
    + 8.1 G (NTTs) = 70.3 G multiply-adds with the committed window tables"""
    import bendg
    hdr = [1 << 18, 1, (1 << 18) + 1, 19, (1 << 18) + 2, (1 << 18) + 2, (1 << 19) - 1, 1 << 18]
    w = bench.proof_imad(bendg.lib(), hdr)
    assert abs(w - 70.28e9) < 0.01e9
