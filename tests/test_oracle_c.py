"""The C oracle (CPU baseline and large-size checker) agrees with the pinned Python oracle
and the golden fixtures."""
import os
import random

import numpy as np
import pytest

import bn254_ref as o
import oracle_c
from conftest import GOLDEN


def test_c_oracle_msm_vectors():
    for n in (8, 64, 1024):
        buf = open(os.path.join(GOLDEN, "vectors", "msm_small_%d.bin" % n), "rb").read()
        w = np.frombuffer(buf, dtype="<u4", offset=4).astype(np.uint32)
        got = oracle_c.msm_g1(w[: 32 * n], w[32 * n: 48 * n], n, threads=4)
        assert np.array_equal(got, w[48 * n: 48 * n + 32])


def test_c_oracle_msm_g2_small():
    rng = random.Random(3)
    f = o.FixedBase(o.G2, o.G2.gen)
    pts = [f.mul(rng.randrange(1, o.P_FR)) for _ in range(20)] + [None]
    sc = [rng.randrange(o.P_FR) for _ in range(21)]
    from gpu_helpers import g2_wire, scalars_wire, g2_from_aff_wire
    got = oracle_c.msm_g2(g2_wire(pts), scalars_wire(sc), 21, threads=3)
    assert g2_from_aff_wire(got) == o.msm_naive(o.G2, pts, sc)


@pytest.mark.parametrize("n", [8, 64, 1024])
def test_c_oracle_ntt_vectors(n):
    buf = open(os.path.join(GOLDEN, "vectors", "ntt_small_%d.bin" % n), "rb").read()
    w = np.frombuffer(buf, dtype="<u4", offset=4 + 128).astype(np.uint32).reshape(3, n * 16)
    lg = n.bit_length() - 1
    assert np.array_equal(oracle_c.ntt(w[0], lg, 0, threads=2), w[1])
    assert np.array_equal(oracle_c.ntt(w[1], lg, 1, threads=2), w[2])


@pytest.mark.parametrize("k", [4, 10])
def test_c_oracle_qap_and_prove(k):
    d = os.path.join(GOLDEN, "k%d" % k)
    hdr = np.fromfile(os.path.join(d, "header.bin"), dtype="<u4")
    n = 1 << int(hdr[3])
    abc = np.fromfile(os.path.join(d, "abc_evals.bin"), dtype="<u4").astype(np.uint32).reshape(3, n * 16)
    href = np.fromfile(os.path.join(d, "h_ref.bin"), dtype="<u4").astype(np.uint32)
    assert np.array_equal(oracle_c.qap_h(abc[0], abc[1], abc[2], int(hdr[3]), threads=4), href)
    proof, ms = oracle_c.prove_dir(d, threads=4)
    ref = np.fromfile(os.path.join(d, "proof_ref.bin"), dtype="<u4").astype(np.uint32)
    assert np.array_equal(proof, ref)
    assert ms["total"] > 0
