"""NTT and QAP-quotient parity: golden ntt_small vectors (arkworks-shaped fft/ifft), coset
transforms against the oracle, h against the reference's own ref_qap.py output (h_ref.bin),
and full-size round trips / point evaluations."""
import os
import random
import struct

import numpy as np
import pytest

import bendg
import bn254_ref as o
from conftest import GOLDEN
from gpu_helpers import fr_from_wire_mont, fr_wire_mont

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n", [8, 64, 1024])
def test_ntt_small_vectors(ctx, n):
    buf = open(os.path.join(GOLDEN, "vectors", "ntt_small_%d.bin" % n), "rb").read()
    w = np.frombuffer(buf, dtype="<u4", offset=4 + 128).astype(np.uint32).reshape(3, n * 16)
    lg = n.bit_length() - 1
    assert np.array_equal(ctx.ntt(w[0], lg, bendg.NTT_FORWARD), w[1])
    assert np.array_equal(ctx.ntt(w[1], lg, bendg.NTT_INVERSE), w[2])


@pytest.mark.parametrize("lg", [1, 2, 5, 11, 12, 13])
def test_ntt_modes_vs_oracle(ctx, lg):
    rng = random.Random(lg)
    n = 1 << lg
    x = [rng.randrange(o.P_FR) for _ in range(n)]
    xw = fr_wire_mont(x).reshape(-1)
    assert fr_from_wire_mont(ctx.ntt(xw, lg, bendg.NTT_FORWARD)) == o.ntt(x)
    assert fr_from_wire_mont(ctx.ntt(xw, lg, bendg.NTT_INVERSE)) == o.intt(x)
    assert fr_from_wire_mont(ctx.ntt(xw, lg, bendg.NTT_COSET_FORWARD)) == o.coset_ntt(x)
    assert fr_from_wire_mont(ctx.ntt(xw, lg, bendg.NTT_COSET_INVERSE)) == o.coset_intt(x)


@pytest.mark.parametrize("lg", [19, 20, 21])
def test_ntt_full_size_properties(ctx, lg):
    n = 1 << lg
    rng = np.random.default_rng(lg)
    # random canonical values < p as wire words (top limb kept small), Montgomery-form by definition
    w = rng.integers(0, 1 << 16, size=(n, 16), dtype=np.uint32)
    w[:, 15] &= 0x0fff
    xw = w.reshape(-1)
    fwd = ctx.ntt(xw, lg, bendg.NTT_FORWARD)
    import oracle_c
    assert np.array_equal(fwd, oracle_c.ntt(xw, lg, bendg.NTT_FORWARD))
    assert np.array_equal(ctx.ntt(fwd, lg, bendg.NTT_INVERSE), xw)
    cf = ctx.ntt(xw, lg, bendg.NTT_COSET_FORWARD)
    assert np.array_equal(ctx.ntt(cf, lg, bendg.NTT_COSET_INVERSE), xw)
    assert np.array_equal(cf, oracle_c.ntt(xw, lg, bendg.NTT_COSET_FORWARD))
    if lg == 19:
        # evaluation identities at a few indexes: y_j = sum_i x_i w^(ij), coset: sum_i x_i (g w^j)^i
        x = fr_from_wire_mont(xw)
        y = fr_from_wire_mont(fwd[: 16 * 4])
        yc = fr_from_wire_mont(cf[: 16 * 4])
        w1 = o.omega(lg)
        for j in (0, 1, 3):
            assert y[j] == o.poly_eval(x, pow(w1, j, o.P_FR))
            assert yc[j] == o.poly_eval(x, o.GEN * pow(w1, j, o.P_FR) % o.P_FR)


@pytest.mark.parametrize("k", [4, 10])
def test_qap_h_matches_ref_qap(ctx, k):
    d = os.path.join(GOLDEN, "k%d" % k)
    lg = struct.unpack("<8I", open(os.path.join(d, "header.bin"), "rb").read())[3]
    n = 1 << lg
    abc = np.fromfile(os.path.join(d, "abc_evals.bin"), dtype="<u4").astype(np.uint32).reshape(3, n * 16)
    href = np.fromfile(os.path.join(d, "h_ref.bin"), dtype="<u4").astype(np.uint32)
    assert np.array_equal(ctx.qap_h(abc[0], abc[1], abc[2], lg), href)


@pytest.mark.parametrize("lg", [2, 6, 12])
def test_qap_h_random_vs_oracle(ctx, lg):
    rng = random.Random(50 + lg)
    n = 1 << lg
    a = [rng.randrange(o.P_FR) for _ in range(n)]
    b = [rng.randrange(o.P_FR) for _ in range(n)]
    c = [x * y % o.P_FR for x, y in zip(a, b)]  # satisfied on the domain
    h = ctx.qap_h(fr_wire_mont(a), fr_wire_mont(b), fr_wire_mont(c), lg)
    want = o.qap_h(a, b, c)
    assert fr_from_wire_mont(h) == want and want[-1] == 0


def test_qap_h_full_size_vs_c_oracle(ctx):
    """d = 2^21 (the K=20 domain), c = a*b on the domain: h equals the C oracle's bit for bit
    and its top coefficient is 0"""
    import oracle_c
    lg = 21
    n = 1 << lg
    rng = np.random.default_rng(5)
    a = rng.integers(0, 1 << 16, size=(n, 16), dtype=np.uint32)
    b = rng.integers(0, 1 << 16, size=(n, 16), dtype=np.uint32)
    a[:, 15] &= 0x0fff
    b[:, 15] &= 0x0fff
    c = ctx.field_op(bendg.FIELD_FR, bendg.FOP_MUL, a, b)
    h = ctx.qap_h(a.reshape(-1), b.reshape(-1), c, lg)
    assert np.array_equal(h, oracle_c.qap_h(a.reshape(-1), b.reshape(-1), c, lg))
    assert not h[-16:].any()
