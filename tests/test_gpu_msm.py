"""MSM parity (Msm.g1 / Msm.g2 of bend2/src/msm.bend:297, :529 via the seam's C ABI):
golden vectors, edge cases, and full-size checks through the discrete-log identity
sum s_i (k_i G) = (sum s_i k_i) G."""
import os
import random
import struct

import numpy as np
import pytest

import bendg
import bn254_ref as o
from conftest import GOLDEN
from gpu_helpers import (g1_from_aff_wire, g1_from_jac_wire, g1_wire, g2_from_aff_wire, g2_from_jac_wire, g2_wire,
                         scalars_wire)

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n", [8, 64, 1024])
def test_msm_small_vectors(ctx, n):
    buf = open(os.path.join(GOLDEN, "vectors", "msm_small_%d.bin" % n), "rb").read()
    w = np.frombuffer(buf, dtype="<u4", offset=4).astype(np.uint32)
    pts, sc, res = w[: 32 * n], w[32 * n: 48 * n], w[48 * n: 48 * n + 32]
    got = g1_from_jac_wire(ctx.msm_g1(pts, sc, n))
    assert got == g1_from_aff_wire(res)


def random_g1(rng, n):
    f = o.FixedBase(o.G1, o.G1.gen)
    ks = [rng.randrange(1, o.P_FR) for _ in range(n)]
    return ks, [f.mul(k) for k in ks]


def random_g2(rng, n):
    f = o.FixedBase(o.G2, o.G2.gen)
    ks = [rng.randrange(1, o.P_FR) for _ in range(n)]
    return ks, [f.mul(k) for k in ks]


EDGE = ["zero_scalars", "infinity_points", "repeated_point", "negated_pairs", "max_scalars", "single", "one_each"]


def edge_case(kind, rng, pts):
    n = len(pts)
    sc = [rng.randrange(o.P_FR) for _ in range(n)]
    pts = list(pts)
    if kind == "zero_scalars":
        sc = [0 if i % 3 else s for i, s in enumerate(sc)]
    elif kind == "infinity_points":
        pts = [None if i % 4 == 1 else p for i, p in enumerate(pts)]
    elif kind == "repeated_point":
        pts = [pts[0]] * n          # every bucket adds P + P (doubling branch)
        sc = [sc[0]] * (n // 2) + sc[n // 2:]
    elif kind == "negated_pairs":
        curve = o.G1 if isinstance(pts[0][0], int) else o.G2
        pts = [pts[i // 2] if i % 2 == 0 else curve.neg(pts[i // 2]) for i in range(n)]
        sc = [sc[i // 2] for i in range(n)]  # P and -P with equal scalars cancel
    elif kind == "max_scalars":
        sc = [o.P_FR - 1 - (i % 3) for i in range(n)]
    elif kind == "single":
        pts, sc = pts[:1], sc[:1]
    elif kind == "one_each":
        sc = [1] * n
    return pts, sc


@pytest.mark.parametrize("kind", EDGE)
def test_msm_g1_edges(ctx, kind):
    rng = random.Random(hash(kind) & 0xffff)
    _, base = random_g1(rng, 48)
    pts, sc = edge_case(kind, rng, base)
    want = o.msm_naive(o.G1, pts, sc)
    assert g1_from_jac_wire(ctx.msm_g1(g1_wire(pts), scalars_wire(sc), len(pts))) == want


@pytest.mark.parametrize("kind", EDGE)
def test_msm_g2_edges(ctx, kind):
    rng = random.Random(1000 + (hash(kind) & 0xffff))
    _, base = random_g2(rng, 24)
    pts, sc = edge_case(kind, rng, base)
    want = o.msm_naive(o.G2, pts, sc)
    assert g2_from_jac_wire(ctx.msm_g2(g2_wire(pts), scalars_wire(sc), len(pts))) == want


def test_msm_empty(ctx):
    z = np.zeros(0, dtype=np.uint32)
    assert g1_from_jac_wire(ctx.msm_g1(z, z, 0)) is None
    assert g2_from_jac_wire(ctx.msm_g2(z, z, 0)) is None


def test_msm_rejects_out_of_range_scalar(ctx):
    rng = random.Random(7)
    _, pts = random_g1(rng, 4)
    sc = [1, 2, 1 << 255, 3]
    with pytest.raises(bendg.BgError) as e:
        ctx.msm_g1(g1_wire(pts), scalars_wire(sc), 4)
    assert e.value.status == bendg.BG_E_ARG
    # the context stays usable
    assert g1_from_jac_wire(ctx.msm_g1(g1_wire(pts), scalars_wire([1, 2, 3, 4]), 4)) == \
        o.msm_naive(o.G1, pts, [1, 2, 3, 4])


def gpu_points(ctx, curve, ks):
    """k_i * G on the device (bg_curve_op MUL), spot-checked against the oracle"""
    gen = g1_wire([o.G1.gen]) if curve == bendg.CURVE_G1 else g2_wire([o.G2.gen])
    n = len(ks)
    p = np.repeat(gen, n, axis=0)
    out = ctx.curve_op(curve, bendg.COP_MUL, p, k16=scalars_wire(ks))
    pw = 32 if curve == bendg.CURVE_G1 else 64
    out = out.reshape(n, pw)
    conv = g1_from_aff_wire if curve == bendg.CURVE_G1 else g2_from_aff_wire
    c = o.G1 if curve == bendg.CURVE_G1 else o.G2
    for i in (0, n // 2, n - 1):
        assert conv(out[i]) == c.mul(c.gen, ks[i])
    return out


@pytest.mark.parametrize("log2n", [12, 16, 20])
def test_msm_g1_dlog_identity(ctx, log2n):
    n = 1 << log2n
    rng = np.random.default_rng(log2n)
    ks = [int.from_bytes(rng.bytes(32), "little") % o.P_FR for _ in range(n)]
    pts = gpu_points(ctx, bendg.CURVE_G1, ks)
    sc = [int.from_bytes(rng.bytes(32), "little") % o.P_FR for _ in range(n)]
    got = g1_from_jac_wire(ctx.msm_g1(pts, scalars_wire(sc), n))
    want = o.FixedBase(o.G1, o.G1.gen).mul(sum(a * b for a, b in zip(ks, sc)) % o.P_FR)
    assert got == want


@pytest.mark.parametrize("log2n", [10, 14, 18])
def test_msm_g2_dlog_identity(ctx, log2n):
    n = 1 << log2n
    rng = np.random.default_rng(100 + log2n)
    ks = [int.from_bytes(rng.bytes(32), "little") % o.P_FR for _ in range(n)]
    pts = gpu_points(ctx, bendg.CURVE_G2, ks)
    sc = [int.from_bytes(rng.bytes(32), "little") % o.P_FR for _ in range(n)]
    got = g2_from_jac_wire(ctx.msm_g2(pts, scalars_wire(sc), n))
    want = o.G2.mul(o.G2.gen, sum(a * b for a, b in zip(ks, sc)) % o.P_FR)
    assert got == want


@pytest.mark.parametrize("curve", [bendg.CURVE_G1, bendg.CURVE_G2])
def test_msm_heavy_buckets(ctx, curve):
    """scalars from {1, 2, r - 1}: a few buckets receive thousands of entries each, cut into
    hundreds of slices that the hierarchical partial folding must join"""
    n = 1 << 15 if curve == bendg.CURVE_G1 else 1 << 12
    rng = np.random.default_rng(31 + curve)
    ks = [int.from_bytes(rng.bytes(32), "little") % o.P_FR for _ in range(n)]
    pts = gpu_points(ctx, curve, ks)
    choices = [1, 2, o.P_FR - 1]
    sc = [choices[int(v)] for v in rng.integers(0, 3, size=n)]
    c = o.G1 if curve == bendg.CURVE_G1 else o.G2
    want = c.mul(c.gen, sum(a * b for a, b in zip(ks, sc)) % o.P_FR)
    if curve == bendg.CURVE_G1:
        assert g1_from_jac_wire(ctx.msm_g1(pts, scalars_wire(sc), n)) == want
    else:
        assert g2_from_jac_wire(ctx.msm_g2(pts, scalars_wire(sc), n)) == want
