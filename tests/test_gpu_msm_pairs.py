"""The batch-affine pair rounds of the MSM bucket accumulation (msm_pairs.cuh), forced on with
bg_msm_pair_rounds_override at sizes where the cost model would not use them: every edge case of
the MSM tests (zero scalars, points at infinity, P + P and P + (-P) inside a bucket, one bucket
holding every entry), heavy buckets, and the discrete-log identity at mid sizes, each checked
against the oracle and against the accumulation without rounds.  Results must not depend on
the number of rounds (an MSM's value is a unique group element)."""
import random

import numpy as np
import pytest

import bendg
import bn254_ref as o
from gpu_helpers import g1_from_jac_wire, g1_wire, g2_from_jac_wire, g2_wire, scalars_wire
from test_gpu_msm import EDGE, edge_case, gpu_points, random_g1, random_g2

pytestmark = pytest.mark.gpu


@pytest.fixture
def rounds(ctx):
    """set the round count for one test; the session context returns to the model afterwards"""
    yield lambda r: ctx.pair_rounds_override(r)
    ctx.pair_rounds_override(-1)


@pytest.mark.parametrize("kind", EDGE)
def test_pair_rounds_g1_edges(ctx, rounds, kind):
    rng = random.Random(500 + (hash(kind) & 0xffff))
    _, base = random_g1(rng, 64)
    pts, sc = edge_case(kind, rng, base)
    want = o.msm_naive(o.G1, pts, sc)
    for r in (0, 1, 2, 3, 6):
        rounds(r)
        assert g1_from_jac_wire(ctx.msm_g1(g1_wire(pts), scalars_wire(sc), len(pts))) == want, (kind, r)


@pytest.mark.parametrize("kind", EDGE)
def test_pair_rounds_g2_edges(ctx, rounds, kind):
    rng = random.Random(600 + (hash(kind) & 0xffff))
    _, base = random_g2(rng, 32)
    pts, sc = edge_case(kind, rng, base)
    want = o.msm_naive(o.G2, pts, sc)
    for r in (0, 1, 2, 5):
        rounds(r)
        assert g2_from_jac_wire(ctx.msm_g2(g2_wire(pts), scalars_wire(sc), len(pts))) == want, (kind, r)


@pytest.mark.parametrize("curve,log2n,rs", [(bendg.CURVE_G1, 14, (1, 3, 5)), (bendg.CURVE_G2, 12, (1, 2, 4))])
def test_pair_rounds_dlog_identity(ctx, rounds, curve, log2n, rs):
    n = 1 << log2n
    rng = np.random.default_rng(700 + log2n)
    ks = [int.from_bytes(rng.bytes(32), "little") % o.P_FR for _ in range(n)]
    pts = gpu_points(ctx, curve, ks)
    sc = [int.from_bytes(rng.bytes(32), "little") % o.P_FR for _ in range(n)]
    c = o.G1 if curve == bendg.CURVE_G1 else o.G2
    want = c.mul(c.gen, sum(a * b for a, b in zip(ks, sc)) % o.P_FR)
    msm, conv = (ctx.msm_g1, g1_from_jac_wire) if curve == bendg.CURVE_G1 else (ctx.msm_g2, g2_from_jac_wire)
    outs = []
    for r in (0,) + rs:
        rounds(r)
        outs.append(msm(pts, scalars_wire(sc), n))
        assert conv(outs[-1]) == want, r
    assert all(np.array_equal(outs[0], x) for x in outs[1:])


@pytest.mark.parametrize("curve", [bendg.CURVE_G1, bendg.CURVE_G2])
def test_pair_rounds_heavy_buckets(ctx, rounds, curve):
    """scalars from {1, 2, r - 1}: a few buckets of thousands of entries, still hundreds of
    points after the rounds, which the XYZZ accumulation's heavy-bucket pass then joins"""
    n = 1 << 14 if curve == bendg.CURVE_G1 else 1 << 11
    rng = np.random.default_rng(800 + curve)
    ks = [int.from_bytes(rng.bytes(32), "little") % o.P_FR for _ in range(n)]
    pts = gpu_points(ctx, curve, ks)
    choices = [1, 2, o.P_FR - 1]
    sc = [choices[int(v)] for v in rng.integers(0, 3, size=n)]
    c = o.G1 if curve == bendg.CURVE_G1 else o.G2
    want = c.mul(c.gen, sum(a * b for a, b in zip(ks, sc)) % o.P_FR)
    msm, conv = (ctx.msm_g1, g1_from_jac_wire) if curve == bendg.CURVE_G1 else (ctx.msm_g2, g2_from_jac_wire)
    for r in (2, 4):
        rounds(r)
        assert conv(msm(pts, scalars_wire(sc), n)) == want, r
