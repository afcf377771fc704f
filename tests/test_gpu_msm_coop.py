"""The cooperative window reduction (msm_coop.cuh: each point addition shared by a group of 8
lanes), forced on with bg_msm_coop_reduce_override: every MSM edge case (zero scalars, points at
infinity, P + P and P + (-P) inside a bucket -- the doubling and cancelling branches of the
cooperative addition --, one bucket holding every entry), heavy buckets, several reduction
shapes through the sizes, and proofs, each against the oracle and against the thread-per-chain
reduction, word for word."""
import random

import numpy as np
import pytest

import bendg
import bn254_ref as o
from gpu_helpers import g1_from_jac_wire, g1_wire, g2_from_jac_wire, g2_wire, scalars_wire
from test_gpu_msm import EDGE, edge_case, gpu_points, random_g1, random_g2

pytestmark = pytest.mark.gpu


@pytest.fixture
def coop(ctx):
    """set the reduction form for one test; the session context returns to the model afterwards"""
    yield lambda m: ctx.coop_reduce_override(m)
    ctx.coop_reduce_override(-1)


@pytest.mark.parametrize("kind", EDGE)
def test_coop_g1_edges(ctx, coop, kind):
    rng = random.Random(900 + (hash(kind) & 0xffff))
    _, base = random_g1(rng, 64)
    pts, sc = edge_case(kind, rng, base)
    want = o.msm_naive(o.G1, pts, sc)
    for m in (0, 1):
        coop(m)
        assert g1_from_jac_wire(ctx.msm_g1(g1_wire(pts), scalars_wire(sc), len(pts))) == want, (kind, m)


@pytest.mark.parametrize("kind", EDGE)
def test_coop_g2_edges(ctx, coop, kind):
    rng = random.Random(950 + (hash(kind) & 0xffff))
    _, base = random_g2(rng, 32)
    pts, sc = edge_case(kind, rng, base)
    want = o.msm_naive(o.G2, pts, sc)
    for m in (0, 1):
        coop(m)
        assert g2_from_jac_wire(ctx.msm_g2(g2_wire(pts), scalars_wire(sc), len(pts))) == want, (kind, m)


@pytest.mark.parametrize("curve,log2n", [(bendg.CURVE_G1, 10), (bendg.CURVE_G1, 14), (bendg.CURVE_G1, 17),
                                         (bendg.CURVE_G2, 9), (bendg.CURVE_G2, 13)])
def test_coop_dlog_identity(ctx, coop, curve, log2n):
    n = 1 << log2n
    rng = np.random.default_rng(970 + log2n + 100 * curve)
    ks = [int.from_bytes(rng.bytes(32), "little") % o.P_FR for _ in range(n)]
    pts = gpu_points(ctx, curve, ks)
    sc = [int.from_bytes(rng.bytes(32), "little") % o.P_FR for _ in range(n)]
    c = o.G1 if curve == bendg.CURVE_G1 else o.G2
    want = c.mul(c.gen, sum(a * b for a, b in zip(ks, sc)) % o.P_FR)
    msm, conv = (ctx.msm_g1, g1_from_jac_wire) if curve == bendg.CURVE_G1 else (ctx.msm_g2, g2_from_jac_wire)
    outs = []
    for m in (0, 1, -1):
        coop(m)
        outs.append(msm(pts, scalars_wire(sc), n))
        assert conv(outs[-1]) == want, m
    assert all(np.array_equal(outs[0], x) for x in outs[1:])


@pytest.mark.parametrize("curve", [bendg.CURVE_G1, bendg.CURVE_G2])
def test_coop_heavy_buckets(ctx, coop, curve):
    n = 1 << 13 if curve == bendg.CURVE_G1 else 1 << 11
    rng = np.random.default_rng(990 + curve)
    ks = [int.from_bytes(rng.bytes(32), "little") % o.P_FR for _ in range(n)]
    pts = gpu_points(ctx, curve, ks)
    choices = [1, 2, o.P_FR - 1]
    sc = [choices[int(v)] for v in rng.integers(0, 3, size=n)]
    c = o.G1 if curve == bendg.CURVE_G1 else o.G2
    want = c.mul(c.gen, sum(a * b for a, b in zip(ks, sc)) % o.P_FR)
    coop(1)
    msm, conv = (ctx.msm_g1, g1_from_jac_wire) if curve == bendg.CURVE_G1 else (ctx.msm_g2, g2_from_jac_wire)
    assert conv(msm(pts, scalars_wire(sc), n)) == want


@pytest.mark.parametrize("log2n", [10, 12])
def test_coop_proofs_match_c_oracle(ctx, coop, tmp_path, log2n):
    """small proofs, whose reductions all end critical paths, against the C oracle with the
    cooperative form forced on and off (resident key and one-shot)"""
    import oracle_c
    from test_gpu_prove import proof_words
    path = str(tmp_path / "sq")
    ctx.synth_square_chain(log2n, 3131 + log2n, path)
    want, _ = oracle_c.prove_dir(path)
    files = bendg.HostFiles(path)
    key = ctx.pk_upload(files)
    for m in (1, 0, -1):
        coop(m)
        proof, _ = key.prove(files.words("witness"), files.words("rs"))
        assert np.array_equal(proof_words(proof), want), m
        proof, _ = ctx.prove_dir(path)
        assert np.array_equal(proof_words(proof), want), m
    key.release()
