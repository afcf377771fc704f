"""Batched proving (the batch workload's shape: many proofs of uneven K in one call):
every proof in the mix is bit-identical to the same proof made alone, and valid."""
import os
import random

import numpy as np
import pytest

import bendg
import bn254_ref as o
import oracle_io

pytestmark = pytest.mark.gpu


def square_chain_witness(log2n: int, x0: int) -> np.ndarray:
    """z = [1, x_N, x_0 .. x_{N-1}] (Montgomery wire words) for x_{i+1} = x_i^2"""
    n = 1 << log2n
    xs = [x0 % o.P_FR]
    for _ in range(n):
        xs.append(xs[-1] * xs[-1] % o.P_FR)
    z = [1, xs[n]] + xs[:n]
    return bendg.ints_to_wire([o.to_mont(v, o.P_FR) for v in z]).reshape(-1)


def rs_words(r: int, s: int) -> np.ndarray:
    return bendg.ints_to_wire([o.to_mont(r, o.P_FR), o.to_mont(s, o.P_FR)]).reshape(-1)


def test_batch_equals_single(ctx, tmp_path):
    rng = random.Random(2026)
    ks = (6, 8, 10, 12)
    keys, files, paths = {}, {}, {}
    for k in ks:
        p = str(tmp_path / ("sq%d" % k))
        ctx.synth_square_chain(k, 500 + k, p)
        files[k] = bendg.HostFiles(p)
        keys[k] = ctx.pk_upload(files[k])
        paths[k] = p
    jobs = []
    for i in range(14):
        k = ks[i % len(ks)] if i < 8 else rng.choice(ks)
        w = square_chain_witness(k, rng.randrange(o.P_FR))
        jobs.append((k, w, rs_words(rng.randrange(o.P_FR), rng.randrange(o.P_FR))))
    proofs, times, st = ctx.prove_batch([keys[k] for k, _, _ in jobs], [w for _, w, _ in jobs],
                                        [r for _, _, r in jobs], lanes=5)
    assert st == [bendg.BG_OK] * len(jobs)
    for (k, w, r), p in zip(jobs, proofs):
        alone, _ = keys[k].prove(w, r)
        assert ctx.proof_text(p) == ctx.proof_text(alone)
    # and a batch proof is valid: check one per K in the exponent
    for k in ks:
        i = next(i for i, j in enumerate(jobs) if j[0] == k)
        data = oracle_io.load_dir(paths[k])
        data["witness"] = jobs[i][1].astype("<u4").tobytes()
        data["rs"] = jobs[i][2].astype("<u4").tobytes()
        trap = oracle_io.trapdoor_from_bin(data["trapdoor"])
        assert oracle_io.square_chain_trapdoor_check(data, trap, oracle_io.parse_proof_text(ctx.proof_text(proofs[i])))
    for k in ks:
        keys[k].release()


def test_batch_rejects_foreign_key(ctx, tmp_path):
    p = str(tmp_path / "sq5")
    ctx.synth_square_chain(5, 5, p)
    files = bendg.HostFiles(p)
    with bendg.Context(0) as other:
        key = other.pk_upload(files)
        with pytest.raises(bendg.BgError) as e:
            ctx.prove_batch([key], [files.words("witness")], [files.words("rs")], lanes=1)
        assert e.value.status == bendg.BG_E_ARG
        key.release()
