"""The serving loop (the serving workload's shape): requests of different K submitted while
others are proving are admitted as lanes and memory free up; every result is the same proof
made alone; a tight HBM budget serialises admission; an over-budget request is refused."""
import random
import time

import pytest

import bendg
import bn254_ref as o
from test_gpu_batch import rs_words, square_chain_witness

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def keys(ctx, tmp_path_factory):
    out = {}
    for k in (6, 8, 10, 12):
        p = str(tmp_path_factory.mktemp("serve") / ("sq%d" % k))
        ctx.synth_square_chain(k, 900 + k, p)
        out[k] = ctx.pk_upload(bendg.HostFiles(p))
    yield out
    for key in out.values():
        key.release()


def make_requests(n, seed):
    rng = random.Random(seed)
    reqs = []
    for tag in range(n):
        k = rng.choice((6, 8, 10, 12))
        reqs.append((tag, k, square_chain_witness(k, rng.randrange(o.P_FR)),
                     rs_words(rng.randrange(o.P_FR), rng.randrange(o.P_FR))))
    return reqs


def test_served_results_equal_alone(ctx, keys):
    reqs = make_requests(24, 7)
    srv = bendg.Server(ctx, lanes=6)
    for i, (tag, k, w, rs) in enumerate(reqs):
        srv.submit(keys[k], w, rs, tag)
        if i % 5 == 4:
            time.sleep(0.002)  # later requests arrive while earlier ones are on the GPU
    got = {}
    while len(got) < len(reqs):
        r = srv.wait(120000)
        assert r is not None, "server stalled"
        tag, proof, _, lat, q, st = r
        assert st == bendg.BG_OK and lat >= q >= 0
        got[tag] = ctx.proof_text(proof)
    srv.close()
    for tag, k, w, rs in reqs:
        alone, _ = keys[k].prove(w, rs)
        assert got[tag] == ctx.proof_text(alone)


def test_served_mix_matches_c_oracle(ctx, tmp_path_factory):
    """a bounded mix of the serving workload's smaller sizes (K in {12, 14, 16}) submitted while
    earlier requests are proving: the request carrying an instance's own witness and r, s must
    equal the C oracle's proof of that instance word for word, every other served proof the
    same request proved alone, and one proof per K must pass the pairing verifier"""
    import numpy as np
    import oracle_c
    from test_gpu_prove import proof_words
    from test_verify import read_vk
    rng = random.Random(1216)
    inst = {}
    for k in (12, 14, 16):
        p = str(tmp_path_factory.mktemp("mix") / ("sq%d" % k))
        ctx.synth_square_chain(k, 1200 + k, p)
        f = bendg.HostFiles(p)
        want, _ = oracle_c.prove_dir(p)
        inst[k] = (p, f, ctx.pk_upload(f), want)
    reqs = []
    for tag in range(18):
        k = (12, 14, 16)[tag % 3] if tag < 3 else rng.choice((12, 14, 16))
        p, f, key, _ = inst[k]
        if tag < 3:  # the instance's own witness and randomness: the C oracle's proof
            w, rs = f.words("witness").copy(), f.words("rs").copy()
        else:
            w = square_chain_witness(k, rng.randrange(o.P_FR))
            rs = rs_words(rng.randrange(o.P_FR), rng.randrange(o.P_FR))
        reqs.append((tag, k, w, rs))
    srv = bendg.Server(ctx, lanes=4)
    for i, (tag, k, w, rs) in enumerate(reqs):
        srv.submit(inst[k][2], w, rs, tag)
        if i % 4 == 3:
            time.sleep(0.003)
    got = {}
    while len(got) < len(reqs):
        r = srv.wait(300000)
        assert r is not None, "server stalled"
        assert r[5] == bendg.BG_OK
        got[r[0]] = proof_words(r[1]).copy()
    srv.close()
    verified = set()
    for tag, k, w, rs in reqs:
        p, f, key, want = inst[k]
        if tag < 3:
            assert np.array_equal(got[tag], want), k
        alone, _ = key.prove(w, rs)
        assert np.array_equal(got[tag], proof_words(alone)), (tag, k)
        if k not in verified:
            from test_verify import proof_from_words
            assert bendg.verify(*read_vk(p), w[16:32], proof_from_words(got[tag]))
            verified.add(k)
    assert verified == {12, 14, 16}
    for p, f, key, _ in inst.values():
        key.release()


def test_tight_budget_serialises(ctx, keys):
    fp = keys[12].footprint()
    assert fp > 0
    srv = bendg.Server(ctx, lanes=4, hbm_budget_bytes=fp + fp // 2)  # room for one K=12 proof at a time
    reqs = [r for r in make_requests(12, 8)]
    for tag, k, w, rs in reqs:
        srv.submit(keys[k], w, rs, tag)
    done = 0
    while done < len(reqs):
        r = srv.wait(120000)
        assert r is not None and r[5] == bendg.BG_OK
        done += 1
        assert srv.reserved_bytes() <= fp + fp // 2
    srv.close()


def test_over_budget_request_refused(ctx, keys):
    srv = bendg.Server(ctx, lanes=1, hbm_budget_bytes=1 << 20)
    tag, k, w, rs = make_requests(1, 9)[0]
    with pytest.raises(bendg.BgError) as e:
        srv.submit(keys[12], w if k == 12 else square_chain_witness(12, 5), rs, tag)
    assert e.value.status == bendg.BG_E_OOM
    assert srv.wait(10) is None
    srv.close()
