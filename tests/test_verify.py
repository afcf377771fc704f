"""The host Groth16 verifier (bg_verify) and pairing (bg_pairing), the role of
`groth16-ref verify` (ref/src/verify.rs:8-27).  Host code only: these run without a GPU.

The pairing is checked for bilinearity and non-degeneracy on oracle points; the verifier must
accept the golden proofs (made by the oracle, checked in the exponent against the fixture's
trapdoor) under a verifying key rebuilt from that trapdoor, and reject tampered proofs, wrong
public inputs and points off the curve."""
import json
import os
import random

import numpy as np
import pytest

import bendg
import bn254_ref as o
from conftest import GOLDEN


def wire(b: bytes) -> np.ndarray:
    return np.frombuffer(b, dtype="<u4").astype(np.uint32)


def g1w(P):
    return wire(o.g1_bytes(P))


def g2w(P):
    return wire(o.g2_bytes(P))


def test_pairing_bilinear_and_nondegenerate(built_lib):
    rng = random.Random(7)
    P, Q = o.G1.gen, o.G2.gen
    a, b = rng.randrange(1, o.P_FR), rng.randrange(1, o.P_FR)
    e_ab = bendg.pairing(g1w(o.G1.mul(P, a)), g2w(o.G2.mul(Q, b)))
    assert np.array_equal(e_ab, bendg.pairing(g1w(o.G1.mul(P, a * b % o.P_FR)), g2w(Q)))
    assert np.array_equal(e_ab, bendg.pairing(g1w(P), g2w(o.G2.mul(Q, a * b % o.P_FR))))
    one = np.zeros(192, dtype=np.uint32)
    one[:16] = wire(o.fe_bytes_mont(1, o.P_FQ))
    e = bendg.pairing(g1w(P), g2w(Q))
    assert not np.array_equal(e, one)                               # non-degenerate
    assert np.array_equal(bendg.pairing(g1w(None), g2w(Q)), one)    # e(O, Q) = 1
    assert not np.array_equal(e, bendg.pairing(g1w(o.G1.neg(P)), g2w(Q)))


def test_pairing_rejects_points_off_the_curve(built_lib):
    bad = g1w(o.G1.gen).copy()
    bad[16] ^= 1  # y + 1 (Montgomery limb flip) is no longer on y^2 = x^3 + 3
    with pytest.raises(bendg.BgError):
        bendg.pairing(bad, g2w(o.G2.gen))


def golden_vk(k: int):
    """the verifying key of a golden fixture, rebuilt from its recorded setup seeds"""
    t = json.load(open(os.path.join(GOLDEN, "k%d" % k, "trapdoor.json")))
    x0 = random.Random(t["seed_witness"]).randrange(o.P_FR)
    setup = o.Setup(o.SquareChain(k, x0), t["seed_setup"])
    assert "%x" % setup.tau == t["tau"][2:]
    f1 = o.FixedBase(o.G1, o.G1.gen)
    return (g1w(f1.mul(setup.alpha)), g2w(o.G2.mul(o.G2.gen, setup.beta)), g2w(o.G2.mul(o.G2.gen, setup.gamma)),
            g2w(o.G2.mul(o.G2.gen, setup.delta)), np.concatenate([g1w(f1.mul(s)) for s in setup.ic_scalars]))


def golden_proof(k: int):
    raw = wire(open(os.path.join(GOLDEN, "k%d" % k, "proof_ref.bin"), "rb").read())
    p = bendg.Proof()
    np.ctypeslib.as_array(p.a)[:] = raw[:32]
    np.ctypeslib.as_array(p.b)[:] = raw[32:96]
    np.ctypeslib.as_array(p.c)[:] = raw[96:128]
    return p


@pytest.mark.parametrize("k", [4, 10])
def test_verify_golden_proofs(built_lib, k):
    vk = golden_vk(k)
    proof = golden_proof(k)
    pub_hex = json.load(open(os.path.join(GOLDEN, "k%d" % k, "public.json")))["inputs"]
    pub = np.concatenate([wire(o.fe_bytes_mont(int(h, 16), o.P_FR)) for h in pub_hex])
    assert bendg.verify(*vk, pub, proof)
    # a wrong public input, a tampered proof and a swapped proof all fail
    wrong = np.concatenate([wire(o.fe_bytes_mont((int(h, 16) + 1) % o.P_FR, o.P_FR)) for h in pub_hex])
    assert not bendg.verify(*vk, wrong, proof)
    swapped = golden_proof(k)
    a = np.ctypeslib.as_array(swapped.a).copy()
    np.ctypeslib.as_array(swapped.a)[:] = np.ctypeslib.as_array(swapped.c)
    np.ctypeslib.as_array(swapped.c)[:] = a
    assert not bendg.verify(*vk, pub, swapped)
    # the cases of ref/src/verify.rs:35-51: C at infinity is a valid point and a rejected proof;
    # A (or C) off the curve cannot be decoded and is an error, not a rejection
    c_inf = golden_proof(k)
    np.ctypeslib.as_array(c_inf.c)[:] = 0
    assert not bendg.verify(*vk, pub, c_inf)
    for field, word in (("a", 0), ("c", 16)):
        off = golden_proof(k)
        np.ctypeslib.as_array(getattr(off, field))[word] ^= 1
        with pytest.raises(bendg.BgError) as err:
            bendg.verify(*vk, pub, off)
        assert err.value.status == bendg.BG_E_FORMAT
    # a public input not below r is undecodable too
    big = np.concatenate([wire(o.fe_bytes_mont(0, o.P_FR)) for _ in pub_hex])
    big[:16] = 0xFFFF
    with pytest.raises(bendg.BgError) as err:
        bendg.verify(*vk, big, proof)
    assert err.value.status == bendg.BG_E_FORMAT


def test_verify_rejects_wrong_public_count(built_lib):
    vk = golden_vk(4)
    with pytest.raises(bendg.BgError) as e:
        bendg.verify(*vk, np.zeros(32, dtype=np.uint32), golden_proof(4))
    assert e.value.status == bendg.BG_E_ARG


def read_vk(path):
    """vk.bin of a generated instance: alpha_g1, beta_g2, gamma_g2, delta_g2, u32 n_ic, IC points"""
    w = np.fromfile(os.path.join(path, "vk.bin"), dtype="<u4").astype(np.uint32)
    n_ic = int(w[224])
    assert w.size == 225 + 32 * n_ic
    return w[0:32], w[32:96], w[96:160], w[160:224], w[225:225 + 32 * n_ic]


def proof_from_words(words):
    p = bendg.Proof()
    np.ctypeslib.as_array(p.a)[:] = words[:32]
    np.ctypeslib.as_array(p.b)[:] = words[32:96]
    np.ctypeslib.as_array(p.c)[:] = words[96:128]
    return p


def test_verify_generated_instance(built_lib, tmp_path):
    """the C oracle's instance generator writes vk.bin; its proof of the instance verifies"""
    import ctypes
    import oracle_c
    L = oracle_c.lib()
    L.bgo_synth_square_chain.argtypes = [ctypes.c_uint32, ctypes.c_uint64, ctypes.c_char_p, ctypes.c_int]
    assert L.bgo_synth_square_chain(6, 2024, str(tmp_path).encode(), 4) == 0
    vk = read_vk(str(tmp_path))
    words, _ = oracle_c.prove_dir(str(tmp_path), threads=4)
    z = np.fromfile(os.path.join(tmp_path, "witness.bin"), dtype="<u4").astype(np.uint32)
    pub = z[16:32]  # x_N, the one public input
    assert bendg.verify(*vk, pub, proof_from_words(words))
    bad = words.copy()
    bad[96:128] = words[0:32]  # C := A
    assert not bendg.verify(*vk, pub, proof_from_words(bad))
