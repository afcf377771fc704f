"""The oracle, pinned: checked against the golden fixtures the reference's own tooling
produced (tests/golden/gen_golden.py) and against constants in the reference sources."""
import json
import os
import struct

import pytest

import bn254_ref as o
from conftest import GOLDEN


def rd(name):
    return open(os.path.join(GOLDEN, name), "rb").read()


def test_bend_constants():
    # Montgomery literals of bend2/src/ntt.bend:24-41 and bend2/src/fr.bend / fq.bend
    assert o.words16(o.to_mont(o.ROOT_2_28, o.P_FR)) == [15772, 32977, 29525, 25454, 65494, 9285, 62324, 41515,
                                                         984, 7858, 10944, 22085, 63975, 10595, 61332, 6240]
    assert o.words16(o.to_mont(5, o.P_FR)) == [65510, 40959, 3833, 6925, 37183, 41770, 26787, 60090, 1673,
                                                55517, 60278, 18392, 48067, 8437, 2133, 5584]
    assert o.words16(o.to_mont(pow(2, -1, o.P_FR), o.P_FR)) == [65534, 8191, 5336, 30780, 7901, 3213, 12143,
                                                                 44952, 20293, 64765, 29842, 36703, 49068,
                                                                 15772, 25370, 7991]
    assert o.words16(o.to_mont(1, o.P_FR)) == [65531, 20479, 13340, 44182, 52521, 40800, 30357, 14076, 17966,
                                                30841, 41839, 26222, 57135, 39431, 30657, 3594]
    assert o.words16(o.to_mont(1, o.P_FQ)) == [3485, 50575, 17293, 54109, 2877, 62919, 60200, 2680, 17964,
                                                30841, 41839, 26222, 57135, 39431, 30657, 3594]
    assert o.words16(o.P_FQ) == [64839, 55420, 35862, 15392, 51853, 26737, 27281, 38785, 22621, 33153, 17846,
                                 47184, 41001, 57649, 20082, 12388]
    assert (-pow(o.P_FR, -1, 1 << 16)) % (1 << 16) == 65535  # n0' of bend2/src/fr.bend:4
    assert (-pow(o.P_FQ, -1, 1 << 16)) % (1 << 16) == 25481  # n0' of bend2/src/fq.bend:4


def test_curve_constants():
    assert o.G1.on_curve(o.G1.gen) and o.G2.on_curve(o.G2.gen)
    assert o.G1.mul(o.G1.gen, o.P_FR) is None and o.G2.mul(o.G2.gen, o.P_FR) is None


def test_montmul_pairs():
    buf = rd("montmul_fr.bin")
    (count,) = struct.unpack_from("<I", buf, 0)
    assert count == 1000
    for i in range(count):
        a, b, want = (o.from_words16(struct.unpack_from("<16I", buf, 4 + 64 * (3 * i + j))) for j in range(3))
        assert o.mont_mul(a, b, o.P_FR) == want


@pytest.mark.parametrize("name,p", [("fr_ops", o.P_FR), ("fq_ops", o.P_FQ)])
def test_field_vectors(name, p):
    buf = rd("vectors/%s.bin" % name)
    (count,) = struct.unpack_from("<I", buf, 0)
    for c in range(count):
        v = [o.read_fe(buf, 4 + 64 * (9 * c + j), p) for j in range(8)]
        a, b, add, sub, mul, neg, inv, sq = v
        assert (a + b) % p == add and (a - b) % p == sub and a * b % p == mul
        assert (-a) % p == neg and a * inv % p == 1 and a * a % p == sq
        assert o.read_fe(buf, 4 + 64 * (9 * c + 8), p, mont=False) == a


@pytest.mark.parametrize("name,curve,size,reader", [("g1_ops", o.G1, 128, o.read_g1), ("g2_ops", o.G2, 256, o.read_g2)])
def test_curve_vectors(name, curve, size, reader):
    buf = rd("vectors/%s.bin" % name)
    (count,) = struct.unpack_from("<I", buf, 0)
    off = 4
    for c in range(count):
        p = reader(buf, off)
        q = reader(buf, off + size)
        k = o.read_fe(buf, off + 2 * size, o.P_FR, mont=False)
        add, dbl, neg, mul = (reader(buf, off + 2 * size + 64 + size * j) for j in range(4))
        off += 6 * size + 64
        assert curve.on_curve(p) and curve.on_curve(q)
        assert curve.add(p, q) == add and curve.double(p) == dbl and curve.neg(p) == neg
        assert curve.mul(p, k) == mul
        if c == 0:
            assert p is None
        if c == 2:
            assert add is None


@pytest.mark.parametrize("n", [8, 64, 1024])
def test_msm_vectors(n):
    buf = rd("vectors/msm_small_%d.bin" % n)
    assert struct.unpack_from("<I", buf, 0)[0] == n
    pts = [o.read_g1(buf, 4 + 128 * i) for i in range(n)]
    sc = [o.read_fe(buf, 4 + 128 * n + 64 * i, o.P_FR, mont=False) for i in range(n)]
    res = o.read_g1(buf, 4 + 192 * n)
    if n <= 64:
        assert o.msm_naive(o.G1, pts, sc) == res
    assert o.msm_pippenger(o.G1, pts, sc) == res


@pytest.mark.parametrize("n", [8, 64, 1024])
def test_ntt_vectors(n):
    buf = rd("vectors/ntt_small_%d.bin" % n)
    assert struct.unpack_from("<I", buf, 0)[0] == n
    lg = n.bit_length() - 1
    assert o.read_fe(buf, 4, o.P_FR) == o.omega(lg)
    assert o.read_fe(buf, 68, o.P_FR) == pow(n, -1, o.P_FR)
    coeffs = [o.read_fe(buf, 132 + 64 * i, o.P_FR) for i in range(n)]
    evals = [o.read_fe(buf, 132 + 64 * (n + i), o.P_FR) for i in range(n)]
    assert o.ntt(coeffs) == evals and o.intt(evals) == coeffs


@pytest.mark.parametrize("k", [4, 10])
def test_qap_h_against_ref_qap(k):
    """h_ref.bin was written by the reference's bend2/gen/ref_qap.py"""
    d = os.path.join(GOLDEN, "k%d" % k)
    lg = struct.unpack("<8I", open(os.path.join(d, "header.bin"), "rb").read())[3]
    n = 1 << lg
    abc = open(os.path.join(d, "abc_evals.bin"), "rb").read()
    href = open(os.path.join(d, "h_ref.bin"), "rb").read()
    a, b, c = ([o.read_fe(abc, 64 * (j * n + i), o.P_FR) for i in range(n)] for j in range(3))
    h = [o.read_fe(href, 64 * i, o.P_FR) for i in range(n)]
    assert o.qap_h(a, b, c) == h


@pytest.mark.parametrize("k", [4, 10])
def test_proof_ref_trapdoor(k):
    """the committed proof is valid (checked in the exponent with the fixture's trapdoor)"""
    from oracle_io import load_dir, square_chain_trapdoor_check
    d = os.path.join(GOLDEN, "k%d" % k)
    data = load_dir(d)
    trap = json.load(open(os.path.join(d, "trapdoor.json")))
    proof = (o.read_g1(data["proof_ref"], 0), o.read_g2(data["proof_ref"], 128), o.read_g1(data["proof_ref"], 384))
    assert square_chain_trapdoor_check(data, {k2: int(v, 16) for k2, v in trap.items() if k2 in
                                              ("tau", "alpha", "beta", "gamma", "delta")}, proof)
