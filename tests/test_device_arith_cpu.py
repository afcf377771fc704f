"""The device's field and curve arithmetic (fp.cuh, fp_wide.cuh, ec.cuh), its PTX carry chains
emulated on the host (tests/device_emul.py), against the Python oracle: Fr/Fq add, sub, neg,
CIOS product, squaring product, inverse and Montgomery -> canonical; the 512-bit Karatsuba and
squaring products over the whole 256-bit operand range; the Montgomery reduction over its whole
input range [0, p R); the lazy-reduction forms a b - c d; Fq2 (bend2/src/fq2.bend:31-50); the
XYZZ formulas of G1 and G2 with every special case (infinity on either side, P = Q, P = -Q).
The committed golden vectors (field ops, the 1000 Montgomery pairs, G1/G2 ops) go through the
same emulated functions, and the MSM's window layout and signed-digit recoding (msm.cu) are
checked for every window width.  Every asm statement must also set the carry flag before reading it.
No GPU is involved."""
import random

import pytest

import bn254_ref as o
import device_emul

PQ, PR = o.P_FQ, o.P_FR
RINV_Q = pow(o.R256, -1, PQ)
RINV_R = pow(o.R256, -1, PR)


@pytest.fixture(scope="module")
def dev(tmp_path_factory):
    d = device_emul.DeviceArith(device_emul.build(str(tmp_path_factory.mktemp("device_emul"))))
    yield d
    assert d.fault() == 0, "an asm statement read the carry flag before setting it (line %d)" % d.fault()


def edges(p):
    return [0, 1, 2, 3, p - 1, p - 2, (p - 1) // 2, (p + 1) // 2, o.R256 % p, (1 << 255) % p, (1 << 254) % p]


def operands(p, seed, n):
    rng = random.Random(seed)
    e = edges(p)
    pairs = [(a, b) for a in e for b in e]
    pairs += [(rng.randrange(p), rng.randrange(p)) for _ in range(n)]
    return pairs


@pytest.mark.parametrize("pfx,p,rinv", [("fq", PQ, RINV_Q), ("fr", PR, RINV_R)])
def test_field_ops(dev, pfx, p, rinv):
    W = dev.words
    for a, b in operands(p, 11, 1500):
        assert dev.call(pfx + "_add", [W(a), W(b)], 8) == (a + b) % p
        assert dev.call(pfx + "_sub", [W(a), W(b)], 8) == (a - b) % p
        assert dev.call(pfx + "_mul", [W(a), W(b)], 8) == a * b * rinv % p
        assert dev.call(pfx + "_sqr", [W(a)], 8) == a * a * rinv % p
        assert dev.call(pfx + "_neg", [W(a)], 8) == (-a) % p
        assert dev.call(pfx + "_from_mont", [W(a)], 8) == a * rinv % p
    rng = random.Random(12)
    for a in edges(p)[:6] + [rng.randrange(p) for _ in range(40)]:
        # Montgomery inverse: inv(a R) = a^-1 R, and inv(0) = 0 (bend2/src/fq.bend:1991)
        want = 0 if a == 0 else pow(a * rinv, -1, p) * o.R256 % p
        assert dev.call(pfx + "_inv", [W(a)], 8) == want


@pytest.mark.parametrize("pfx,p,rinv", [("fq", PQ, RINV_Q), ("fr", PR, RINV_R)])
def test_binary_euclid_inverse(dev, pfx, p, rinv):
    """inv_binary (the single inversion of a batch-affine round) is the Montgomery inverse on
    edge operands (small values, powers of two -- the longest runs of halvings -- values next to
    p and to the Montgomery one) and on random ones; inv(0) = 0"""
    W = dev.words
    rng = random.Random(21)
    vals = edges(p) + [1 << k for k in range(0, 254, 7)] + [p - (1 << k) for k in range(1, 250, 13)]
    vals += [o.R256 % p + 1, (o.R256 * o.R256) % p] + [rng.randrange(p) for _ in range(400)]
    for a in vals:
        want = 0 if a == 0 else pow(a * rinv, -1, p) * o.R256 % p
        assert dev.call(pfx + "_inv_binary", [W(a)], 8) == want, hex(a)


def test_wide_products_full_range(dev):
    """the 512-bit products are exact for any 256-bit operands (the Fq2 Karatsuba sums reach 2p)"""
    W = dev.words
    rng = random.Random(13)
    vals = [0, 1, 2, (1 << 128) - 1, 1 << 128, (1 << 255), (1 << 256) - 1, PQ - 1, 2 * PQ - 1, 2 * PQ - 2]
    cases = [(a, b) for a in vals for b in vals] + [(rng.getrandbits(256), rng.getrandbits(256)) for _ in range(3000)]
    for a, b in cases:
        assert dev.call("wide_mul_raw", [W(a), W(b)], 16) == a * b
        assert dev.call("wide_sqr_raw", [W(a)], 16) == a * a


@pytest.mark.parametrize("pfx,p,rinv", [("fq", PQ, RINV_Q), ("fr", PR, RINV_R)])
def test_reduction_whole_input_range(dev, pfx, p, rinv):
    """redc returns t R^-1 mod p, fully reduced, for every t < p R"""
    rng = random.Random(14)
    top = p * o.R256
    ts = [0, 1, p - 1, p, p * p - 1, p * p, 4 * p * p - 1, top - 1, top - p, top - (1 << 256)]
    ts += [rng.randrange(top) for _ in range(3000)] + [rng.randrange(4 * p * p) for _ in range(1000)]
    for t in ts:
        assert dev.call(pfx + "_redc", [dev.words(t, 16)], 8) == t * rinv % p


def test_lazy_fq_products(dev):
    W = dev.words
    rng = random.Random(15)
    for a, b in operands(PQ, 16, 1500):
        assert dev.call("fq_fmul", [W(a), W(b)], 8) == a * b * RINV_Q % PQ
        assert dev.call("fq_fsqr", [W(a)], 8) == a * a * RINV_Q % PQ
        c, d = rng.choice(edges(PQ) + [rng.randrange(PQ)]), rng.randrange(PQ)
        assert dev.call("fq_fmul_sub", [W(a), W(b), W(c), W(d)], 8) == (a * b - c * d) * RINV_Q % PQ
    # extremes of a b - c d: both products zero, maximal positive, maximal negative
    m = PQ - 1
    for a, b, c, d in [(0, 0, 0, 0), (m, m, 0, 0), (0, 0, m, m), (m, m, m, m), (1, 0, m, m)]:
        assert dev.call("fq_fmul_sub", [W(a), W(b), W(c), W(d)], 8) == (a * b - c * d) * RINV_Q % PQ


def f2_words(dev, a):
    """Fq2 (c0, c1), canonical -> device words (Montgomery)"""
    return dev.words(o.to_mont(a[0], PQ) | (o.to_mont(a[1], PQ) << 256), 16)


def f2_value(v):
    return (o.from_mont(v & ((1 << 256) - 1), PQ), o.from_mont(v >> 256, PQ))


def test_fq2(dev):
    rng = random.Random(17)
    e = [0, 1, PQ - 1, (PQ - 1) // 2]
    vals = [(x, y) for x in e for y in e] + [(rng.randrange(PQ), rng.randrange(PQ)) for _ in range(300)]
    for i, a in enumerate(vals):
        b = vals[(i * 7 + 3) % len(vals)]
        c, d = vals[(i * 5 + 1) % len(vals)], vals[(i * 3 + 2) % len(vals)]
        A, B, C, D = (f2_words(dev, x) for x in (a, b, c, d))
        ab = o.f2_mul(a, b)
        assert f2_value(dev.call("fq2_mul", [A, B], 16)) == ab
        assert f2_value(dev.call("fq2_fmul", [A, B], 16)) == ab
        assert f2_value(dev.call("fq2_sqr", [A], 16)) == o.f2_sqr(a)
        assert f2_value(dev.call("fq2_fsqr", [A], 16)) == o.f2_sqr(a)
        assert f2_value(dev.call("fq2_fmul_sub", [A, B, C, D], 16)) == o.f2_sub(ab, o.f2_mul(c, d))
        if i % 10 == 0:
            want = (0, 0) if a == (0, 0) else o.f2_inv(a)
            assert f2_value(dev.call("fq2_inv", [A], 16)) == want
        if i % 3 == 0:
            want = (0, 0) if a == (0, 0) else o.f2_inv(a)
            assert f2_value(dev.call("fq2_inv_fast", [A], 16)) == want


class CurveIO:
    """device words of affine and XYZZ points of one curve, from and to the oracle's affine form"""

    def __init__(self, dev, curve, g2: bool):
        self.dev, self.curve, self.g2 = dev, curve, g2
        self.fw = 16 if g2 else 8  # words per field element

    def fe(self, x) -> int:
        if self.g2:
            return o.to_mont(x[0], PQ) | (o.to_mont(x[1], PQ) << 256)
        return o.to_mont(x, PQ)

    def fe_value(self, v):
        if self.g2:
            return f2_value(v)
        return o.from_mont(v, PQ)

    def mul(self, a, b):
        return o.f2_mul(a, b) if self.g2 else a * b % PQ

    def inv(self, a):
        return o.f2_inv(a) if self.g2 else pow(a, -1, PQ)

    def one(self):
        return (1, 0) if self.g2 else 1

    def pack(self, elems) -> int:
        bits = 32 * self.fw
        return sum(self.fe(x) << (bits * i) for i, x in enumerate(elems))

    def affine(self, P):
        if P is None:
            return self.dev.words(0, 2 * self.fw)
        return self.dev.words(self.pack([P[0], P[1]]), 2 * self.fw)

    def xyzz(self, P, lam):
        """P with ZZ = lam^2, ZZZ = lam^3; infinity as the device writes it (ZZ = 0)"""
        if P is None:
            one = self.one()
            zero = (0, 0) if self.g2 else 0
            return self.dev.words(self.pack([one, one, zero, zero]), 4 * self.fw)
        zz = self.mul(lam, lam)
        zzz = self.mul(zz, lam)
        return self.dev.words(self.pack([self.mul(P[0], zz), self.mul(P[1], zzz), zz, zzz]), 4 * self.fw)

    def from_xyzz(self, v):
        bits = 32 * self.fw
        mask = (1 << bits) - 1
        x, y, zz, zzz = (self.fe_value((v >> (bits * i)) & mask) for i in range(4))
        zero = (0, 0) if self.g2 else 0
        if zz == zero:
            return None
        # the XYZZ invariant ZZ^3 = ZZZ^2
        assert self.mul(self.mul(zz, zz), zz) == self.mul(zzz, zzz)
        P = (self.mul(x, self.inv(zz)), self.mul(y, self.inv(zzz)))
        assert self.curve.on_curve(P)
        return P

    def rand_lam(self, rng):
        return (rng.randrange(1, PQ), rng.randrange(PQ)) if self.g2 else rng.randrange(1, PQ)


@pytest.mark.parametrize("g2", [False, True], ids=["g1", "g2"])
def test_xyzz_formulas(dev, g2):
    curve = o.G2 if g2 else o.G1
    io = CurveIO(dev, curve, g2)
    pfx = "g2" if g2 else "g1"
    rng = random.Random(18 + g2)
    f = o.FixedBase(curve, curve.gen)
    pts = [f.mul(rng.randrange(1, PR)) for _ in range(12 if g2 else 30)]
    nw = 4 * io.fw
    for i, P in enumerate(pts):
        Q = pts[(i + 1) % len(pts)]
        lp, lq = io.rand_lam(rng), io.rand_lam(rng)
        cases = [(P, Q), (P, P), (P, curve.neg(P)), (None, Q), (P, None), (None, None)]
        for A, B in cases:
            want = curve.add(A, B)
            got = io.from_xyzz(dev.call(pfx + "_madd", [io.xyzz(A, lp), io.affine(B)], nw))
            assert got == want, (pfx, "madd", i, A is None, B is None)
            got = io.from_xyzz(dev.call(pfx + "_add", [io.xyzz(A, lp), io.xyzz(B, lq)], nw))
            assert got == want, (pfx, "add", i, A is None, B is None)
            # commuted (the reference's commuted-add case, bend2/tests/test_g1.bend)
            got = io.from_xyzz(dev.call(pfx + "_madd", [io.xyzz(B, lq), io.affine(A)], nw))
            assert got == want, (pfx, "madd commuted", i, A is None, B is None)
        assert io.from_xyzz(dev.call(pfx + "_dbl", [io.xyzz(P, lp)], nw)) == curve.double(P)
        assert io.from_xyzz(dev.call(pfx + "_dbl", [io.xyzz(None, lp)], nw)) is None
        assert io.from_xyzz(dev.call(pfx + "_dbl_affine", [io.affine(P)], nw)) == curve.double(P)
        assert io.from_xyzz(dev.call(pfx + "_from_affine", [io.affine(P)], nw)) == P
        assert io.from_xyzz(dev.call(pfx + "_from_affine", [io.affine(None)], nw)) is None


@pytest.mark.parametrize("g2", [False, True], ids=["g1", "g2"])
def test_affine_pair_additions(dev, g2):
    """the affine pair addition of the batch-affine rounds (pair_kind + pair_finish) with every
    case: the chord, the tangent (P = Q), P = -Q, infinity on either side or both"""
    import ctypes
    curve = o.G2 if g2 else o.G1
    io = CurveIO(dev, curve, g2)
    pfx = "g2" if g2 else "g1"
    rng = random.Random(22 + g2)
    f = o.FixedBase(curve, curve.gen)
    pts = [f.mul(rng.randrange(1, PR)) for _ in range(10 if g2 else 30)]
    nw = 2 * io.fw
    bits = 32 * io.fw

    def add(A, B):
        kind = ctypes.c_uint32()
        out = (ctypes.c_uint32 * nw)()
        getattr(dev.lib, pfx + "_pair_add")(io.affine(A), io.affine(B), ctypes.byref(kind), out)
        v = dev.value(out)
        x, y = io.fe_value(v & ((1 << bits) - 1)), io.fe_value(v >> bits)
        zero = (0, 0) if g2 else 0
        return kind.value, (None if (x, y) == (zero, zero) else (x, y))

    for i, P in enumerate(pts):
        Q = pts[(i + 1) % len(pts)]
        for A, B, k in [(P, Q, 0), (P, P, 1), (P, curve.neg(P), 2), (P, None, 3), (None, Q, 4), (None, None, 4)]:
            kind, got = add(A, B)
            assert kind == k and got == curve.add(A, B), (pfx, i, k)
            if got is not None:
                assert curve.on_curve(got)


def _mutated_build(tmp_path, edit):
    """the emulation built from a copy of the headers with one planted mistake"""
    import shutil
    src = tmp_path / "csrc"
    src.mkdir()
    for h in device_emul.HEADERS:
        shutil.copy(f"{device_emul.CSRC}/{h}", src / h)
    edit(src)
    old = device_emul.CSRC
    device_emul.CSRC = str(src)
    try:
        return device_emul.DeviceArith(device_emul.build(str(tmp_path / "out")))
    finally:
        device_emul.CSRC = old


def test_emulation_sees_a_dropped_carry(tmp_path):
    """planting a carry-chain mistake in a copy of fp_wide.cuh (one madc.hi that ignores the
    incoming carry) makes the products disagree with the oracle: the emulation runs the chains,
    it does not restate the arithmetic"""
    def edit(src):
        t = (src / "fp_wide.cuh").read_text()
        i = t.index("madc.hi.cc.u32", t.index("BG_DEV void wide_mul("))
        (src / "fp_wide.cuh").write_text(t[:i] + "mad.hi.cc.u32 " + t[i + len("madc.hi.cc.u32"):])
    d = _mutated_build(tmp_path, edit)
    rng = random.Random(19)
    bad = sum(d.call("wide_mul_raw", [d.words(a), d.words(b)], 16) != a * b
              for a, b in ((rng.getrandbits(256), rng.getrandbits(256)) for _ in range(200)))
    assert bad > 20  # the carry is set in about a quarter of random products


def test_emulation_flags_an_unset_carry(tmp_path):
    """a chain whose first instruction reads the carry flag (left over from another asm
    statement on the device) is reported"""
    def edit(src):
        t = (src / "fp.cuh").read_text()
        i = t.index('asm("add.cc.u32', t.index("BG_DEV Fp<P> add("))
        (src / "fp.cuh").write_text(t[:i] + 'asm("addc.cc.u32' + t[i + len('asm("add.cc.u32'):])
    d = _mutated_build(tmp_path, edit)
    assert d.fault() == 0
    d.call("fq_add", [d.words(1), d.words(2)], 8)
    assert d.fault() != 0


def _records(name, cols):
    import os
    import struct

    import numpy as np
    from conftest import GOLDEN
    buf = open(os.path.join(GOLDEN, *name), "rb").read()
    (n,) = struct.unpack_from("<I", buf, 0)
    return np.frombuffer(buf, dtype="<u4", offset=4).reshape(n, cols).astype(np.uint32)


def _v16(words) -> int:
    """a bend2/FORMAT.md field element (16 words of 16-bit limbs) as an integer"""
    return o.from_words16([int(x) for x in words])


@pytest.mark.parametrize("name,pfx", [("fr_ops", "fr"), ("fq_ops", "fq")])
def test_golden_field_vectors(dev, name, pfx):
    """the committed field vectors (shapes of bend2/tests/test_fr.bend, test_fq.bend) through the
    device arithmetic: a, b, a + b, a - b, a b, -a, 1/a, a^2, canonical a"""
    rec = _records(("vectors", name + ".bin"), 9 * 16).reshape(-1, 9, 16)
    W = dev.words
    for r in rec:
        a, b = _v16(r[0]), _v16(r[1])
        assert dev.call(pfx + "_add", [W(a), W(b)], 8) == _v16(r[2])
        assert dev.call(pfx + "_sub", [W(a), W(b)], 8) == _v16(r[3])
        assert dev.call(pfx + "_mul", [W(a), W(b)], 8) == _v16(r[4])
        assert dev.call(pfx + "_neg", [W(a)], 8) == _v16(r[5])
        assert dev.call(pfx + "_inv", [W(a)], 8) == _v16(r[6])
        assert dev.call(pfx + "_sqr", [W(a)], 8) == _v16(r[7])
        assert dev.call(pfx + "_from_mont", [W(a)], 8) == _v16(r[8])
        if pfx == "fq":
            assert dev.call("fq_fmul", [W(a), W(b)], 8) == _v16(r[4])
            assert dev.call("fq_fsqr", [W(a)], 8) == _v16(r[7])


def test_golden_montmul_pairs(dev):
    """the 1000 Montgomery products from the reference's check_montmul.py operand generator"""
    rec = _records(("montmul_fr.bin",), 3 * 16).reshape(-1, 3, 16)
    W = dev.words
    for r in rec:
        assert dev.call("fr_mul", [W(_v16(r[0])), W(_v16(r[1]))], 8) == _v16(r[2])


@pytest.mark.parametrize("name,g2", [("g1_ops", False), ("g2_ops", True)], ids=["g1", "g2"])
def test_golden_curve_vectors(dev, name, g2):
    """the committed curve vectors (shapes of bend2/tests/test_g1.bend, test_g2.bend; cases 0-2
    are infinity, P = Q and P = -Q): P + Q by the mixed addition and 2P by the XYZZ doubling of
    the device, normalised to affine on the host"""
    pw = 64 if g2 else 32
    rec = _records(("vectors", name + ".bin"), 6 * pw + 16)
    curve = o.G2 if g2 else o.G1
    io = CurveIO(dev, curve, g2)
    fe = 16  # wire words per Fq element

    def aff(words):
        vals = [o.from_mont(_v16(words[i * fe:(i + 1) * fe]), PQ) for i in range(pw // fe)]
        if not any(vals):
            return None
        return ((vals[0], vals[1]), (vals[2], vals[3])) if g2 else (vals[0], vals[1])

    pfx = "g2" if g2 else "g1"
    nw = 4 * io.fw
    for r in rec:
        P, Q = aff(r[0:pw]), aff(r[pw:2 * pw])
        want_add, want_dbl = aff(r[2 * pw + 16:3 * pw + 16]), aff(r[3 * pw + 16:4 * pw + 16])
        xp = dev.call(pfx + "_from_affine", [io.affine(P)], nw)
        got = io.from_xyzz(dev.call(pfx + "_madd", [dev.words(xp, nw), io.affine(Q)], nw))
        assert got == want_add
        assert io.from_xyzz(dev.call(pfx + "_dbl", [dev.words(xp, nw)], nw)) == want_dbl


@pytest.fixture(scope="module")
def digits_lib(tmp_path_factory):
    import ctypes
    return ctypes.CDLL(device_emul.build_digits(str(tmp_path_factory.mktemp("digits_emul"))))


def test_msm_window_layout_and_signed_digits(digits_lib):
    """the MSM's balanced windows and signed-digit recoding (msm.cu, used by k_digits_hist and
    k_scatter) for every window width the library accepts: the W = floor(254 / c) + 1 windows
    tile bits [0, 255) with widths of at most c, every digit's magnitude is at most 2^(b-1) for
    its b-bit window (so its bucket index fits 2^(c-1) buckets), no carry leaves the top window,
    and sum_w +-|d_w| 2^(o_w) gives the scalar back -- for edge scalars (0, 1, r - 1, 2^254 - 1,
    all-ones and alternating bit patterns, runs that make carries ripple) and random ones"""
    import ctypes
    L = digits_lib
    L.digits.restype = ctypes.c_uint32
    rng = random.Random(20)
    top = (1 << 254) - 1
    edge = [0, 1, 2, PR - 1, top, top // 3, (top // 3) * 2, (1 << 253), (1 << 253) - 1]
    edge += [((1 << k) - 1) for k in (15, 16, 17, 31, 32, 33, 127, 128, 200, 253)]
    for c in range(2, 23):
        W = 254 // c + 1
        widths = [L.digit_window_width(w, W) for w in range(W)]
        offsets = [L.digit_window_offset(w, W) for w in range(W)]
        assert sum(widths) == 255 and max(widths) <= c and min(widths) >= max(widths) - 1
        assert offsets == [sum(widths[:w]) for w in range(W)]
        # scalars whose every window digit sits at the sign boundary 2^(b-1) and just above it
        half = sum(1 << (o + b - 1) for o, b in zip(offsets, widths)) & top
        above = sum(((1 << (b - 1)) + 1) << o for o, b in zip(offsets, widths)) & top
        cases = edge + [half, above] + [rng.getrandbits(254) for _ in range(300 if c < 8 else 60)]
        mags = (ctypes.c_uint32 * W)()
        negs = (ctypes.c_uint8 * W)()
        for s in cases:
            words = (ctypes.c_uint32 * 8)(*[(s >> (32 * i)) & 0xFFFFFFFF for i in range(8)])
            carry = L.digits(words, W, mags, negs)
            assert carry == 0, (c, s)
            total = 0
            for w in range(W):
                assert mags[w] <= 1 << (widths[w] - 1), (c, s, w)
                # a window of all ones plus a carry gives magnitude 0 (flagged negative, with
                # the carry passed up): no bucket entry, as the kernels skip magnitude 0
                total += (-1 if negs[w] else 1) * mags[w] << offsets[w]
            assert total == s, (c, s)


def test_emulation_rejects_a_read_of_an_unwritten_output(tmp_path):
    """a chain that reads one of its own write-only outputs before writing it (undefined on the
    device) is refused when the headers are translated"""
    def edit(src):
        t = (src / "fp.cuh").read_text()
        i = t.index('asm("add.cc.u32  %0, %8,', t.index("BG_DEV Fp<P> add("))
        (src / "fp.cuh").write_text(t[:i] + 'asm("add.cc.u32  %0, %1,' + t[i + len('asm("add.cc.u32  %0, %8,'):])
    with pytest.raises(ValueError, match="no value yet"):
        _mutated_build(tmp_path, edit)
