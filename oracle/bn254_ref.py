"""CPU oracle (test infrastructure, not product code) for the Groth16/BN254 prover hot path.

Pure-Python big-int restatement of the reference's algorithms.  Only the tests, the smoke
check and the CPU-baseline leg of the benchmark use this module, and only as the checker.

What it restates (reference paths are relative to the bend-groth16 project root):
  * Fr / Fq field, Montgomery form with R = 2^256, 16-bit-limb wire words
      bend2/FORMAT.md:5-12, bend2/src/fr.bend:1-30, bend2/src/fq.bend:1-30
  * Fq2 = Fq[u]/(u^2+1), Karatsuba mul / complex square / norm inverse
      bend2/src/fq2.bend:1-50
  * G1 / G2 short Weierstrass (a = 0), affine infinity encoded as (0, 0)
      bend2/src/g1.bend:1-75, bend2/src/g2.bend:1-20
  * Pippenger MSM semantics (sum_i s_i P_i, canonical scalars, Jacobian result)
      bend2/src/msm.bend:34-58, :192-239, :297
  * radix-2 NTT / iNTT / coset NTT over arkworks' Radix2EvaluationDomain and the
    LibsnarkReduction quotient h(x)
      bend2/gen/ref_qap.py:18-72, bend2/src/ntt.bend:22-77, :446-459
  * R1CS evaluation vectors incl. libsnark input-consistency rows
      bend2/src/groth16.bend:162-188, bend2/gen/ref_qap.py:105-107
  * Groth16 proof combination A / B / C
      ref/README.md:24-32, bend2/src/groth16.bend:298-308
  * SquareChain(N) circuit and assignment z = [1, x_N, x_0..x_{N-1}]
      ref/src/circuit.rs:21-74, ref/src/gen.rs:78-93
  * a seeded Groth16 setup of our own with a known trapdoor (tau, alpha, beta, gamma,
    delta); the arkworks setup RNG is not reproduced.  With the trapdoor every proof can
    be checked without pairings: A = a_s*G1, B = b_s*G2, C = c_s*G1 for scalars a_s, b_s,
    c_s computed in Fr (trapdoor_check).
"""
from __future__ import annotations

import random
import struct

# ---------------------------------------------------------------- fields

P_FR = 21888242871839275222246405745257275088548364400416034343698204186575808495617
P_FQ = 21888242871839275222246405745257275088696311157297823662689037894645226208583
R256 = 1 << 256
# 2-adic root of unity of order 2^28 and the coset generator g = Fr::GENERATOR = 5
# (bend2/gen/gen_ntt.py:9-11, bend2/gen/ref_qap.py:18-20)
ROOT_2_28 = 19103219067921713944291392827692070036145651957329286315305642004821462161904
GEN = 5
TWO_ADICITY = 28


def to_mont(x: int, p: int) -> int:
    return x * R256 % p


def from_mont(x: int, p: int) -> int:
    return x * pow(R256, -1, p) % p


def mont_mul(a: int, b: int, p: int) -> int:
    """a*b*2^-256 mod p: the product the CIOS kernels compute (bend2/gen/gen_field.py:105-135)."""
    return a * b * pow(R256, -1, p) % p


# ---- FORMAT.md wire words: 16 x u32, each holding one 16-bit limb, little-endian

def words16(x: int) -> list[int]:
    return [(x >> (16 * j)) & 0xFFFF for j in range(16)]


def from_words16(w) -> int:
    return sum(int(v) << (16 * j) for j, v in enumerate(w))


def words32(x: int) -> list[int]:
    """packed layout used on the device: 8 x u32 limbs, little-endian"""
    return [(x >> (32 * j)) & 0xFFFFFFFF for j in range(8)]


def from_words32(w) -> int:
    return sum(int(v) << (32 * j) for j, v in enumerate(w))


# ---------------------------------------------------------------- Fq2 (bend2/src/fq2.bend)

def f2_add(a, b):
    return ((a[0] + b[0]) % P_FQ, (a[1] + b[1]) % P_FQ)


def f2_sub(a, b):
    return ((a[0] - b[0]) % P_FQ, (a[1] - b[1]) % P_FQ)


def f2_neg(a):
    return ((-a[0]) % P_FQ, (-a[1]) % P_FQ)


def f2_mul(a, b):
    """Karatsuba, u^2 = -1 (bend2/src/fq2.bend:31-38)"""
    t0 = a[0] * b[0] % P_FQ
    t1 = a[1] * b[1] % P_FQ
    t2 = (a[0] + a[1]) * (b[0] + b[1]) % P_FQ
    return ((t0 - t1) % P_FQ, (t2 - t0 - t1) % P_FQ)


def f2_sqr(a):
    """complex squaring (bend2/src/fq2.bend:40-44)"""
    return ((a[0] + a[1]) * (a[0] - a[1]) % P_FQ, 2 * a[0] * a[1] % P_FQ)


def f2_inv(a):
    """(a0 - a1 u)/(a0^2 + a1^2); inv(0) = 0 (bend2/src/fq2.bend:46-50)"""
    n = (a[0] * a[0] + a[1] * a[1]) % P_FQ
    ni = pow(n, -1, P_FQ) if n else 0
    return (a[0] * ni % P_FQ, (-a[1] * ni) % P_FQ)


def f2_mul_scalar(a, k):
    return (a[0] * k % P_FQ, a[1] * k % P_FQ)


F2_ZERO = (0, 0)
F2_ONE = (1, 0)

# ---------------------------------------------------------------- curves
# Generic affine arithmetic over a field given by its ops; None = point at infinity.


class _Fq:
    zero, one = 0, 1
    add = staticmethod(lambda a, b: (a + b) % P_FQ)
    sub = staticmethod(lambda a, b: (a - b) % P_FQ)
    mul = staticmethod(lambda a, b: a * b % P_FQ)
    neg = staticmethod(lambda a: (-a) % P_FQ)
    inv = staticmethod(lambda a: pow(a, -1, P_FQ))
    small = staticmethod(lambda k: k % P_FQ)


class _Fq2:
    zero, one = F2_ZERO, F2_ONE
    add = staticmethod(f2_add)
    sub = staticmethod(f2_sub)
    mul = staticmethod(f2_mul)
    neg = staticmethod(f2_neg)
    inv = staticmethod(f2_inv)
    small = staticmethod(lambda k: (k % P_FQ, 0))


class Curve:
    """y^2 = x^3 + b over field F (a = 0).  Points are affine tuples (x, y) or None."""

    def __init__(self, F, b, gen):
        self.F, self.b, self.gen = F, b, gen

    def on_curve(self, P):
        if P is None:
            return True
        F = self.F
        x, y = P
        return F.sub(F.mul(y, y), F.add(F.mul(F.mul(x, x), x), self.b)) == F.zero

    def neg(self, P):
        return None if P is None else (P[0], self.F.neg(P[1]))

    def add(self, P, Q):
        F = self.F
        if P is None:
            return Q
        if Q is None:
            return P
        if P[0] == Q[0]:
            if P[1] != Q[1] or P[1] == F.zero:
                return None
            return self.double(P)
        lam = F.mul(F.sub(Q[1], P[1]), F.inv(F.sub(Q[0], P[0])))
        x3 = F.sub(F.sub(F.mul(lam, lam), P[0]), Q[0])
        return (x3, F.sub(F.mul(lam, F.sub(P[0], x3)), P[1]))

    def double(self, P):
        F = self.F
        if P is None or P[1] == F.zero:
            return None
        x2 = F.mul(P[0], P[0])
        lam = F.mul(F.add(F.add(x2, x2), x2), F.inv(F.add(P[1], P[1])))
        x3 = F.sub(F.mul(lam, lam), F.add(P[0], P[0]))
        return (x3, F.sub(F.mul(lam, F.sub(P[0], x3)), P[1]))

    def mul(self, P, k: int):
        """k*P by double-and-add over the bits of the integer k >= 0
        (bend2/src/g1.bend:175-191 walks all 256 bits of a canonical scalar)"""
        R = None
        for bit in bin(k)[2:] if k > 0 else "":
            R = self.double(R)
            if bit == "1":
                R = self.add(R, P)
        return R


# BN254 G1: y^2 = x^3 + 3, generator (1, 2)
G1 = Curve(_Fq, 3, (1, 2))
# BN254 G2 on the sextic twist y^2 = x^3 + 3/(9+u), standard (EIP-197) generator
_B2 = f2_mul((3, 0), f2_inv((9, 1)))
_G2_GEN = (
    (10857046999023057135944570762232829481370756359578518086990519993285655852781,
     11559732032986387107991004021392285783925812861821192530917403151452391805634),
    (8495653923123431417604973247489272438418190587263600148770280649306958101930,
     4082367875863433681332203403145435568316851327593401208105741076214120093531),
)
G2 = Curve(_Fq2, _B2, _G2_GEN)
assert G1.on_curve(G1.gen) and G2.on_curve(G2.gen), "curve constants mistyped"


class FixedBase:
    """k*G for many k from a table of 2^i*G (one affine add per set bit)."""

    def __init__(self, curve: Curve, base, bits=256):
        self.curve = curve
        self.tab = []
        P = base
        for _ in range(bits):
            self.tab.append(P)
            P = curve.double(P)

    def mul(self, k: int):
        R = None
        i = 0
        while k:
            if k & 1:
                R = self.curve.add(R, self.tab[i])
            k >>= 1
            i += 1
        return R


# ---- jacobian helpers matching the reference seam's result type (bend2/src/g1.bend:13-17)

def jacobian_to_affine(curve: Curve, X, Y, Z):
    """(X/Z^2, Y/Z^3); Z = 0 is infinity (bend2/src/g1.bend:44-57)"""
    F = curve.F
    if Z == F.zero:
        return None
    zi = F.inv(Z)
    zi2 = F.mul(zi, zi)
    return (F.mul(X, zi2), F.mul(Y, F.mul(zi, zi2)))


# ---------------------------------------------------------------- MSM

def msm_naive(curve: Curve, points, scalars):
    acc = None
    for P, k in zip(points, scalars):
        acc = curve.add(acc, curve.mul(P, k))
    return acc


def msm_pippenger(curve: Curve, points, scalars, c=None):
    """unsigned c-bit windows, running-sum bucket reduction, Horner window combine
    (bend2/src/msm.bend:34-58 windows / digit, :192-205 red, :225-239 wtree)"""
    n = len(points)
    if c is None:
        c = 8 if n < (1 << 20) else 10  # Msm.pick_c, bend2/src/msm.bend:40-41
    w_count = 253 // c + 1  # Msm.windows, bend2/src/msm.bend:34-35
    mask = (1 << c) - 1
    total = None
    for w in reversed(range(w_count)):
        for _ in range(c):
            total = curve.double(total)
        buckets = [None] * (1 << c)
        for P, k in zip(points, scalars):
            d = (k >> (w * c)) & mask
            if d:
                buckets[d] = curve.add(buckets[d], P)
        run, acc = None, None
        for j in range((1 << c) - 1, 0, -1):
            run = curve.add(run, buckets[j])
            acc = curve.add(acc, run)
        total = curve.add(total, acc)
    return total


# ---------------------------------------------------------------- NTT (bend2/gen/ref_qap.py:23-72)

def omega(log2: int) -> int:
    """generator of the size-2^log2 radix-2 domain (bend2/src/ntt.bend:73-74)"""
    return pow(ROOT_2_28, 1 << (TWO_ADICITY - log2), P_FR)


def bitrev_permute(a):
    n = len(a)
    lg = n.bit_length() - 1
    out = [0] * n
    for i in range(n):
        out[int(format(i, "0%db" % lg)[::-1], 2) if lg else 0] = a[i]
    return out


def fft(a, w):
    """natural order in and out, radix-2 DIT; w generates the size-len(a) domain"""
    n = len(a)
    a = bitrev_permute(list(a))
    m = 1
    while m < n:
        wm = pow(w, n // (2 * m), P_FR)
        for k in range(0, n, 2 * m):
            t = 1
            for j in range(m):
                u, v = a[k + j], a[k + j + m] * t % P_FR
                a[k + j], a[k + j + m] = (u + v) % P_FR, (u - v) % P_FR
                t = t * wm % P_FR
        m *= 2
    return a


def ntt(a):
    return fft(a, omega(len(a).bit_length() - 1))


def intt(a):
    n = len(a)
    lg = n.bit_length() - 1
    ninv = pow(n, -1, P_FR)
    return [x * ninv % P_FR for x in fft(a, pow(omega(lg), -1, P_FR))]


def coset_ntt(a):
    return ntt([x * pow(GEN, j, P_FR) % P_FR for j, x in enumerate(a)])


def coset_intt(a):
    ginv = pow(GEN, -1, P_FR)
    return [x * pow(ginv, j, P_FR) % P_FR for j, x in enumerate(intt(a))]


def qap_h(a, b, c):
    """h = coset_iNTT((coset_NTT(iNTT a) * coset_NTT(iNTT b) - coset_NTT(iNTT c)) / (g^d - 1))
    (bend2/gen/ref_qap.py:68-72, bend2/src/ntt.bend:446-459)"""
    d = len(a)
    A, B, C = (coset_ntt(intt(v)) for v in (a, b, c))
    zinv = pow((pow(GEN, d, P_FR) - 1) % P_FR, -1, P_FR)
    return coset_intt([(x * y - z) % P_FR * zinv % P_FR for x, y, z in zip(A, B, C)])


def poly_eval(coeffs, x):
    acc = 0
    for cf in reversed(coeffs):
        acc = (acc * x + cf) % P_FR
    return acc


# ---------------------------------------------------------------- SquareChain circuit

def domain_log2(n_constraints: int, n_instance: int = 2) -> int:
    """smallest 2^k >= N + num_instance (ref/src/gen.rs:91-93, ref/README.md:19)"""
    need = n_constraints + n_instance
    k = 0
    while (1 << k) < need:
        k += 1
    return k


class SquareChain:
    """x_{i+1} = x_i^2, N constraints, z = [1, x_N, x_0..x_{N-1}] (ref/src/circuit.rs:21-74)"""

    def __init__(self, log2n: int, x0: int):
        self.n = 1 << log2n
        xs = [x0 % P_FR]
        for _ in range(self.n):
            xs.append(xs[-1] * xs[-1] % P_FR)
        self.xs = xs
        self.z = [1, xs[self.n]] + xs[: self.n]
        self.num_instance = 2
        self.num_witness = self.n

    def rows(self):
        """R1CS rows: A = B = [(2+i, 1)], C = [(3+i, 1)] or [(1, 1)] for the last row
        (the frozen shape asserted at ref/src/gen.rs:78-83)"""
        n = self.n
        a = [[(2 + i, 1)] for i in range(n)]
        b = [[(2 + i, 1)] for i in range(n)]
        c = [[(3 + i, 1) if i + 1 < n else (1, 1)] for i in range(n)]
        return a, b, c


def eval_rows(rows, z):
    return [sum(coef * z[col] for col, coef in row) % P_FR for row in rows]


def evals(rows_a, rows_b, rows_c, z, n_instance, d):
    """a_i = <A_i, z>, plus libsnark input-consistency rows a[N+i] = z[i]; b, c likewise
    without them; zero elsewhere (bend2/src/groth16.bend:162-188, bend2/gen/ref_qap.py:105-107)"""
    n = len(rows_a)
    a = eval_rows(rows_a, z) + z[:n_instance] + [0] * (d - n - n_instance)
    b = eval_rows(rows_b, z) + [0] * (d - n)
    c = eval_rows(rows_c, z) + [0] * (d - n)
    return a, b, c


# ---------------------------------------------------------------- Groth16 setup (own, seeded)

def lagrange_at(tau: int, log2d: int):
    """L_k(tau) for the size-d radix-2 domain: Z(tau) w^k / (d (tau - w^k))"""
    d = 1 << log2d
    w = omega(log2d)
    zt = (pow(tau, d, P_FR) - 1) % P_FR
    dinv = pow(d, -1, P_FR)
    out = []
    wk = 1
    for _ in range(d):
        out.append(zt * wk % P_FR * dinv % P_FR * pow((tau - wk) % P_FR, -1, P_FR) % P_FR)
        wk = wk * w % P_FR
    return out


def rng_fr(rng: random.Random) -> int:
    return rng.randrange(P_FR)


class Setup:
    """Circuit-specific Groth16 setup with a seeded trapdoor.  Column polynomials follow
    the libsnark reduction: A gets the input-consistency rows N+i for instance columns."""

    def __init__(self, circ: SquareChain, seed: int):
        rng = random.Random(seed)
        self.tau, self.alpha, self.beta, self.gamma, self.delta = (rng_fr(rng) for _ in range(5))
        n, ni = circ.n, circ.num_instance
        self.log2d = domain_log2(n, ni)
        d = 1 << self.log2d
        self.d = d
        lag = lagrange_at(self.tau, self.log2d)
        m = ni + circ.num_witness
        A = [0] * m
        B = [0] * m
        C = [0] * m
        ra, rb, rc = circ.rows()
        for i, row in enumerate(ra):
            for col, cf in row:
                A[col] = (A[col] + cf * lag[i]) % P_FR
        for i, row in enumerate(rb):
            for col, cf in row:
                B[col] = (B[col] + cf * lag[i]) % P_FR
        for i, row in enumerate(rc):
            for col, cf in row:
                C[col] = (C[col] + cf * lag[i]) % P_FR
        for i in range(ni):
            A[i] = (A[i] + lag[n + i]) % P_FR
        self.A, self.B, self.C = A, B, C
        zt = (pow(self.tau, d, P_FR) - 1) % P_FR
        dinv = pow(self.delta, -1, P_FR)
        ginv = pow(self.gamma, -1, P_FR)
        self.h_scalars = [pow(self.tau, k, P_FR) * zt % P_FR * dinv % P_FR for k in range(d - 1)]
        self.l_scalars = [(self.beta * A[ni + j] + self.alpha * B[ni + j] + C[ni + j]) * dinv % P_FR
                          for j in range(circ.num_witness)]
        self.ic_scalars = [(self.beta * A[i] + self.alpha * B[i] + C[i]) * ginv % P_FR for i in range(ni)]
        self.ni = ni

    def keys(self):
        """all proving-key points (affine, None = infinity) in ref/README.md's pk.json roles"""
        f1 = FixedBase(G1, G1.gen)
        f2 = FixedBase(G2, G2.gen)
        pk = {
            "alpha_g1": f1.mul(self.alpha), "beta_g1": f1.mul(self.beta), "delta_g1": f1.mul(self.delta),
            "beta_g2": f2.mul(self.beta), "delta_g2": f2.mul(self.delta), "gamma_g2": f2.mul(self.gamma),
            "a_query": [f1.mul(k) for k in self.A],
            "b_g1_query": [f1.mul(k) for k in self.B],
            "b_g2_query": [f2.mul(k) for k in self.B],
            "h_query": [f1.mul(k) for k in self.h_scalars],
            "l_query": [f1.mul(k) for k in self.l_scalars],
            "gamma_abc_g1": [f1.mul(k) for k in self.ic_scalars],
        }
        return pk


# ---------------------------------------------------------------- Groth16 prove

def to_canonical_scalar(x: int) -> int:
    return x % P_FR


def prove(pk, z, h, r: int, s: int, n_witness_start: int = 2):
    """A = alpha + sum z_i a_i + r delta; B2 = beta2 + sum z_i b2_i + s delta2;
    B1 likewise; C = s A + r B1 - r s delta1 + sum_j z[2+j] l_j + sum_k h_k h_query_k
    (ref/README.md:24-32, bend2/src/groth16.bend:298-308)"""
    mA = msm_naive(G1, pk["a_query"], z)
    mB1 = msm_naive(G1, pk["b_g1_query"], z)
    mB2 = msm_naive(G2, pk["b_g2_query"], z)
    mL = msm_naive(G1, pk["l_query"], z[n_witness_start:])
    mH = msm_naive(G1, pk["h_query"], h[: len(pk["h_query"])])
    A = G1.add(G1.add(mA, G1.mul(pk["delta_g1"], r)), pk["alpha_g1"])
    B1 = G1.add(G1.add(mB1, G1.mul(pk["delta_g1"], s)), pk["beta_g1"])
    B2 = G2.add(G2.add(mB2, G2.mul(pk["delta_g2"], s)), pk["beta_g2"])
    C = G1.add(G1.add(G1.mul(A, s), G1.mul(B1, r)),
               G1.add(G1.neg(G1.mul(pk["delta_g1"], r * s % P_FR)), G1.add(mL, mH)))
    return A, B2, C


def trapdoor_scalars(setup: Setup, z, h, r: int, s: int):
    """the discrete logs of A (base G1), B (base G2), C (base G1) for an honest proof"""
    ni = setup.ni
    a_s = (setup.alpha + sum(zi * ai for zi, ai in zip(z, setup.A)) + r * setup.delta) % P_FR
    b_s = (setup.beta + sum(zi * bi for zi, bi in zip(z, setup.B)) + s * setup.delta) % P_FR
    lsum = sum(z[ni + j] * setup.l_scalars[j] for j in range(len(setup.l_scalars)))
    hsum = sum(h[k] * setup.h_scalars[k] for k in range(len(setup.h_scalars)))
    c_s = (s * a_s + r * b_s - r * s * setup.delta + lsum + hsum) % P_FR
    return a_s, b_s, c_s


def trapdoor_check(setup: Setup, z, r: int, s: int, proof) -> bool:
    """Proof validity without pairings: the QAP identity makes c_s equal the value the
    verification equation needs iff h is the true quotient; comparing A, B, C against
    a_s G1, b_s G2, c_s G1 (with h from the oracle's qap_h) pins every MSM and the NTTs."""
    A, B, C = proof
    # verification identity in the exponent: a_s b_s = alpha beta + ic + c_s delta
    a_s = (setup.alpha + sum(zi * ai for zi, ai in zip(z, setup.A)) + r * setup.delta) % P_FR
    b_s = (setup.beta + sum(zi * bi for zi, bi in zip(z, setup.B)) + s * setup.delta) % P_FR
    ic = sum(z[i] * setup.ic_scalars[i] for i in range(setup.ni)) % P_FR
    c_s = (a_s * b_s - setup.alpha * setup.beta - ic * setup.gamma) * pow(setup.delta, -1, P_FR) % P_FR
    f1 = FixedBase(G1, G1.gen)
    return A == f1.mul(a_s) and B == G2.mul(G2.gen, b_s) and C == f1.mul(c_s)


# ---------------------------------------------------------------- arkworks JSON encoding (ref/README.md:13-22)

def hx(v: int) -> str:
    return "0x%x" % v


def g1_json(P):
    return {"inf": True} if P is None else {"x": hx(P[0]), "y": hx(P[1])}


def g2_json(P):
    if P is None:
        return {"inf": True}
    return {"x": [hx(P[0][0]), hx(P[0][1])], "y": [hx(P[1][0]), hx(P[1][1])]}


def g1_from_json(j):
    return None if j.get("inf") else (int(j["x"], 16), int(j["y"], 16))


def g2_from_json(j):
    if j.get("inf"):
        return None
    return ((int(j["x"][0], 16), int(j["x"][1], 16)), (int(j["y"][0], 16), int(j["y"][1], 16)))


# ---------------------------------------------------------------- FORMAT.md binary encoders

def fe_bytes_mont(x: int, p: int) -> bytes:
    return struct.pack("<16I", *words16(to_mont(x, p)))


def g1_bytes(P) -> bytes:
    if P is None:
        return bytes(128)
    return fe_bytes_mont(P[0], P_FQ) + fe_bytes_mont(P[1], P_FQ)


def g2_bytes(P) -> bytes:
    if P is None:
        return bytes(256)
    return b"".join(fe_bytes_mont(v, P_FQ) for v in (P[0][0], P[0][1], P[1][0], P[1][1]))


def read_fe(buf: bytes, off: int, p: int, mont=True) -> int:
    v = from_words16(struct.unpack_from("<16I", buf, off))
    return from_mont(v, p) if mont else v


def read_g1(buf: bytes, off: int):
    x, y = read_fe(buf, off, P_FQ), read_fe(buf, off + 64, P_FQ)
    return None if x == 0 and y == 0 else (x, y)


def read_g2(buf: bytes, off: int):
    v = [read_fe(buf, off + 64 * i, P_FQ) for i in range(4)]
    return None if not any(v) else ((v[0], v[1]), (v[2], v[3]))
