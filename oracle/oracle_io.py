"""Oracle side of the file format and the pairing-free proof check (test infrastructure).

load_dir reads a bend2/FORMAT.md directory; square_chain_trapdoor_check verifies a proof in
the exponent from the setup trapdoor: with the column polynomials A_j, B_j, C_j at tau
(Lagrange basis of the size-d radix-2 domain, input-consistency rows N+i in A; the libsnark
reduction of ref/README.md:24-32), an honest Groth16 proof satisfies
    A = a_s G1,  B = b_s G2,  C = c_s G1
    a_s = alpha + sum_i z_i A_i + r delta,   b_s = beta + sum_i z_i B_i + s delta,
    c_s = (a_s b_s - alpha beta - sum_{i<ni} z_i (beta A_i + alpha B_i + C_i)) / delta,
which is the verification equation e(A, B) = e(alpha, beta) e(IC, gamma) e(C, delta) with every
point written as its discrete log.  Work is O(d) field operations and three fixed-base
multiplications, so it runs at full benchmark sizes.
"""
from __future__ import annotations

import os
import struct

import numpy as np

import bn254_ref as o

FILES = ("header", "witness", "r1cs_a", "r1cs_b", "r1cs_c", "pk_g1", "pk_g2", "pk_a", "pk_b1", "pk_b2", "pk_h",
         "pk_l", "rs")


def load_dir(path: str) -> dict:
    out = {}
    for name in FILES + ("proof_ref", "trapdoor"):
        f = os.path.join(path, name + ".bin")
        if os.path.exists(f):
            out[name] = open(f, "rb").read()
    hdr = struct.unpack("<8I", out["header"])
    out["hdr"] = dict(zip(("nc", "ni", "nw", "lg", "na", "nb", "nh", "nl"), hdr))
    return out


def fes(buf: bytes, count: int, p: int, mont=True, offset=0) -> list:
    """`count` field elements of a FORMAT.md buffer as python ints (vectorised limb packing)"""
    w = np.frombuffer(buf, dtype="<u4", count=16 * count, offset=offset).astype("<u2")
    raw = w.tobytes()
    vals = [int.from_bytes(raw[32 * i: 32 * i + 32], "little") for i in range(count)]
    if mont:
        rinv = pow(o.R256, -1, p)
        vals = [v * rinv % p for v in vals]
    return vals


def csr_rows(buf: bytes, nc: int):
    """(row, col, coeff) triples of a CSR file: nnz; offsets[nc+1]; (col, Fr coeff) * nnz"""
    (nnz,) = struct.unpack_from("<I", buf, 0)
    offs = struct.unpack_from("<%dI" % (nc + 1), buf, 4)
    base = 4 * (2 + nc)
    ent = np.frombuffer(buf, dtype="<u4", offset=base, count=17 * nnz).reshape(nnz, 17) if nnz else None
    rinv = pow(o.R256, -1, o.P_FR)
    out = []
    for row in range(nc):
        for e in range(offs[row], offs[row + 1]):
            col = int(ent[e, 0])
            coeff = o.from_words16(ent[e, 1:]) * rinv % o.P_FR
            out.append((row, col, coeff))
    return out


def batch_inv(vals, p):
    pre, acc = [], 1
    for v in vals:
        pre.append(acc)
        acc = acc * v % p
    inv = pow(acc, -1, p)
    out = [0] * len(vals)
    for i in range(len(vals) - 1, -1, -1):
        out[i] = inv * pre[i] % p
        inv = inv * vals[i] % p
    return out


def lagrange_basis_at(tau: int, lg: int):
    d = 1 << lg
    w = o.omega(lg)
    wk, acc = [], 1
    for _ in range(d):
        wk.append(acc)
        acc = acc * w % o.P_FR
    zt = (pow(tau, d, o.P_FR) - 1) % o.P_FR
    scale = zt * pow(d, -1, o.P_FR) % o.P_FR
    inv = batch_inv([(tau - x) % o.P_FR for x in wk], o.P_FR)
    return [scale * x % o.P_FR * y % o.P_FR for x, y in zip(wk, inv)]


def column_polys(data: dict, tau: int):
    h = data["hdr"]
    m = h["ni"] + h["nw"]
    lag = lagrange_basis_at(tau, h["lg"])
    cols = []
    for name in ("r1cs_a", "r1cs_b", "r1cs_c"):
        v = [0] * m
        for row, col, cf in csr_rows(data[name], h["nc"]):
            v[col] = (v[col] + cf * lag[row]) % o.P_FR
        cols.append(v)
    A, B, C = cols
    for i in range(h["ni"]):
        A[i] = (A[i] + lag[h["nc"] + i]) % o.P_FR
    return A, B, C


def square_chain_trapdoor_check(data: dict, trap: dict, proof) -> bool:
    """True iff proof = (A, B, C) (affine tuples / None) is the honest proof for the
    directory's witness and r, s under the setup trapdoor `trap` (tau/alpha/beta/gamma/delta)."""
    h = data["hdr"]
    P = o.P_FR
    z = fes(data["witness"], h["ni"] + h["nw"], P)
    r, s = fes(data["rs"], 2, P)
    A, B, C = column_polys(data, trap["tau"])
    al, be, de = trap["alpha"], trap["beta"], trap["delta"]
    a_s = (al + sum(zi * x for zi, x in zip(z, A)) + r * de) % P
    b_s = (be + sum(zi * x for zi, x in zip(z, B)) + s * de) % P
    ic = sum(z[i] * (be * A[i] + al * B[i] + C[i]) for i in range(h["ni"])) % P
    c_s = (a_s * b_s - al * be - ic) * pow(de, -1, P) % P
    f1 = o.FixedBase(o.G1, o.G1.gen)
    pa, pb, pc = proof
    return pa == f1.mul(a_s) and pb == o.G2.mul(o.G2.gen, b_s) and pc == f1.mul(c_s)


def trapdoor_from_bin(buf: bytes) -> dict:
    vals = fes(buf, 5, o.P_FR, mont=False)
    return dict(zip(("tau", "alpha", "beta", "gamma", "delta"), vals))


def parse_proof_text(text: str):
    """`A x y` / `B x0 x1 y0 y1` / `C x y` lines (canonical hex) -> affine tuples"""
    pts = {}
    for line in text.splitlines():
        parts = line.split()
        if parts and parts[0] in ("A", "B", "C"):
            pts[parts[0]] = [int(v, 16) for v in parts[1:]]
    a, b, c = pts["A"], pts["B"], pts["C"]
    g1 = lambda v: None if v == [0, 0] else (v[0], v[1])  # noqa: E731
    bb = None if b == [0, 0, 0, 0] else ((b[0], b[1]), (b[2], b[3]))
    return g1(a), bb, g1(c)
