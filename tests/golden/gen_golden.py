#!/usr/bin/env python3
"""Generate the committed golden fixtures under tests/golden/ (run once, in a container that
holds the bend-groth16 reference checkout; the GPU tests only read the committed outputs).

Pinning strategy.  arkworks (the reference's own oracle) cannot be built here, so the
fixtures are produced by the CPU oracle (oracle/bn254_ref.py) in arkworks' frozen JSON
encoding (ref/README.md:13-22) and then pushed through the reference's OWN tooling:
  * bend2/tools/export_bin.py   JSON -> FORMAT.md .bin          (pins the wire format)
  * bend2/tools/verify_bin.py   .bin -> JSON round-trip check    (pins the encoder)
  * bend2/gen/ref_qap.py        the reference's stdlib qap_h     (pins h; abc_evals.bin, h_ref.bin)
  * bend2/tools/proof_to_json.py proof line parser / comparator  (pins the A/B/C stdout format)
  * bend2/probe/check_montmul.py deterministic Montgomery pairs  (pins a*b*R^-1 mod p)
The oracle's own qap_h must agree with ref_qap.py's h bit for bit before anything is written.

Usage: python tests/golden/gen_golden.py REFERENCE_ROOT
       (or set BEND_GROTH16_REF to the checkout's root and give no argument)
"""
from __future__ import annotations

import ast
import contextlib
import io
import json
import os
import random
import shutil
import struct
import sys
import tempfile
from pathlib import Path

HERE = Path(__file__).resolve().parent
REPO = HERE.parents[1]
sys.path.insert(0, str(REPO / "oracle"))
import bn254_ref as o  # noqa: E402

SEED_SETUP = 42
SEED_WITNESS = 42 ^ 0x5157_4E45_5353  # ref/src/circuit.rs:37-41 uses the same seed value
SEED_VECTORS = 42


def load_ref_module(ref: Path, rel: str, name: str):
    import importlib.util
    spec = importlib.util.spec_from_file_location(name, ref / rel)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def montmul_pairs(ref: Path, count: int):
    """The deterministic operand generator of bend2/probe/check_montmul.py (its function
    definitions only; the script body would run a Bend binary)."""
    src = (ref / "bend2/probe/check_montmul.py").read_text()
    tree = ast.parse(src)
    keep = [n for n in tree.body if isinstance(n, (ast.FunctionDef, ast.Import, ast.ImportFrom))
            or (isinstance(n, ast.Assign) and all(isinstance(t, ast.Name) and t.id in ("P", "R", "RINV", "M32")
                                                  for t in n.targets))]
    ns: dict = {}
    exec(compile(ast.Module(body=keep, type_ignores=[]), "check_montmul_defs", "exec"), ns)
    out = []
    for i in range(count):
        a, b = ns["rnd"](2 * i), ns["rnd"](2 * i + 1)
        want = a * b * ns["RINV"] % ns["P"]
        assert want == o.mont_mul(a, b, o.P_FR)
        out.append((a, b, want))
    return out


# ---------------------------------------------------------------- vectors (mirrors ref/src/vectors.rs:166-210)

def field_cases(rng, p, n):
    cases = []
    for _ in range(n):
        a, b = rng.randrange(p), rng.randrange(p)
        mul = a * b % p
        cases.append({
            "a": o.hx(a), "b": o.hx(b), "add": o.hx((a + b) % p), "sub": o.hx((a - b) % p),
            "mul": o.hx(mul), "neg_a": o.hx((-a) % p), "inv_a": o.hx(pow(a, -1, p) if a else 0),
            "sq_a": o.hx(a * a % p), "a_mont": o.hx(a * o.R256 % p), "mul_mont": o.hx(mul * o.R256 % p),
        })
    consts = {"p": o.hx(p), "r_mod_p": o.hx(o.R256 % p), "r2_mod_p": o.hx(o.R256 * o.R256 % p)}
    for bits in (12, 24, 32, 64):
        consts["n_prime_%d" % bits] = o.hx((-pow(p, -1, 1 << bits)) % (1 << bits))
    return {"constants": consts, "cases": cases}


def curve_cases(rng, curve, fb, to_json, n):
    """cases 0..2 are infinity, P == Q, P == -Q (ref/src/vectors.rs:129-131)"""
    out = []
    for i in range(n):
        p = fb.mul(rng.randrange(1, o.P_FR))
        q = fb.mul(rng.randrange(1, o.P_FR))
        if i == 0:
            p = None
        elif i == 1:
            q = p
        elif i == 2:
            q = curve.neg(p)
        k = rng.randrange(o.P_FR)
        out.append({"p": to_json(p), "q": to_json(q), "k": o.hx(k), "add": to_json(curve.add(p, q)),
                    "double_p": to_json(curve.double(p)), "neg_p": to_json(curve.neg(p)),
                    "mul_pk": to_json(curve.mul(p, k))})
    return out


def build_vectors(dst: Path, export_bin, verify_bin):
    rng = random.Random(SEED_VECTORS)
    tmp = Path(tempfile.mkdtemp(prefix="bg_vec_"))
    f1, f2 = o.FixedBase(o.G1, o.G1.gen), o.FixedBase(o.G2, o.G2.gen)
    (tmp / "fr_ops.json").write_text(json.dumps(field_cases(rng, o.P_FR, 64)))
    (tmp / "fq_ops.json").write_text(json.dumps(field_cases(rng, o.P_FQ, 64)))
    (tmp / "g1_ops.json").write_text(json.dumps(curve_cases(rng, o.G1, f1, o.g1_json, 32)))
    (tmp / "g2_ops.json").write_text(json.dumps(curve_cases(rng, o.G2, f2, o.g2_json, 16)))
    msm = []
    for size in (8, 64, 1024):
        ks = [rng.randrange(1, o.P_FR) for _ in range(size)]
        pts = [f1.mul(k) for k in ks]
        sc = [rng.randrange(o.P_FR) for _ in range(size)]
        res = o.msm_pippenger(o.G1, pts, sc) if size > 8 else o.msm_naive(o.G1, pts, sc)
        assert res == f1.mul(sum(a * b for a, b in zip(ks, sc)) % o.P_FR)
        msm.append({"size": size, "points": [o.g1_json(p) for p in pts], "scalars": [o.hx(s) for s in sc],
                    "result": o.g1_json(res)})
    (tmp / "msm_small.json").write_text(json.dumps(msm))
    ntt = []
    for size in (8, 64, 1024):
        lg = size.bit_length() - 1
        coeffs = [rng.randrange(o.P_FR) for _ in range(size)]
        evals = o.ntt(coeffs)
        icoeffs = o.intt(evals)
        assert icoeffs == coeffs
        assert all(evals[j] == o.poly_eval(coeffs, pow(o.omega(lg), j, o.P_FR)) for j in (0, 1, size - 1))
        ntt.append({"size": size, "omega": o.hx(o.omega(lg)), "domain_size_inv": o.hx(pow(size, -1, o.P_FR)),
                    "coeffs": [o.hx(v) for v in coeffs], "evals": [o.hx(v) for v in evals],
                    "icoeffs_of_evals": [o.hx(v) for v in icoeffs]})
    (tmp / "ntt_small.json").write_text(json.dumps(ntt))
    with contextlib.redirect_stdout(io.StringIO()):
        export_bin.export_vectors(str(tmp))
        bad = verify_bin.verify_vectors(str(tmp))
    assert bad == 0, "verify_bin found mismatches in the vectors"
    dst.mkdir(parents=True, exist_ok=True)
    for f in sorted((tmp / "bend").glob("*.bin")):
        shutil.copy(f, dst / f.name)
    shutil.rmtree(tmp)


# ---------------------------------------------------------------- circuits

def build_circuit(log2n: int, dst: Path, export_bin, verify_bin, ref_qap, proof_to_json):
    wrng = random.Random(SEED_WITNESS + log2n)
    circ = o.SquareChain(log2n, wrng.randrange(o.P_FR))
    setup = o.Setup(circ, SEED_SETUP + log2n)
    pk = setup.keys()
    rrng = random.Random(SEED_SETUP * 1000 + log2n)
    r, s = rrng.randrange(o.P_FR), rrng.randrange(o.P_FR)
    ra, rb, rc = circ.rows()
    d = setup.d
    a, b, c = o.evals(ra, rb, rc, circ.z, circ.num_instance, d)
    h = o.qap_h(a, b, c)
    assert h[-1] == 0
    proof = prove_pippenger(pk, circ.z, h, r, s)
    assert o.trapdoor_check(setup, circ.z, r, s, proof), "oracle proof failed the trapdoor check"

    tmp = Path(tempfile.mkdtemp(prefix="bg_k%d_" % log2n))
    rows_json = lambda rows: [[[col, o.hx(cf)] for col, cf in row] for row in rows]  # noqa: E731
    (tmp / "r1cs.json").write_text(json.dumps({
        "num_constraints": circ.n, "num_instance": 2, "num_witness": circ.n,
        "a": rows_json(ra), "b": rows_json(rb), "c": rows_json(rc)}))
    (tmp / "witness.json").write_text(json.dumps({"z": [o.hx(v) for v in circ.z]}))
    (tmp / "public.json").write_text(json.dumps({"inputs": [o.hx(circ.z[1])]}))
    (tmp / "proof_ref_rs.json").write_text(json.dumps({"r": o.hx(r), "s": o.hx(s)}))
    A, B, C = proof
    (tmp / "proof_ref.json").write_text(json.dumps({"a": o.g1_json(A), "b": o.g2_json(B), "c": o.g1_json(C)}))
    vk = {"alpha_g1": o.g1_json(pk["alpha_g1"]), "beta_g2": o.g2_json(pk["beta_g2"]),
          "gamma_g2": o.g2_json(pk["gamma_g2"]), "delta_g2": o.g2_json(pk["delta_g2"]),
          "gamma_abc_g1": [o.g1_json(p) for p in pk["gamma_abc_g1"]]}
    (tmp / "pk.json").write_text(json.dumps({
        "domain_size": d,
        "alpha_g1": o.g1_json(pk["alpha_g1"]), "beta_g1": o.g1_json(pk["beta_g1"]),
        "beta_g2": o.g2_json(pk["beta_g2"]), "delta_g1": o.g1_json(pk["delta_g1"]),
        "delta_g2": o.g2_json(pk["delta_g2"]),
        "a_query": [o.g1_json(p) for p in pk["a_query"]],
        "b_g1_query": [o.g1_json(p) for p in pk["b_g1_query"]],
        "b_g2_query": [o.g2_json(p) for p in pk["b_g2_query"]],
        "h_query": [o.g1_json(p) for p in pk["h_query"]],
        "l_query": [o.g1_json(p) for p in pk["l_query"]],
        "vk": vk}))
    with contextlib.redirect_stdout(io.StringIO()):
        export_bin.export_circuit(str(tmp))
        ref_qap.main(str(tmp))
        bad = verify_bin.verify_circuit(str(tmp))
    assert bad == 0, "verify_bin found mismatches for K=%d" % log2n
    # the reference's own qap_h must agree with the oracle's, element for element
    href = (tmp / "bend" / "h_ref.bin").read_bytes()
    got = [o.read_fe(href, 64 * i, o.P_FR) for i in range(d)]
    assert got == h, "oracle qap_h differs from bend2/gen/ref_qap.py"
    # the reference's proof-line parser accepts the oracle's printed lines and finds them EQUAL
    lines = proof_lines(proof)
    parsed = proof_to_json.parse(lines)
    for k in ("a", "b", "c"):
        ref_pt = json.loads((tmp / "proof_ref.json").read_text())[k]
        assert proof_to_json.norm(parsed[k]) == proof_to_json.norm(ref_pt)
    dst.mkdir(parents=True, exist_ok=True)
    for f in sorted((tmp / "bend").glob("*.bin")):
        shutil.copy(f, dst / f.name)
    for name in ("proof_ref.json", "public.json", "proof_ref_rs.json"):
        shutil.copy(tmp / name, dst / name)
    (dst / "proof_ref.txt").write_text(lines)
    (dst / "trapdoor.json").write_text(json.dumps({
        "note": "seeded setup trapdoor of this fixture (tests only): discrete logs of the pk points",
        "tau": o.hx(setup.tau), "alpha": o.hx(setup.alpha), "beta": o.hx(setup.beta),
        "gamma": o.hx(setup.gamma), "delta": o.hx(setup.delta), "r": o.hx(r), "s": o.hx(s),
        "seed_setup": SEED_SETUP + log2n, "seed_witness": SEED_WITNESS + log2n}, indent=1))
    shutil.rmtree(tmp)


def prove_pippenger(pk, z, h, r, s):
    G1, G2 = o.G1, o.G2
    mA = o.msm_pippenger(G1, pk["a_query"], z)
    mB1 = o.msm_pippenger(G1, pk["b_g1_query"], z)
    mB2 = o.msm_pippenger(G2, pk["b_g2_query"], z)
    mL = o.msm_pippenger(G1, pk["l_query"], z[2:])
    mH = o.msm_pippenger(G1, pk["h_query"], h[: len(pk["h_query"])])
    A = G1.add(G1.add(mA, G1.mul(pk["delta_g1"], r)), pk["alpha_g1"])
    B1 = G1.add(G1.add(mB1, G1.mul(pk["delta_g1"], s)), pk["beta_g1"])
    B2 = G2.add(G2.add(mB2, G2.mul(pk["delta_g2"], s)), pk["beta_g2"])
    C = G1.add(G1.add(G1.mul(A, s), G1.mul(B1, r)),
               G1.add(G1.neg(G1.mul(pk["delta_g1"], r * s % o.P_FR)), G1.add(mL, mH)))
    return A, B2, C


def proof_lines(proof) -> str:
    """the prover's stdout proof lines: canonical big-endian 0x hex (bend2/FORMAT.md:33)"""
    A, B, C = proof
    hx = lambda v: "0x%064x" % v  # noqa: E731
    return "A %s %s\nB %s %s %s %s\nC %s %s\n" % (
        hx(A[0]), hx(A[1]), hx(B[0][0]), hx(B[0][1]), hx(B[1][0]), hx(B[1][1]), hx(C[0]), hx(C[1]))


def main():
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("BEND_GROTH16_REF")
    if not root:
        sys.exit("usage: gen_golden.py REFERENCE_ROOT (or set BEND_GROTH16_REF): the bend-groth16 checkout")
    ref = Path(root)
    if not (ref / "bend2" / "FORMAT.md").is_file():
        sys.exit("%s does not hold a bend-groth16 checkout (no bend2/FORMAT.md)" % ref)
    export_bin = load_ref_module(ref, "bend2/tools/export_bin.py", "ref_export_bin")
    verify_bin = load_ref_module(ref, "bend2/tools/verify_bin.py", "ref_verify_bin")
    ref_qap = load_ref_module(ref, "bend2/gen/ref_qap.py", "ref_ref_qap")
    proof_to_json = load_ref_module(ref, "bend2/tools/proof_to_json.py", "ref_proof_to_json")

    pairs = montmul_pairs(ref, 1000)
    with open(HERE / "montmul_fr.bin", "wb") as f:
        f.write(struct.pack("<I", len(pairs)))
        for a, b, want in pairs:
            for v in (a, b, want):
                f.write(struct.pack("<16I", *o.words16(v)))
    build_vectors(HERE / "vectors", export_bin, verify_bin)
    for k in (4, 10):
        build_circuit(k, HERE / ("k%d" % k), export_bin, verify_bin, ref_qap, proof_to_json)
    print("golden fixtures written under", HERE)


if __name__ == "__main__":
    main()
