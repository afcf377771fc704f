"""Whole proofs: the golden SquareChain fixtures must reproduce proof_ref bit for bit (the
role of bend2/tests/test_prove.sh), through every entry point (directory, host buffers,
resident key, the prove_bin CLI); synthetic instances are checked in the exponent."""
import os
import subprocess

import numpy as np
import pytest

import bendg
import oracle_io
from conftest import GOLDEN, ROOT

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("k", [4, 10])
def test_prove_dir_equals_proof_ref(ctx, k):
    d = os.path.join(GOLDEN, "k%d" % k)
    proof, t = ctx.prove_dir(d)
    assert ctx.proof_text(proof) == open(os.path.join(d, "proof_ref.txt")).read()
    assert all(v >= 0 for v in t.values())


@pytest.mark.parametrize("k", [4, 10])
def test_prove_host_and_resident_agree(ctx, k):
    d = os.path.join(GOLDEN, "k%d" % k)
    want = open(os.path.join(d, "proof_ref.txt")).read()
    files = bendg.HostFiles(d, pinned=(k == 10))
    proof, _ = ctx.prove_host(files)
    assert ctx.proof_text(proof) == want
    key = ctx.pk_upload(files)
    for _ in range(2):  # repeated proofs against the resident key
        proof, _ = key.prove(files.words("witness"), files.words("rs"))
        assert ctx.proof_text(proof) == want
    key.release()


def test_prove_bin_cli(built_lib):
    d = os.path.join(GOLDEN, "k4")
    env = dict(os.environ, BENDG_DATA=d, BENDG_GPU="1")
    out = subprocess.run([bendg.PROVE_BIN], env=env, capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stderr
    lines = out.stdout.splitlines()
    assert "\n".join(lines[:3]) + "\n" == open(os.path.join(d, "proof_ref.txt")).read()
    assert [ln.split()[1] for ln in lines[3:]] == list(bendg.PHASES)


def test_prove_bin_missing_dir(built_lib):
    env = dict(os.environ, BENDG_DATA="/nonexistent/dir")
    out = subprocess.run([bendg.PROVE_BIN], env=env, capture_output=True, text=True, timeout=120)
    assert out.returncode == 1 and "cannot read" in out.stderr


def test_truncated_file_rejected(ctx, tmp_path):
    import shutil
    d = os.path.join(GOLDEN, "k4")
    for f in os.listdir(d):
        shutil.copy(os.path.join(d, f), tmp_path / f)
    data = open(tmp_path / "pk_h.bin", "rb").read()
    open(tmp_path / "pk_h.bin", "wb").write(data[:-128])
    with pytest.raises(bendg.BgError) as e:
        ctx.prove_dir(str(tmp_path))
    assert e.value.status == bendg.BG_E_FORMAT
    proof, _ = ctx.prove_dir(d)  # context still usable
    assert ctx.proof_text(proof) == open(os.path.join(d, "proof_ref.txt")).read()


@pytest.mark.parametrize("log2n", [6, 12, 16])
def test_synthetic_instance_trapdoor(ctx, tmp_path, log2n):
    path = str(tmp_path / ("sq%d" % log2n))
    ctx.synth_square_chain(log2n, 1234 + log2n, path)
    data = oracle_io.load_dir(path)
    trap = oracle_io.trapdoor_from_bin(data["trapdoor"])
    proof, _ = ctx.prove_dir(path)
    pts = oracle_io.parse_proof_text(ctx.proof_text(proof))
    assert oracle_io.square_chain_trapdoor_check(data, trap, pts)


def test_synth_gpu_equals_cpu(ctx, tmp_path):
    """the device fixed-base generator and the C oracle's CPU generator write identical files"""
    import ctypes
    import oracle_c
    L = oracle_c.lib()
    L.bgo_synth_square_chain.argtypes = [ctypes.c_uint32, ctypes.c_uint64, ctypes.c_char_p, ctypes.c_int]
    g, c = tmp_path / "gpu", tmp_path / "cpu"
    os.makedirs(c)
    ctx.synth_square_chain(10, 77, str(g))
    assert L.bgo_synth_square_chain(10, 77, str(c).encode(), 8) == 0
    for f in sorted(os.listdir(c)):
        assert open(g / f, "rb").read() == open(c / f, "rb").read(), f


@pytest.mark.parametrize("log2n", [14, 18, 20])
def test_prove_matches_c_oracle(ctx, tmp_path, log2n):
    """full-size proof bit-identical to the C oracle's on the same synthetic instance"""
    import oracle_c
    path = str(tmp_path / "sq")
    ctx.synth_square_chain(log2n, 4242 + log2n, path)
    want, _ = oracle_c.prove_dir(path)
    proof, _ = ctx.prove_dir(path)
    assert np.array_equal(proof_words(proof), want)
    # the resident key proves through its window tables (one shared bucket set per MSM)
    files = bendg.HostFiles(path)
    key = ctx.pk_upload(files)
    proof, _ = key.prove(files.words("witness"), files.words("rs"))
    key.release()
    assert np.array_equal(proof_words(proof), want)


def proof_words(proof):
    return np.concatenate([np.ctypeslib.as_array(proof.a), np.ctypeslib.as_array(proof.b),
                           np.ctypeslib.as_array(proof.c)])


@pytest.mark.parametrize("x0", [0, 1, -1])
def test_degenerate_witness_matches_c_oracle(ctx, tmp_path, x0):
    """SquareChain witnesses from x0 in {0, 1, -1}: every MSM scalar is 0 or 1, so one bucket
    receives all n entries of its MSM (cut into n / 32 slices: the heavy-bucket path of the
    fixup) or none at all; every entry point must still equal the C oracle."""
    import shutil
    import oracle_c
    import bn254_ref as o
    src = str(tmp_path / "sq")
    ctx.synth_square_chain(12, 99, src)
    dst = tmp_path / "deg"
    shutil.copytree(src, dst)
    n = 1 << 12
    xs = [x0 % o.P_FR]
    for _ in range(n):
        xs.append(xs[-1] * xs[-1] % o.P_FR)  # x_0 .. x_N
    z = [1, xs[n]] + xs[:n]
    mont = [v * (1 << 256) % o.P_FR for v in z]
    bendg.ints_to_wire(mont).astype("<u4").tofile(str(dst / "witness.bin"))
    want, _ = oracle_c.prove_dir(str(dst))
    proof, _ = ctx.prove_dir(str(dst))
    assert np.array_equal(proof_words(proof), want)
    files = bendg.HostFiles(str(dst))
    key = ctx.pk_upload(files)
    for _ in range(2):
        proof, _ = key.prove(files.words("witness"), files.words("rs"))
        assert np.array_equal(proof_words(proof), want)
    key.release()


@pytest.mark.parametrize("log2n", [12, 16])
def test_gpu_proofs_verify(ctx, tmp_path, log2n):
    """proofs from every entry point pass the pairing verifier under the instance's vk.bin"""
    from test_verify import read_vk, proof_from_words
    path = str(tmp_path / "sq")
    ctx.synth_square_chain(log2n, 555 + log2n, path)
    vk = read_vk(path)
    files = bendg.HostFiles(path)
    pub = files.words("witness")[16:32]
    proof, _ = ctx.prove_dir(path)
    assert bendg.verify(*vk, pub, proof)
    key = ctx.pk_upload(files)
    proof, _ = key.prove(files.words("witness"), files.words("rs"))
    key.release()
    assert bendg.verify(*vk, pub, proof)
    w = proof_words(proof).copy()
    w[0:32], w[96:128] = w[96:128].copy(), w[0:32].copy()  # A and C swapped
    assert not bendg.verify(*vk, pub, proof_from_words(w))
