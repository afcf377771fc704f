"""Field and curve primitives on the GPU against the golden vectors (the shapes of the
reference's bend2/tests/test_fr.bend, test_fq.bend, test_g1.bend, test_g2.bend)."""
import os
import struct

import numpy as np
import pytest

import bendg
import bn254_ref as o
from conftest import GOLDEN

pytestmark = pytest.mark.gpu


def words(buf, off, count):
    return np.frombuffer(buf, dtype="<u4", count=16 * count, offset=off).astype(np.uint32)


@pytest.mark.parametrize("name,field", [("fr_ops", bendg.FIELD_FR), ("fq_ops", bendg.FIELD_FQ)])
def test_field_ops(ctx, name, field):
    buf = open(os.path.join(GOLDEN, "vectors", name + ".bin"), "rb").read()
    (n,) = struct.unpack_from("<I", buf, 0)
    rec = np.frombuffer(buf, dtype="<u4", offset=4).reshape(n, 9, 16).astype(np.uint32)
    a, b = rec[:, 0].copy(), rec[:, 1].copy()
    ops = [(bendg.FOP_ADD, 2), (bendg.FOP_SUB, 3), (bendg.FOP_MUL, 4), (bendg.FOP_NEG, 5), (bendg.FOP_INV, 6),
           (bendg.FOP_SQR, 7)]
    for op, col in ops:
        got = ctx.field_op(field, op, a, b).reshape(n, 16)
        assert np.array_equal(got, rec[:, col]), (name, op)
    # from / to Montgomery against the canonical column
    assert np.array_equal(ctx.field_op(field, bendg.FOP_FROM_MONT, a).reshape(n, 16), rec[:, 8])
    assert np.array_equal(ctx.field_op(field, bendg.FOP_TO_MONT, rec[:, 8].copy()).reshape(n, 16), a)


def test_montmul_pairs(ctx):
    buf = open(os.path.join(GOLDEN, "montmul_fr.bin"), "rb").read()
    (n,) = struct.unpack_from("<I", buf, 0)
    rec = np.frombuffer(buf, dtype="<u4", offset=4).reshape(n, 3, 16).astype(np.uint32)
    got = ctx.field_op(bendg.FIELD_FR, bendg.FOP_MUL, rec[:, 0].copy(), rec[:, 1].copy()).reshape(n, 16)
    assert np.array_equal(got, rec[:, 2])


@pytest.mark.parametrize("name,curve,pw", [("g1_ops", bendg.CURVE_G1, 32), ("g2_ops", bendg.CURVE_G2, 64)])
def test_curve_ops(ctx, name, curve, pw):
    buf = open(os.path.join(GOLDEN, "vectors", name + ".bin"), "rb").read()
    (n,) = struct.unpack_from("<I", buf, 0)
    rec = np.frombuffer(buf, dtype="<u4", offset=4).reshape(n, 6 * pw + 16).astype(np.uint32)
    p = rec[:, 0:pw].copy()
    q = rec[:, pw:2 * pw].copy()
    k = rec[:, 2 * pw:2 * pw + 16].copy()
    exp = [rec[:, 2 * pw + 16 + j * pw: 2 * pw + 16 + (j + 1) * pw] for j in range(4)]
    assert np.array_equal(ctx.curve_op(curve, bendg.COP_ADD, p, q).reshape(n, pw), exp[0])
    assert np.array_equal(ctx.curve_op(curve, bendg.COP_DOUBLE, p).reshape(n, pw), exp[1])
    assert np.array_equal(ctx.curve_op(curve, bendg.COP_NEG, p).reshape(n, pw), exp[2])
    assert np.array_equal(ctx.curve_op(curve, bendg.COP_MUL, p, k16=k).reshape(n, pw), exp[3])


def test_bad_wire_word_rejected(ctx):
    a = np.zeros((4, 16), dtype=np.uint32)
    a[1, 3] = 0x10000  # a limb above 16 bits violates bend2/FORMAT.md
    with pytest.raises(bendg.BgError) as e:
        ctx.field_op(bendg.FIELD_FR, bendg.FOP_NEG, a)
    assert e.value.status == bendg.BG_E_FORMAT
