"""Conversions between the oracle's python-int points and the C ABI's wire words."""
import numpy as np

import bendg
import bn254_ref as o


def g1_wire(points):
    """affine G1 (None = infinity) -> (n, 32) wire words, Montgomery"""
    vals = []
    for p in points:
        vals += [0, 0] if p is None else [o.to_mont(p[0], o.P_FQ), o.to_mont(p[1], o.P_FQ)]
    return bendg.ints_to_wire(vals).reshape(len(points), 32)


def g2_wire(points):
    vals = []
    for p in points:
        if p is None:
            vals += [0, 0, 0, 0]
        else:
            vals += [o.to_mont(v, o.P_FQ) for v in (p[0][0], p[0][1], p[1][0], p[1][1])]
    return bendg.ints_to_wire(vals).reshape(len(points), 64)


def scalars_wire(scalars):
    return bendg.ints_to_wire(scalars).reshape(len(scalars), 16)


def fr_wire_mont(vals):
    return bendg.ints_to_wire([o.to_mont(v, o.P_FR) for v in vals]).reshape(len(vals), 16)


def fr_from_wire_mont(words):
    return [o.from_mont(v, o.P_FR) for v in bendg.wire_to_ints(words)]


def g1_from_jac_wire(words):
    x, y, z = (o.from_mont(v, o.P_FQ) for v in bendg.wire_to_ints(words))
    if z == 0:
        assert y == 1 and x == 0
        return None
    assert z == 1
    return (x, y)


def g2_from_jac_wire(words):
    v = [o.from_mont(t, o.P_FQ) for t in bendg.wire_to_ints(words)]
    if v[4] == 0 and v[5] == 0:
        assert v[2:4] == [1, 0] and v[0:2] == [0, 0]
        return None
    assert v[4:6] == [1, 0]
    return ((v[0], v[1]), (v[2], v[3]))


def g1_from_aff_wire(words):
    x, y = (o.from_mont(v, o.P_FQ) for v in bendg.wire_to_ints(words))
    return None if x == 0 and y == 0 else (x, y)


def g2_from_aff_wire(words):
    v = [o.from_mont(t, o.P_FQ) for t in bendg.wire_to_ints(words)]
    return None if not any(v) else ((v[0], v[1]), (v[2], v[3]))


def proof_points(ctx, proof):
    import oracle_io
    return oracle_io.parse_proof_text(ctx.proof_text(proof))
