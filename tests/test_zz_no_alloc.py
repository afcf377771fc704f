"""bg_msm_g1_noalloc, the G1 MSM that allocates nothing, against the allocating bg_msm_g1_dev.

Callers that may not allocate device memory (a program whose GPU memory is all held by its
own pool, a latency-critical loop that cannot take the synchronisation of cudaMalloc/cudaFree)
use this entry point; its scratch is a fixed array inside the library and its size limit is
16384 points.  Two calls in a row must each give the allocating path's result (the second
call sees the first call's leftovers in the shared array).  This file is collected last.
"""
import ctypes

import numpy as np
import pytest

import bendg
import bn254_ref as o
from gpu_helpers import g1_wire, scalars_wire

pytestmark = pytest.mark.gpu

MAX_POINTS = 1 << 14


def packed(wire_rows: np.ndarray) -> np.ndarray:
    """wire words (16-bit limbs) -> packed 32-bit limbs"""
    w = np.ascontiguousarray(wire_rows, dtype=np.uint32).reshape(-1, 2)
    return (w[:, 0] | (w[:, 1] << 16)).astype(np.uint32)


def test_noalloc_matches_allocating_msm(ctx):
    import torch
    L = bendg.lib()
    rng = np.random.default_rng(99)
    n_pts = MAX_POINTS
    ks = [int.from_bytes(rng.bytes(32), "little") % o.P_FR for _ in range(n_pts)]
    gen = np.repeat(g1_wire([o.G1.gen]), n_pts, axis=0)
    pts_wire = ctx.curve_op(bendg.CURVE_G1, bendg.COP_MUL, gen, k16=scalars_wire(ks))
    d_pts = torch.from_numpy(packed(pts_wire).view(np.int32)).cuda()

    for n in (MAX_POINTS, 5000):  # two calls in a row, the second smaller than the first
        sc = [int.from_bytes(rng.bytes(32), "little") % o.P_FR for _ in range(n)]
        d_sc = torch.from_numpy(packed(scalars_wire(sc)).view(np.int32)).cuda()
        torch.cuda.synchronize()
        want = ctx.msm_g1_dev(d_pts.data_ptr(), d_sc.data_ptr(), n)
        got = np.zeros(16, dtype=np.uint32)
        st = L.bg_msm_g1_noalloc(d_pts.data_ptr(), d_sc.data_ptr(), n, None, got.ctypes.data_as(ctypes.c_void_p))
        assert st == bendg.BG_OK, L.bg_last_error(None)
        assert np.array_equal(got, want)
        if n == 5000:  # and the value itself, through the discrete logs of the points
            x, y = (o.from_mont(v, o.P_FQ) for v in bendg.wire_to_ints(
                np.stack([got & 0xffff, got >> 16], axis=1).reshape(-1)))
            assert (x, y) == o.FixedBase(o.G1, o.G1.gen).mul(sum(a * b for a, b in zip(ks, sc)) % o.P_FR)

    # small n take the fallback width rule (narrow windows, many of them), where the layout's
    # guards are tightest; n = 0 gives infinity (all zero) like the allocating path
    for n in (1, 8, 200, 1000, 0):
        sc = [int.from_bytes(rng.bytes(32), "little") % o.P_FR for _ in range(max(n, 1))]
        d_sc = torch.from_numpy(packed(scalars_wire(sc)).view(np.int32)).cuda()
        torch.cuda.synchronize()
        want = ctx.msm_g1_dev(d_pts.data_ptr(), d_sc.data_ptr(), n)
        got = np.full(16, 0xdead, dtype=np.uint32)
        st = L.bg_msm_g1_noalloc(d_pts.data_ptr(), d_sc.data_ptr(), n, None, got.ctypes.data_as(ctypes.c_void_p))
        assert st == bendg.BG_OK, L.bg_last_error(None)
        assert np.array_equal(got, want), n

    # a scalar not below 2^254 is rejected, and the next valid call is unaffected
    n = 200
    sc = [int.from_bytes(rng.bytes(32), "little") % o.P_FR for _ in range(n)]
    bad = packed(scalars_wire(sc))
    bad[8 * 17 + 7] |= 0xC0000000
    d_bad = torch.from_numpy(bad.view(np.int32)).cuda()
    torch.cuda.synchronize()
    got = np.zeros(16, dtype=np.uint32)
    st = L.bg_msm_g1_noalloc(d_pts.data_ptr(), d_bad.data_ptr(), n, None, got.ctypes.data_as(ctypes.c_void_p))
    assert st == bendg.BG_E_ARG and b"2^254" in L.bg_last_error(None)
    d_sc = torch.from_numpy(packed(scalars_wire(sc)).view(np.int32)).cuda()
    torch.cuda.synchronize()
    want = ctx.msm_g1_dev(d_pts.data_ptr(), d_sc.data_ptr(), n)
    st = L.bg_msm_g1_noalloc(d_pts.data_ptr(), d_sc.data_ptr(), n, None, got.ctypes.data_as(ctypes.c_void_p))
    assert st == bendg.BG_OK, L.bg_last_error(None)
    assert np.array_equal(got, want)

    too_many = np.zeros(16, dtype=np.uint32)
    st = L.bg_msm_g1_noalloc(d_pts.data_ptr(), d_pts.data_ptr(), MAX_POINTS + 1, None,
                             too_many.ctypes.data_as(ctypes.c_void_p))
    assert st == bendg.BG_E_ARG and b"maximum" in L.bg_last_error(None)
