"""ctypes binding of the C oracle (oracle/bn254_oracle.c): test checker and CPU baseline only."""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "liboracle.so")
PHASES = ("load", "evals", "qap", "msm_a", "msm_b1", "msm_b2", "msm_h", "msm_l", "total")
_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            import subprocess
            subprocess.run(["make"], cwd=HERE, check=True, capture_output=True)
        L = ctypes.CDLL(LIB)
        vp, sz, i32 = ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int
        L.bgo_msm_g1.argtypes = [vp, vp, sz, i32, vp]
        L.bgo_msm_g2.argtypes = [vp, vp, sz, i32, vp]
        L.bgo_ntt.argtypes = [vp, i32, i32, i32]
        L.bgo_qap_h.argtypes = [vp, vp, vp, i32, i32, vp]
        L.bgo_prove_dir.argtypes = [ctypes.c_char_p, i32, vp, vp]
        for f in (L.bgo_msm_g1, L.bgo_msm_g2, L.bgo_ntt, L.bgo_qap_h, L.bgo_prove_dir):
            f.restype = i32
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def _u32(a):
    return np.ascontiguousarray(np.asarray(a, dtype=np.uint32))


def threads_default():
    return os.cpu_count() or 1


def msm_g1(points16, scalars16, n, threads=None):
    out = np.zeros(32, dtype=np.uint32)
    p, s = _u32(points16), _u32(scalars16)
    lib().bgo_msm_g1(_p(p), _p(s), n, threads or threads_default(), _p(out))
    return out


def msm_g2(points16, scalars16, n, threads=None):
    out = np.zeros(64, dtype=np.uint32)
    p, s = _u32(points16), _u32(scalars16)
    lib().bgo_msm_g2(_p(p), _p(s), n, threads or threads_default(), _p(out))
    return out


def ntt(data16, lg, mode, threads=None):
    d = _u32(data16).copy()
    lib().bgo_ntt(_p(d), lg, mode, threads or threads_default())
    return d


def qap_h(a16, b16, c16, lg, threads=None):
    h = np.zeros((1 << lg) * 16, dtype=np.uint32)
    a, b, c = _u32(a16), _u32(b16), _u32(c16)
    lib().bgo_qap_h(_p(a), _p(b), _p(c), lg, threads or threads_default(), _p(h))
    return h


def prove_dir(path, threads=None):
    """-> (128 proof words: A 32, B 64, C 32 affine Montgomery wire layout, phase ms dict)"""
    out = np.zeros(128, dtype=np.uint32)
    ms = np.zeros(9, dtype=np.float64)
    rc = lib().bgo_prove_dir(path.encode(), threads or threads_default(), _p(out),
                             ms.ctypes.data_as(ctypes.c_void_p))
    if rc:
        raise OSError("bgo_prove_dir: cannot read " + path)
    return out, dict(zip(PHASES, ms.tolist()))
