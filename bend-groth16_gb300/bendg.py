"""Python binding of the C ABI in include/bg.h (ctypes over the in-tree libbg.so).

This is the host-side mirror of the reference's GPU seam (bend2/prove.bend:21-49):
`Context.msm_g1` / `msm_g2` / `qap_h` take and return arrays in the bend2/FORMAT.md wire
layout (16 uint32 words per field element, each a 16-bit limb), exactly what Pr.g1_run /
Pr.g2_run / Pr.qap_run consume and produce.  Errors raise `BgError` carrying the status code;
nothing falls back to a CPU path.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libbg.so")
PROVE_BIN = os.path.join(HERE, "prove_bin")

BG_OK, BG_E_ARG, BG_E_OOM, BG_E_FORMAT, BG_E_TIMEOUT, BG_E_DEVICE, BG_E_IO = range(7)
NTT_FORWARD, NTT_INVERSE, NTT_COSET_FORWARD, NTT_COSET_INVERSE = range(4)
FIELD_FR, FIELD_FQ = 0, 1
FOP_ADD, FOP_SUB, FOP_MUL, FOP_NEG, FOP_INV, FOP_SQR, FOP_TO_MONT, FOP_FROM_MONT = range(8)
CURVE_G1, CURVE_G2 = 0, 1
COP_ADD, COP_DOUBLE, COP_NEG, COP_MUL = range(4)
PHASES = ("load", "evals", "qap", "msm_a", "msm_b1", "msm_b2", "msm_h", "msm_l", "total")
BIN_FILES = ("header", "witness", "r1cs_a", "r1cs_b", "r1cs_c", "pk_g1", "pk_g2", "pk_a", "pk_b1", "pk_b2",
             "pk_h", "pk_l", "rs")

# every symbol include/bg.h declares
EXPORTS = (
    "bg_ctx_create", "bg_ctx_destroy", "bg_strerror", "bg_last_error", "bg_ctx_stream", "bg_ctx_launches",
    "bg_host_alloc", "bg_host_free", "bg_msm_g1", "bg_msm_g2", "bg_qap_h", "bg_prove_dir", "bg_prove_host",
    "bg_pk_upload", "bg_pk_release", "bg_prove_resident", "bg_proof_format", "bg_ntt", "bg_field_op",
    "bg_curve_op", "bg_msm_g1_dev", "bg_msm_g2_dev", "bg_ntt_dev", "bg_repack_to_packed_dev",
    "bg_repack_to_wire_dev", "bg_synth_square_chain", "bg_msm_window_bits", "bg_ctx_profile",
    "bg_ctx_kernel_stats", "bg_probe_imad", "bg_msm_g1_noalloc", "bg_prove_batch", "bg_prove_footprint",
    "bg_server_create", "bg_server_submit", "bg_server_wait", "bg_server_reserved_bytes", "bg_server_destroy",
    "bg_ctx_timeline", "bg_msm_table_window_bits", "bg_ctx_transfer_bytes", "bg_verify", "bg_pairing",
    "bg_msm_window_override", "bg_msm_proof_window_bits", "bg_msm_pair_rounds_override", "bg_msm_pair_rounds",
    "bg_msm_coop_reduce_override",
)


class BgError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__("%s (status %d)" % (message, status))
        self.status = status


class Proof(ctypes.Structure):
    _fields_ = [("a", ctypes.c_uint32 * 32), ("b", ctypes.c_uint32 * 64), ("c", ctypes.c_uint32 * 32)]


class PhaseMs(ctypes.Structure):
    _fields_ = [(name, ctypes.c_double) for name in PHASES]

    def as_dict(self):
        return {name: getattr(self, name) for name in PHASES}


class Vk(ctypes.Structure):
    _fields_ = [("alpha_g1", ctypes.c_void_p), ("beta_g2", ctypes.c_void_p), ("gamma_g2", ctypes.c_void_p),
                ("delta_g2", ctypes.c_void_p), ("gamma_abc_g1", ctypes.c_void_p), ("n_ic", ctypes.c_size_t)]


class Inputs(ctypes.Structure):
    _fields_ = sum(([(name, ctypes.c_void_p), (name + "_bytes", ctypes.c_size_t)] for name in BIN_FILES), [])


_lib = None

u32p = ctypes.POINTER(ctypes.c_uint32)


def lib():
    """the loaded libbg.so; raises if the CUDA library was not built"""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise FileNotFoundError("libbg.so is not built (run __graft_entry__.build()): " + LIB_PATH)
    L = ctypes.CDLL(LIB_PATH)
    vp, sz, i32, u32, u64 = ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int, ctypes.c_uint32, ctypes.c_uint64
    sig = {
        "bg_ctx_create": (i32, [i32, ctypes.POINTER(vp)]),
        "bg_ctx_destroy": (None, [vp]),
        "bg_strerror": (ctypes.c_char_p, [i32]),
        "bg_last_error": (ctypes.c_char_p, [vp]),
        "bg_ctx_stream": (vp, [vp]),
        "bg_ctx_launches": (u64, [vp]),
        "bg_host_alloc": (i32, [sz, ctypes.POINTER(vp)]),
        "bg_host_free": (None, [vp]),
        "bg_msm_g1": (i32, [vp, vp, vp, sz, vp]),
        "bg_msm_g2": (i32, [vp, vp, vp, sz, vp]),
        "bg_qap_h": (i32, [vp, vp, vp, vp, u32, vp]),
        "bg_prove_dir": (i32, [vp, ctypes.c_char_p, ctypes.POINTER(Proof), ctypes.POINTER(PhaseMs)]),
        "bg_prove_host": (i32, [vp, ctypes.POINTER(Inputs), ctypes.POINTER(Proof), ctypes.POINTER(PhaseMs)]),
        "bg_pk_upload": (i32, [vp, ctypes.POINTER(Inputs), ctypes.POINTER(vp)]),
        "bg_pk_release": (None, [vp]),
        "bg_prove_resident": (i32, [vp, vp, vp, vp, ctypes.POINTER(Proof), ctypes.POINTER(PhaseMs)]),
        "bg_proof_format": (i32, [ctypes.POINTER(Proof), ctypes.c_char_p, sz]),
        "bg_ntt": (i32, [vp, vp, u32, i32]),
        "bg_field_op": (i32, [vp, i32, i32, vp, vp, vp, sz]),
        "bg_curve_op": (i32, [vp, i32, i32, vp, vp, vp, vp, sz]),
        "bg_msm_g1_dev": (i32, [vp, vp, vp, sz, vp]),
        "bg_msm_g2_dev": (i32, [vp, vp, vp, sz, vp]),
        "bg_ntt_dev": (i32, [vp, vp, u32, i32]),
        "bg_repack_to_packed_dev": (i32, [vp, vp, vp, sz]),
        "bg_repack_to_wire_dev": (i32, [vp, vp, vp, sz]),
        "bg_synth_square_chain": (i32, [vp, u32, u64, ctypes.c_char_p]),
        "bg_msm_window_bits": (i32, [sz, i32]),
        "bg_msm_table_window_bits": (i32, [sz, i32]),
        "bg_msm_proof_window_bits": (i32, [sz, i32]),
        "bg_msm_window_override": (i32, [vp, i32, i32, i32]),
        "bg_msm_pair_rounds_override": (i32, [vp, i32]),
        "bg_msm_pair_rounds": (i32, [sz, i32]),
        "bg_msm_coop_reduce_override": (i32, [vp, i32]),
        "bg_ctx_profile": (i32, [vp, i32]),
        "bg_ctx_timeline": (i32, [vp, i32, ctypes.c_char_p, ctypes.c_size_t]),
        "bg_ctx_transfer_bytes": (i32, [vp, ctypes.POINTER(u64), ctypes.POINTER(u64)]),
        "bg_ctx_kernel_stats": (i32, [vp, ctypes.c_char_p, ctypes.POINTER(u64), ctypes.POINTER(ctypes.c_double)]),
        "bg_probe_imad": (i32, [vp, i32, u32, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double)]),
        "bg_msm_g1_noalloc": (i32, [vp, vp, sz, vp, vp]),
        "bg_prove_batch": (i32, [vp, vp, vp, vp, sz, i32, ctypes.POINTER(Proof), ctypes.POINTER(PhaseMs),
                                 ctypes.POINTER(i32)]),
        "bg_prove_footprint": (sz, [vp]),
        "bg_server_create": (i32, [vp, i32, sz, ctypes.POINTER(vp)]),
        "bg_server_submit": (i32, [vp, vp, vp, vp, u64]),
        "bg_server_wait": (i32, [vp, i32, ctypes.POINTER(u64), ctypes.POINTER(Proof), ctypes.POINTER(PhaseMs),
                                 ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double),
                                 ctypes.POINTER(i32)]),
        "bg_server_reserved_bytes": (sz, [vp]),
        "bg_server_destroy": (None, [vp]),
        "bg_verify": (i32, [ctypes.POINTER(Vk), vp, sz, ctypes.POINTER(Proof), ctypes.POINTER(i32)]),
        "bg_pairing": (i32, [vp, vp, vp]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


def _ptr(a: np.ndarray):
    assert a.dtype == np.uint32 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(ctypes.c_void_p)


def _u32(a) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(a, dtype=np.uint32))


def _noctx_check(st: int, what: str):
    if st != 0:
        msg = lib().bg_last_error(None)
        raise BgError(st, "%s: %s" % (what, msg.decode() if msg else "error"))


def verify(alpha_g1, beta_g2, gamma_g2, delta_g2, gamma_abc_g1, public, proof: Proof) -> bool:
    """Groth16 verification on the host (bg_verify); points and public inputs in the wire
    layout (uint32 words of 16-bit limbs, Montgomery), gamma_abc_g1 as (n_ic, 32) words"""
    keep = [_u32(alpha_g1).reshape(-1), _u32(beta_g2).reshape(-1), _u32(gamma_g2).reshape(-1),
            _u32(delta_g2).reshape(-1), _u32(gamma_abc_g1).reshape(-1), _u32(public).reshape(-1)]
    n_ic = keep[4].size // 32
    vk = Vk(*[_ptr(a) for a in keep[:5]], n_ic)
    ok = ctypes.c_int()
    _noctx_check(lib().bg_verify(ctypes.byref(vk), _ptr(keep[5]) if keep[5].size else None, keep[5].size // 16,
                                 ctypes.byref(proof), ctypes.byref(ok)), "bg_verify")
    return ok.value == 1


def pairing(p_g1, q_g2) -> np.ndarray:
    """e(P, Q) (bg_pairing): 192 uint32 words, 12 Fq elements in tower order, wire layout"""
    p, q = _u32(p_g1).reshape(-1), _u32(q_g2).reshape(-1)
    out = np.zeros(192, dtype=np.uint32)
    _noctx_check(lib().bg_pairing(_ptr(p), _ptr(q), _ptr(out)), "bg_pairing")
    return out


# ---------------------------------------------------------------- wire-format helpers

def ints_to_wire(vals) -> np.ndarray:
    """python ints (< 2^256) -> (n, 16) uint32 words of 16-bit limbs"""
    vals = list(vals)
    raw = b"".join(int(v).to_bytes(32, "little") for v in vals)
    return np.frombuffer(raw, dtype="<u2").astype(np.uint32).reshape(len(vals), 16)


def wire_to_ints(words) -> list:
    w = np.asarray(words, dtype=np.uint32).reshape(-1, 16)
    raw = w.astype("<u2").tobytes()
    return [int.from_bytes(raw[32 * i: 32 * i + 32], "little") for i in range(w.shape[0])]


class Context:
    """One device context (CUDA stream + workspace) of the prover library."""

    def __init__(self, device: int = 0):
        self._L = lib()
        h = ctypes.c_void_p()
        st = self._L.bg_ctx_create(device, ctypes.byref(h))
        if st != BG_OK:
            raise BgError(st, "bg_ctx_create: " + self._L.bg_last_error(None).decode())
        self.h = h

    def close(self):
        if self.h:
            self._L.bg_ctx_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, st: int, what: str):
        if st != BG_OK:
            raise BgError(st, "%s: %s: %s" % (what, self._L.bg_strerror(st).decode(),
                                              self._L.bg_last_error(self.h).decode()))

    @property
    def stream(self) -> int:
        return self._L.bg_ctx_stream(self.h) or 0

    def launches(self) -> int:
        return int(self._L.bg_ctx_launches(self.h))

    def profile(self, enable: bool):
        self._check(self._L.bg_ctx_profile(self.h, 1 if enable else 0), "bg_ctx_profile")

    def window_override(self, layout: int, curve: int, c: int):
        """force the MSM window width (layout 0: bucket set per window, 1: tables of keys uploaded
        afterwards); c = 0 restores the library's choice"""
        self._check(self._L.bg_msm_window_override(self.h, layout, curve, c), "bg_msm_window_override")

    def pair_rounds_override(self, rounds: int):
        """force the number of batch-affine pair rounds of later MSMs (-1: the library's model,
        0: none); results do not depend on it"""
        self._check(self._L.bg_msm_pair_rounds_override(self.h, rounds), "bg_msm_pair_rounds_override")

    def coop_reduce_override(self, mode: int):
        """latency-critical window reductions on groups of 8 lanes per addition: -1 the
        library's model, 0 never, 1 always; results do not depend on it"""
        self._check(self._L.bg_msm_coop_reduce_override(self.h, mode), "bg_msm_coop_reduce_override")

    def transfer_bytes(self):
        """(host-to-device, device-to-host) bytes copied by this context so far"""
        a, b = ctypes.c_uint64(), ctypes.c_uint64()
        self._check(self._L.bg_ctx_transfer_bytes(self.h, ctypes.byref(a), ctypes.byref(b)), "bg_ctx_transfer_bytes")
        return int(a.value), int(b.value)

    def timeline(self, enable: bool):
        """enable=True starts recording launch spans; enable=False stops and returns
        [(family, start_ms, end_ms)] in issue order"""
        if enable:
            self._check(self._L.bg_ctx_timeline(self.h, 1, None, 0), "bg_ctx_timeline")
            return []
        buf = ctypes.create_string_buffer(1 << 22)
        self._check(self._L.bg_ctx_timeline(self.h, 0, buf, len(buf)), "bg_ctx_timeline")
        out = []
        for ln in buf.value.decode().splitlines():
            name, a, b = ln.split()
            out.append((name, float(a), float(b)))
        return out

    def kernel_stats(self, name: str):
        n, ms = ctypes.c_uint64(), ctypes.c_double()
        self._check(self._L.bg_ctx_kernel_stats(self.h, name.encode(), ctypes.byref(n), ctypes.byref(ms)),
                    "bg_ctx_kernel_stats")
        return int(n.value), float(ms.value)

    def probe_imad(self, which: int, iters: int):
        ops, ms = ctypes.c_double(), ctypes.c_double()
        self._check(self._L.bg_probe_imad(self.h, which, iters, ctypes.byref(ops), ctypes.byref(ms)),
                    "bg_probe_imad")
        return ops.value, ms.value

    # ---- the seam
    def msm_g1(self, points16, scalars16, n: int | None = None) -> np.ndarray:
        p, s = _u32(points16), _u32(scalars16)
        n = s.size // 16 if n is None else n
        out = np.zeros(48, dtype=np.uint32)
        self._check(self._L.bg_msm_g1(self.h, _ptr(p), _ptr(s), n, _ptr(out)), "bg_msm_g1")
        return out

    def msm_g2(self, points16, scalars16, n: int | None = None) -> np.ndarray:
        p, s = _u32(points16), _u32(scalars16)
        n = s.size // 16 if n is None else n
        out = np.zeros(96, dtype=np.uint32)
        self._check(self._L.bg_msm_g2(self.h, _ptr(p), _ptr(s), n, _ptr(out)), "bg_msm_g2")
        return out

    def qap_h(self, a16, b16, c16, log2d: int) -> np.ndarray:
        a, b, c = _u32(a16), _u32(b16), _u32(c16)
        h = np.zeros((1 << log2d) * 16, dtype=np.uint32)
        self._check(self._L.bg_qap_h(self.h, _ptr(a), _ptr(b), _ptr(c), log2d, _ptr(h)), "bg_qap_h")
        return h

    # ---- primitives
    def ntt(self, data16, log2n: int, mode: int) -> np.ndarray:
        d = _u32(data16).copy()
        self._check(self._L.bg_ntt(self.h, _ptr(d), log2n, mode), "bg_ntt")
        return d

    def field_op(self, field: int, op: int, a16, b16=None) -> np.ndarray:
        a = _u32(a16)
        b = _u32(b16) if b16 is not None else None
        n = a.size // 16
        out = np.zeros(n * 16, dtype=np.uint32)
        self._check(self._L.bg_field_op(self.h, field, op, _ptr(a), _ptr(b) if b is not None else None,
                                        _ptr(out), n), "bg_field_op")
        return out

    def curve_op(self, curve: int, op: int, p16, q16=None, k16=None) -> np.ndarray:
        p = _u32(p16)
        per = 32 if curve == CURVE_G1 else 64
        n = p.size // per
        q = _u32(q16) if q16 is not None else None
        k = _u32(k16) if k16 is not None else None
        out = np.zeros(n * per, dtype=np.uint32)
        self._check(self._L.bg_curve_op(self.h, curve, op, _ptr(p), _ptr(q) if q is not None else None,
                                        _ptr(k) if k is not None else None, _ptr(out), n), "bg_curve_op")
        return out

    # ---- whole proofs
    def prove_dir(self, path: str):
        proof, t = Proof(), PhaseMs()
        self._check(self._L.bg_prove_dir(self.h, path.encode(), ctypes.byref(proof), ctypes.byref(t)),
                    "bg_prove_dir")
        return proof, t.as_dict()

    def prove_inputs(self, inputs: "Inputs"):
        """bg_prove_host on an Inputs record whose pointers the caller set (host, pinned, or
        device memory for the five query sets)"""
        proof, t = Proof(), PhaseMs()
        self._check(self._L.bg_prove_host(self.h, ctypes.byref(inputs), ctypes.byref(proof), ctypes.byref(t)),
                    "bg_prove_host")
        return proof, t.as_dict()

    def prove_host(self, files: "HostFiles"):
        proof, t = Proof(), PhaseMs()
        self._check(self._L.bg_prove_host(self.h, ctypes.byref(files.inputs), ctypes.byref(proof),
                                          ctypes.byref(t)), "bg_prove_host")
        return proof, t.as_dict()

    def pk_upload(self, files: "HostFiles") -> "ResidentKey":
        h = ctypes.c_void_p()
        self._check(self._L.bg_pk_upload(self.h, ctypes.byref(files.inputs), ctypes.byref(h)), "bg_pk_upload")
        return ResidentKey(self, h)

    def prove_batch(self, keys, witnesses, rss, lanes: int = 8):
        """proofs i = (keys[i], witnesses[i], rss[i]) made concurrently; witnesses / rss are
        numpy uint32 arrays (host) or integer pointers (host or device).
        Returns (proofs, phase dicts, statuses)."""
        n = len(keys)
        keep = []  # host arrays stay referenced until the call returns

        def ptr(x):
            if isinstance(x, int):
                return x
            a = _u32(x)
            keep.append(a)
            return a.ctypes.data

        PK = ctypes.c_void_p * n
        PP = ctypes.c_void_p * n
        pks = PK(*[k.h.value for k in keys])
        ws = PP(*[ptr(w) for w in witnesses])
        rs = PP(*[ptr(r) for r in rss])
        proofs = (Proof * n)()
        times = (PhaseMs * n)()
        st = (ctypes.c_int * n)()
        self._check(self._L.bg_prove_batch(self.h, pks, ws, rs, n, lanes, proofs, times, st), "bg_prove_batch")
        del keep
        return list(proofs), [t.as_dict() for t in times], list(st)

    def synth_square_chain(self, log2n: int, seed: int, path: str):
        os.makedirs(path, exist_ok=True)
        self._check(self._L.bg_synth_square_chain(self.h, log2n, seed, path.encode()), "bg_synth_square_chain")

    def proof_text(self, proof: Proof) -> str:
        buf = ctypes.create_string_buffer(1024)
        self._check(self._L.bg_proof_format(ctypes.byref(proof), buf, 1024), "bg_proof_format")
        return buf.value.decode()

    # ---- device-resident primitives (pointers from a torch.cuda tensor or the like)
    def msm_g1_dev(self, d_points: int, d_scalars: int, n: int) -> np.ndarray:
        out = np.zeros(16, dtype=np.uint32)
        self._check(self._L.bg_msm_g1_dev(self.h, d_points, d_scalars, n, _ptr(out)), "bg_msm_g1_dev")
        return out

    def msm_g2_dev(self, d_points: int, d_scalars: int, n: int) -> np.ndarray:
        out = np.zeros(32, dtype=np.uint32)
        self._check(self._L.bg_msm_g2_dev(self.h, d_points, d_scalars, n, _ptr(out)), "bg_msm_g2_dev")
        return out

    def ntt_dev(self, d_data: int, log2n: int, mode: int):
        self._check(self._L.bg_ntt_dev(self.h, d_data, log2n, mode), "bg_ntt_dev")

    def repack_to_packed_dev(self, d_wire: int, d_packed: int, n: int):
        self._check(self._L.bg_repack_to_packed_dev(self.h, d_wire, d_packed, n), "bg_repack_to_packed_dev")


class Server:
    """Continuous-batching prove server over resident keys (bg_server_*)."""

    def __init__(self, ctx: Context, lanes: int = 8, hbm_budget_bytes: int = 64 << 30):
        self.ctx = ctx
        h = ctypes.c_void_p()
        ctx._check(ctx._L.bg_server_create(ctx.h, lanes, hbm_budget_bytes, ctypes.byref(h)), "bg_server_create")
        self.h = h
        self._keep = {}

    def submit(self, key: "ResidentKey", witness16, rs16, tag: int):
        w, r = _u32(witness16), _u32(rs16)
        self._keep[tag] = (w, r)  # the buffers must outlive the request
        self.ctx._check(self.ctx._L.bg_server_submit(self.h, key.h, _ptr(w), _ptr(r), tag), "bg_server_submit")

    def wait(self, timeout_ms: int = 60000):
        """-> (tag, proof, phases, latency_ms, queue_ms, status) or None on timeout"""
        tag = ctypes.c_uint64()
        proof, t = Proof(), PhaseMs()
        lat, q, st = ctypes.c_double(), ctypes.c_double(), ctypes.c_int()
        rc = self.ctx._L.bg_server_wait(self.h, timeout_ms, ctypes.byref(tag), ctypes.byref(proof), ctypes.byref(t),
                                        ctypes.byref(lat), ctypes.byref(q), ctypes.byref(st))
        if rc == BG_E_TIMEOUT:
            return None
        self.ctx._check(rc, "bg_server_wait")
        self._keep.pop(tag.value, None)
        return tag.value, proof, t.as_dict(), lat.value, q.value, st.value

    def reserved_bytes(self) -> int:
        return int(self.ctx._L.bg_server_reserved_bytes(self.h))

    def close(self):
        if self.h:
            self.ctx._L.bg_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class ResidentKey:
    def __init__(self, ctx: Context, h):
        self.ctx, self.h = ctx, h

    def footprint(self) -> int:
        return int(self.ctx._L.bg_prove_footprint(self.h))

    def prove(self, witness16: np.ndarray, rs16: np.ndarray):
        proof, t = Proof(), PhaseMs()
        w, rs = _u32(witness16), _u32(rs16)
        self.ctx._check(self.ctx._L.bg_prove_resident(self.ctx.h, self.h, _ptr(w), _ptr(rs), ctypes.byref(proof),
                                                      ctypes.byref(t)), "bg_prove_resident")
        return proof, t.as_dict()

    def prove_ptr(self, witness_ptr: int, rs_ptr: int):
        proof, t = Proof(), PhaseMs()
        self.ctx._check(self.ctx._L.bg_prove_resident(self.ctx.h, self.h, witness_ptr, rs_ptr, ctypes.byref(proof),
                                                      ctypes.byref(t)), "bg_prove_resident")
        return proof, t.as_dict()

    def release(self):
        if self.h:
            self.ctx._L.bg_pk_release(self.h)
            self.h = None

    def __del__(self):
        try:
            self.release()
        except Exception:
            pass


class HostFiles:
    """The .bin files of one data directory held in host memory (optionally pinned)."""

    def __init__(self, path: str, pinned: bool = False, ctx: Context | None = None):
        self.bufs = {}
        self._pinned = []
        self.inputs = Inputs()
        for name in BIN_FILES:
            raw = open(os.path.join(path, name + ".bin"), "rb").read()
            if pinned:
                L = lib()
                p = ctypes.c_void_p()
                st = L.bg_host_alloc(max(len(raw), 1), ctypes.byref(p))
                if st != BG_OK:
                    raise BgError(st, "bg_host_alloc")
                self._pinned.append(p)
                ctypes.memmove(p, raw, len(raw))
                arr = np.ctypeslib.as_array(ctypes.cast(p, ctypes.POINTER(ctypes.c_uint8)), shape=(len(raw),))
            else:
                arr = np.frombuffer(bytearray(raw), dtype=np.uint8)
            self.bufs[name] = arr
            setattr(self.inputs, name, arr.ctypes.data_as(ctypes.c_void_p).value if len(raw) else None)
            setattr(self.inputs, name + "_bytes", len(raw))

    def words(self, name: str) -> np.ndarray:
        return self.bufs[name].view(np.uint32)

    def nbytes(self) -> int:
        return sum(b.size for b in self.bufs.values())

    def free(self):
        L = lib()
        for p in self._pinned:
            L.bg_host_free(p)
        self._pinned = []

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass
