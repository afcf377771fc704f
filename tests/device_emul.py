"""The device field and curve arithmetic, executed on the host for CPU tests.

`bend-groth16_gb300/csrc/fp.cuh`, `fp_wide.cuh` and `ec.cuh` compute every Fr/Fq/Fq2 product
and every G1/G2 addition with PTX carry chains written as inline `asm` statements.  This
module checks those chains without a GPU: it runs the C preprocessor over the headers,
rewrites each `asm(...)` statement into C++ that executes the same PTX instructions on 32-bit
integers with an explicit carry flag, compiles the result with g++ into a shared library and
binds it with ctypes.  Everything outside the asm statements (the CIOS row loop, the Karatsuba
split, the lazy-reduction bookkeeping, the XYZZ formulas and their special cases) is the
device source itself, compiled for the host.

PTX semantics emulated (PTX ISA, integer arithmetic instructions, extended precision):
`add/sub{.cc}`, `addc/subc{.cc}`, `mad{.cc}.lo/.hi`, `madc{.cc}.lo/.hi`, `mul.lo/.hi`, all
`.u32`.  `.cc` writes the carry flag (a borrow for `sub`/`subc`), `addc`/`subc`/`madc` read
it.  The flag starts undefined in every asm statement, as it does on the device (the compiler
may clobber it between statements): an instruction that reads it before one in the same
statement wrote it records a fault, which the tests assert never happens.  Likewise a
write-only output (`=r`) or a scratch register declared in the statement must be written before
it is read, and every `=r` output must be written; the translation checks this (each asm
statement is straight-line code) and fails otherwise.  Any other opcode, type or operand
constraint makes the translation fail loudly too.
"""
import ctypes
import os
import re
import subprocess
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "bend-groth16_gb300", "csrc")
HEADERS = ("fp.cuh", "fp_wide.cuh", "ec.cuh")

_ASM = re.compile(r"\basm\s*(?:volatile\s*)?\(")
_OPCODE = re.compile(r"^(add|addc|sub|subc|mul|mad|madc)((?:\.lo|\.hi)?)((?:\.cc)?)\.u32$")


def _skip_string(s: str, i: int) -> int:
    """index just past the string literal that starts at s[i] == '"'"""
    i += 1
    while s[i] != '"':
        i += 2 if s[i] == "\\" else 1
    return i + 1


def _split_top(s: str, sep: str) -> list[str]:
    """split s at `sep` outside string literals and parentheses"""
    parts, depth, start, i = [], 0, 0, 0
    while i < len(s):
        c = s[i]
        if c == '"':
            i = _skip_string(s, i)
            continue
        if c in "([":
            depth += 1
        elif c in ")]":
            depth -= 1
        elif c == sep and depth == 0:
            parts.append(s[start:i])
            start = i + 1
        i += 1
    parts.append(s[start:])
    return parts


def _template(s: str) -> str:
    """concatenated value of the adjacent string literals in s"""
    out, i = [], 0
    while i < len(s):
        if s[i] == '"':
            j = _skip_string(s, i)
            out.append(s[i + 1: j - 1].encode().decode("unicode_escape"))
            i = j
        elif s[i].isspace():
            i += 1
        else:
            raise ValueError("unexpected text in an asm template: %r" % s[i:i + 40])
    return "".join(out)


def _operands(s: str) -> list[tuple[str, str]]:
    ops = []
    for part in _split_top(s, ","):
        part = part.strip()
        if not part:
            continue
        m = re.match(r'^"([^"]*)"\s*\((.*)\)$', part, re.S)
        if not m:
            raise ValueError("unexpected asm operand %r" % part)
        ops.append((m.group(1), m.group(2).strip()))
    return ops


def _operand_expr(tok: str, names: set) -> str:
    tok = tok.strip()
    m = re.fullmatch(r"%(\d+)", tok)
    if m:
        return "_o%s" % m.group(1)
    if re.fullmatch(r"(0[xX][0-9a-fA-F]+|\d+)[uU]?", tok):
        return "((uint32_t)%sull)" % tok.rstrip("uU")
    if tok in names:
        return "_v_" + tok
    raise ValueError("unknown PTX operand %r" % tok)


def _instruction(line: str, names: set, unset: set) -> str:
    """C++ for one PTX instruction; `unset` holds the operands that have no value yet (write-only
    outputs and scratch registers not written so far in this statement): reading one is an
    error, writing one removes it"""
    op, _, rest = line.strip().partition(" ")
    m = _OPCODE.match(op)
    if not m:
        raise ValueError("PTX instruction not emulated: %r" % line)
    base, half, cc = m.group(1), m.group(2), m.group(3)
    args = [_operand_expr(t, names) for t in rest.split(",")]
    need = {"mul": 3, "mad": 4, "madc": 4}.get(base, 3)
    if len(args) != need:
        raise ValueError("wrong operand count in %r" % line)
    for src in args[1:]:
        if src in unset:
            raise ValueError("%r reads an operand that has no value yet" % line)
    unset.discard(args[0])
    if base in ("mul", "mad", "madc") and not half:
        raise ValueError("mul/mad without .lo/.hi: %r" % line)
    d, a, b = args[0], args[1], args[2]
    chk = "if (_cf > 1) g_emul_fault = __LINE__; "
    setcf = cc != ""
    if base in ("mul", "mad", "madc"):
        prod = "((uint64_t)%s * (uint64_t)%s)" % (a, b)
        p = "(uint32_t)(%s >> 32)" % prod if half == ".hi" else "(uint32_t)%s" % prod
        if base == "mul":
            if setcf:
                raise ValueError("mul.cc does not exist: %r" % line)
            return "%s = %s;" % (d, p)
        c = args[3]
        cin = " + (uint64_t)_cf" if base == "madc" else ""
        s = ("{ %suint64_t _t = (uint64_t)%s + (uint64_t)%s%s; %s = (uint32_t)_t;%s }"
             % (chk if base == "madc" else "", p, c, cin, d, " _cf = (int)(_t >> 32);" if setcf else ""))
        return s
    if half:
        raise ValueError("add/sub take no .lo/.hi: %r" % line)
    if base in ("add", "addc"):
        cin = " + (uint64_t)_cf" if base == "addc" else ""
        return ("{ %suint64_t _t = (uint64_t)%s + (uint64_t)%s%s; %s = (uint32_t)_t;%s }"
                % (chk if base == "addc" else "", a, b, cin, d, " _cf = (int)(_t >> 32);" if setcf else ""))
    # sub / subc: the flag is the borrow
    bin_ = "(uint64_t)%s + (uint64_t)_cf" % b if base == "subc" else "(uint64_t)%s" % b
    return ("{ %suint64_t _a = %s, _b = %s; %s = (uint32_t)(_a - _b);%s }"
            % (chk if base == "subc" else "", a, bin_, d, " _cf = _a < _b;" if setcf else ""))


def translate_asm(body: str) -> str:
    """C++ block executing one asm statement's body (the text between `asm(` and `)`)"""
    parts = _split_top(body, ":")
    if not 1 <= len(parts) <= 4:
        raise ValueError("unexpected asm statement shape")
    text = _template(parts[0])
    outs = _operands(parts[1]) if len(parts) > 1 else []
    ins = _operands(parts[2]) if len(parts) > 2 else []
    if len(parts) > 3 and parts[3].strip():
        raise ValueError("asm clobbers are not expected: %r" % parts[3])
    ops = outs + ins
    code = ["{ int _cf = 2;"]
    unset = set()
    for k, (cons, expr) in enumerate(ops):
        if k < len(outs):
            if cons not in ("=r", "+r"):
                raise ValueError("output constraint %r not emulated" % cons)
            if cons == "=r":
                unset.add("_o%d" % k)
            code.append("uint32_t _o%d%s;" % (k, " = (uint32_t)(%s)" % expr if cons == "+r" else ""))
        else:
            if cons not in ("r", "n"):
                raise ValueError("input constraint %r not emulated" % cons)
            code.append("const uint32_t _o%d = (uint32_t)(%s);" % (k, expr))
    names = set()
    for stmt in text.replace("{", ";").replace("}", ";").split(";"):
        stmt = stmt.strip()
        if not stmt:
            continue
        if stmt.startswith(".reg"):
            m = re.fullmatch(r"\.reg\s+\.u32\s+(.+)", stmt)
            if not m:
                raise ValueError("register declaration not emulated: %r" % stmt)
            for nm in m.group(1).split(","):
                nm = nm.strip()
                names.add(nm)
                unset.add("_v_" + nm)
                code.append("uint32_t _v_%s = 0;" % nm)
            continue
        code.append(_instruction(stmt, names, unset))
    never = sorted(u for u in unset if u.startswith("_o"))
    if never:
        raise ValueError("asm outputs never written: %s" % ", ".join(never))
    for k, (cons, expr) in enumerate(outs):
        code.append("(%s) = _o%d;" % (expr, k))
    code.append("(void)_cf; }")
    return "\n".join(code)


def translate_source(src: str) -> tuple[str, int]:
    """src with every asm statement replaced by its emulation; also the statement count"""
    out, i, count = [], 0, 0
    while True:
        m = _ASM.search(src, i)
        if not m:
            out.append(src[i:])
            break
        out.append(src[i:m.start()])
        j = k = m.end()
        depth = 1
        while depth:
            c = src[k]
            if c == '"':
                k = _skip_string(src, k)
                continue
            if c == "(":
                depth += 1
            elif c == ")":
                depth -= 1
            k += 1
        out.append(translate_asm(src[j:k - 1]))
        count += 1
        i = k
    return "".join(out), count


_PRELUDE = r"""
#include <cstdint>
#include <cstring>
struct uint4 { uint32_t x, y, z, w; };
inline uint4 make_uint4(uint32_t x, uint32_t y, uint32_t z, uint32_t w) { return {x, y, z, w}; }
static int g_emul_fault = 0;
"""

_EXPORTS = r"""
using namespace bg;
template <class P> static Fp<P> ld(const uint32_t* s) { Fp<P> r; memcpy(r.v, s, 32); return r; }
template <class P> static void st(uint32_t* d, const Fp<P>& x) { memcpy(d, x.v, 32); }
static Fq2 ld2(const uint32_t* s) { return {ld<FqParams>(s), ld<FqParams>(s + 8)}; }
static void st2(uint32_t* d, const Fq2& x) { st(d, x.c0); st(d + 8, x.c1); }
static void ldf(Fq& r, const uint32_t* s) { r = ld<FqParams>(s); }
static void ldf(Fq2& r, const uint32_t* s) { r = ld2(s); }
static void stf(uint32_t* d, const Fq& x) { st(d, x); }
static void stf(uint32_t* d, const Fq2& x) { st2(d, x); }
template <class F> static XYZZ<F> ldx(const uint32_t* s) {
  constexpr int W = FieldWords<F>::value; XYZZ<F> p;
  ldf(p.x, s); ldf(p.y, s + W); ldf(p.zz, s + 2 * W); ldf(p.zzz, s + 3 * W); return p;
}
template <class F> static void stx(uint32_t* d, const XYZZ<F>& p) {
  constexpr int W = FieldWords<F>::value;
  stf(d, p.x); stf(d + W, p.y); stf(d + 2 * W, p.zz); stf(d + 3 * W, p.zzz);
}
template <class F> static Affine<F> lda(const uint32_t* s) {
  constexpr int W = FieldWords<F>::value; Affine<F> p; ldf(p.x, s); ldf(p.y, s + W); return p;
}
template <class F> static void sta(uint32_t* d, const Affine<F>& p) {
  constexpr int W = FieldWords<F>::value; stf(d, p.x); stf(d + W, p.y);
}
/* one affine pair addition as the batch-affine rounds make it, with a one-element batch: the
 * denominator pair_kind picks, inverted by the binary-Euclid inverse, into pair_finish */
template <class F> static void pair_add_impl(const uint32_t* p, const uint32_t* q, uint32_t* r, uint32_t* kind) {
  const Affine<F> P = lda<F>(p), Q = lda<F>(q);
  F d = field_zero<F>();
  *kind = pair_kind(P, Q, d);
  const F dinv = *kind <= kPairTangent ? field_inv_fast(d) : field_zero<F>();
  sta(r, pair_finish(P, Q, *kind, dinv));
}

#define FIELD_OPS(PFX, PARAMS)                                                                  \
  void PFX##_add(const uint32_t* a, const uint32_t* b, uint32_t* r) { st(r, add(ld<PARAMS>(a), ld<PARAMS>(b))); } \
  void PFX##_sub(const uint32_t* a, const uint32_t* b, uint32_t* r) { st(r, sub(ld<PARAMS>(a), ld<PARAMS>(b))); } \
  void PFX##_neg(const uint32_t* a, uint32_t* r) { st(r, neg(ld<PARAMS>(a))); }                 \
  void PFX##_mul(const uint32_t* a, const uint32_t* b, uint32_t* r) { st(r, mul(ld<PARAMS>(a), ld<PARAMS>(b))); } \
  void PFX##_sqr(const uint32_t* a, uint32_t* r) { st(r, sqr(ld<PARAMS>(a))); }                 \
  void PFX##_inv(const uint32_t* a, uint32_t* r) { st(r, inv(ld<PARAMS>(a))); }                 \
  void PFX##_inv_binary(const uint32_t* a, uint32_t* r) { st(r, inv_binary(ld<PARAMS>(a))); }   \
  void PFX##_from_mont(const uint32_t* a, uint32_t* r) { st(r, from_mont(ld<PARAMS>(a))); }     \
  void PFX##_redc(const uint32_t* t16, uint32_t* r) { Wide t; memcpy(t.v, t16, 64); st(r, redc<PARAMS>(t)); }

extern "C" {
int emu_fault(void) { return g_emul_fault; }
void emu_clear_fault(void) { g_emul_fault = 0; }
FIELD_OPS(fq, FqParams)
FIELD_OPS(fr, FrParams)
void wide_mul_raw(const uint32_t* a, const uint32_t* b, uint32_t* t16) { Wide t; wide_mul(t, a, b); memcpy(t16, t.v, 64); }
void wide_sqr_raw(const uint32_t* a, uint32_t* t16) { Wide t; wide_sqr(t, a); memcpy(t16, t.v, 64); }
void fq_fmul(const uint32_t* a, const uint32_t* b, uint32_t* r) { st(r, fmul(ld<FqParams>(a), ld<FqParams>(b))); }
void fq_fsqr(const uint32_t* a, uint32_t* r) { st(r, fsqr(ld<FqParams>(a))); }
void fq_fmul_sub(const uint32_t* a, const uint32_t* b, const uint32_t* c, const uint32_t* d, uint32_t* r) {
  st(r, fmul_sub(ld<FqParams>(a), ld<FqParams>(b), ld<FqParams>(c), ld<FqParams>(d)));
}
void fq2_mul(const uint32_t* a, const uint32_t* b, uint32_t* r) { st2(r, mul(ld2(a), ld2(b))); }
void fq2_sqr(const uint32_t* a, uint32_t* r) { st2(r, sqr(ld2(a))); }
void fq2_fmul(const uint32_t* a, const uint32_t* b, uint32_t* r) { st2(r, fmul(ld2(a), ld2(b))); }
void fq2_fsqr(const uint32_t* a, uint32_t* r) { st2(r, fsqr(ld2(a))); }
void fq2_fmul_sub(const uint32_t* a, const uint32_t* b, const uint32_t* c, const uint32_t* d, uint32_t* r) {
  st2(r, fmul_sub(ld2(a), ld2(b), ld2(c), ld2(d)));
}
void fq2_inv(const uint32_t* a, uint32_t* r) { st2(r, field_inv_any(ld2(a))); }
void fq2_inv_fast(const uint32_t* a, uint32_t* r) { st2(r, field_inv_fast(ld2(a))); }
void g1_pair_add(const uint32_t* p, const uint32_t* q, uint32_t* kind, uint32_t* r) { pair_add_impl<Fq>(p, q, r, kind); }
void g2_pair_add(const uint32_t* p, const uint32_t* q, uint32_t* kind, uint32_t* r) { pair_add_impl<Fq2>(p, q, r, kind); }

#define CURVE_OPS(PFX, F)                                                                       \
  void PFX##_madd(const uint32_t* p, const uint32_t* q, uint32_t* r) { stx(r, xyzz_madd(ldx<F>(p), lda<F>(q))); } \
  void PFX##_add(const uint32_t* p, const uint32_t* q, uint32_t* r) { stx(r, xyzz_add(ldx<F>(p), ldx<F>(q))); } \
  void PFX##_dbl(const uint32_t* p, uint32_t* r) { stx(r, xyzz_dbl(ldx<F>(p))); }               \
  void PFX##_dbl_affine(const uint32_t* q, uint32_t* r) { stx(r, xyzz_dbl_affine(lda<F>(q))); } \
  void PFX##_from_affine(const uint32_t* q, uint32_t* r) { stx(r, xyzz_from_affine(lda<F>(q))); }
CURVE_OPS(g1, Fq)
CURVE_OPS(g2, Fq2)
}
"""


def build(out_dir: str | None = None) -> str:
    """translate and compile the headers; returns the shared library's path"""
    out_dir = out_dir or tempfile.mkdtemp(prefix="device_emul_")
    fake = os.path.join(out_dir, "fakeinc")
    os.makedirs(fake, exist_ok=True)
    for h in ("cstdint",):
        open(os.path.join(fake, h), "w").close()
    top = os.path.join(out_dir, "top.cpp")
    with open(top, "w") as f:
        f.write('#include "ec.cuh"\n')
    pre = subprocess.run(
        ["g++", "-E", "-P", "-nostdinc", "-I", fake, "-I", CSRC, "-D__device__=", "-D__forceinline__=",
         "-D__noinline__=", "-DBG_DEV=inline", "-x", "c++", top],
        check=True, capture_output=True, text=True).stdout
    body, count = translate_source(pre)
    if count < 40:
        raise RuntimeError("only %d asm statements found in %s" % (count, ", ".join(HEADERS)))
    src = os.path.join(out_dir, "device_emul.cpp")
    with open(src, "w") as f:
        f.write(_PRELUDE + body + _EXPORTS)
    so = os.path.join(out_dir, "libdevice_emul.so")
    subprocess.run(["g++", "-O1", "-std=c++17", "-shared", "-fPIC", "-w", "-o", so, src], check=True)
    return so


_DIGITS_EXPORTS = r"""
extern "C" {
int digit_window_width(int w, int W) { return bg::window_width(w, W); }
int digit_window_offset(int w, int W) { return bg::window_offset(w, W); }
/* signed digits of one scalar (8 limbs) over W windows, as k_digits_hist and k_scatter make
 * them; returns the carry left after the top window */
uint32_t digits(const uint32_t* s, int W, uint32_t* mags, uint8_t* negs) {
  uint32_t carry = 0;
  for (int w = 0; w < W; w++) {
    bool ng = false;
    mags[w] = bg::signed_digit(s, w, W, carry, ng);
    negs[w] = ng ? 1 : 0;
  }
  return carry;
}
}
"""


def build_digits(out_dir: str) -> str:
    """the MSM's window layout and signed-digit recoding (the digits section of msm.cu, from
    window_bits to signed_digit, which k_digits_hist and k_scatter call) compiled for the host;
    returns the shared library's path"""
    src_text = open(os.path.join(CSRC, "msm.cu")).read()
    start = src_text.index("BG_DEV uint32_t window_bits(")
    end = src_text.index("__global__ void k_digits_hist(")
    section = src_text[start:end]
    os.makedirs(out_dir, exist_ok=True)
    src = os.path.join(out_dir, "digits_emul.cpp")
    with open(src, "w") as f:
        f.write(_PRELUDE + "#define BG_DEV inline\n#define __host__\n#define __device__\n#define __restrict__\n"
                + "namespace bg {\n" + section + "}  // namespace bg\n" + _DIGITS_EXPORTS)
    so = os.path.join(out_dir, "libdigits_emul.so")
    subprocess.run(["g++", "-O1", "-std=c++17", "-shared", "-fPIC", "-w", "-o", so, src], check=True)
    return so


class DeviceArith:
    """ctypes view of the compiled emulation; values are Python ints, Montgomery form where
    the device keeps them so (the caller converts)"""

    def __init__(self, so_path: str):
        self.lib = ctypes.CDLL(so_path)

    @staticmethod
    def words(x: int, n: int = 8):
        if not 0 <= x < 1 << (32 * n):
            raise ValueError("value does not fit %d words" % n)
        return (ctypes.c_uint32 * n)(*[(x >> (32 * i)) & 0xFFFFFFFF for i in range(n)])

    @staticmethod
    def value(w) -> int:
        return sum(int(v) << (32 * i) for i, v in enumerate(w))

    def fault(self) -> int:
        return self.lib.emu_fault()

    def call(self, name: str, args: list, out_words: int) -> int:
        out = (ctypes.c_uint32 * out_words)()
        getattr(self.lib, name)(*args, out)
        return self.value(out)
