// BN254 base field Fq and scalar field Fr on the device: 8 x 32-bit little-endian limbs,
// Montgomery form with R = 2^256 (the value stored for x is x*2^256 mod p).
//
// Reference: the Bend prover keeps the same Montgomery representation in 16 x 16-bit limbs
// (bend2/FORMAT.md:5-12; Fr.mul CIOS at bend2/src/fr.bend:269, Fq.mul at bend2/src/fq.bend:269,
// n0' at fr.bend:4 / fq.bend:4).  Here one limb is 32 bits, so a product is 8 rows of
// coarsely-integrated operand scanning (CIOS, Koc-Acar-Kaliski 1996) written as PTX
// mad.lo/hi.cc carry chains.  Every carry chain lives inside a single asm statement so no
// compiler-generated instruction can sit between two .cc instructions.
//
// Invariants: inputs and outputs of add/sub/mul are fully reduced (< p).  Both moduli are
// below 2^254, so a CIOS row's running value stays below 2^288 (9 limbs) and the final
// result is below 2p; one conditional subtraction reduces it.
#pragma once
#include <cstdint>

#ifndef BG_DEV
#define BG_DEV __device__ __forceinline__
#endif

namespace bg {

// ---------------------------------------------------------------- moduli and constants
struct FqParams {
  static constexpr uint32_t P0 = 0xd87cfd47u, P1 = 0x3c208c16u, P2 = 0x6871ca8du, P3 = 0x97816a91u,
                            P4 = 0x8181585du, P5 = 0xb85045b6u, P6 = 0xe131a029u, P7 = 0x30644e72u;
  static constexpr uint32_t N0 = 0xe4866389u;  // -p^-1 mod 2^32
  // R mod p (Montgomery one)
  static constexpr uint32_t ONE0 = 0xc58f0d9du, ONE1 = 0xd35d438du, ONE2 = 0xf5c70b3du, ONE3 = 0x0a78eb28u,
                            ONE4 = 0x7879462cu, ONE5 = 0x666ea36fu, ONE6 = 0x9a07df2fu, ONE7 = 0x0e0a77c1u;
  // R^3 mod p (turns the inverse of a Montgomery representative into a Montgomery inverse)
  static constexpr uint32_t R3_0 = 0xda1530dfu, R3_1 = 0xb1cd6dafu, R3_2 = 0xa7283db6u, R3_3 = 0x62f210e6u,
                            R3_4 = 0x0ada0afbu, R3_5 = 0xef7f0b0cu, R3_6 = 0x2d592544u, R3_7 = 0x20fd6e90u;
};
struct FrParams {
  static constexpr uint32_t P0 = 0xf0000001u, P1 = 0x43e1f593u, P2 = 0x79b97091u, P3 = 0x2833e848u,
                            P4 = 0x8181585du, P5 = 0xb85045b6u, P6 = 0xe131a029u, P7 = 0x30644e72u;
  static constexpr uint32_t N0 = 0xefffffffu;
  static constexpr uint32_t ONE0 = 0x4ffffffbu, ONE1 = 0xac96341cu, ONE2 = 0x9f60cd29u, ONE3 = 0x36fc7695u,
                            ONE4 = 0x7879462eu, ONE5 = 0x666ea36fu, ONE6 = 0x9a07df2fu, ONE7 = 0x0e0a77c1u;
  static constexpr uint32_t R3_0 = 0xb4bf0040u, R3_1 = 0x5e94d8e1u, R3_2 = 0x1cfbb6b8u, R3_3 = 0x2a489cbeu,
                            R3_4 = 0xa19fcfedu, R3_5 = 0x893cc664u, R3_6 = 0x7fcc657cu, R3_7 = 0x0cf8594bu;
};

template <class P>
struct Fp {
  uint32_t v[8];
};
using Fq = Fp<FqParams>;
using Fr = Fp<FrParams>;

// ---------------------------------------------------------------- basic predicates
template <class P>
BG_DEV bool is_zero(const Fp<P>& a) {
  uint32_t o = a.v[0] | a.v[1] | a.v[2] | a.v[3] | a.v[4] | a.v[5] | a.v[6] | a.v[7];
  return o == 0;
}
template <class P>
BG_DEV bool eq(const Fp<P>& a, const Fp<P>& b) {
  uint32_t o = 0;
#pragma unroll
  for (int i = 0; i < 8; i++) o |= a.v[i] ^ b.v[i];
  return o == 0;
}
template <class P>
BG_DEV Fp<P> fp_zero() {
  Fp<P> r;
#pragma unroll
  for (int i = 0; i < 8; i++) r.v[i] = 0;
  return r;
}
template <class P>
BG_DEV Fp<P> fp_one() {
  Fp<P> r;
  r.v[0] = P::ONE0; r.v[1] = P::ONE1; r.v[2] = P::ONE2; r.v[3] = P::ONE3;
  r.v[4] = P::ONE4; r.v[5] = P::ONE5; r.v[6] = P::ONE6; r.v[7] = P::ONE7;
  return r;
}

// ---------------------------------------------------------------- reduction helper
// r = t - p if t >= p else t   (t < 2p, 8 limbs)
template <class P>
BG_DEV void reduce_once(uint32_t* r, const uint32_t* t) {
  uint32_t d0, d1, d2, d3, d4, d5, d6, d7, bw;
  asm("sub.cc.u32  %0, %9,  %17;\n\t"
      "subc.cc.u32 %1, %10, %18;\n\t"
      "subc.cc.u32 %2, %11, %19;\n\t"
      "subc.cc.u32 %3, %12, %20;\n\t"
      "subc.cc.u32 %4, %13, %21;\n\t"
      "subc.cc.u32 %5, %14, %22;\n\t"
      "subc.cc.u32 %6, %15, %23;\n\t"
      "subc.cc.u32 %7, %16, %24;\n\t"
      "subc.u32    %8, 0, 0;"
      : "=r"(d0), "=r"(d1), "=r"(d2), "=r"(d3), "=r"(d4), "=r"(d5), "=r"(d6), "=r"(d7), "=r"(bw)
      : "r"(t[0]), "r"(t[1]), "r"(t[2]), "r"(t[3]), "r"(t[4]), "r"(t[5]), "r"(t[6]), "r"(t[7]),
        "n"(P::P0), "n"(P::P1), "n"(P::P2), "n"(P::P3), "n"(P::P4), "n"(P::P5), "n"(P::P6), "n"(P::P7));
  // bw = 0xffffffff when t < p (borrow): keep t
  const bool keep = bw != 0;
  r[0] = keep ? t[0] : d0;
  r[1] = keep ? t[1] : d1;
  r[2] = keep ? t[2] : d2;
  r[3] = keep ? t[3] : d3;
  r[4] = keep ? t[4] : d4;
  r[5] = keep ? t[5] : d5;
  r[6] = keep ? t[6] : d6;
  r[7] = keep ? t[7] : d7;
}

// ---------------------------------------------------------------- add / sub / neg
template <class P>
BG_DEV Fp<P> add(const Fp<P>& a, const Fp<P>& b) {
  uint32_t t[8];
  asm("add.cc.u32  %0, %8,  %16;\n\t"
      "addc.cc.u32 %1, %9,  %17;\n\t"
      "addc.cc.u32 %2, %10, %18;\n\t"
      "addc.cc.u32 %3, %11, %19;\n\t"
      "addc.cc.u32 %4, %12, %20;\n\t"
      "addc.cc.u32 %5, %13, %21;\n\t"
      "addc.cc.u32 %6, %14, %22;\n\t"
      "addc.u32    %7, %15, %23;"
      : "=r"(t[0]), "=r"(t[1]), "=r"(t[2]), "=r"(t[3]), "=r"(t[4]), "=r"(t[5]), "=r"(t[6]), "=r"(t[7])
      : "r"(a.v[0]), "r"(a.v[1]), "r"(a.v[2]), "r"(a.v[3]), "r"(a.v[4]), "r"(a.v[5]), "r"(a.v[6]), "r"(a.v[7]),
        "r"(b.v[0]), "r"(b.v[1]), "r"(b.v[2]), "r"(b.v[3]), "r"(b.v[4]), "r"(b.v[5]), "r"(b.v[6]), "r"(b.v[7]));
  Fp<P> r;
  reduce_once<P>(r.v, t);
  return r;
}

template <class P>
BG_DEV Fp<P> sub(const Fp<P>& a, const Fp<P>& b) {
  uint32_t t[8], bw;
  asm("sub.cc.u32  %0, %9,  %17;\n\t"
      "subc.cc.u32 %1, %10, %18;\n\t"
      "subc.cc.u32 %2, %11, %19;\n\t"
      "subc.cc.u32 %3, %12, %20;\n\t"
      "subc.cc.u32 %4, %13, %21;\n\t"
      "subc.cc.u32 %5, %14, %22;\n\t"
      "subc.cc.u32 %6, %15, %23;\n\t"
      "subc.cc.u32 %7, %16, %24;\n\t"
      "subc.u32    %8, 0, 0;"
      : "=r"(t[0]), "=r"(t[1]), "=r"(t[2]), "=r"(t[3]), "=r"(t[4]), "=r"(t[5]), "=r"(t[6]), "=r"(t[7]), "=r"(bw)
      : "r"(a.v[0]), "r"(a.v[1]), "r"(a.v[2]), "r"(a.v[3]), "r"(a.v[4]), "r"(a.v[5]), "r"(a.v[6]), "r"(a.v[7]),
        "r"(b.v[0]), "r"(b.v[1]), "r"(b.v[2]), "r"(b.v[3]), "r"(b.v[4]), "r"(b.v[5]), "r"(b.v[6]), "r"(b.v[7]));
  // on borrow add p back (mask p by bw)
  Fp<P> r;
  asm("add.cc.u32  %0, %8,  %16;\n\t"
      "addc.cc.u32 %1, %9,  %17;\n\t"
      "addc.cc.u32 %2, %10, %18;\n\t"
      "addc.cc.u32 %3, %11, %19;\n\t"
      "addc.cc.u32 %4, %12, %20;\n\t"
      "addc.cc.u32 %5, %13, %21;\n\t"
      "addc.cc.u32 %6, %14, %22;\n\t"
      "addc.u32    %7, %15, %23;"
      : "=r"(r.v[0]), "=r"(r.v[1]), "=r"(r.v[2]), "=r"(r.v[3]), "=r"(r.v[4]), "=r"(r.v[5]), "=r"(r.v[6]), "=r"(r.v[7])
      : "r"(t[0]), "r"(t[1]), "r"(t[2]), "r"(t[3]), "r"(t[4]), "r"(t[5]), "r"(t[6]), "r"(t[7]),
        "r"(P::P0 & bw), "r"(P::P1 & bw), "r"(P::P2 & bw), "r"(P::P3 & bw), "r"(P::P4 & bw), "r"(P::P5 & bw),
        "r"(P::P6 & bw), "r"(P::P7 & bw));
  return r;
}

template <class P>
BG_DEV Fp<P> neg(const Fp<P>& a) {
  // p - a, and 0 stays 0
  return sub(fp_zero<P>(), a);
}

template <class P>
BG_DEV Fp<P> dbl(const Fp<P>& a) { return add(a, a); }

// ---------------------------------------------------------------- Montgomery product
// one CIOS row: t += a*bi; m = t0*n0'; t += m*p; (t0 becomes 0; the caller shifts)
#define BG_CIOS_ROW(P)                                                                          \
  asm("{\n\t.reg .u32 m;\n\t"                                                                   \
      "mad.lo.cc.u32  %0, %9,  %17, %0;\n\t"                                                   \
      "madc.lo.cc.u32 %1, %10, %17, %1;\n\t"                                                   \
      "madc.lo.cc.u32 %2, %11, %17, %2;\n\t"                                                   \
      "madc.lo.cc.u32 %3, %12, %17, %3;\n\t"                                                   \
      "madc.lo.cc.u32 %4, %13, %17, %4;\n\t"                                                   \
      "madc.lo.cc.u32 %5, %14, %17, %5;\n\t"                                                   \
      "madc.lo.cc.u32 %6, %15, %17, %6;\n\t"                                                   \
      "madc.lo.cc.u32 %7, %16, %17, %7;\n\t"                                                   \
      "addc.u32       %8, %8, 0;\n\t"                                                          \
      "mad.hi.cc.u32  %1, %9,  %17, %1;\n\t"                                                   \
      "madc.hi.cc.u32 %2, %10, %17, %2;\n\t"                                                   \
      "madc.hi.cc.u32 %3, %11, %17, %3;\n\t"                                                   \
      "madc.hi.cc.u32 %4, %12, %17, %4;\n\t"                                                   \
      "madc.hi.cc.u32 %5, %13, %17, %5;\n\t"                                                   \
      "madc.hi.cc.u32 %6, %14, %17, %6;\n\t"                                                   \
      "madc.hi.cc.u32 %7, %15, %17, %7;\n\t"                                                   \
      "madc.hi.u32    %8, %16, %17, %8;\n\t"                                                   \
      "mul.lo.u32     m, %0, %18;\n\t"                                                         \
      "mad.lo.cc.u32  %0, m, %19, %0;\n\t"                                                     \
      "madc.lo.cc.u32 %1, m, %20, %1;\n\t"                                                     \
      "madc.lo.cc.u32 %2, m, %21, %2;\n\t"                                                     \
      "madc.lo.cc.u32 %3, m, %22, %3;\n\t"                                                     \
      "madc.lo.cc.u32 %4, m, %23, %4;\n\t"                                                     \
      "madc.lo.cc.u32 %5, m, %24, %5;\n\t"                                                     \
      "madc.lo.cc.u32 %6, m, %25, %6;\n\t"                                                     \
      "madc.lo.cc.u32 %7, m, %26, %7;\n\t"                                                     \
      "addc.u32       %8, %8, 0;\n\t"                                                          \
      "mad.hi.cc.u32  %1, m, %19, %1;\n\t"                                                     \
      "madc.hi.cc.u32 %2, m, %20, %2;\n\t"                                                     \
      "madc.hi.cc.u32 %3, m, %21, %3;\n\t"                                                     \
      "madc.hi.cc.u32 %4, m, %22, %4;\n\t"                                                     \
      "madc.hi.cc.u32 %5, m, %23, %5;\n\t"                                                     \
      "madc.hi.cc.u32 %6, m, %24, %6;\n\t"                                                     \
      "madc.hi.cc.u32 %7, m, %25, %7;\n\t"                                                     \
      "madc.hi.u32    %8, m, %26, %8;\n\t}"                                                    \
      : "+r"(t0), "+r"(t1), "+r"(t2), "+r"(t3), "+r"(t4), "+r"(t5), "+r"(t6), "+r"(t7), "+r"(t8) \
      : "r"(a.v[0]), "r"(a.v[1]), "r"(a.v[2]), "r"(a.v[3]), "r"(a.v[4]), "r"(a.v[5]),         \
        "r"(a.v[6]), "r"(a.v[7]), "r"(bi), "n"(P::N0), "n"(P::P0), "n"(P::P1), "n"(P::P2),     \
        "n"(P::P3), "n"(P::P4), "n"(P::P5), "n"(P::P6), "n"(P::P7))

template <class P>
BG_DEV Fp<P> mul(const Fp<P>& a, const Fp<P>& b) {
  uint32_t t0 = 0, t1 = 0, t2 = 0, t3 = 0, t4 = 0, t5 = 0, t6 = 0, t7 = 0, t8 = 0;
#pragma unroll
  for (int i = 0; i < 8; i++) {
    const uint32_t bi = b.v[i];
    BG_CIOS_ROW(P);
    // t0 is now zero: shift one limb down
    t0 = t1; t1 = t2; t2 = t3; t3 = t4; t4 = t5; t5 = t6; t6 = t7; t7 = t8; t8 = 0;
  }
  uint32_t t[8] = {t0, t1, t2, t3, t4, t5, t6, t7};
  Fp<P> r;
  reduce_once<P>(r.v, t);
  return r;
}
#undef BG_CIOS_ROW

// squaring product (28 off-diagonal limb products doubled, then one reduction; fp_wide.cuh)
template <class P>
BG_DEV Fp<P> sqr_wide(const Fp<P>& a);
template <class P>
BG_DEV Fp<P> sqr(const Fp<P>& a) { return sqr_wide(a); }

// x * 2^-256: Montgomery -> canonical (multiply by the raw integer 1)
template <class P>
BG_DEV Fp<P> from_mont(const Fp<P>& a) {
  Fp<P> one_raw = fp_zero<P>();
  one_raw.v[0] = 1;
  return mul(a, one_raw);
}

// a^e for a 256-bit exponent given as 8 limbs (square-and-multiply, MSB first)
template <class P>
BG_DEV Fp<P> pow_limbs(const Fp<P>& a, const uint32_t* e) {
  Fp<P> r = fp_one<P>();
  for (int i = 7; i >= 0; i--) {
    for (int b = 31; b >= 0; b--) {
      r = sqr(r);
      if ((e[i] >> b) & 1u) r = mul(r, a);
    }
  }
  return r;
}

// 1/a = a^(p-2) (Fermat); inv(0) = 0 as in bend2/src/fq.bend:1991
template <class P>
BG_DEV Fp<P> inv(const Fp<P>& a) {
  const uint32_t e[8] = {P::P0 - 2u, P::P1, P::P2, P::P3, P::P4, P::P5, P::P6, P::P7};
  return pow_limbs(a, e);
}

// ---------------------------------------------------------------- inversion by binary Euclid
// 1/a for a Montgomery element a (0 -> 0).  Binary extended Euclid (Hankerson, Menezes and
// Vanstone, Guide to Elliptic Curve Cryptography, Algorithm 2.22) on the representative aR,
// with the invariants (aR) x1 = u and (aR) x2 = v (mod p) from u = aR, v = p: strip the factors
// of two from u (x1 follows with x1 / 2^k mod p), subtract the smaller of the odd u, v from the
// larger (x1 or x2 follows), until u or v is 1; one Montgomery product by R^3 mod p then turns
// (aR)^-1 into a^-1 R.  The k trailing zeros of u leave in one step: x1 / 2^k mod p is the exact
// quotient (x1 + m p) / 2^k with m = x1 (-p^-1) mod 2^k, which is below p for x1 < p, so a
// pass is a subtraction, a shift and one 8-limb multiply-add, about 250 passes in all.  One
// thread computes the inversion that a whole CTA of the batch-affine bucket accumulation waits
// for, so its latency is what counts (the Fermat power is 320 dependent products).  Variable
// time (the inputs are public bucket coordinates).  Requires a < p (every stored element is).
namespace binv {
BG_DEV bool is_one8(const uint32_t* u) {
  return u[0] == 1u && (u[1] | u[2] | u[3] | u[4] | u[5] | u[6] | u[7]) == 0u;
}
BG_DEV int ctz32(uint32_t x) {
#ifdef __CUDA_ARCH__
  return __ffs((int)x) - 1;
#else
  return __builtin_ctz(x);
#endif
}
// u >>= k, 1 <= k <= 31
BG_DEV void shr8(uint32_t* u, int k) {
#pragma unroll
  for (int i = 0; i < 7; i++) u[i] = (u[i] >> k) | (u[i + 1] << (32 - k));
  u[7] >>= k;
}
// x = x / 2^k mod p for x < p, 1 <= k <= 31: (x + m p) / 2^k, m = x n0' mod 2^k
BG_DEV void div2k_mod(uint32_t* x, int k, const uint32_t* p, uint32_t n0) {
  const uint32_t m = (x[0] * n0) & ((1u << k) - 1u);
  uint32_t t[9];
  uint64_t c = 0;
#pragma unroll
  for (int i = 0; i < 8; i++) {
    c += (uint64_t)x[i] + (uint64_t)m * p[i];
    t[i] = (uint32_t)c;
    c >>= 32;
  }
  t[8] = (uint32_t)c;
#pragma unroll
  for (int i = 0; i < 8; i++) x[i] = (t[i] >> k) | (t[i + 1] << (32 - k));
}
// strip the factors of two of u (u != 0), dividing x by the same power of two mod p
BG_DEV void strip2(uint32_t* u, uint32_t* x, const uint32_t* p, uint32_t n0) {
  for (int limb = 0; limb < 8 && u[0] == 0u; limb++) {  // rare: a whole zero limb, two steps of 16 bits
#pragma unroll
    for (int i = 0; i < 7; i++) u[i] = u[i + 1];
    u[7] = 0u;
    div2k_mod(x, 16, p, n0);
    div2k_mod(x, 16, p, n0);
  }
  if (u[0] == 0u) return;  // u = 0: only for an input that is 0 mod p
  const int k = ctz32(u[0]);
  if (k) {
    shr8(u, k);
    div2k_mod(x, k, p, n0);
  }
}
// u -= v when u >= v (returns true), else leaves u and returns false
BG_DEV bool sub_if_geq(uint32_t* u, const uint32_t* v) {
  uint32_t d[8];
  uint64_t b = 0;
#pragma unroll
  for (int i = 0; i < 8; i++) {
    const uint64_t t = (uint64_t)u[i] - v[i] - b;
    d[i] = (uint32_t)t;
    b = t >> 63;
  }
  if (b) return false;
#pragma unroll
  for (int i = 0; i < 8; i++) u[i] = d[i];
  return true;
}
BG_DEV void sub8(uint32_t* u, const uint32_t* v) {
  uint64_t b = 0;
#pragma unroll
  for (int i = 0; i < 8; i++) {
    const uint64_t t = (uint64_t)u[i] - v[i] - b;
    u[i] = (uint32_t)t;
    b = t >> 63;
  }
}
// x = x - y mod p (x, y < p)
BG_DEV void sub_mod(uint32_t* x, const uint32_t* y, const uint32_t* p) {
  uint64_t b = 0;
#pragma unroll
  for (int i = 0; i < 8; i++) {
    const uint64_t t = (uint64_t)x[i] - y[i] - b;
    x[i] = (uint32_t)t;
    b = t >> 63;
  }
  if (b) {
    uint64_t c = 0;
#pragma unroll
    for (int i = 0; i < 8; i++) {
      c += (uint64_t)x[i] + p[i];
      x[i] = (uint32_t)c;
      c >>= 32;
    }
  }
}
}  // namespace binv

template <class P>
BG_DEV Fp<P> inv_binary(const Fp<P>& a) {
  if (is_zero(a)) return a;
  const uint32_t p[8] = {P::P0, P::P1, P::P2, P::P3, P::P4, P::P5, P::P6, P::P7};
  uint32_t u[8], v[8], x1[8], x2[8];
#pragma unroll
  for (int i = 0; i < 8; i++) {
    u[i] = a.v[i];
    v[i] = p[i];
    x1[i] = 0;
    x2[i] = 0;
  }
  x1[0] = 1;
  // v is odd from the start and after every strip; each pass removes at least one bit from
  // u v (below 2^508), so 512 passes always suffice
  for (int pass = 0; pass < 512; pass++) {
    binv::strip2(u, x1, p, P::N0);
    if (binv::is_one8(u) || binv::is_one8(v)) break;
    if (binv::sub_if_geq(u, v)) {
      binv::sub_mod(x1, x2, p);
    } else {
      binv::sub8(v, u);
      binv::sub_mod(x2, x1, p);
      binv::strip2(v, x2, p, P::N0);
    }
  }
  Fp<P> r, r3;
#pragma unroll
  for (int i = 0; i < 8; i++) r.v[i] = binv::is_one8(u) ? x1[i] : x2[i];
  r3.v[0] = P::R3_0; r3.v[1] = P::R3_1; r3.v[2] = P::R3_2; r3.v[3] = P::R3_3;
  r3.v[4] = P::R3_4; r3.v[5] = P::R3_5; r3.v[6] = P::R3_6; r3.v[7] = P::R3_7;
  return mul(r, r3);
}

// ---------------------------------------------------------------- Fq2 = Fq[u]/(u^2 + 1)
// bend2/src/fq2.bend:31-50: Karatsuba product (3M), complex square (2M)
struct Fq2 {
  Fq c0, c1;
};

BG_DEV bool is_zero(const Fq2& a) { return is_zero(a.c0) && is_zero(a.c1); }
BG_DEV bool eq(const Fq2& a, const Fq2& b) { return eq(a.c0, b.c0) && eq(a.c1, b.c1); }
BG_DEV Fq2 add(const Fq2& a, const Fq2& b) { return {add(a.c0, b.c0), add(a.c1, b.c1)}; }
BG_DEV Fq2 sub(const Fq2& a, const Fq2& b) { return {sub(a.c0, b.c0), sub(a.c1, b.c1)}; }
BG_DEV Fq2 neg(const Fq2& a) { return {neg(a.c0), neg(a.c1)}; }
BG_DEV Fq2 dbl(const Fq2& a) { return {dbl(a.c0), dbl(a.c1)}; }
BG_DEV Fq2 mul(const Fq2& a, const Fq2& b) {
  const Fq t0 = mul(a.c0, b.c0);
  const Fq t1 = mul(a.c1, b.c1);
  const Fq t2 = mul(add(a.c0, a.c1), add(b.c0, b.c1));
  return {sub(t0, t1), sub(sub(t2, t0), t1)};
}
BG_DEV Fq2 sqr(const Fq2& a) {
  return {mul(add(a.c0, a.c1), sub(a.c0, a.c1)), mul(dbl(a.c0), a.c1)};
}

template <class F>
BG_DEV F field_zero();
template <>
BG_DEV Fq field_zero<Fq>() { return fp_zero<FqParams>(); }
template <>
BG_DEV Fr field_zero<Fr>() { return fp_zero<FrParams>(); }
template <>
BG_DEV Fq2 field_zero<Fq2>() { return {fp_zero<FqParams>(), fp_zero<FqParams>()}; }

template <class F>
BG_DEV F field_one();
template <>
BG_DEV Fq field_one<Fq>() { return fp_one<FqParams>(); }
template <>
BG_DEV Fr field_one<Fr>() { return fp_one<FrParams>(); }
template <>
BG_DEV Fq2 field_one<Fq2>() { return {fp_one<FqParams>(), fp_zero<FqParams>()}; }

// ---------------------------------------------------------------- global memory helpers
// 128-bit loads/stores of packed elements (an element is 32 bytes, 32-byte aligned)
template <class P>
BG_DEV Fp<P> load_fp(const uint32_t* src) {
  const uint4 a = reinterpret_cast<const uint4*>(src)[0];
  const uint4 b = reinterpret_cast<const uint4*>(src)[1];
  Fp<P> r;
  r.v[0] = a.x; r.v[1] = a.y; r.v[2] = a.z; r.v[3] = a.w;
  r.v[4] = b.x; r.v[5] = b.y; r.v[6] = b.z; r.v[7] = b.w;
  return r;
}
template <class P>
BG_DEV void store_fp(uint32_t* dst, const Fp<P>& x) {
  reinterpret_cast<uint4*>(dst)[0] = make_uint4(x.v[0], x.v[1], x.v[2], x.v[3]);
  reinterpret_cast<uint4*>(dst)[1] = make_uint4(x.v[4], x.v[5], x.v[6], x.v[7]);
}

}  // namespace bg

#include "fp_wide.cuh"
