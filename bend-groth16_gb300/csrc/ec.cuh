// Short Weierstrass curves y^2 = x^3 + b (a = 0) over Fq (G1) and Fq2 (G2) on the device.
//
// Affine points use the wire convention of the reference: infinity is (0, 0), which is not
// on the curve (bend2/FORMAT.md:14-16, bend2/src/g1.bend:19-25).  Accumulators use
// extended Jacobian "XYZZ" coordinates (x = X/ZZ, y = Y/ZZZ, ZZ^3 = ZZZ^2), infinity is
// ZZ = 0.  Formulas are the Explicit-Formulas Database ones for XYZZ with a = 0:
//   madd-2008-s (XYZZ + affine, 8M + 2S), add-2008-s (XYZZ + XYZZ, 12M + 2S),
//   dbl-2008-s-1 (XYZZ, 6M + 3S), mdbl-2008-s (affine -> XYZZ double, 3M + 2S).
// The reference's Jacobian madd-2007-bl / add-2007-bl / dbl-2009-l (bend2/src/g1.bend:76-172)
// compute the same group law; only the projective representation differs, and every
// result leaving the device is normalised (affine, or Jacobian with Z = 1).
// Special cases (infinity, P == Q, P == -Q) are resolved by branches before the generic
// formula; they are rare on random inputs, so the branch is almost never divergent.
#pragma once
#include "fp.cuh"

namespace bg {

// Products used by the curve formulas: three shared out-of-line bodies (fp_wide.cuh) -- a
// 512-bit Karatsuba product, a 512-bit square and a Montgomery reduction -- so squares cost a
// squaring product, Y3 = u v - w z costs one reduction for two products, and an Fq2 product
// two reductions for three products, while the hot loops keep one small copy of each body in
// the instruction cache (measured against out-of-line CIOS products: G1 accumulation -3%,
// SquareChain(2^18) proof 11.6 -> 10.7 ms).
BG_DEV Fq fmul(const Fq& a, const Fq& b) { return redc_ool(wide_mul_ool(a, b)); }
BG_DEV Fq fsqr(const Fq& a) { return redc_ool(wide_sqr_ool(a)); }
BG_DEV Fq fmul_sub(const Fq& a, const Fq& b, const Fq& c, const Fq& d) {
  Wide t = wide_mul_ool(a, b);
  wide_add_2p2(t);
  const Wide u = wide_mul_ool(c, d);
  wide_sub(t, u);
  return redc_ool(t);
}
BG_DEV Fq2 fmul(const Fq2& a, const Fq2& b) { return fq2_mul_ool(a, b); }
BG_DEV Fq2 fsqr(const Fq2& a) {
  return {fmul(add(a.c0, a.c1), sub(a.c0, a.c1)), fmul(dbl(a.c0), a.c1)};
}
BG_DEV Fq2 fmul_sub(const Fq2& a, const Fq2& b, const Fq2& c, const Fq2& d) {
  return fq2_mul_sub_mul_ool(a, b, c, d);
}

// 1/a (0 -> 0): Fermat in Fq; in Fq2 through the norm a0^2 + a1^2 (bend2/src/fq2.bend:46-50)
BG_DEV Fq field_inv_any(const Fq& a) { return inv(a); }
BG_DEV Fq2 field_inv_any(const Fq2& a) {
  const Fq ni = inv(add(fsqr(a.c0), fsqr(a.c1)));
  return {fmul(a.c0, ni), neg(fmul(a.c1, ni))};
}

// 1/a by binary Euclid (fp.cuh): the latency-critical single inversion of a batch
BG_DEV Fq field_inv_fast(const Fq& a) { return inv_binary(a); }
BG_DEV Fq2 field_inv_fast(const Fq2& a) {
  const Fq ni = inv_binary(add(fsqr(a.c0), fsqr(a.c1)));
  return {fmul(a.c0, ni), neg(fmul(a.c1, ni))};
}

template <class F>
struct Affine {
  F x, y;
};

template <class F>
struct XYZZ {
  F x, y, zz, zzz;
};

template <class F>
BG_DEV bool is_inf(const Affine<F>& p) { return is_zero(p.x) && is_zero(p.y); }

template <class F>
BG_DEV bool is_inf(const XYZZ<F>& p) { return is_zero(p.zz); }

template <class F>
BG_DEV XYZZ<F> xyzz_inf() {
  XYZZ<F> r;
  r.x = field_one<F>();
  r.y = field_one<F>();
  r.zz = field_zero<F>();
  r.zzz = field_zero<F>();
  return r;
}

template <class F>
BG_DEV XYZZ<F> xyzz_from_affine(const Affine<F>& p) {
  if (is_inf(p)) return xyzz_inf<F>();
  XYZZ<F> r;
  r.x = p.x;
  r.y = p.y;
  r.zz = field_one<F>();
  r.zzz = field_one<F>();
  return r;
}

template <class F>
BG_DEV Affine<F> affine_neg(const Affine<F>& p) {
  Affine<F> r;
  r.x = p.x;
  r.y = neg(p.y);  // neg(0) = 0 keeps the (0, 0) infinity encoding
  return r;
}

template <class F>
BG_DEV XYZZ<F> xyzz_neg(const XYZZ<F>& p) {
  XYZZ<F> r = p;
  r.y = neg(p.y);
  return r;
}

// 2P for affine P != infinity, y != 0 (mdbl-2008-s)
template <class F>
BG_DEV XYZZ<F> xyzz_dbl_affine(const Affine<F>& p) {
  const F u = dbl(p.y);
  const F v = fsqr(u);
  const F w = fmul(u, v);
  const F s = fmul(p.x, v);
  const F x2 = fsqr(p.x);
  const F m = add(dbl(x2), x2);
  XYZZ<F> r;
  r.x = sub(fsqr(m), dbl(s));
  r.y = fmul_sub(m, sub(s, r.x), w, p.y);
  r.zz = v;
  r.zzz = w;
  return r;
}

// 2P (dbl-2008-s-1)
template <class F>
BG_DEV XYZZ<F> xyzz_dbl(const XYZZ<F>& p) {
  if (is_inf(p)) return p;
  const F u = dbl(p.y);
  const F v = fsqr(u);
  const F w = fmul(u, v);
  const F s = fmul(p.x, v);
  const F x2 = fsqr(p.x);
  const F m = add(dbl(x2), x2);
  XYZZ<F> r;
  r.x = sub(fsqr(m), dbl(s));
  r.y = fmul_sub(m, sub(s, r.x), w, p.y);
  r.zz = fmul(v, p.zz);
  r.zzz = fmul(w, p.zzz);
  return r;
}

// P + Q for XYZZ P and affine Q (madd-2008-s)
template <class F>
BG_DEV XYZZ<F> xyzz_madd(const XYZZ<F>& p, const Affine<F>& q) {
  if (is_inf(q)) return p;
  if (is_inf(p)) return xyzz_from_affine(q);
  const F u2 = fmul(q.x, p.zz);
  const F s2 = fmul(q.y, p.zzz);
  const F pp_ = sub(u2, p.x);
  const F r_ = sub(s2, p.y);
  if (is_zero(pp_)) {
    if (is_zero(r_)) return xyzz_dbl_affine(q);
    return xyzz_inf<F>();
  }
  const F pp = fsqr(pp_);
  const F ppp = fmul(pp_, pp);
  const F qq = fmul(p.x, pp);
  XYZZ<F> r;
  r.x = sub(sub(fsqr(r_), ppp), dbl(qq));
  r.y = fmul_sub(r_, sub(qq, r.x), p.y, ppp);
  r.zz = fmul(p.zz, pp);
  r.zzz = fmul(p.zzz, ppp);
  return r;
}

// P + Q for XYZZ P, Q (add-2008-s).  The products that read p and q come first, so neither
// input is live past them: (u1, s1, zz1 zz2, zzz1 zzz2) is p itself in other coordinates
// (x = u1 / (zz1 zz2), y = s1 / (zzz1 zzz2)), and the P = Q case doubles that.
template <class F>
BG_DEV XYZZ<F> xyzz_add(const XYZZ<F>& p, const XYZZ<F>& q) {
  if (is_inf(q)) return p;
  if (is_inf(p)) return q;
  const F u1 = fmul(p.x, q.zz);
  const F u2 = fmul(q.x, p.zz);
  const F s1 = fmul(p.y, q.zzz);
  const F s2 = fmul(q.y, p.zzz);
  const F zz12 = fmul(p.zz, q.zz);
  const F zzz12 = fmul(p.zzz, q.zzz);
  const F pp_ = sub(u2, u1);
  const F r_ = sub(s2, s1);
  if (is_zero(pp_)) {
    if (is_zero(r_)) return xyzz_dbl(XYZZ<F>{u1, s1, zz12, zzz12});
    return xyzz_inf<F>();
  }
  const F pp = fsqr(pp_);
  const F ppp = fmul(pp_, pp);
  const F qq = fmul(u1, pp);
  XYZZ<F> r;
  r.x = sub(sub(fsqr(r_), ppp), dbl(qq));
  r.y = fmul_sub(r_, sub(qq, r.x), s1, ppp);
  r.zz = fmul(zz12, pp);
  r.zzz = fmul(zzz12, ppp);
  return r;
}

// ---------------------------------------------------------------- affine pair additions
// P + Q for affine P and Q where the caller supplies 1/d for the denominator d: the
// batch-affine accumulation inverts the denominators of many additions at once (Montgomery's
// simultaneous inversion), so an addition costs the chord slope and the new coordinates
// (two products and a square) plus its three products of the shared inversion, against
// madd-2008-s's eight products and two squares.  pair_kind picks the case and its denominator:
// the chord (x_Q - x_P), the tangent (2 y_P) when P = Q, or none (a result of infinity, or one
// input at infinity).  The affine infinity is (0, 0) as everywhere on the device.
enum : uint32_t { kPairChord = 0, kPairTangent = 1, kPairInf = 2, kPairFirst = 3, kPairSecond = 4 };

template <class F>
BG_DEV uint32_t pair_kind(const Affine<F>& p, const Affine<F>& q, F& d) {
  if (is_inf(p)) return kPairSecond;
  if (is_inf(q)) return kPairFirst;
  d = sub(q.x, p.x);
  if (!is_zero(d)) return kPairChord;
  if (eq(p.y, q.y) && !is_zero(p.y)) {
    d = dbl(p.y);
    return kPairTangent;
  }
  return kPairInf;  // Q = -P (or a point of order two, which the prime-order groups lack)
}

// the sum for the case pair_kind chose; dinv = 1 / d for the chord and tangent cases
template <class F>
BG_DEV Affine<F> pair_finish(const Affine<F>& p, const Affine<F>& q, uint32_t kind, const F& dinv) {
  if (kind == kPairFirst) return p;
  if (kind == kPairSecond) return q;
  Affine<F> r;
  if (kind == kPairInf) {
    r.x = field_zero<F>();
    r.y = field_zero<F>();
    return r;
  }
  F num;
  if (kind == kPairChord) {
    num = sub(q.y, p.y);
  } else {
    const F x2 = fsqr(p.x);
    num = add(dbl(x2), x2);
  }
  const F l = fmul(num, dinv);
  r.x = sub(sub(fsqr(l), p.x), q.x);  // the tangent case has q.x = p.x
  r.y = sub(fmul(l, sub(p.x, r.x)), p.y);
  return r;
}

// ---------------------------------------------------------------- packed memory layout
// G1 affine: x[8] y[8] (64 B).  G2 affine: x.c0 x.c1 y.c0 y.c1 (128 B).
// XYZZ: x, y, zz, zzz (4 field elements).
BG_DEV void load_elem(Fq& r, const uint32_t* src) { r = load_fp<FqParams>(src); }
BG_DEV void load_elem(Fq2& r, const uint32_t* src) {
  r.c0 = load_fp<FqParams>(src);
  r.c1 = load_fp<FqParams>(src + 8);
}
BG_DEV void store_elem(uint32_t* dst, const Fq& x) { store_fp(dst, x); }
BG_DEV void store_elem(uint32_t* dst, const Fq2& x) {
  store_fp(dst, x.c0);
  store_fp(dst + 8, x.c1);
}

template <class F>
struct FieldWords;
template <>
struct FieldWords<Fq> {
  static constexpr int value = 8;
};
template <>
struct FieldWords<Fq2> {
  static constexpr int value = 16;
};

template <class F>
BG_DEV Affine<F> load_affine(const uint32_t* src) {
  constexpr int W = FieldWords<F>::value;
  Affine<F> p;
  load_elem(p.x, src);
  load_elem(p.y, src + W);
  return p;
}
template <class F>
BG_DEV void store_affine(uint32_t* dst, const Affine<F>& p) {
  constexpr int W = FieldWords<F>::value;
  store_elem(dst, p.x);
  store_elem(dst + W, p.y);
}
template <class F>
BG_DEV XYZZ<F> load_xyzz(const uint32_t* src) {
  constexpr int W = FieldWords<F>::value;
  XYZZ<F> p;
  load_elem(p.x, src);
  load_elem(p.y, src + W);
  load_elem(p.zz, src + 2 * W);
  load_elem(p.zzz, src + 3 * W);
  return p;
}
template <class F>
BG_DEV void store_xyzz(uint32_t* dst, const XYZZ<F>& p) {
  constexpr int W = FieldWords<F>::value;
  store_elem(dst, p.x);
  store_elem(dst + W, p.y);
  store_elem(dst + 2 * W, p.zz);
  store_elem(dst + 3 * W, p.zzz);
}

}  // namespace bg
