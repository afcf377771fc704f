// Host-side BN254 arithmetic for the library's serial steps: the window combination of an
// MSM (a few hundred doublings), normalisation to affine, the Groth16 combine
// (bend2/src/groth16.bend:298-308), NTT twiddle / coset table seeds, and canonical
// conversion for printing.  4 x 64-bit little-endian limbs, Montgomery form with R = 2^256
// (the same integers the device holds as 8 x 32-bit limbs on a little-endian host).
#pragma once
#include <cstdint>
#include <cstring>

namespace bgh {

typedef unsigned __int128 u128;

struct Mod {
  uint64_t p[4];
  uint64_t n0;      // -p^-1 mod 2^64
  uint64_t one[4];  // R mod p
  uint64_t r2[4];   // R^2 mod p
};

extern const Mod FQ;
extern const Mod FR;

struct Fe {
  uint64_t v[4];
};

inline bool fe_is_zero(const Fe& a) { return (a.v[0] | a.v[1] | a.v[2] | a.v[3]) == 0; }
inline bool fe_eq(const Fe& a, const Fe& b) {
  return a.v[0] == b.v[0] && a.v[1] == b.v[1] && a.v[2] == b.v[2] && a.v[3] == b.v[3];
}
inline Fe fe_zero() { return Fe{{0, 0, 0, 0}}; }
inline Fe fe_one(const Mod& m) { return Fe{{m.one[0], m.one[1], m.one[2], m.one[3]}}; }
inline Fe fe_raw(uint64_t x) { return Fe{{x, 0, 0, 0}}; }

// a >= b as 256-bit integers
inline bool geq(const uint64_t* a, const uint64_t* b) {
  for (int i = 3; i >= 0; i--) {
    if (a[i] != b[i]) return a[i] > b[i];
  }
  return true;
}
inline uint64_t sub4(uint64_t* r, const uint64_t* a, const uint64_t* b) {
  uint64_t borrow = 0;
  for (int i = 0; i < 4; i++) {
    u128 d = (u128)a[i] - b[i] - borrow;
    r[i] = (uint64_t)d;
    borrow = (uint64_t)(d >> 64) & 1;
  }
  return borrow;
}
inline uint64_t add4(uint64_t* r, const uint64_t* a, const uint64_t* b) {
  uint64_t c = 0;
  for (int i = 0; i < 4; i++) {
    u128 s = (u128)a[i] + b[i] + c;
    r[i] = (uint64_t)s;
    c = (uint64_t)(s >> 64);
  }
  return c;
}

inline Fe fe_add(const Mod& m, const Fe& a, const Fe& b) {
  Fe r;
  add4(r.v, a.v, b.v);  // < 2p < 2^255, no carry out
  if (geq(r.v, m.p)) sub4(r.v, r.v, m.p);
  return r;
}
inline Fe fe_sub(const Mod& m, const Fe& a, const Fe& b) {
  Fe r;
  if (sub4(r.v, a.v, b.v)) add4(r.v, r.v, m.p);
  return r;
}
inline Fe fe_neg(const Mod& m, const Fe& a) { return fe_sub(m, fe_zero(), a); }
inline Fe fe_dbl(const Mod& m, const Fe& a) { return fe_add(m, a, a); }

// CIOS Montgomery product a*b*2^-256 mod p
inline Fe fe_mul(const Mod& m, const Fe& a, const Fe& b) {
  uint64_t t[6] = {0, 0, 0, 0, 0, 0};
  for (int i = 0; i < 4; i++) {
    uint64_t c = 0;
    for (int j = 0; j < 4; j++) {
      u128 s = (u128)a.v[j] * b.v[i] + t[j] + c;
      t[j] = (uint64_t)s;
      c = (uint64_t)(s >> 64);
    }
    u128 s = (u128)t[4] + c;
    t[4] = (uint64_t)s;
    t[5] = (uint64_t)(s >> 64);
    const uint64_t q = t[0] * m.n0;
    s = (u128)q * m.p[0] + t[0];
    c = (uint64_t)(s >> 64);
    for (int j = 1; j < 4; j++) {
      s = (u128)q * m.p[j] + t[j] + c;
      t[j - 1] = (uint64_t)s;
      c = (uint64_t)(s >> 64);
    }
    s = (u128)t[4] + c;
    t[3] = (uint64_t)s;
    t[4] = t[5] + (uint64_t)(s >> 64);
  }
  Fe r{{t[0], t[1], t[2], t[3]}};
  if (t[4] || geq(r.v, m.p)) sub4(r.v, r.v, m.p);
  return r;
}
inline Fe fe_sqr(const Mod& m, const Fe& a) { return fe_mul(m, a, a); }
inline Fe fe_to_mont(const Mod& m, const Fe& a) {
  return fe_mul(m, a, Fe{{m.r2[0], m.r2[1], m.r2[2], m.r2[3]}});
}
inline Fe fe_from_mont(const Mod& m, const Fe& a) { return fe_mul(m, a, fe_raw(1)); }

inline Fe fe_pow(const Mod& m, const Fe& a, const uint64_t e[4]) {
  Fe r = fe_one(m);
  for (int i = 3; i >= 0; i--)
    for (int b = 63; b >= 0; b--) {
      r = fe_sqr(m, r);
      if ((e[i] >> b) & 1) r = fe_mul(m, r, a);
    }
  return r;
}
inline Fe fe_pow_u64(const Mod& m, const Fe& a, uint64_t e) {
  const uint64_t ee[4] = {e, 0, 0, 0};
  return fe_pow(m, a, ee);
}
// 1/a (Fermat); 0 -> 0
inline Fe fe_inv(const Mod& m, const Fe& a) {
  uint64_t e[4] = {m.p[0] - 2, m.p[1], m.p[2], m.p[3]};
  return fe_pow(m, a, e);
}

// ---------------------------------------------------------------- Fq2 = Fq[u]/(u^2+1)
struct Fe2 {
  Fe c0, c1;
};
inline bool fe_is_zero(const Fe2& a) { return fe_is_zero(a.c0) && fe_is_zero(a.c1); }
inline bool fe_eq(const Fe2& a, const Fe2& b) { return fe_eq(a.c0, b.c0) && fe_eq(a.c1, b.c1); }

// Field adaptors so curve code is generic over Fq and Fq2
struct FqOps {
  typedef Fe T;
  static T zero() { return fe_zero(); }
  static T one() { return fe_one(FQ); }
  static T add(const T& a, const T& b) { return fe_add(FQ, a, b); }
  static T sub(const T& a, const T& b) { return fe_sub(FQ, a, b); }
  static T neg(const T& a) { return fe_neg(FQ, a); }
  static T mul(const T& a, const T& b) { return fe_mul(FQ, a, b); }
  static T sqr(const T& a) { return fe_mul(FQ, a, a); }
  static T inv(const T& a) { return fe_inv(FQ, a); }
  static bool is_zero(const T& a) { return fe_is_zero(a); }
  static bool eq(const T& a, const T& b) { return fe_eq(a, b); }
  static constexpr int WORDS = 8;  // 32-bit words
};
struct Fq2Ops {
  typedef Fe2 T;
  static T zero() { return {fe_zero(), fe_zero()}; }
  static T one() { return {fe_one(FQ), fe_zero()}; }
  static T add(const T& a, const T& b) { return {fe_add(FQ, a.c0, b.c0), fe_add(FQ, a.c1, b.c1)}; }
  static T sub(const T& a, const T& b) { return {fe_sub(FQ, a.c0, b.c0), fe_sub(FQ, a.c1, b.c1)}; }
  static T neg(const T& a) { return {fe_neg(FQ, a.c0), fe_neg(FQ, a.c1)}; }
  static T mul(const T& a, const T& b) {
    Fe t0 = fe_mul(FQ, a.c0, b.c0), t1 = fe_mul(FQ, a.c1, b.c1);
    Fe t2 = fe_mul(FQ, fe_add(FQ, a.c0, a.c1), fe_add(FQ, b.c0, b.c1));
    return {fe_sub(FQ, t0, t1), fe_sub(FQ, fe_sub(FQ, t2, t0), t1)};
  }
  static T sqr(const T& a) {
    return {fe_mul(FQ, fe_add(FQ, a.c0, a.c1), fe_sub(FQ, a.c0, a.c1)), fe_mul(FQ, fe_dbl(FQ, a.c0), a.c1)};
  }
  static T inv(const T& a) {
    Fe n = fe_add(FQ, fe_sqr(FQ, a.c0), fe_sqr(FQ, a.c1));
    Fe ni = fe_inv(FQ, n);
    return {fe_mul(FQ, a.c0, ni), fe_neg(FQ, fe_mul(FQ, a.c1, ni))};
  }
  static bool is_zero(const T& a) { return fe_is_zero(a); }
  static bool eq(const T& a, const T& b) { return fe_eq(a, b); }
  static constexpr int WORDS = 16;
};

// ---------------------------------------------------------------- curve points
template <class F>
struct Aff {
  typename F::T x, y;
  bool inf;
};
template <class F>
struct Xyzz {
  typename F::T x, y, zz, zzz;
};

template <class F>
Xyzz<F> xyzz_inf() {
  return {F::one(), F::one(), F::zero(), F::zero()};
}
template <class F>
bool xyzz_is_inf(const Xyzz<F>& p) {
  return F::is_zero(p.zz);
}
template <class F>
Xyzz<F> xyzz_from(const Aff<F>& a) {
  if (a.inf) return xyzz_inf<F>();
  return {a.x, a.y, F::one(), F::one()};
}
template <class F>
Xyzz<F> xyzz_dbl(const Xyzz<F>& p) {
  if (xyzz_is_inf(p)) return p;
  auto u = F::add(p.y, p.y);
  auto v = F::sqr(u);
  auto w = F::mul(u, v);
  auto s = F::mul(p.x, v);
  auto x2 = F::sqr(p.x);
  auto m = F::add(F::add(x2, x2), x2);
  Xyzz<F> r;
  r.x = F::sub(F::sqr(m), F::add(s, s));
  r.y = F::sub(F::mul(m, F::sub(s, r.x)), F::mul(w, p.y));
  r.zz = F::mul(v, p.zz);
  r.zzz = F::mul(w, p.zzz);
  return r;
}
template <class F>
Xyzz<F> xyzz_add(const Xyzz<F>& p, const Xyzz<F>& q) {
  if (xyzz_is_inf(q)) return p;
  if (xyzz_is_inf(p)) return q;
  auto u1 = F::mul(p.x, q.zz);
  auto u2 = F::mul(q.x, p.zz);
  auto s1 = F::mul(p.y, q.zzz);
  auto s2 = F::mul(q.y, p.zzz);
  auto pp_ = F::sub(u2, u1);
  auto r_ = F::sub(s2, s1);
  if (F::is_zero(pp_)) {
    if (F::is_zero(r_)) return xyzz_dbl(p);
    return xyzz_inf<F>();
  }
  auto pp = F::sqr(pp_);
  auto ppp = F::mul(pp_, pp);
  auto qq = F::mul(u1, pp);
  Xyzz<F> r;
  r.x = F::sub(F::sub(F::sqr(r_), ppp), F::add(qq, qq));
  r.y = F::sub(F::mul(r_, F::sub(qq, r.x)), F::mul(s1, ppp));
  r.zz = F::mul(F::mul(p.zz, q.zz), pp);
  r.zzz = F::mul(F::mul(p.zzz, q.zzz), ppp);
  return r;
}
template <class F>
Xyzz<F> xyzz_neg(const Xyzz<F>& p) {
  Xyzz<F> r = p;
  r.y = F::neg(p.y);
  return r;
}
template <class F>
Aff<F> xyzz_to_affine(const Xyzz<F>& p) {
  Aff<F> a;
  if (xyzz_is_inf(p)) {
    a.x = F::zero();
    a.y = F::zero();
    a.inf = true;
    return a;
  }
  // x = X/ZZ, y = Y/ZZZ with one inversion: 1/(ZZ*ZZZ)
  auto t = F::inv(F::mul(p.zz, p.zzz));
  a.x = F::mul(p.x, F::mul(t, p.zzz));
  a.y = F::mul(p.y, F::mul(t, p.zz));
  a.inf = false;
  return a;
}
// k*P for a canonical scalar k (4 x 64 little-endian), 4-bit fixed window
template <class F>
Xyzz<F> xyzz_mul(const Xyzz<F>& p, const uint64_t k[4]) {
  Xyzz<F> tab[16];
  tab[0] = xyzz_inf<F>();
  for (int i = 1; i < 16; i++) tab[i] = xyzz_add(tab[i - 1], p);
  Xyzz<F> r = xyzz_inf<F>();
  for (int i = 63; i >= 0; i--) {
    for (int d = 0; d < 4; d++) r = xyzz_dbl(r);
    unsigned nib = (unsigned)(k[i / 16] >> (4 * (i % 16))) & 15u;
    if (nib) r = xyzz_add(r, tab[nib]);
  }
  return r;
}

// k*P for a 64-bit k, the same 4-bit fixed window
template <class F>
Xyzz<F> xyzz_mul64(const Xyzz<F>& p, uint64_t k) {
  Xyzz<F> tab[16];
  tab[0] = xyzz_inf<F>();
  for (int i = 1; i < 16; i++) tab[i] = xyzz_add(tab[i - 1], p);
  Xyzz<F> r = xyzz_inf<F>();
  for (int i = 15; i >= 0; i--) {
    for (int d = 0; d < 4; d++) r = xyzz_dbl(r);
    const unsigned nib = (unsigned)(k >> (4 * i)) & 15u;
    if (nib) r = xyzz_add(r, tab[nib]);
  }
  return r;
}

// ---------------------------------------------------------------- wire-format conversion
// FORMAT.md element: 16 words, each a 16-bit limb (bend2/FORMAT.md:7-8)
inline Fe fe_from_words16(const uint32_t* w) {
  Fe r;
  for (int i = 0; i < 4; i++) {
    r.v[i] = (uint64_t)(w[4 * i] & 0xffff) | ((uint64_t)(w[4 * i + 1] & 0xffff) << 16) |
             ((uint64_t)(w[4 * i + 2] & 0xffff) << 32) | ((uint64_t)(w[4 * i + 3] & 0xffff) << 48);
  }
  return r;
}
inline void fe_to_words16(uint32_t* w, const Fe& a) {
  for (int i = 0; i < 16; i++) w[i] = (uint32_t)(a.v[i / 4] >> (16 * (i % 4))) & 0xffffu;
}
inline Fe fe_from_words32(const uint32_t* w) {
  Fe r;
  for (int i = 0; i < 4; i++) r.v[i] = (uint64_t)w[2 * i] | ((uint64_t)w[2 * i + 1] << 32);
  return r;
}
inline void fe_to_words32(uint32_t* w, const Fe& a) {
  for (int i = 0; i < 8; i++) w[i] = (uint32_t)(a.v[i / 2] >> (32 * (i % 2)));
}

template <class F>
void elem_from_words32(typename F::T& r, const uint32_t* w);
template <>
inline void elem_from_words32<FqOps>(Fe& r, const uint32_t* w) {
  r = fe_from_words32(w);
}
template <>
inline void elem_from_words32<Fq2Ops>(Fe2& r, const uint32_t* w) {
  r.c0 = fe_from_words32(w);
  r.c1 = fe_from_words32(w + 8);
}
template <class F>
void elem_to_words32(uint32_t* w, const typename F::T& a);
template <>
inline void elem_to_words32<FqOps>(uint32_t* w, const Fe& a) {
  fe_to_words32(w, a);
}
template <>
inline void elem_to_words32<Fq2Ops>(uint32_t* w, const Fe2& a) {
  fe_to_words32(w, a.c0);
  fe_to_words32(w + 8, a.c1);
}
template <class F>
Xyzz<F> xyzz_from_words32(const uint32_t* w) {
  Xyzz<F> p;
  elem_from_words32<F>(p.x, w);
  elem_from_words32<F>(p.y, w + F::WORDS);
  elem_from_words32<F>(p.zz, w + 2 * F::WORDS);
  elem_from_words32<F>(p.zzz, w + 3 * F::WORDS);
  return p;
}
template <class F>
Aff<F> aff_from_words32(const uint32_t* w) {
  Aff<F> a;
  elem_from_words32<F>(a.x, w);
  elem_from_words32<F>(a.y, w + F::WORDS);
  a.inf = F::is_zero(a.x) && F::is_zero(a.y);
  return a;
}
template <class F>
void aff_to_words32(uint32_t* w, const Aff<F>& a) {
  if (a.inf) {
    memset(w, 0, sizeof(uint32_t) * 2 * F::WORDS);
    return;
  }
  elem_to_words32<F>(w, a.x);
  elem_to_words32<F>(w + F::WORDS, a.y);
}

}  // namespace bgh
