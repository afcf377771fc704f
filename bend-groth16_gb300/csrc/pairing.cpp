// Optimal ate pairing over BN254 and the Groth16 verification equation, on the host.
//
// Reference semantics: the arkworks verifier the reference's harness calls
// (ref/src/verify.rs:8-27; ark-groth16 0.5.0 verify_proof over ark-bn254 0.5.0, not vendored
// in the reference): e(A, B) = e(alpha, beta) e(vk_x, gamma) e(C, delta) with
// vk_x = IC_0 + sum_i x_i IC_i.  This file restates the published algorithm (Vercauteren's
// optimal ate pairing for BN curves: a Miller loop over 6u + 2, two lines through Frobenius
// images of Q, and the final exponentiation by (p^12 - 1) / r), written for clarity rather than
// speed: affine Miller-loop steps with one Fq2 inversion each, and the final exponentiation by
// plain square-and-multiply over exact big-integer exponents.  It verifies a proof in a few
// milliseconds; it is a self-check for proofs and keys, not part of proving.
//
// Tower: Fq2 = Fq[u]/(u^2 + 1), Fq6 = Fq2[v]/(v^3 - xi), Fq12 = Fq6[w]/(w^2 - v), xi = 9 + u.
// G2 lives on the sextic twist y^2 = x^3 + 3/xi over Fq2; psi(x, y) = (x w^2, y w^3) maps it
// into E(Fq12).  Every derived constant is computed at first use from p, r and the BN
// parameter u, and u is checked against p = 36u^4 + 36u^3 + 24u^2 + 6u + 1 and
// r = 36u^4 + 36u^3 + 18u^2 + 6u + 1.
#include "pairing.hpp"

#include <algorithm>
#include <stdexcept>
#include <string>
#include <vector>

#include "host_ff.hpp"

namespace bgh {
namespace {

// ---------------------------------------------------------------- big unsigned integers
typedef std::vector<uint64_t> Big;  // little-endian 64-bit limbs

void big_trim(Big& a) {
  while (!a.empty() && a.back() == 0) a.pop_back();
}
Big big_from(const uint64_t* v, int n) {
  Big a(v, v + n);
  big_trim(a);
  return a;
}
Big big_small(uint64_t x) { return big_from(&x, 1); }
Big big_add(const Big& a, const Big& b) {
  Big r(std::max(a.size(), b.size()) + 1, 0);
  u128 c = 0;
  for (size_t i = 0; i < r.size(); i++) {
    c += (u128)(i < a.size() ? a[i] : 0) + (i < b.size() ? b[i] : 0);
    r[i] = (uint64_t)c;
    c >>= 64;
  }
  big_trim(r);
  return r;
}
int big_cmp(const Big& a, const Big& b) {
  if (a.size() != b.size()) return a.size() < b.size() ? -1 : 1;
  for (size_t i = a.size(); i-- > 0;)
    if (a[i] != b[i]) return a[i] < b[i] ? -1 : 1;
  return 0;
}
Big big_sub(const Big& a, const Big& b) {  // a >= b
  Big r(a.size(), 0);
  uint64_t br = 0;
  for (size_t i = 0; i < a.size(); i++) {
    const u128 d = (u128)a[i] - (i < b.size() ? b[i] : 0) - br;
    r[i] = (uint64_t)d;
    br = (uint64_t)(d >> 64) & 1;
  }
  big_trim(r);
  return r;
}
Big big_mul(const Big& a, const Big& b) {
  Big r(a.size() + b.size() + 1, 0);
  for (size_t i = 0; i < a.size(); i++) {
    u128 c = 0;
    for (size_t j = 0; j < b.size(); j++) {
      c += (u128)a[i] * b[j] + r[i + j];
      r[i + j] = (uint64_t)c;
      c >>= 64;
    }
    for (size_t k = i + b.size(); c; k++) {
      c += r[k];
      r[k] = (uint64_t)c;
      c >>= 64;
    }
  }
  big_trim(r);
  return r;
}
size_t big_bits(const Big& a) {
  if (a.empty()) return 0;
  size_t n = 64 * (a.size() - 1);
  for (uint64_t t = a.back(); t; t >>= 1) n++;
  return n;
}
bool big_bit(const Big& a, size_t i) { return i / 64 < a.size() && ((a[i / 64] >> (i % 64)) & 1); }
// quotient and remainder by bit-serial long division
void big_divmod(const Big& a, const Big& d, Big& q, Big& rem) {
  q.assign(a.size(), 0);
  rem.clear();
  for (size_t i = big_bits(a); i-- > 0;) {
    rem = big_add(rem, rem);
    if (big_bit(a, i)) rem = big_add(rem, big_small(1));
    if (big_cmp(rem, d) >= 0) {
      rem = big_sub(rem, d);
      q[i / 64] |= 1ull << (i % 64);
    }
  }
  big_trim(q);
}

// ---------------------------------------------------------------- Fq, Fq2 helpers
typedef Fq2Ops F2;
Fe fq_small(uint64_t x) { return fe_to_mont(FQ, fe_raw(x)); }
Fe2 f2(const Fe& a, const Fe& b) { return Fe2{a, b}; }
Fe2 f2_conj(const Fe2& a) { return {a.c0, fe_neg(FQ, a.c1)}; }
Fe2 f2_scale(const Fe2& a, const Fe& k) { return {fe_mul(FQ, a.c0, k), fe_mul(FQ, a.c1, k)}; }
Fe2 f2_pow(const Fe2& a, const Big& e) {
  Fe2 r = F2::one();
  for (size_t i = big_bits(e); i-- > 0;) {
    r = F2::sqr(r);
    if (big_bit(e, i)) r = F2::mul(r, a);
  }
  return r;
}

// ---------------------------------------------------------------- Fq6, Fq12
struct Fe6 {
  Fe2 c0, c1, c2;
};
struct Fe12 {
  Fe6 g, h;  // g + h w
};

struct Consts {
  Fe2 xi;             // 9 + u
  Fe2 twist_b;        // 3 / xi
  Fe g1_b;            // 3
  Fe2 frob_x, frob_y;  // xi^((p-1)/3), xi^((p-1)/2)
  Fe frob2_x, frob2_y;  // their norms: xi^((p^2-1)/3), xi^((p^2-1)/2)
  Big ate;            // 6u + 2
  Big exp_easy2;      // p^2 + 1
  Big exp_hard;       // (p^4 - p^2 + 1) / r
  uint64_t r[4];
  Consts() {
    const uint64_t u = 4965661367192848881ull;  // BN254 curve parameter
    const Big U = big_small(u), P = big_from(FQ.p, 4), R = big_from(FR.p, 4);
    const Big u2 = big_mul(U, U), u3 = big_mul(u2, U), u4 = big_mul(u3, U);
    auto k = [](uint64_t c, const Big& x) { return big_mul(big_small(c), x); };
    const Big base = big_add(big_add(k(36, u4), k(36, u3)), big_add(k(6, U), big_small(1)));
    if (big_cmp(big_add(base, k(24, u2)), P) != 0 || big_cmp(big_add(base, k(18, u2)), R) != 0)
      throw std::logic_error("pairing: BN parameter does not reproduce p and r");
    ate = big_add(k(6, U), big_small(2));
    xi = f2(fq_small(9), fq_small(1));
    twist_b = F2::mul(f2(fq_small(3), fe_zero()), F2::inv(xi));
    g1_b = fq_small(3);
    Big q, rem;
    const Big pm1 = big_sub(P, big_small(1));
    big_divmod(pm1, big_small(3), q, rem);
    if (!rem.empty()) throw std::logic_error("pairing: p - 1 not divisible by 3");
    frob_x = f2_pow(xi, q);
    big_divmod(pm1, big_small(2), q, rem);
    frob_y = f2_pow(xi, q);
    // y^((p^2-1)/k) = (y^((p-1)/k))^(p+1) = y' * conj(y') for y' in Fq2
    frob2_x = F2::mul(frob_x, f2_conj(frob_x)).c0;
    frob2_y = F2::mul(frob_y, f2_conj(frob_y)).c0;
    const Big p2 = big_mul(P, P);
    exp_easy2 = big_add(p2, big_small(1));
    const Big num = big_add(big_sub(big_mul(p2, p2), p2), big_small(1));
    big_divmod(num, R, exp_hard, rem);
    if (!rem.empty()) throw std::logic_error("pairing: r does not divide p^4 - p^2 + 1");
    for (int i = 0; i < 4; i++) r[i] = FR.p[i];
  }
};
const Consts& C() {
  static const Consts c;
  return c;
}

Fe2 mul_xi(const Fe2& a) { return F2::mul(a, C().xi); }
Fe6 f6_zero() { return {F2::zero(), F2::zero(), F2::zero()}; }
Fe6 f6_one() { return {F2::one(), F2::zero(), F2::zero()}; }
Fe6 f6_add(const Fe6& a, const Fe6& b) { return {F2::add(a.c0, b.c0), F2::add(a.c1, b.c1), F2::add(a.c2, b.c2)}; }
Fe6 f6_sub(const Fe6& a, const Fe6& b) { return {F2::sub(a.c0, b.c0), F2::sub(a.c1, b.c1), F2::sub(a.c2, b.c2)}; }
Fe6 f6_neg(const Fe6& a) { return {F2::neg(a.c0), F2::neg(a.c1), F2::neg(a.c2)}; }
Fe6 f6_mul(const Fe6& a, const Fe6& b) {
  // v^3 = xi
  const Fe2 a0b0 = F2::mul(a.c0, b.c0), a1b1 = F2::mul(a.c1, b.c1), a2b2 = F2::mul(a.c2, b.c2);
  const Fe2 c0 = F2::add(a0b0, mul_xi(F2::add(F2::mul(a.c1, b.c2), F2::mul(a.c2, b.c1))));
  const Fe2 c1 = F2::add(F2::add(F2::mul(a.c0, b.c1), F2::mul(a.c1, b.c0)), mul_xi(a2b2));
  const Fe2 c2 = F2::add(F2::add(F2::mul(a.c0, b.c2), a1b1), F2::mul(a.c2, b.c0));
  return {c0, c1, c2};
}
Fe6 f6_mul_v(const Fe6& a) { return {mul_xi(a.c2), a.c0, a.c1}; }
Fe6 f6_inv(const Fe6& a) {
  const Fe2 t0 = F2::sub(F2::sqr(a.c0), mul_xi(F2::mul(a.c1, a.c2)));
  const Fe2 t1 = F2::sub(mul_xi(F2::sqr(a.c2)), F2::mul(a.c0, a.c1));
  const Fe2 t2 = F2::sub(F2::sqr(a.c1), F2::mul(a.c0, a.c2));
  const Fe2 det = F2::add(F2::mul(a.c0, t0), mul_xi(F2::add(F2::mul(a.c2, t1), F2::mul(a.c1, t2))));
  const Fe2 di = F2::inv(det);
  return {F2::mul(t0, di), F2::mul(t1, di), F2::mul(t2, di)};
}
bool f6_eq(const Fe6& a, const Fe6& b) { return F2::eq(a.c0, b.c0) && F2::eq(a.c1, b.c1) && F2::eq(a.c2, b.c2); }

Fe12 f12_one() { return {f6_one(), f6_zero()}; }
Fe12 f12_mul(const Fe12& a, const Fe12& b) {
  // (g1 + h1 w)(g2 + h2 w) = g1 g2 + h1 h2 v + (g1 h2 + h1 g2) w
  const Fe6 gg = f6_mul(a.g, b.g), hh = f6_mul(a.h, b.h);
  const Fe6 cross = f6_sub(f6_sub(f6_mul(f6_add(a.g, a.h), f6_add(b.g, b.h)), gg), hh);
  return {f6_add(gg, f6_mul_v(hh)), cross};
}
Fe12 f12_conj(const Fe12& a) { return {a.g, f6_neg(a.h)}; }  // a^(p^6)
Fe12 f12_inv(const Fe12& a) {
  const Fe6 d = f6_inv(f6_sub(f6_mul(a.g, a.g), f6_mul_v(f6_mul(a.h, a.h))));
  return {f6_mul(a.g, d), f6_neg(f6_mul(a.h, d))};
}
Fe12 f12_pow(const Fe12& a, const Big& e) {
  Fe12 r = f12_one();
  for (size_t i = big_bits(e); i-- > 0;) {
    r = f12_mul(r, r);
    if (big_bit(e, i)) r = f12_mul(r, a);
  }
  return r;
}
bool f12_is_one(const Fe12& a) { return f6_eq(a.g, f6_one()) && f6_eq(a.h, f6_zero()); }

// ---------------------------------------------------------------- Miller loop
struct G1A {
  Fe x, y;
  bool inf;
};
struct G2A {
  Fe2 x, y;
  bool inf;
};

// line through T with slope lambda, evaluated at psi^-1-side point P:
// y_P - lambda x_P w + (lambda x_T - y_T) w^3
Fe12 line(const Fe2& lambda, const G2A& t, const G1A& p) {
  Fe12 l = {f6_zero(), f6_zero()};
  l.g.c0 = f2(p.y, fe_zero());
  l.h.c0 = F2::neg(f2_scale(lambda, p.x));
  l.h.c1 = F2::sub(F2::mul(lambda, t.x), t.y);
  return l;
}
// T <- T + Q (T != +-Q), multiplying f by the line through T and Q
void add_step(Fe12& f, G2A& t, const G2A& q, const G1A& p) {
  const Fe2 lambda = F2::mul(F2::sub(q.y, t.y), F2::inv(F2::sub(q.x, t.x)));
  f = f12_mul(f, line(lambda, t, p));
  const Fe2 x3 = F2::sub(F2::sub(F2::sqr(lambda), t.x), q.x);
  t.y = F2::sub(F2::mul(lambda, F2::sub(t.x, x3)), t.y);
  t.x = x3;
}
void dbl_step(Fe12& f, G2A& t, const G1A& p) {
  const Fe2 x2 = F2::sqr(t.x);
  const Fe2 lambda = F2::mul(F2::add(F2::add(x2, x2), x2), F2::inv(F2::add(t.y, t.y)));
  f = f12_mul(f12_mul(f, f), line(lambda, t, p));
  const Fe2 x3 = F2::sub(F2::sqr(lambda), F2::add(t.x, t.x));
  t.y = F2::sub(F2::mul(lambda, F2::sub(t.x, x3)), t.y);
  t.x = x3;
}
Fe12 miller(const G1A& p, const G2A& q) {
  if (p.inf || q.inf) return f12_one();
  const Consts& k = C();
  Fe12 f = f12_one();
  G2A t = q;
  for (size_t i = big_bits(k.ate) - 1; i-- > 0;) {
    dbl_step(f, t, p);
    if (big_bit(k.ate, i)) add_step(f, t, q, p);
  }
  // Frobenius images on the twist: pi(Q) and -pi^2(Q)
  const G2A q1 = {F2::mul(f2_conj(q.x), k.frob_x), F2::mul(f2_conj(q.y), k.frob_y), false};
  const G2A q2n = {f2_scale(q.x, k.frob2_x), F2::neg(f2_scale(q.y, k.frob2_y)), false};
  add_step(f, t, q1, p);
  const Fe2 lambda = F2::mul(F2::sub(q2n.y, t.y), F2::inv(F2::sub(q2n.x, t.x)));
  return f12_mul(f, line(lambda, t, p));
}
Fe12 final_exp(const Fe12& f) {
  const Consts& k = C();
  Fe12 r = f12_mul(f12_conj(f), f12_inv(f));  // f^(p^6 - 1)
  r = f12_pow(r, k.exp_easy2);                 // ^(p^2 + 1)
  return f12_pow(r, k.exp_hard);               // ^((p^4 - p^2 + 1) / r)
}

// ---------------------------------------------------------------- points from the wire
G1A g1_from_wire(const uint32_t* w) {
  G1A a{fe_from_words16(w), fe_from_words16(w + 16), false};
  a.inf = fe_is_zero(a.x) && fe_is_zero(a.y);
  return a;
}
G2A g2_from_wire(const uint32_t* w) {
  G2A a{{fe_from_words16(w), fe_from_words16(w + 16)}, {fe_from_words16(w + 32), fe_from_words16(w + 48)}, false};
  a.inf = F2::is_zero(a.x) && F2::is_zero(a.y);
  return a;
}
bool limbs_ok(const uint32_t* w, size_t words) {
  for (size_t i = 0; i < words; i++)
    if (w[i] >> 16) return false;
  return true;
}
bool below(const Fe& a, const Mod& m) { return !geq(a.v, m.p); }
bool g1_valid(const G1A& a) {
  if (a.inf) return true;
  if (!below(a.x, FQ) || !below(a.y, FQ)) return false;
  const Fe rhs = fe_add(FQ, fe_mul(FQ, fe_sqr(FQ, a.x), a.x), C().g1_b);
  return fe_eq(fe_sqr(FQ, a.y), rhs);  // cofactor 1: on the curve = in G1
}
bool g2_valid(const G2A& a) {
  if (a.inf) return true;
  if (!below(a.x.c0, FQ) || !below(a.x.c1, FQ) || !below(a.y.c0, FQ) || !below(a.y.c1, FQ)) return false;
  const Fe2 rhs = F2::add(F2::mul(F2::sqr(a.x), a.x), C().twist_b);
  if (!F2::eq(F2::sqr(a.y), rhs)) return false;
  const Aff<Fq2Ops> aff{a.x, a.y, false};
  return xyzz_is_inf(xyzz_mul(xyzz_from(aff), C().r));  // order r
}
G1A g1_neg(const G1A& a) { return {a.x, fe_neg(FQ, a.y), a.inf}; }

}  // namespace

int groth16_verify(const VkWire& vk, const uint32_t* public16, size_t n_public, const uint32_t* a32,
                   const uint32_t* b64, const uint32_t* c32) {
  if (!vk.alpha_g1 || !vk.beta_g2 || !vk.gamma_g2 || !vk.delta_g2 || !vk.gamma_abc_g1 || !a32 || !b64 || !c32)
    throw std::invalid_argument("bg_verify: null pointer");
  if (vk.n_ic == 0 || n_public + 1 != vk.n_ic)
    throw std::invalid_argument("bg_verify: " + std::to_string(n_public) + " public inputs for a key with " +
                                std::to_string(vk.n_ic) + " IC points");
  if (n_public && !public16) throw std::invalid_argument("bg_verify: null public inputs");
  if (!limbs_ok(vk.alpha_g1, 32) || !limbs_ok(vk.beta_g2, 64) || !limbs_ok(vk.gamma_g2, 64) ||
      !limbs_ok(vk.delta_g2, 64) || !limbs_ok(vk.gamma_abc_g1, 32 * vk.n_ic) || !limbs_ok(a32, 32) ||
      !limbs_ok(b64, 64) || !limbs_ok(c32, 32) || (n_public && !limbs_ok(public16, 16 * n_public)))
    throw MalformedInput("bg_verify: a wire word has bits above its 16-bit limb");
  const G1A alpha = g1_from_wire(vk.alpha_g1), A = g1_from_wire(a32), Cp = g1_from_wire(c32);
  const G2A beta = g2_from_wire(vk.beta_g2), gamma = g2_from_wire(vk.gamma_g2), delta = g2_from_wire(vk.delta_g2);
  const G2A B = g2_from_wire(b64);
  if (!g1_valid(alpha) || !g1_valid(A) || !g1_valid(Cp) || !g2_valid(beta) || !g2_valid(gamma) ||
      !g2_valid(delta) || !g2_valid(B))
    throw MalformedInput("bg_verify: a proof or key point is off its curve or outside the order-r subgroup");
  // vk_x = IC_0 + sum_i x_i IC_{i+1}
  Xyzz<FqOps> acc = xyzz_inf<FqOps>();
  for (size_t i = 0; i < vk.n_ic; i++) {
    const G1A ic = g1_from_wire(vk.gamma_abc_g1 + 32 * i);
    if (!g1_valid(ic)) throw MalformedInput("bg_verify: an IC point is off the curve");
    const Aff<FqOps> p{ic.x, ic.y, ic.inf};
    if (i == 0) {
      acc = xyzz_add(acc, xyzz_from(p));
      continue;
    }
    const Fe xm = fe_from_words16(public16 + 16 * (i - 1));
    if (!below(xm, FR)) throw MalformedInput("bg_verify: a public input is not below r");
    const Fe x = fe_from_mont(FR, xm);
    acc = xyzz_add(acc, xyzz_mul(xyzz_from(p), x.v));
  }
  const Aff<FqOps> vx = xyzz_to_affine(acc);
  const G1A vkx{vx.x, vx.y, vx.inf};
  // e(A, B) e(-alpha, beta) e(-vk_x, gamma) e(-C, delta) = 1
  Fe12 f = miller(A, B);
  f = f12_mul(f, miller(g1_neg(alpha), beta));
  f = f12_mul(f, miller(g1_neg(vkx), gamma));
  f = f12_mul(f, miller(g1_neg(Cp), delta));
  return f12_is_one(final_exp(f)) ? 1 : 0;
}

void pairing_wire(const uint32_t* p32, const uint32_t* q64, uint32_t* out192) {
  const G1A p = g1_from_wire(p32);
  const G2A q = g2_from_wire(q64);
  if (!g1_valid(p) || !g2_valid(q)) throw std::invalid_argument("bg_pairing: point not in G1 / G2");
  const Fe12 e = final_exp(miller(p, q));
  const Fe2* parts[6] = {&e.g.c0, &e.g.c1, &e.g.c2, &e.h.c0, &e.h.c1, &e.h.c2};
  for (int i = 0; i < 6; i++) {
    fe_to_words16(out192 + 32 * i, parts[i]->c0);
    fe_to_words16(out192 + 32 * i + 16, parts[i]->c1);
  }
}

}  // namespace bgh
