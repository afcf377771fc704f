/* CPU oracle in C (test infrastructure and the timed CPU baseline; never linked into the
 * product).  A restatement of the reference prover's algorithms over 4 x 64-bit Montgomery
 * limbs, multithreaded with pthreads:
 *   field      CIOS Montgomery product, R = 2^256 (bend2/gen/gen_field.py:105-135)
 *   Fq2        Karatsuba / complex square / norm inverse (bend2/src/fq2.bend:31-50)
 *   curves     Jacobian dbl-2009-l, add-2007-bl, madd-2007-bl with the special cases of
 *              bend2/src/g1.bend:76-172 (same formulas for G2 over Fq2, bend2/src/g2.bend)
 *   MSM        unsigned c-bit windows, per-window buckets, running-sum reduction and a
 *              Horner window combine (bend2/src/msm.bend:34-58, :133-239); windows are
 *              spread over threads
 *   NTT        radix-2 DIT with a bit-reversal, arkworks domain w = root^(2^(28-L))
 *              (bend2/gen/ref_qap.py:27-65, bend2/src/ntt.bend:73-74)
 *   qap_h      LibsnarkReduction quotient (bend2/gen/ref_qap.py:68-72)
 *   prove      evals (bend2/src/groth16.bend:162-188), the five MSMs and the combine
 *              (bend2/src/groth16.bend:298-308) from a bend2/FORMAT.md directory.
 * Plain C11, no architecture-specific code: it builds and gives identical results on x86-64
 * and aarch64. */
#include <pthread.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

typedef unsigned __int128 u128;
typedef struct { uint64_t v[4]; } fe;
typedef struct { uint64_t p[4], n0, one[4], r2[4]; } modulus;

static const modulus FQ = {{0x3c208c16d87cfd47ull, 0x97816a916871ca8dull, 0xb85045b68181585dull, 0x30644e72e131a029ull},
                           0x87d20782e4866389ull,
                           {0xd35d438dc58f0d9dull, 0x0a78eb28f5c70b3dull, 0x666ea36f7879462cull, 0x0e0a77c19a07df2full},
                           {0xf32cfc5b538afa89ull, 0xb5e71911d44501fbull, 0x47ab1eff0a417ff6ull, 0x06d89f71cab8351full}};
static const modulus FR = {{0x43e1f593f0000001ull, 0x2833e84879b97091ull, 0xb85045b68181585dull, 0x30644e72e131a029ull},
                           0xc2e1f593efffffffull,
                           {0xac96341c4ffffffbull, 0x36fc76959f60cd29ull, 0x666ea36f7879462eull, 0x0e0a77c19a07df2full},
                           {0x1bb8e645ae216da7ull, 0x53fe3ab1e35c59e3ull, 0x8c49833d53bb8085ull, 0x0216d0b17f4e44a5ull}};

/* ------------------------------------------------------------------ field */
static int geq4(const uint64_t *a, const uint64_t *b) {
  for (int i = 3; i >= 0; i--)
    if (a[i] != b[i]) return a[i] > b[i];
  return 1;
}
static uint64_t sub4(uint64_t *r, const uint64_t *a, const uint64_t *b) {
  uint64_t br = 0;
  for (int i = 0; i < 4; i++) {
    u128 d = (u128)a[i] - b[i] - br;
    r[i] = (uint64_t)d;
    br = (uint64_t)(d >> 64) & 1;
  }
  return br;
}
static void add4(uint64_t *r, const uint64_t *a, const uint64_t *b) {
  uint64_t c = 0;
  for (int i = 0; i < 4; i++) {
    u128 s = (u128)a[i] + b[i] + c;
    r[i] = (uint64_t)s;
    c = (uint64_t)(s >> 64);
  }
}
static inline fe f_add(const modulus *m, fe a, fe b) {
  fe r;
  add4(r.v, a.v, b.v);
  if (geq4(r.v, m->p)) sub4(r.v, r.v, m->p);
  return r;
}
static inline fe f_sub(const modulus *m, fe a, fe b) {
  fe r;
  if (sub4(r.v, a.v, b.v)) add4(r.v, r.v, m->p);
  return r;
}
static inline fe f_mul(const modulus *m, fe a, fe b) {
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
    uint64_t q = t[0] * m->n0;
    s = (u128)q * m->p[0] + t[0];
    c = (uint64_t)(s >> 64);
    for (int j = 1; j < 4; j++) {
      s = (u128)q * m->p[j] + t[j] + c;
      t[j - 1] = (uint64_t)s;
      c = (uint64_t)(s >> 64);
    }
    s = (u128)t[4] + c;
    t[3] = (uint64_t)s;
    t[4] = t[5] + (uint64_t)(s >> 64);
  }
  fe r = {{t[0], t[1], t[2], t[3]}};
  if (t[4] || geq4(r.v, m->p)) sub4(r.v, r.v, m->p);
  return r;
}
static inline int f_is_zero(fe a) { return (a.v[0] | a.v[1] | a.v[2] | a.v[3]) == 0; }
static inline int f_eq(fe a, fe b) { return !memcmp(&a, &b, sizeof a); }
static inline fe f_zero(void) { fe r = {{0, 0, 0, 0}}; return r; }
static inline fe f_one(const modulus *m) { fe r; memcpy(r.v, m->one, 32); return r; }
static fe f_pow(const modulus *m, fe a, const uint64_t *e) {
  fe r = f_one(m);
  for (int i = 3; i >= 0; i--)
    for (int b = 63; b >= 0; b--) {
      r = f_mul(m, r, r);
      if ((e[i] >> b) & 1) r = f_mul(m, r, a);
    }
  return r;
}
static fe f_inv(const modulus *m, fe a) {
  uint64_t e[4] = {m->p[0] - 2, m->p[1], m->p[2], m->p[3]};
  return f_pow(m, a, e);
}
static fe f_to_mont(const modulus *m, fe a) { fe r2; memcpy(r2.v, m->r2, 32); return f_mul(m, a, r2); }
static fe f_from_mont(const modulus *m, fe a) { fe one = {{1, 0, 0, 0}}; return f_mul(m, a, one); }

/* FORMAT.md element: 16 u32 words, each a 16-bit limb */
static fe fe_read16(const uint32_t *w) {
  fe r;
  for (int i = 0; i < 4; i++)
    r.v[i] = (uint64_t)(w[4 * i] & 0xffff) | ((uint64_t)(w[4 * i + 1] & 0xffff) << 16) |
             ((uint64_t)(w[4 * i + 2] & 0xffff) << 32) | ((uint64_t)(w[4 * i + 3] & 0xffff) << 48);
  return r;
}
static void fe_write16(uint32_t *w, fe a) {
  for (int i = 0; i < 16; i++) w[i] = (uint32_t)(a.v[i / 4] >> (16 * (i % 4))) & 0xffffu;
}

/* ------------------------------------------------------------------ Fq2 */
typedef struct { fe c0, c1; } fe2;
static inline fe2 f2_add(fe2 a, fe2 b) { fe2 r = {f_add(&FQ, a.c0, b.c0), f_add(&FQ, a.c1, b.c1)}; return r; }
static inline fe2 f2_sub(fe2 a, fe2 b) { fe2 r = {f_sub(&FQ, a.c0, b.c0), f_sub(&FQ, a.c1, b.c1)}; return r; }
static inline fe2 f2_mul(fe2 a, fe2 b) {
  fe t0 = f_mul(&FQ, a.c0, b.c0), t1 = f_mul(&FQ, a.c1, b.c1);
  fe t2 = f_mul(&FQ, f_add(&FQ, a.c0, a.c1), f_add(&FQ, b.c0, b.c1));
  fe2 r = {f_sub(&FQ, t0, t1), f_sub(&FQ, f_sub(&FQ, t2, t0), t1)};
  return r;
}
static inline fe2 f2_sqr(fe2 a) {
  fe2 r = {f_mul(&FQ, f_add(&FQ, a.c0, a.c1), f_sub(&FQ, a.c0, a.c1)), f_mul(&FQ, f_add(&FQ, a.c0, a.c0), a.c1)};
  return r;
}
static inline int f2_is_zero(fe2 a) { return f_is_zero(a.c0) && f_is_zero(a.c1); }
static fe2 f2_inv(fe2 a) {
  fe ni = f_inv(&FQ, f_add(&FQ, f_mul(&FQ, a.c0, a.c0), f_mul(&FQ, a.c1, a.c1)));
  fe2 r = {f_mul(&FQ, a.c0, ni), f_sub(&FQ, f_zero(), f_mul(&FQ, a.c1, ni))};
  return r;
}

/* ------------------------------------------------------------------ curves (Jacobian)
 * The same code is instantiated for G1 (Fq) and G2 (Fq2) through macros. */
#define DEFINE_CURVE(P, F, ADD, SUB, MUL, SQR, ISZ, INV, ZERO, ONE)                                \
  typedef struct { F x, y, z; } P##_jac;                                                            \
  typedef struct { F x, y; int inf; } P##_aff;                                                      \
  static inline P##_jac P##_inf(void) { P##_jac r = {ZERO, ONE, ZERO}; return r; }                 \
  static inline int P##_is_inf(const P##_jac *p) { return ISZ(p->z); }                             \
  /* dbl-2009-l */                                                                                  \
  static P##_jac P##_dbl(P##_jac p) {                                                              \
    if (ISZ(p.z)) return p;                                                                         \
    F a = SQR(p.x), b = SQR(p.y), c = SQR(b);                                                       \
    F t = SQR(ADD(p.x, b));                                                                         \
    F d = SUB(SUB(t, a), c);                                                                        \
    d = ADD(d, d);                                                                                  \
    F e = ADD(ADD(a, a), a), f = SQR(e);                                                            \
    P##_jac r;                                                                                      \
    r.x = SUB(f, ADD(d, d));                                                                        \
    F c8 = ADD(c, c); c8 = ADD(c8, c8); c8 = ADD(c8, c8);                                           \
    r.y = SUB(MUL(e, SUB(d, r.x)), c8);                                                             \
    F yz = MUL(p.y, p.z);                                                                           \
    r.z = ADD(yz, yz);                                                                              \
    return r;                                                                                       \
  }                                                                                                 \
  /* add-2007-bl with the special cases resolved first */                                           \
  static P##_jac P##_add(P##_jac p, P##_jac q) {                                                   \
    if (ISZ(p.z)) return q;                                                                         \
    if (ISZ(q.z)) return p;                                                                         \
    F z1z1 = SQR(p.z), z2z2 = SQR(q.z);                                                             \
    F u1 = MUL(p.x, z2z2), u2 = MUL(q.x, z1z1);                                                     \
    F s1 = MUL(MUL(p.y, q.z), z2z2), s2 = MUL(MUL(q.y, p.z), z1z1);                                 \
    F h = SUB(u2, u1), rr = SUB(s2, s1);                                                            \
    if (ISZ(h)) { if (ISZ(rr)) return P##_dbl(p); return P##_inf(); }                               \
    F i = SQR(ADD(h, h)), j = MUL(h, i);                                                            \
    F r2 = ADD(rr, rr), v = MUL(u1, i);                                                             \
    P##_jac o;                                                                                      \
    o.x = SUB(SUB(SQR(r2), j), ADD(v, v));                                                          \
    F s1j = MUL(s1, j);                                                                             \
    o.y = SUB(MUL(r2, SUB(v, o.x)), ADD(s1j, s1j));                                                 \
    o.z = MUL(SUB(SUB(SQR(ADD(p.z, q.z)), z1z1), z2z2), h);                                         \
    return o;                                                                                       \
  }                                                                                                 \
  /* madd-2007-bl */                                                                                \
  static P##_jac P##_madd(P##_jac p, const P##_aff *q) {                                           \
    if (q->inf) return p;                                                                           \
    if (ISZ(p.z)) { P##_jac r = {q->x, q->y, ONE}; return r; }                                      \
    F z1z1 = SQR(p.z);                                                                              \
    F u2 = MUL(q->x, z1z1), s2 = MUL(MUL(q->y, p.z), z1z1);                                         \
    F h = SUB(u2, p.x), rr0 = SUB(s2, p.y);                                                         \
    if (ISZ(h)) {                                                                                   \
      if (ISZ(rr0)) { P##_jac t = {q->x, q->y, ONE}; return P##_dbl(t); }                           \
      return P##_inf();                                                                             \
    }                                                                                               \
    F hh = SQR(h), i = ADD(hh, hh); i = ADD(i, i);                                                  \
    F j = MUL(h, i), rr = ADD(rr0, rr0), v = MUL(p.x, i);                                           \
    P##_jac o;                                                                                      \
    o.x = SUB(SUB(SQR(rr), j), ADD(v, v));                                                          \
    F y1j = MUL(p.y, j);                                                                            \
    o.y = SUB(MUL(rr, SUB(v, o.x)), ADD(y1j, y1j));                                                 \
    o.z = SUB(SUB(SQR(ADD(p.z, h)), z1z1), hh);                                                     \
    return o;                                                                                       \
  }                                                                                                 \
  static P##_aff P##_to_aff(P##_jac p) {                                                           \
    P##_aff a;                                                                                      \
    if (ISZ(p.z)) { a.x = ZERO; a.y = ZERO; a.inf = 1; return a; }                                  \
    F zi = INV(p.z), zi2 = SQR(zi);                                                                 \
    a.x = MUL(p.x, zi2); a.y = MUL(p.y, MUL(zi, zi2)); a.inf = 0;                                   \
    return a;                                                                                       \
  }                                                                                                 \
  static P##_jac P##_from_aff(const P##_aff *a) {                                                  \
    if (a->inf) return P##_inf();                                                                   \
    P##_jac r = {a->x, a->y, ONE};                                                                  \
    return r;                                                                                       \
  }                                                                                                 \
  /* double-and-add over 256 bits of a canonical scalar (bend2/src/g1.bend:175-191) */              \
  static P##_jac P##_mul(P##_jac p, fe k) {                                                        \
    P##_jac acc = P##_inf();                                                                        \
    for (int i = 255; i >= 0; i--) {                                                                \
      acc = P##_dbl(acc);                                                                           \
      if ((k.v[i / 64] >> (i % 64)) & 1) acc = P##_add(acc, p);                                     \
    }                                                                                               \
    return acc;                                                                                     \
  }

#define Q_ADD(a, b) f_add(&FQ, a, b)
#define Q_SUB(a, b) f_sub(&FQ, a, b)
#define Q_MUL(a, b) f_mul(&FQ, a, b)
#define Q_SQR(a) f_mul(&FQ, a, a)
#define Q_INV(a) f_inv(&FQ, a)
static inline fe q_zero(void) { return f_zero(); }
static inline fe q_one(void) { return f_one(&FQ); }
DEFINE_CURVE(g1, fe, Q_ADD, Q_SUB, Q_MUL, Q_SQR, f_is_zero, Q_INV, q_zero(), q_one())

static inline fe2 q2_zero(void) { fe2 r = {f_zero(), f_zero()}; return r; }
static inline fe2 q2_one(void) { fe2 r = {f_one(&FQ), f_zero()}; return r; }
DEFINE_CURVE(g2, fe2, f2_add, f2_sub, f2_mul, f2_sqr, f2_is_zero, f2_inv, q2_zero(), q2_one())

static g1_aff g1_read16(const uint32_t *w) {
  g1_aff a;
  a.x = fe_read16(w);
  a.y = fe_read16(w + 16);
  a.inf = f_is_zero(a.x) && f_is_zero(a.y);
  return a;
}
static g2_aff g2_read16(const uint32_t *w) {
  g2_aff a;
  a.x.c0 = fe_read16(w);
  a.x.c1 = fe_read16(w + 16);
  a.y.c0 = fe_read16(w + 32);
  a.y.c1 = fe_read16(w + 48);
  a.inf = f2_is_zero(a.x) && f2_is_zero(a.y);
  return a;
}
static void g1_write16(uint32_t *w, const g1_aff *a) {
  fe_write16(w, a->x);
  fe_write16(w + 16, a->y);
}
static void g2_write16(uint32_t *w, const g2_aff *a) {
  fe_write16(w, a->x.c0);
  fe_write16(w + 16, a->x.c1);
  fe_write16(w + 32, a->y.c0);
  fe_write16(w + 48, a->y.c1);
}

/* ------------------------------------------------------------------ MSM (Pippenger) */
static int pick_c(size_t n) {
  int lg = 0;
  while (((size_t)1 << (lg + 1)) <= n) lg++;
  int c = lg - 4;
  if (c < 4) c = 4;
  if (c > 16) c = 16;
  return c;
}
static inline uint32_t digit(const fe *k, int bit, int c) {
  int limb = bit / 64, sh = bit % 64;
  if (limb >= 4) return 0;
  uint64_t v = k->v[limb] >> sh;
  if (sh > 64 - c && limb + 1 < 4) v |= k->v[limb + 1] << (64 - sh);
  return (uint32_t)(v & ((1ull << c) - 1));
}

#define DEFINE_MSM(P)                                                                               \
  typedef struct {                                                                                  \
    const P##_aff *pts; const fe *sc; size_t n; int c, W, next, nthreads;                           \
    P##_jac *win; pthread_mutex_t mu;                                                               \
  } P##_msm_job;                                                                                    \
  static void *P##_msm_worker(void *arg) {                                                         \
    P##_msm_job *j = (P##_msm_job *)arg;                                                            \
    const uint32_t nb = 1u << j->c;                                                                 \
    P##_jac *b = (P##_jac *)malloc(sizeof(P##_jac) * nb);                                           \
    for (;;) {                                                                                      \
      pthread_mutex_lock(&j->mu);                                                                   \
      int w = j->next++;                                                                            \
      pthread_mutex_unlock(&j->mu);                                                                 \
      if (w >= j->W) break;                                                                         \
      for (uint32_t i = 0; i < nb; i++) b[i] = P##_inf();                                           \
      for (size_t i = 0; i < j->n; i++) {                                                           \
        uint32_t d = digit(&j->sc[i], w * j->c, j->c);                                              \
        if (d) b[d] = P##_madd(b[d], &j->pts[i]);                                                   \
      }                                                                                             \
      P##_jac run = P##_inf(), acc = P##_inf();                                                     \
      for (uint32_t i = nb - 1; i >= 1; i--) {                                                      \
        run = P##_add(run, b[i]);                                                                   \
        acc = P##_add(acc, run);                                                                    \
      }                                                                                             \
      j->win[w] = acc;                                                                              \
    }                                                                                               \
    free(b);                                                                                        \
    return NULL;                                                                                    \
  }                                                                                                 \
  static P##_jac P##_msm(const P##_aff *pts, const fe *sc, size_t n, int threads) {                \
    P##_msm_job j;                                                                                  \
    j.pts = pts; j.sc = sc; j.n = n; j.c = pick_c(n); j.W = 256 / j.c + (256 % j.c ? 1 : 0);        \
    j.next = 0; j.nthreads = threads;                                                               \
    j.win = (P##_jac *)malloc(sizeof(P##_jac) * j.W);                                               \
    pthread_mutex_init(&j.mu, NULL);                                                                \
    int nt = threads < j.W ? threads : j.W;                                                         \
    if (nt < 1) nt = 1;                                                                             \
    pthread_t th[256];                                                                              \
    for (int t = 0; t < nt; t++) pthread_create(&th[t], NULL, P##_msm_worker, &j);                  \
    for (int t = 0; t < nt; t++) pthread_join(th[t], NULL);                                         \
    P##_jac total = P##_inf();                                                                      \
    for (int w = j.W - 1; w >= 0; w--) {                                                            \
      for (int d = 0; d < j.c; d++) total = P##_dbl(total);                                         \
      total = P##_add(total, j.win[w]);                                                             \
    }                                                                                               \
    free(j.win);                                                                                    \
    pthread_mutex_destroy(&j.mu);                                                                   \
    return total;                                                                                   \
  }
DEFINE_MSM(g1)
DEFINE_MSM(g2)

/* ------------------------------------------------------------------ NTT */
static fe omega_mont(int L) {
  fe root = {{0x9bd61b6e725b19f0ull, 0x402d111e41112ed4ull, 0x00e0a7eb8ef62abcull, 0x2a3c09f0a58a7e85ull}};
  fe w = f_to_mont(&FR, root);
  for (int i = L; i < 28; i++) w = f_mul(&FR, w, w);
  return w;
}
static fe fr_small(uint64_t x) { fe r = {{x, 0, 0, 0}}; return f_to_mont(&FR, r); }

typedef struct {
  fe *a; const fe *tw; size_t n; int L, nthreads, id;
  pthread_barrier_t *bar;
} ntt_job;

static void *ntt_worker(void *arg) {
  ntt_job *j = (ntt_job *)arg;
  const size_t n = j->n, half = n / 2;
  /* bit reversal: thread-partitioned swaps */
  for (size_t i = j->id; i < n; i += j->nthreads) {
    size_t r = 0;
    for (int b = 0; b < j->L; b++) r |= ((i >> b) & 1) << (j->L - 1 - b);
    if (i < r) { fe t = j->a[i]; j->a[i] = j->a[r]; j->a[r] = t; }
  }
  pthread_barrier_wait(j->bar);
  for (int s = 0; s < j->L; s++) {
    const size_t m = (size_t)1 << s;
    const size_t stride = half >> s; /* twiddle index step: w_(2m)^k = w_n^(k n/(2m)) */
    size_t lo = half * j->id / j->nthreads, hi = half * (j->id + 1) / j->nthreads;
    for (size_t b = lo; b < hi; b++) {
      size_t k = b & (m - 1), blk = b >> s;
      size_t i1 = blk * 2 * m + k, i2 = i1 + m;
      fe u = j->a[i1], v = f_mul(&FR, j->a[i2], j->tw[k * stride]);
      j->a[i1] = f_add(&FR, u, v);
      j->a[i2] = f_sub(&FR, u, v);
    }
    pthread_barrier_wait(j->bar);
  }
  return NULL;
}

/* natural-order radix-2 DIT on n = 2^L Montgomery elements; w = generator (Montgomery) */
static void ntt_core(fe *a, int L, fe w, int threads) {
  const size_t n = (size_t)1 << L;
  if (L == 0) return;
  fe *tw = (fe *)malloc(sizeof(fe) * (n / 2));
  fe x = f_one(&FR);
  for (size_t i = 0; i < n / 2; i++) { tw[i] = x; x = f_mul(&FR, x, w); }
  int nt = threads < 1 ? 1 : threads;
  if ((size_t)nt > n / 2) nt = (int)(n / 2);
  pthread_barrier_t bar;
  pthread_barrier_init(&bar, NULL, nt);
  pthread_t th[256];
  ntt_job jobs[256];
  for (int t = 0; t < nt; t++) {
    jobs[t].a = a; jobs[t].tw = tw; jobs[t].n = n; jobs[t].L = L; jobs[t].nthreads = nt; jobs[t].id = t;
    jobs[t].bar = &bar;
    pthread_create(&th[t], NULL, ntt_worker, &jobs[t]);
  }
  for (int t = 0; t < nt; t++) pthread_join(th[t], NULL);
  pthread_barrier_destroy(&bar);
  free(tw);
}

static void scale_powers(fe *a, size_t n, fe first, fe step) {
  fe x = first;
  for (size_t i = 0; i < n; i++) { a[i] = f_mul(&FR, a[i], x); x = f_mul(&FR, x, step); }
}

/* mode: 0 fft, 1 ifft, 2 coset fft, 3 coset ifft (bend2/gen/ref_qap.py:27-65) */
static void ntt_mode(fe *a, int L, int mode, int threads) {
  const size_t n = (size_t)1 << L;
  fe w = omega_mont(L), g = fr_small(5), one = f_one(&FR);
  if (mode == 2) scale_powers(a, n, one, g);
  if (mode == 0 || mode == 2) {
    ntt_core(a, L, w, threads);
    return;
  }
  ntt_core(a, L, f_inv(&FR, w), threads);
  fe ninv = f_inv(&FR, fr_small(n));
  if (mode == 1) scale_powers(a, n, ninv, one);
  else scale_powers(a, n, ninv, f_inv(&FR, g));
}

static void qap_h_core(fe *a, fe *b, fe *c, int L, int threads) {
  const size_t n = (size_t)1 << L;
  fe *v[3] = {a, b, c};
  for (int i = 0; i < 3; i++) { ntt_mode(v[i], L, 1, threads); ntt_mode(v[i], L, 2, threads); }
  fe g = fr_small(5);
  uint64_t e[4] = {n, 0, 0, 0};
  fe zinv = f_inv(&FR, f_sub(&FR, f_pow(&FR, g, e), f_one(&FR)));
  for (size_t i = 0; i < n; i++) a[i] = f_mul(&FR, f_sub(&FR, f_mul(&FR, a[i], b[i]), c[i]), zinv);
  ntt_mode(a, L, 3, threads);
}

/* ------------------------------------------------------------------ exported oracle API */
static fe *read_fes(const uint32_t *w16, size_t n) {
  fe *a = (fe *)malloc(sizeof(fe) * (n ? n : 1));
  for (size_t i = 0; i < n; i++) a[i] = fe_read16(w16 + 16 * i);
  return a;
}

int bgo_msm_g1(const uint32_t *pts16, const uint32_t *sc16, size_t n, int threads, uint32_t *out_aff16) {
  g1_aff *p = (g1_aff *)malloc(sizeof(g1_aff) * (n ? n : 1));
  for (size_t i = 0; i < n; i++) p[i] = g1_read16(pts16 + 32 * i);
  fe *s = read_fes(sc16, n);
  g1_aff r = g1_to_aff(g1_msm(p, s, n, threads));
  g1_write16(out_aff16, &r);
  free(p);
  free(s);
  return 0;
}

int bgo_msm_g2(const uint32_t *pts16, const uint32_t *sc16, size_t n, int threads, uint32_t *out_aff16) {
  g2_aff *p = (g2_aff *)malloc(sizeof(g2_aff) * (n ? n : 1));
  for (size_t i = 0; i < n; i++) p[i] = g2_read16(pts16 + 64 * i);
  fe *s = read_fes(sc16, n);
  g2_aff r = g2_to_aff(g2_msm(p, s, n, threads));
  g2_write16(out_aff16, &r);
  free(p);
  free(s);
  return 0;
}

int bgo_ntt(uint32_t *data16, int L, int mode, int threads) {
  const size_t n = (size_t)1 << L;
  fe *a = read_fes(data16, n);
  ntt_mode(a, L, mode, threads);
  for (size_t i = 0; i < n; i++) fe_write16(data16 + 16 * i, a[i]);
  free(a);
  return 0;
}

int bgo_qap_h(const uint32_t *a16, const uint32_t *b16, const uint32_t *c16, int L, int threads, uint32_t *h16) {
  const size_t n = (size_t)1 << L;
  fe *a = read_fes(a16, n), *b = read_fes(b16, n), *c = read_fes(c16, n);
  qap_h_core(a, b, c, L, threads);
  for (size_t i = 0; i < n; i++) fe_write16(h16 + 16 * i, a[i]);
  free(a); free(b); free(c);
  return 0;
}

/* ------------------------------------------------------------------ whole proof */
static uint32_t *slurp(const char *dir, const char *name, size_t *words) {
  char path[4096];
  snprintf(path, sizeof path, "%s/%s.bin", dir, name);
  FILE *f = fopen(path, "rb");
  if (!f) return NULL;
  fseek(f, 0, SEEK_END);
  long sz = ftell(f);
  fseek(f, 0, SEEK_SET);
  uint32_t *buf = (uint32_t *)malloc(sz > 0 ? (size_t)sz : 4);
  size_t got = sz > 0 ? fread(buf, 1, (size_t)sz, f) : 0;
  fclose(f);
  if ((long)got != sz) { free(buf); return NULL; }
  *words = (size_t)sz / 4;
  return buf;
}

static double now_ms(void) {
  struct timespec t;
  clock_gettime(CLOCK_MONOTONIC, &t);
  return t.tv_sec * 1e3 + t.tv_nsec / 1e6;
}

/* CSR row sums: ev[i] = sum coeff z[col] (bend2/src/groth16.bend:129-162) */
static void evals_csr(const uint32_t *csr, uint32_t nc, const fe *z, size_t nz, fe *ev) {
  const uint32_t *offs = csr + 1;
  const uint32_t *ent = csr + 2 + nc;
  for (uint32_t i = 0; i < nc; i++) {
    fe acc = f_zero();
    for (uint32_t e = offs[i]; e < offs[i + 1]; e++) {
      uint32_t col = ent[17 * e];
      if (col >= nz) continue;
      acc = f_add(&FR, acc, f_mul(&FR, fe_read16(ent + 17 * e + 1), z[col]));
    }
    ev[i] = acc;
  }
}

/* Proof from a FORMAT.md directory.  out16: A (32 words), B (64), C (32) affine Montgomery;
 * ms: 9 phase times (load evals qap msm_a msm_b1 msm_b2 msm_h msm_l total). */
int bgo_prove_dir(const char *dir, int threads, uint32_t *out16, double *ms) {
  double t0 = now_ms();
  static const char *names[13] = {"header", "witness", "r1cs_a", "r1cs_b", "r1cs_c", "pk_g1", "pk_g2",
                                  "pk_a",   "pk_b1",   "pk_b2",  "pk_h",   "pk_l",   "rs"};
  uint32_t *f[13];
  size_t nw[13];
  for (int i = 0; i < 13; i++) {
    f[i] = slurp(dir, names[i], &nw[i]);
    if (!f[i]) { for (int j = 0; j < i; j++) free(f[j]); return 1; }
  }
  const uint32_t *h = f[0];
  const uint32_t nc = h[0], ni = h[1], nwit = h[2], lg = h[3], na = h[4], nb = h[5], nh = h[6], nl = h[7];
  const size_t d = (size_t)1 << lg, nz = (size_t)ni + nwit;
  fe *z = read_fes(f[1], nz);
  g1_aff *pa = malloc(sizeof(g1_aff) * na), *pb1 = malloc(sizeof(g1_aff) * nb);
  g1_aff *ph = malloc(sizeof(g1_aff) * (nh ? nh : 1)), *pl = malloc(sizeof(g1_aff) * (nl ? nl : 1));
  g2_aff *pb2 = malloc(sizeof(g2_aff) * nb);
  for (uint32_t i = 0; i < na; i++) pa[i] = g1_read16(f[7] + 32 * i);
  for (uint32_t i = 0; i < nb; i++) pb1[i] = g1_read16(f[8] + 32 * i);
  for (uint32_t i = 0; i < nb; i++) pb2[i] = g2_read16(f[9] + 64 * i);
  for (uint32_t i = 0; i < nh; i++) ph[i] = g1_read16(f[10] + 32 * i);
  for (uint32_t i = 0; i < nl; i++) pl[i] = g1_read16(f[11] + 32 * i);
  double t1 = now_ms();
  fe *ea = calloc(d, sizeof(fe)), *eb = calloc(d, sizeof(fe)), *ec = calloc(d, sizeof(fe));
  evals_csr(f[2], nc, z, nz, ea);
  evals_csr(f[3], nc, z, nz, eb);
  evals_csr(f[4], nc, z, nz, ec);
  for (uint32_t i = 0; i < ni && nc + i < d; i++) ea[nc + i] = z[i];
  fe *zc = malloc(sizeof(fe) * nz);
  for (size_t i = 0; i < nz; i++) zc[i] = f_from_mont(&FR, z[i]);
  double t2 = now_ms();
  qap_h_core(ea, eb, ec, (int)lg, threads);
  for (size_t i = 0; i < d; i++) ea[i] = f_from_mont(&FR, ea[i]);
  double t3 = now_ms();
  g1_jac mA = g1_msm(pa, zc, na, threads);
  double t4 = now_ms();
  g1_jac mB1 = g1_msm(pb1, zc, nb, threads);
  double t5 = now_ms();
  g2_jac mB2 = g2_msm(pb2, zc, nb, threads);
  double t6 = now_ms();
  g1_jac mH = g1_msm(ph, ea, nh, threads);
  double t7 = now_ms();
  g1_jac mL = g1_msm(pl, zc + ni, nl, threads);
  double t8 = now_ms();
  /* combine (bend2/src/groth16.bend:298-308) */
  g1_aff alpha = g1_read16(f[5]), beta = g1_read16(f[5] + 32), delta = g1_read16(f[5] + 64);
  g2_aff beta2 = g2_read16(f[6]), delta2 = g2_read16(f[6] + 64);
  fe rm = fe_read16(f[12]), sm = fe_read16(f[12] + 16);
  fe r = f_from_mont(&FR, rm), s = f_from_mont(&FR, sm), rs = f_from_mont(&FR, f_mul(&FR, rm, sm));
  g1_jac dj = g1_from_aff(&delta);
  g1_jac A = g1_madd(g1_add(mA, g1_mul(dj, r)), &alpha);
  g1_jac B1 = g1_madd(g1_add(mB1, g1_mul(dj, s)), &beta);
  g2_jac B2 = g2_madd(g2_add(mB2, g2_mul(g2_from_aff(&delta2), s)), &beta2);
  g1_jac nrs = g1_mul(dj, rs);
  nrs.y = f_sub(&FQ, f_zero(), nrs.y);
  g1_jac C = g1_add(g1_add(g1_add(g1_mul(A, s), g1_mul(B1, r)), nrs), g1_add(mL, mH));
  g1_aff Aa = g1_to_aff(A), Ca = g1_to_aff(C);
  g2_aff Ba = g2_to_aff(B2);
  g1_write16(out16, &Aa);
  g2_write16(out16 + 32, &Ba);
  g1_write16(out16 + 96, &Ca);
  double t9 = now_ms();
  if (ms) {
    double v[9] = {t1 - t0, t2 - t1, t3 - t2, t4 - t3, t5 - t4, t6 - t5, t7 - t6, t8 - t7, t9 - t0};
    memcpy(ms, v, sizeof v);
  }
  free(z); free(zc); free(pa); free(pb1); free(pb2); free(ph); free(pl); free(ea); free(eb); free(ec);
  for (int i = 0; i < 13; i++) free(f[i]);
  return 0;
}

/* ------------------------------------------------------------------ synthetic instance
 * The SquareChain(2^k) instance of the library's bg_synth_square_chain, computed on the CPU:
 * same splitmix64 stream, same trapdoor draws, same column polynomials (ref/src/circuit.rs,
 * ref/src/gen.rs:78-93), so the files must be byte-identical. */
typedef struct { uint64_t s; } splitmix;
static uint64_t sm_next(splitmix *r) {
  uint64_t z = (r->s += 0x9e3779b97f4a7c15ull);
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}
static fe sm_fr(splitmix *r) {
  for (;;) {
    fe x;
    x.v[0] = sm_next(r); x.v[1] = sm_next(r); x.v[2] = sm_next(r); x.v[3] = sm_next(r) & 0x3fffffffffffffffull;
    if (!geq4(x.v, FR.p)) return x;
  }
}
static void batch_inv_fr(fe *v, size_t n) {
  fe *pre = (fe *)malloc(sizeof(fe) * (n ? n : 1));
  fe acc = f_one(&FR);
  for (size_t i = 0; i < n; i++) { pre[i] = acc; if (!f_is_zero(v[i])) acc = f_mul(&FR, acc, v[i]); }
  fe inv = f_inv(&FR, acc);
  for (size_t i = n; i-- > 0;) {
    if (f_is_zero(v[i])) continue;
    fe vi = v[i];
    v[i] = f_mul(&FR, inv, pre[i]);
    inv = f_mul(&FR, inv, vi);
  }
  free(pre);
}

typedef struct { const void *table; const fe *k; size_t lo, hi; void *out; int g2; } fb_job;

static void *fb_worker(void *arg) {
  fb_job *j = (fb_job *)arg;
  for (size_t i = j->lo; i < j->hi; i++) {
    if (!j->g2) {
      const g1_aff *t = (const g1_aff *)j->table;
      g1_jac acc = g1_inf();
      for (int w = 0; w < 32; w++) {
        unsigned d = (unsigned)(j->k[i].v[w / 8] >> (8 * (w % 8))) & 0xffu;
        if (d) acc = g1_madd(acc, &t[w * 255 + d - 1]);
      }
      ((g1_aff *)j->out)[i] = g1_to_aff(acc);
    } else {
      const g2_aff *t = (const g2_aff *)j->table;
      g2_jac acc = g2_inf();
      for (int w = 0; w < 32; w++) {
        unsigned d = (unsigned)(j->k[i].v[w / 8] >> (8 * (w % 8))) & 0xffu;
        if (d) acc = g2_madd(acc, &t[w * 255 + d - 1]);
      }
      ((g2_aff *)j->out)[i] = g2_to_aff(acc);
    }
  }
  return NULL;
}

static void fixed_base(const void *table, int g2, const fe *k, size_t n, void *out, int threads) {
  int nt = threads < 1 ? 1 : (threads > 256 ? 256 : threads);
  pthread_t th[256];
  fb_job jobs[256];
  for (int t = 0; t < nt; t++) {
    jobs[t].table = table; jobs[t].k = k; jobs[t].lo = n * t / nt; jobs[t].hi = n * (t + 1) / nt;
    jobs[t].out = out; jobs[t].g2 = g2;
    pthread_create(&th[t], NULL, fb_worker, &jobs[t]);
  }
  for (int t = 0; t < nt; t++) pthread_join(th[t], NULL);
}

static int write_u32(const char *dir, const char *name, const uint32_t *w, size_t n) {
  char path[4096];
  snprintf(path, sizeof path, "%s/%s.bin", dir, name);
  FILE *f = fopen(path, "wb");
  if (!f) return 1;
  size_t put = n ? fwrite(w, 4, n, f) : 0;
  fclose(f);
  return put != n;
}

int bgo_synth_square_chain(uint32_t log2n, uint64_t seed, const char *dir, int threads) {
  if (log2n < 1 || log2n > 24) return 2;
  const uint64_t N = 1ull << log2n, ni = 2, nw = N, m = ni + nw;
  uint32_t lg = 0;
  while ((1ull << lg) < N + ni) lg++;
  const uint64_t d = 1ull << lg;
  splitmix rng = {seed};
  fe x0 = sm_fr(&rng);
  fe tau = sm_fr(&rng), alpha = sm_fr(&rng), beta = sm_fr(&rng), gamma = sm_fr(&rng), delta = sm_fr(&rng);
  fe r = sm_fr(&rng), s = sm_fr(&rng);
  const fe one = f_one(&FR);
  int bad = 0;

  /* witness */
  uint32_t *wit = (uint32_t *)malloc(4 * 16 * m);
  fe x = f_to_mont(&FR, x0);
  fe *xs = (fe *)malloc(sizeof(fe) * (N + 1));
  xs[0] = x;
  for (uint64_t i = 0; i < N; i++) xs[i + 1] = f_mul(&FR, xs[i], xs[i]);
  fe_write16(wit, one);
  fe_write16(wit + 16, xs[N]);
  for (uint64_t i = 0; i < N; i++) fe_write16(wit + 16 * (2 + i), xs[i]);
  bad |= write_u32(dir, "witness", wit, 16 * m);
  free(wit);
  free(xs);

  /* Lagrange basis at tau */
  fe w = omega_mont((int)lg);
  fe taum = f_to_mont(&FR, tau);
  uint64_t e[4] = {d, 0, 0, 0};
  fe zt = f_sub(&FR, f_pow(&FR, taum, e), one);
  fe zd = f_mul(&FR, zt, f_inv(&FR, fr_small(d)));
  fe *wk = (fe *)malloc(sizeof(fe) * d), *den = (fe *)malloc(sizeof(fe) * d);
  fe acc = one;
  for (uint64_t k = 0; k < d; k++) { wk[k] = acc; den[k] = f_sub(&FR, taum, acc); acc = f_mul(&FR, acc, w); }
  batch_inv_fr(den, d);
#define LAG(k) f_mul(&FR, f_mul(&FR, zd, wk[k]), den[k])
  fe *A = (fe *)calloc(m, sizeof(fe)), *B = (fe *)calloc(m, sizeof(fe)), *C = (fe *)calloc(m, sizeof(fe));
  for (uint64_t i = 0; i < N; i++) {
    fe li = LAG(i);
    A[2 + i] = f_add(&FR, A[2 + i], li);
    B[2 + i] = f_add(&FR, B[2 + i], li);
    uint64_t cc = (i + 1 < N) ? 3 + i : 1;
    C[cc] = f_add(&FR, C[cc], li);
  }
  for (uint64_t i = 0; i < ni; i++) A[i] = f_add(&FR, A[i], LAG(N + i));
#undef LAG
  fe am = f_to_mont(&FR, alpha), bm = f_to_mont(&FR, beta), dm = f_to_mont(&FR, delta);
  fe dinv = f_inv(&FR, dm);
  fe *ka = (fe *)malloc(sizeof(fe) * m), *kb = (fe *)malloc(sizeof(fe) * m);
  fe *kh = (fe *)malloc(sizeof(fe) * d), *kl = (fe *)malloc(sizeof(fe) * nw);
  for (uint64_t j = 0; j < m; j++) { ka[j] = f_from_mont(&FR, A[j]); kb[j] = f_from_mont(&FR, B[j]); }
  fe tp = f_mul(&FR, zt, dinv);
  for (uint64_t k = 0; k + 1 < d; k++) { kh[k] = f_from_mont(&FR, tp); tp = f_mul(&FR, tp, taum); }
  for (uint64_t j = 0; j < nw; j++) {
    fe v = f_add(&FR, f_mul(&FR, bm, A[2 + j]), f_mul(&FR, am, B[2 + j]));
    v = f_add(&FR, v, C[2 + j]);
    kl[j] = f_from_mont(&FR, f_mul(&FR, v, dinv));
  }
  /* verifying key: IC_i = (beta A_i + alpha B_i + C_i)(tau) / gamma for the instance columns */
  fe ginv = f_inv(&FR, f_to_mont(&FR, gamma));
  fe kic[2];
  for (uint64_t i = 0; i < ni; i++) {
    fe v = f_add(&FR, f_mul(&FR, bm, A[i]), f_mul(&FR, am, B[i]));
    v = f_add(&FR, v, C[i]);
    kic[i] = f_from_mont(&FR, f_mul(&FR, v, ginv));
  }
  free(wk); free(den); free(A); free(B); free(C);

  /* fixed-base tables T[w][d-1] = d 2^(8w) G */
  g1_aff g1g;
  g1g.x = f_to_mont(&FQ, (fe){{1, 0, 0, 0}});
  g1g.y = f_to_mont(&FQ, (fe){{2, 0, 0, 0}});
  g1g.inf = 0;
  g2_aff g2g;
  g2g.x.c0 = f_to_mont(&FQ, (fe){{0x46debd5cd992f6edull, 0x674322d4f75edaddull, 0x426a00665e5c4479ull, 0x1800deef121f1e76ull}});
  g2g.x.c1 = f_to_mont(&FQ, (fe){{0x97e485b7aef312c2ull, 0xf1aa493335a9e712ull, 0x7260bfb731fb5d25ull, 0x198e9393920d483aull}});
  g2g.y.c0 = f_to_mont(&FQ, (fe){{0x4ce6cc0166fa7daaull, 0xe3d1e7690c43d37bull, 0x4aab71808dcb408full, 0x12c85ea5db8c6debull}});
  g2g.y.c1 = f_to_mont(&FQ, (fe){{0x55acdadcd122975bull, 0xbc4b313370b38ef3ull, 0xec9e99ad690c3395ull, 0x090689d0585ff075ull}});
  g2g.inf = 0;
  g1_aff *t1 = (g1_aff *)malloc(sizeof(g1_aff) * 32 * 255);
  g2_aff *t2 = (g2_aff *)malloc(sizeof(g2_aff) * 32 * 255);
  g1_jac b1 = g1_from_aff(&g1g);
  g2_jac b2 = g2_from_aff(&g2g);
  for (int ww = 0; ww < 32; ww++) {
    g1_jac a1 = b1;
    g2_jac a2 = b2;
    for (int dd = 1; dd <= 255; dd++) {
      t1[ww * 255 + dd - 1] = g1_to_aff(a1);
      t2[ww * 255 + dd - 1] = g2_to_aff(a2);
      a1 = g1_add(a1, b1);
      a2 = g2_add(a2, b2);
    }
    for (int i = 0; i < 8; i++) { b1 = g1_dbl(b1); b2 = g2_dbl(b2); }
  }
  fe kg1[3] = {alpha, beta, delta}, kg2[2] = {beta, delta}, kvk1[1] = {alpha}, kvk2[3] = {beta, gamma, delta};
  struct { const fe *k; size_t n; int g2; const char *name; } outs[10] = {
      {ka, m, 0, "pk_a"}, {kb, m, 0, "pk_b1"}, {kb, m, 1, "pk_b2"}, {kh, d - 1, 0, "pk_h"},
      {kl, nw, 0, "pk_l"}, {kg1, 3, 0, "pk_g1"}, {kg2, 2, 1, "pk_g2"},
      {kvk1, 1, 0, NULL}, {kvk2, 3, 1, NULL}, {kic, ni, 0, NULL}};
  /* vk.bin: alpha_g1, beta_g2, gamma_g2, delta_g2, u32 n_ic, IC_0 .. IC_{n_ic-1} */
  uint32_t vk[32 + 3 * 64 + 1 + 2 * 32];
  size_t vk_off[3] = {0, 32, 32 + 3 * 64 + 1};
  vk[32 + 3 * 64] = (uint32_t)ni;
  for (int o = 0; o < 10; o++) {
    size_t n = outs[o].n;
    size_t pw = outs[o].g2 ? 64 : 32;
    void *pts = malloc((outs[o].g2 ? sizeof(g2_aff) : sizeof(g1_aff)) * (n ? n : 1));
    fixed_base(outs[o].g2 ? (const void *)t2 : (const void *)t1, outs[o].g2, outs[o].k, n, pts, threads);
    uint32_t *wbuf = (uint32_t *)malloc(4 * pw * (n ? n : 1));
    for (size_t i = 0; i < n; i++) {
      if (outs[o].g2) {
        g2_aff a = ((g2_aff *)pts)[i];
        if (a.inf) memset(wbuf + pw * i, 0, 4 * pw); else g2_write16(wbuf + pw * i, &a);
      } else {
        g1_aff a = ((g1_aff *)pts)[i];
        if (a.inf) memset(wbuf + pw * i, 0, 4 * pw); else g1_write16(wbuf + pw * i, &a);
      }
    }
    if (outs[o].name) bad |= write_u32(dir, outs[o].name, wbuf, pw * n);
    else memcpy(vk + vk_off[o - 7], wbuf, 4 * pw * n);
    free(wbuf);
    free(pts);
  }
  free(t1); free(t2); free(ka); free(kb); free(kh); free(kl);

  /* CSR, header, r/s, trapdoor */
  for (int which = 0; which < 3; which++) {
    size_t words = 2 + N + 17 * N;
    uint32_t *f = (uint32_t *)malloc(4 * words);
    f[0] = (uint32_t)N;
    for (uint64_t i = 0; i <= N; i++) f[1 + i] = (uint32_t)i;
    for (uint64_t i = 0; i < N; i++) {
      uint32_t col = which < 2 ? (uint32_t)(2 + i) : (i + 1 < N ? (uint32_t)(3 + i) : 1u);
      f[2 + N + 17 * i] = col;
      fe_write16(f + 2 + N + 17 * i + 1, one);
    }
    bad |= write_u32(dir, which == 0 ? "r1cs_a" : which == 1 ? "r1cs_b" : "r1cs_c", f, words);
    free(f);
  }
  uint32_t header[8] = {(uint32_t)N, (uint32_t)ni, (uint32_t)nw, lg, (uint32_t)m, (uint32_t)m, (uint32_t)(d - 1),
                        (uint32_t)nw};
  bad |= write_u32(dir, "header", header, 8);
  uint32_t rs[32], trap[80];
  fe_write16(rs, f_to_mont(&FR, r));
  fe_write16(rs + 16, f_to_mont(&FR, s));
  bad |= write_u32(dir, "rs", rs, 32);
  fe tv[5] = {tau, alpha, beta, gamma, delta};
  for (int i = 0; i < 5; i++) fe_write16(trap + 16 * i, tv[i]);
  bad |= write_u32(dir, "trapdoor", trap, 80);
  bad |= write_u32(dir, "vk", vk, sizeof(vk) / 4);
  return bad;
}
