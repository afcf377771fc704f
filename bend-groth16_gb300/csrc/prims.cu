// Element-wise primitives: wire-layout repacking (bend2/FORMAT.md 16-bit limbs <-> packed
// 8 x 32-bit limbs), field and curve op vectors (the shapes of the reference's unit tests
// bend2/tests/test_fr.bend:9-16, test_g1.bend:9-20, test_g2.bend:13-20), Montgomery <->
// canonical conversion, and an integer multiply-add throughput probe used as the MSM
// roofline denominator.
#include "common.cuh"
#include "ec.cuh"
#include "prims.h"

namespace bg {

// ---------------------------------------------------------------- repacking
// element i: 16 words (low 16 bits significant) -> 8 words.  Upper halves of wire words must
// be zero; a nonzero one sets BG_DSTATUS_FORMAT.
__global__ void k_wire_to_packed(const uint32_t* __restrict__ wire, uint32_t* __restrict__ packed, size_t n,
                                 uint32_t* __restrict__ status) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint4* src = reinterpret_cast<const uint4*>(wire + 16 * i);
  const uint4 a = src[0], b = src[1], c = src[2], d = src[3];
  const uint32_t hi = (a.x | a.y | a.z | a.w | b.x | b.y | b.z | b.w | c.x | c.y | c.z | c.w | d.x | d.y | d.z | d.w) >> 16;
  if (hi && status) atomicOr(status, BG_DSTATUS_FORMAT);
  uint4* dst = reinterpret_cast<uint4*>(packed + 8 * i);
  dst[0] = make_uint4((a.x & 0xffff) | (a.y << 16), (a.z & 0xffff) | (a.w << 16), (b.x & 0xffff) | (b.y << 16),
                      (b.z & 0xffff) | (b.w << 16));
  dst[1] = make_uint4((c.x & 0xffff) | (c.y << 16), (c.z & 0xffff) | (c.w << 16), (d.x & 0xffff) | (d.y << 16),
                      (d.z & 0xffff) | (d.w << 16));
}

__global__ void k_packed_to_wire(const uint32_t* __restrict__ packed, uint32_t* __restrict__ wire, size_t n) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint4 p0 = reinterpret_cast<const uint4*>(packed + 8 * i)[0];
  const uint4 p1 = reinterpret_cast<const uint4*>(packed + 8 * i)[1];
  uint4* dst = reinterpret_cast<uint4*>(wire + 16 * i);
  dst[0] = make_uint4(p0.x & 0xffff, p0.x >> 16, p0.y & 0xffff, p0.y >> 16);
  dst[1] = make_uint4(p0.z & 0xffff, p0.z >> 16, p0.w & 0xffff, p0.w >> 16);
  dst[2] = make_uint4(p1.x & 0xffff, p1.x >> 16, p1.y & 0xffff, p1.y >> 16);
  dst[3] = make_uint4(p1.z & 0xffff, p1.z >> 16, p1.w & 0xffff, p1.w >> 16);
}

void wire_to_packed(cudaStream_t st, const uint32_t* d_wire, uint32_t* d_packed, size_t n, uint32_t* d_status) {
  if (n == 0) return;
  k_wire_to_packed<<<ceil_div(n, 256), 256, 0, st>>>(d_wire, d_packed, n, d_status);
  BG_CHECK_LAUNCH();
}
void packed_to_wire(cudaStream_t st, const uint32_t* d_packed, uint32_t* d_wire, size_t n) {
  if (n == 0) return;
  k_packed_to_wire<<<ceil_div(n, 256), 256, 0, st>>>(d_packed, d_wire, n);
  BG_CHECK_LAUNCH();
}

// ---------------------------------------------------------------- Montgomery <-> canonical
__global__ void k_fr_from_mont(const uint32_t* __restrict__ in, uint32_t* __restrict__ out, size_t n) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  store_fp(out + 8 * i, from_mont(load_fp<FrParams>(in + 8 * i)));
}
void fr_from_mont(cudaStream_t st, const uint32_t* d_in, uint32_t* d_out, size_t n) {
  if (n == 0) return;
  k_fr_from_mont<<<ceil_div(n, 256), 256, 0, st>>>(d_in, d_out, n);
  BG_CHECK_LAUNCH();
}

// ---------------------------------------------------------------- field op vectors
template <class P>
BG_DEV Fp<P> r_squared();
template <>
BG_DEV Fp<FqParams> r_squared<FqParams>() {
  Fp<FqParams> r;
  const uint32_t v[8] = {0x538afa89u, 0xf32cfc5bu, 0xd44501fbu, 0xb5e71911u,
                         0x0a417ff6u, 0x47ab1effu, 0xcab8351fu, 0x06d89f71u};
#pragma unroll
  for (int i = 0; i < 8; i++) r.v[i] = v[i];
  return r;
}
template <>
BG_DEV Fp<FrParams> r_squared<FrParams>() {
  Fp<FrParams> r;
  const uint32_t v[8] = {0xae216da7u, 0x1bb8e645u, 0xe35c59e3u, 0x53fe3ab1u,
                         0x53bb8085u, 0x8c49833du, 0x7f4e44a5u, 0x0216d0b1u};
#pragma unroll
  for (int i = 0; i < 8; i++) r.v[i] = v[i];
  return r;
}

template <class P>
__global__ void k_field_op(int op, const uint32_t* __restrict__ a, const uint32_t* __restrict__ b,
                           uint32_t* __restrict__ out, size_t n) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const Fp<P> x = load_fp<P>(a + 8 * i);
  Fp<P> y;
  if (b) y = load_fp<P>(b + 8 * i);
  Fp<P> r;
  switch (op) {
    case BG_FOP_ADD: r = add(x, y); break;
    case BG_FOP_SUB: r = sub(x, y); break;
    case BG_FOP_MUL: r = mul(x, y); break;
    case BG_FOP_NEG: r = neg(x); break;
    case BG_FOP_INV: r = inv(x); break;
    case BG_FOP_SQR: r = sqr(x); break;
    case BG_FOP_TO_MONT: r = mul(x, r_squared<P>()); break;
    default: r = from_mont(x); break;
  }
  store_fp(out + 8 * i, r);
}

void field_op(cudaStream_t st, int field, int op, const uint32_t* a, const uint32_t* b, uint32_t* out, size_t n) {
  if (n == 0) return;
  if (field == BG_FIELD_FR)
    k_field_op<FrParams><<<ceil_div(n, 128), 128, 0, st>>>(op, a, b, out, n);
  else
    k_field_op<FqParams><<<ceil_div(n, 128), 128, 0, st>>>(op, a, b, out, n);
  BG_CHECK_LAUNCH();
}

// ---------------------------------------------------------------- curve op vectors
BG_DEV Fq field_inv(const Fq& a) { return inv(a); }
BG_DEV Fq2 field_inv(const Fq2& a) {
  const Fq ni = inv(add(sqr(a.c0), sqr(a.c1)));
  return {mul(a.c0, ni), neg(mul(a.c1, ni))};
}

template <class F>
BG_DEV Affine<F> to_affine(const XYZZ<F>& p) {
  Affine<F> r;
  if (is_inf(p)) {
    r.x = field_zero<F>();
    r.y = field_zero<F>();
    return r;
  }
  const F t = field_inv(mul(p.zz, p.zzz));
  r.x = mul(p.x, mul(t, p.zzz));
  r.y = mul(p.y, mul(t, p.zz));
  return r;
}

// k*P, MSB-first double-and-add over the 256 bits of a canonical scalar
// (the shape of G1.mul_scalar, bend2/src/g1.bend:175-191)
template <class F>
BG_DEV XYZZ<F> scalar_mul(const Affine<F>& p, const uint32_t* k) {
  XYZZ<F> acc = xyzz_inf<F>();
  for (int i = 255; i >= 0; i--) {
    acc = xyzz_dbl(acc);
    if ((k[i >> 5] >> (i & 31)) & 1u) acc = xyzz_madd(acc, p);
  }
  return acc;
}

template <class F>
__global__ void k_curve_op(int op, const uint32_t* __restrict__ p, const uint32_t* __restrict__ q,
                           const uint32_t* __restrict__ k, uint32_t* __restrict__ out, size_t n) {
  constexpr int FW = FieldWords<F>::value;
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const Affine<F> a = load_affine<F>(p + 2 * FW * i);
  Affine<F> r;
  switch (op) {
    case BG_COP_ADD: {
      const Affine<F> b = load_affine<F>(q + 2 * FW * i);
      r = to_affine(xyzz_madd(xyzz_from_affine(a), b));
      break;
    }
    case BG_COP_DOUBLE:
      r = to_affine(xyzz_dbl(xyzz_from_affine(a)));
      break;
    case BG_COP_NEG:
      r = affine_neg(a);
      break;
    default: {
      uint32_t kk[8];
#pragma unroll
      for (int j = 0; j < 8; j++) kk[j] = k[8 * i + j];
      r = to_affine(scalar_mul(a, kk));
      break;
    }
  }
  store_affine(out + 2 * FW * i, r);
}

void curve_op(cudaStream_t st, int curve, int op, const uint32_t* p, const uint32_t* q, const uint32_t* k,
              uint32_t* out, size_t n) {
  if (n == 0) return;
  if (curve == BG_CURVE_G1)
    k_curve_op<Fq><<<ceil_div(n, 64), 64, 0, st>>>(op, p, q, k, out, n);
  else
    k_curve_op<Fq2><<<ceil_div(n, 64), 64, 0, st>>>(op, p, q, k, out, n);
  BG_CHECK_LAUNCH();
}

// ---------------------------------------------------------------- throughput probes
// Independent 32-bit multiply-add chains: 8 accumulators x `iters` x 2 (lo and hi) per thread.
__global__ void k_imad_probe(uint32_t* __restrict__ sink, uint32_t iters, uint32_t seed) {
  uint32_t a[8], b = seed * 2654435761u + threadIdx.x;
#pragma unroll
  for (int j = 0; j < 8; j++) a[j] = seed ^ (threadIdx.x * 7919u + j);
  for (uint32_t it = 0; it < iters; it++) {
#pragma unroll
    for (int j = 0; j < 8; j++) {
      asm volatile("mad.lo.u32 %0, %0, %1, %2;" : "+r"(a[j]) : "r"(b), "r"(a[(j + 1) & 7]));
      asm volatile("mad.hi.u32 %0, %0, %1, %2;" : "+r"(a[j]) : "r"(b), "r"(a[(j + 3) & 7]));
    }
  }
  uint32_t x = 0;
#pragma unroll
  for (int j = 0; j < 8; j++) x ^= a[j];
  if (x == 0x12345678u) sink[0] = x;
}

// Fq Montgomery products: 4 independent chains per thread
__global__ void k_fqmul_probe(uint32_t* __restrict__ sink, uint32_t iters, uint32_t seed) {
  Fq x[4];
  Fq m = fp_one<FqParams>();
  m.v[0] ^= seed;
#pragma unroll
  for (int j = 0; j < 4; j++) {
    x[j] = fp_one<FqParams>();
    x[j].v[1] ^= threadIdx.x + j;
  }
  for (uint32_t it = 0; it < iters; it++) {
#pragma unroll
    for (int j = 0; j < 4; j++) x[j] = mul(x[j], m);
  }
  uint32_t o = 0;
#pragma unroll
  for (int j = 0; j < 4; j++) o ^= x[j].v[0];
  if (o == 0x12345678u) sink[0] = o;
}

// single-form chains: 16 independent accumulators, one instruction form each
// (form 2: mad.lo.u32, 3: mad.hi.u32, 4: mad.wide.u32 into 64-bit accumulators)
template <int FORM>
__global__ void k_imad_form_probe(uint32_t* __restrict__ sink, uint32_t iters, uint32_t seed) {
  uint32_t a[16];
  unsigned long long w[16];
  const uint32_t b = seed * 2654435761u + threadIdx.x;
#pragma unroll
  for (int j = 0; j < 16; j++) {
    a[j] = seed ^ (threadIdx.x * 7919u + j);
    w[j] = a[j];
  }
  for (uint32_t it = 0; it < iters; it++) {
#pragma unroll
    for (int j = 0; j < 16; j++) {
      if (FORM == 2) asm volatile("mad.lo.u32 %0, %0, %1, %2;" : "+r"(a[j]) : "r"(b), "r"(a[(j + 5) & 15]));
      if (FORM == 3) asm volatile("mad.hi.u32 %0, %0, %1, %2;" : "+r"(a[j]) : "r"(b), "r"(a[(j + 5) & 15]));
      if (FORM == 4) asm volatile("mad.wide.u32 %0, %1, %2, %0;" : "+l"(w[j]) : "r"(a[j]), "r"(b));
    }
    if (FORM == 4) {
#pragma unroll
      for (int j = 0; j < 16; j++) a[j] ^= (uint32_t)(w[j] >> 32);
    }
  }
  uint32_t x = 0;
#pragma unroll
  for (int j = 0; j < 16; j++) x ^= a[j] ^ (uint32_t)w[j];
  if (x == 0x12345678u) sink[0] = x;
}

void imad_probe(cudaStream_t st, int blocks, int threads, uint32_t iters, uint32_t* sink, int which) {
  switch (which) {
    case 0: k_imad_probe<<<blocks, threads, 0, st>>>(sink, iters, 12345u); break;
    case 1: k_fqmul_probe<<<blocks, threads, 0, st>>>(sink, iters, 12345u); break;
    case 2: k_imad_form_probe<2><<<blocks, threads, 0, st>>>(sink, iters, 12345u); break;
    case 3: k_imad_form_probe<3><<<blocks, threads, 0, st>>>(sink, iters, 12345u); break;
    default: k_imad_form_probe<4><<<blocks, threads, 0, st>>>(sink, iters, 12345u); break;
  }
  BG_CHECK_LAUNCH();
}

}  // namespace bg
