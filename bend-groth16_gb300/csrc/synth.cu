// Seeded synthetic SquareChain(2^k) instance in bend2/FORMAT.md files: the input generator
// for benchmarks at sizes where no committed fixture exists (the role `groth16-ref gen`,
// ref/src/gen.rs:95-164, plays for the reference).  It is not on the proving path.
//
// Circuit (ref/src/circuit.rs:21-74): x_{i+1} = x_i^2, N = 2^k constraints, z = [1, x_N,
// x_0 .. x_{N-1}]; row i: A = B = [(2+i, 1)], C = [(3+i, 1)], last row C = [(1, 1)]
// (ref/src/gen.rs:78-83).  Setup: own seeded trapdoor (tau, alpha, beta, gamma, delta), the
// arkworks RNG is not reproduced.  Column polynomials at tau use the size-d Lagrange basis,
// with libsnark's input-consistency rows N+i in A for the instance columns; then
//   a_query[j] = A_j(tau) G1, b_g1_query[j] = B_j(tau) G1, b_g2_query[j] = B_j(tau) G2,
//   h_query[k] = tau^k Z(tau)/delta G1 (k < d-1),
//   l_query[j] = (beta A_{2+j} + alpha B_{2+j} + C_{2+j})(tau)/delta G1.
// The trapdoor is also written to trapdoor.bin (5 canonical Fr, 16-bit-limb words) so tests
// can check proofs without pairings, and the verifying key to vk.bin (the .bin counterpart of
// the reference's vk.json: alpha_g1, beta_g2, gamma_g2, delta_g2, u32 n_ic, n_ic IC points,
// IC_i = (beta A_i + alpha B_i + C_i)(tau)/gamma G1 for the instance columns).
#include <cstdio>
#include <string>
#include <vector>

#include "common.cuh"
#include "ec.cuh"
#include "host_ff.hpp"
#include "prims.h"

namespace bg {

using bgh::Fe;
using bgh::FR;

namespace {

struct SplitMix {
  uint64_t s;
  uint64_t next() {
    uint64_t z = (s += 0x9e3779b97f4a7c15ull);
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
  }
  // uniform canonical Fr by rejection sampling of 254-bit integers
  Fe fr() {
    while (true) {
      Fe x{{next(), next(), next(), next() & 0x3fffffffffffffffull}};
      if (!bgh::geq(x.v, FR.p)) return x;
    }
  }
};

Fe mont(const Fe& canon) { return bgh::fe_to_mont(FR, canon); }
Fe canon(const Fe& m) { return bgh::fe_from_mont(FR, m); }

void batch_inverse(std::vector<Fe>& v) {
  // Montgomery's trick; zeros stay zero
  std::vector<Fe> pre(v.size());
  Fe acc = bgh::fe_one(FR);
  for (size_t i = 0; i < v.size(); i++) {
    pre[i] = acc;
    if (!bgh::fe_is_zero(v[i])) acc = bgh::fe_mul(FR, acc, v[i]);
  }
  Fe inv = bgh::fe_inv(FR, acc);
  for (size_t i = v.size(); i-- > 0;) {
    if (bgh::fe_is_zero(v[i])) continue;
    Fe vi = v[i];
    v[i] = bgh::fe_mul(FR, inv, pre[i]);
    inv = bgh::fe_mul(FR, inv, vi);
  }
}

// 8-bit fixed-base tables: T[w][d-1] = d 2^(8w) G, d = 1..255, w = 0..31 (affine, packed)
template <class H>
std::vector<uint32_t> fixed_base_table(const bgh::Aff<H>& g) {
  constexpr int PW = 2 * H::WORDS;
  std::vector<bgh::Xyzz<H>> pts;
  pts.reserve(32 * 255);
  bgh::Xyzz<H> base = bgh::xyzz_from(g);
  for (int w = 0; w < 32; w++) {
    bgh::Xyzz<H> acc = base;
    for (int d = 1; d <= 255; d++) {
      pts.push_back(acc);
      acc = bgh::xyzz_add(acc, base);
    }
    for (int i = 0; i < 8; i++) base = bgh::xyzz_dbl(base);
  }
  std::vector<uint32_t> out(pts.size() * PW);
  for (size_t i = 0; i < pts.size(); i++) bgh::aff_to_words32<H>(out.data() + i * PW, bgh::xyzz_to_affine(pts[i]));
  return out;
}

template <class F>
BG_DEV Affine<F> xyzz_to_affine_dev(const XYZZ<F>& p);
template <>
BG_DEV Affine<Fq> xyzz_to_affine_dev<Fq>(const XYZZ<Fq>& p) {
  Affine<Fq> r;
  if (is_inf(p)) {
    r.x = fp_zero<FqParams>();
    r.y = fp_zero<FqParams>();
    return r;
  }
  const Fq t = inv(mul(p.zz, p.zzz));
  r.x = mul(p.x, mul(t, p.zzz));
  r.y = mul(p.y, mul(t, p.zz));
  return r;
}
template <>
BG_DEV Affine<Fq2> xyzz_to_affine_dev<Fq2>(const XYZZ<Fq2>& p) {
  Affine<Fq2> r;
  if (is_inf(p)) {
    r.x = field_zero<Fq2>();
    r.y = field_zero<Fq2>();
    return r;
  }
  const Fq2 m = mul(p.zz, p.zzz);
  const Fq ni = inv(add(sqr(m.c0), sqr(m.c1)));
  const Fq2 t = {mul(m.c0, ni), neg(mul(m.c1, ni))};
  r.x = mul(p.x, mul(t, p.zzz));
  r.y = mul(p.y, mul(t, p.zz));
  return r;
}

// out[i] = k_i G for canonical scalars k (packed, 8 words each)
template <class F>
__global__ void k_fixed_base(const uint32_t* __restrict__ table, const uint32_t* __restrict__ scalars, size_t n,
                             uint32_t* __restrict__ out) {
  constexpr int PW = 2 * FieldWords<F>::value;
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  uint32_t k[8];
#pragma unroll
  for (int j = 0; j < 8; j++) k[j] = scalars[8 * i + j];
  XYZZ<F> acc = xyzz_inf<F>();
  for (int w = 0; w < 32; w++) {
    const uint32_t d = (k[w >> 2] >> (8 * (w & 3))) & 0xffu;
    if (d) acc = xyzz_madd(acc, load_affine<F>(table + ((size_t)w * 255 + d - 1) * PW));
  }
  store_affine(out + PW * i, xyzz_to_affine_dev(acc));
}

template <class F, class H>
std::vector<uint32_t> device_fixed_base(Ctx& c, const std::vector<uint32_t>& table, const std::vector<Fe>& ks) {
  constexpr int PW = 2 * H::WORDS;
  const size_t n = ks.size();
  std::vector<uint32_t> out_wire(n * PW * 2);
  if (n == 0) return out_wire;
  std::vector<uint32_t> sc(n * 8);
  for (size_t i = 0; i < n; i++) bgh::fe_to_words32(sc.data() + 8 * i, ks[i]);
  uint32_t* d_tab = c.ws.get_t<uint32_t>("synth.tab", table.size());
  uint32_t* d_sc = c.ws.get_t<uint32_t>("synth.sc", sc.size());
  uint32_t* d_out = c.ws.get_t<uint32_t>("synth.out", n * PW);
  uint32_t* d_wire = c.ws.get_t<uint32_t>("synth.wire", n * PW * 2);
  BG_CUDA(cudaMemcpyAsync(d_tab, table.data(), table.size() * 4, cudaMemcpyHostToDevice, c.stream));
  BG_CUDA(cudaMemcpyAsync(d_sc, sc.data(), sc.size() * 4, cudaMemcpyHostToDevice, c.stream));
  k_fixed_base<F><<<ceil_div(n, 128), 128, 0, c.stream>>>(d_tab, d_sc, n, d_out);
  BG_CHECK_LAUNCH();
  packed_to_wire(c.stream, d_out, d_wire, n * PW / 8);
  BG_CUDA(cudaMemcpyAsync(out_wire.data(), d_wire, out_wire.size() * 4, cudaMemcpyDeviceToHost, c.stream));
  BG_CUDA(cudaStreamSynchronize(c.stream));
  return out_wire;
}

void put_fe_wire(std::vector<uint32_t>& out, const Fe& x) {
  uint32_t w[16];
  bgh::fe_to_words16(w, x);
  out.insert(out.end(), w, w + 16);
}

void write_file(const std::string& path, const void* data, size_t bytes) {
  FILE* f = fopen(path.c_str(), "wb");
  if (!f) throw Error(BG_E_IO, "cannot write " + path);
  size_t put = bytes ? fwrite(data, 1, bytes, f) : 0;
  fclose(f);
  if (put != bytes) throw Error(BG_E_IO, "short write to " + path);
}

void write_words(const std::string& path, const std::vector<uint32_t>& w) { write_file(path, w.data(), w.size() * 4); }

}  // namespace

void synth_square_chain(Ctx& c, uint32_t log2n, uint64_t seed, const std::string& dir) {
  if (log2n < 1 || log2n > 24) throw Error(BG_E_ARG, "synth: log2n must be in 1..24");
  const uint64_t N = 1ull << log2n;
  const uint32_t ni = 2, nw = (uint32_t)N;
  uint32_t lg = 0;
  while ((1ull << lg) < N + ni) lg++;
  const uint64_t d = 1ull << lg;
  SplitMix rng{seed};
  const Fe x0 = rng.fr();
  const Fe tau = rng.fr(), alpha = rng.fr(), beta = rng.fr(), gamma = rng.fr(), delta = rng.fr();
  const Fe r = rng.fr(), s = rng.fr();
  const Fe one = bgh::fe_one(FR);

  // witness z = [1, x_N, x_0 .. x_{N-1}] (Montgomery)
  std::vector<Fe> xs(N + 1);
  xs[0] = mont(x0);
  for (uint64_t i = 0; i < N; i++) xs[i + 1] = bgh::fe_sqr(FR, xs[i]);
  std::vector<uint32_t> wit;
  wit.reserve((N + 2) * 16);
  put_fe_wire(wit, one);
  put_fe_wire(wit, xs[N]);
  for (uint64_t i = 0; i < N; i++) put_fe_wire(wit, xs[i]);

  // Lagrange basis at tau over the size-d domain: L_k = Z(tau) w^k / (d (tau - w^k))
  Fe w = mont(Fe{{0x9bd61b6e725b19f0ull, 0x402d111e41112ed4ull, 0x00e0a7eb8ef62abcull, 0x2a3c09f0a58a7e85ull}});
  for (uint32_t i = lg; i < 28; i++) w = bgh::fe_sqr(FR, w);
  const Fe taum = mont(tau);
  const Fe zt = bgh::fe_sub(FR, bgh::fe_pow_u64(FR, taum, d), one);
  const Fe dinv_dom = bgh::fe_inv(FR, mont(bgh::fe_raw(d)));
  std::vector<Fe> wk(d), den(d);
  Fe acc = one;
  for (uint64_t k = 0; k < d; k++) {
    wk[k] = acc;
    den[k] = bgh::fe_sub(FR, taum, acc);
    acc = bgh::fe_mul(FR, acc, w);
  }
  batch_inverse(den);
  const Fe zd = bgh::fe_mul(FR, zt, dinv_dom);
  auto lag = [&](uint64_t k) { return bgh::fe_mul(FR, bgh::fe_mul(FR, zd, wk[k]), den[k]); };

  const uint64_t m = ni + nw;
  std::vector<Fe> A(m, bgh::fe_zero()), B(m, bgh::fe_zero()), C(m, bgh::fe_zero());
  for (uint64_t i = 0; i < N; i++) {
    const Fe li = lag(i);
    A[2 + i] = bgh::fe_add(FR, A[2 + i], li);
    B[2 + i] = bgh::fe_add(FR, B[2 + i], li);
    const uint64_t ccol = (i + 1 < N) ? 3 + i : 1;
    C[ccol] = bgh::fe_add(FR, C[ccol], li);
  }
  for (uint64_t i = 0; i < ni; i++) A[i] = bgh::fe_add(FR, A[i], lag(N + i));

  const Fe am = mont(alpha), bm = mont(beta), dm = mont(delta);
  const Fe dinv = bgh::fe_inv(FR, dm);
  std::vector<Fe> ka(m), kb(m), kh(d - 1), kl(nw);
  for (uint64_t j = 0; j < m; j++) {
    ka[j] = canon(A[j]);
    kb[j] = canon(B[j]);
  }
  Fe tp = bgh::fe_mul(FR, zt, dinv);
  for (uint64_t k = 0; k + 1 < d; k++) {
    kh[k] = canon(tp);
    tp = bgh::fe_mul(FR, tp, taum);
  }
  for (uint64_t j = 0; j < nw; j++) {
    Fe v = bgh::fe_add(FR, bgh::fe_mul(FR, bm, A[2 + j]), bgh::fe_mul(FR, am, B[2 + j]));
    v = bgh::fe_add(FR, v, C[2 + j]);
    kl[j] = canon(bgh::fe_mul(FR, v, dinv));
  }
  // verifying key: IC_i = (beta A_i + alpha B_i + C_i)(tau) / gamma for the instance columns
  const Fe ginv = bgh::fe_inv(FR, mont(gamma));
  std::vector<Fe> kic(ni);
  for (uint64_t i = 0; i < ni; i++) {
    Fe v = bgh::fe_add(FR, bgh::fe_mul(FR, bm, A[i]), bgh::fe_mul(FR, am, B[i]));
    v = bgh::fe_add(FR, v, C[i]);
    kic[i] = canon(bgh::fe_mul(FR, v, ginv));
  }

  // generators (canonical coordinates -> Montgomery)
  bgh::Aff<bgh::FqOps> g1;
  g1.x = bgh::fe_to_mont(bgh::FQ, bgh::fe_raw(1));
  g1.y = bgh::fe_to_mont(bgh::FQ, bgh::fe_raw(2));
  g1.inf = false;
  bgh::Aff<bgh::Fq2Ops> g2;
  g2.x.c0 = bgh::fe_to_mont(bgh::FQ, Fe{{0x46debd5cd992f6edull, 0x674322d4f75edaddull, 0x426a00665e5c4479ull,
                                         0x1800deef121f1e76ull}});
  g2.x.c1 = bgh::fe_to_mont(bgh::FQ, Fe{{0x97e485b7aef312c2ull, 0xf1aa493335a9e712ull, 0x7260bfb731fb5d25ull,
                                         0x198e9393920d483aull}});
  g2.y.c0 = bgh::fe_to_mont(bgh::FQ, Fe{{0x4ce6cc0166fa7daaull, 0xe3d1e7690c43d37bull, 0x4aab71808dcb408full,
                                         0x12c85ea5db8c6debull}});
  g2.y.c1 = bgh::fe_to_mont(bgh::FQ, Fe{{0x55acdadcd122975bull, 0xbc4b313370b38ef3ull, 0xec9e99ad690c3395ull,
                                         0x090689d0585ff075ull}});
  g2.inf = false;
  const auto t1 = fixed_base_table<bgh::FqOps>(g1);
  const auto t2 = fixed_base_table<bgh::Fq2Ops>(g2);

  auto pa = device_fixed_base<Fq, bgh::FqOps>(c, t1, ka);
  auto pb1 = device_fixed_base<Fq, bgh::FqOps>(c, t1, kb);
  auto pb2 = device_fixed_base<Fq2, bgh::Fq2Ops>(c, t2, kb);
  auto ph = device_fixed_base<Fq, bgh::FqOps>(c, t1, kh);
  auto pl = device_fixed_base<Fq, bgh::FqOps>(c, t1, kl);
  auto pg1 = device_fixed_base<Fq, bgh::FqOps>(c, t1, {alpha, beta, delta});
  auto pg2 = device_fixed_base<Fq2, bgh::Fq2Ops>(c, t2, {beta, delta});
  // vk.bin: alpha_g1, beta_g2, gamma_g2, delta_g2, u32 n_ic, IC_0 .. IC_{n_ic-1}
  std::vector<uint32_t> vk = device_fixed_base<Fq, bgh::FqOps>(c, t1, {alpha});
  const auto vk2 = device_fixed_base<Fq2, bgh::Fq2Ops>(c, t2, {beta, gamma, delta});
  const auto vkic = device_fixed_base<Fq, bgh::FqOps>(c, t1, kic);
  vk.insert(vk.end(), vk2.begin(), vk2.end());
  vk.push_back(ni);
  vk.insert(vk.end(), vkic.begin(), vkic.end());

  // CSR files: nnz; offsets[N+1]; (col, coeff = Montgomery one) per entry
  auto csr = [&](int which) {
    std::vector<uint32_t> f;
    f.reserve(2 + N + 17 * N);
    f.push_back((uint32_t)N);
    for (uint64_t i = 0; i <= N; i++) f.push_back((uint32_t)i);
    for (uint64_t i = 0; i < N; i++) {
      const uint32_t col = which < 2 ? (uint32_t)(2 + i) : (i + 1 < N ? (uint32_t)(3 + i) : 1u);
      f.push_back(col);
      put_fe_wire(f, one);
    }
    return f;
  };
  const std::vector<uint32_t> header = {(uint32_t)N, ni, nw, lg, (uint32_t)m, (uint32_t)m, (uint32_t)(d - 1), nw};
  std::vector<uint32_t> rs;
  put_fe_wire(rs, mont(r));
  put_fe_wire(rs, mont(s));
  std::vector<uint32_t> trap;
  for (const Fe& v : {tau, alpha, beta, gamma, delta}) put_fe_wire(trap, v);

  write_words(dir + "/header.bin", header);
  write_words(dir + "/witness.bin", wit);
  write_words(dir + "/r1cs_a.bin", csr(0));
  write_words(dir + "/r1cs_b.bin", csr(1));
  write_words(dir + "/r1cs_c.bin", csr(2));
  write_words(dir + "/pk_g1.bin", pg1);
  write_words(dir + "/pk_g2.bin", pg2);
  write_words(dir + "/pk_a.bin", pa);
  write_words(dir + "/pk_b1.bin", pb1);
  write_words(dir + "/pk_b2.bin", pb2);
  write_words(dir + "/pk_h.bin", ph);
  write_words(dir + "/pk_l.bin", pl);
  write_words(dir + "/rs.bin", rs);
  write_words(dir + "/trapdoor.bin", trap);
  write_words(dir + "/vk.bin", vk);
}

}  // namespace bg
