// Radix-2 NTTs over BN254 Fr and the Groth16 QAP quotient h(x).
//
// Reference semantics: Ntt.fft / ifft / coset_fft (bend2/src/ntt.bend:431-438) over
// arkworks' Radix2EvaluationDomain (generator w = root^(2^(28-L)), ntt.bend:73-74), and
// Ntt.qap_h (ntt.bend:446-459) = ark-groth16 LibsnarkReduction:
//   h = coset_iNTT((coset_NTT(iNTT a) * coset_NTT(iNTT b) - coset_NTT(iNTT c)) / (g^d - 1)),
// with g = 5 (bend2/gen/ref_qap.py:59-72).  The reference runs log2(d) Stockham stages on a
// chunk tree with running-product twiddles (ntt.bend:1-18).
//
// Here a transform is a few passes over HBM/L2; each pass loads a tile of up to 1024
// elements into shared memory (limb-major, so a warp's 32 butterflies hit 32 banks), runs up
// to 10 radix-2 stages there with twiddles from a resident table, and writes the tile back.
// 1024-element tiles (32 KiB) give a 2^19 transform 512 CTAs instead of 256 with 64 KiB
// tiles: measured 2^19 0.219 -> 0.210 ms, 2^20 0.407 -> 0.360 ms.
//   DIF (Gentleman-Sande): natural order in -> bit-reversed out (used for inverse transforms)
//   DIT (Cooley-Tukey):    bit-reversed in -> natural order out (forward transforms)
// so iNTT followed by a coset NTT needs no permutation: the coset factor g^j of coefficient j
// is applied in bit-reversed position, fused with n^-1 into the last DIF pass.  Only the final
// h needs one bit-reversal gather.
#include <mutex>

#include "common.cuh"
#include "fp.cuh"
#include "host_ff.hpp"
#include "ntt.h"

namespace bg {

constexpr int kNttThreads = 256;
constexpr int kNttTile = 1024;   // elements per CTA tile (32 KiB of shared memory)
constexpr int kContigMax = 10;   // stages in one pass, contiguous or strided (a 1024-element tile)

enum ScaleMode { SC_NONE = 0, SC_NATURAL = 1, SC_BITREV = 2, SC_CONST = 3 };

struct ScaleTab {
  const uint32_t* lo = nullptr;  // T(i) = lo[i & (2^bits-1)] * hi[i >> bits]
  const uint32_t* hi = nullptr;
  int bits = 0;
};

// a b as the 512-bit Karatsuba product and one Montgomery reduction (232 multiply-adds instead
// of CIOS's 264; the inputs are below r, so the product is below r R): 2^20 forward transform
// 0.357 -> 0.352 ms, bit-identical.  Stage-pair register blocks (radix-4 sets, half the
// shared-memory round trips) were measured slower, 0.40 ms.
BG_DEV Fr mul_kara(const Fr& a, const Fr& b) {
  Wide t;
  wide_mul(t, a.v, b.v);
  return redc<FrParams>(t);
}

BG_DEV Fr scale_factor(int mode, size_t j, int L, const ScaleTab& t) {
  if (mode == SC_CONST) return load_fp<FrParams>(t.hi);
  size_t i = j;
  if (mode == SC_BITREV) i = __brevll((unsigned long long)j) >> (64 - L);
  const Fr a = load_fp<FrParams>(t.lo + 8 * (i & ((size_t(1) << t.bits) - 1)));
  const Fr b = load_fp<FrParams>(t.hi + 8 * (i >> t.bits));
  return mul(a, b);
}

// The tile in shared memory: element e's low and high 16 bytes at uint4 slot e of two arrays
// of E slots, so an element moves in two 128-bit accesses.  The pass is bound by instruction
// issue, and a limb-major tile took eight 32-bit accesses per element for the same wavefronts:
// 2^20 forward transform 0.362 -> 0.333 ms (76 registers, 3 CTAs per SM; forcing 4 CTAs per SM
// at 64 registers spills and measured the same 0.332 ms).
BG_DEV void tile_store(uint32_t* sm, int E, int e, const Fr& x) {
  uint4* lo = reinterpret_cast<uint4*>(sm);
  lo[e] = make_uint4(x.v[0], x.v[1], x.v[2], x.v[3]);
  lo[E + e] = make_uint4(x.v[4], x.v[5], x.v[6], x.v[7]);
}
BG_DEV Fr tile_load(const uint32_t* sm, int E, int e) {
  const uint4* lo = reinterpret_cast<const uint4*>(sm);
  const uint4 a = lo[e], b = lo[E + e];
  Fr x;
  x.v[0] = a.x; x.v[1] = a.y; x.v[2] = a.z; x.v[3] = a.w;
  x.v[4] = b.x; x.v[5] = b.y; x.v[6] = b.z; x.v[7] = b.w;
  return x;
}

// One pass: stages [s0, s0 + k) of a size-2^L transform.  A CTA owns G independent groups of
// 2^k elements; group element t of group (hi, lo) sits at hi*2^(s0+k) + t*2^s0 + lo.
// Up to three vectors transformed by one launch (the QAP's a, b and c), blockIdx.y picks one.
struct NttVecs {
  uint32_t* p[3];
};

template <bool DIT, int NT>
__global__ void __launch_bounds__(NT) k_ntt_pass(NttVecs vecs, const uint32_t* __restrict__ tw, int L, int s0, int k,
                                                 int G, int pre_mode, int post_mode, ScaleTab sc) {
  extern __shared__ __align__(16) uint32_t sm[];
  uint32_t* __restrict__ data = vecs.p[blockIdx.y];
  const int E = G << k;
  const uint32_t kmask = (1u << k) - 1u;
  const size_t lomask = (size_t(1) << s0) - 1;
  const size_t gid0 = (size_t)blockIdx.x * G;

  for (int idx = threadIdx.x; idx < E; idx += blockDim.x) {
    int grp, t;
    if (s0 == 0) {
      grp = idx >> k;
      t = idx & kmask;
    } else {
      grp = idx % G;
      t = idx / G;
    }
    const size_t gid = gid0 + grp;
    const size_t j = (s0 == 0) ? ((gid << k) | (size_t)t)
                               : (((gid >> s0) << (s0 + k)) | ((size_t)t << s0) | (gid & lomask));
    Fr x = load_fp<FrParams>(data + 8 * j);
    if (pre_mode != SC_NONE) x = mul(x, scale_factor(pre_mode, j, L, sc));
    tile_store(sm, E, (grp << k) | t, x);
  }
  __syncthreads();

  const int half = E >> 1;
  for (int rr = 0; rr < k; rr++) {
    const int r = DIT ? rr : (k - 1 - rr);
    const int s = s0 + r;
    const uint32_t rmask = (1u << r) - 1u;
    for (int b = threadIdx.x; b < half; b += blockDim.x) {
      const int grp = b >> (k - 1);
      const uint32_t q = (uint32_t)b & ((1u << (k - 1)) - 1u);
      const uint32_t t1 = ((q >> r) << (r + 1)) | (q & rmask);
      const uint32_t t2 = t1 | (1u << r);
      const size_t lo = (s0 == 0) ? 0 : ((gid0 + grp) & lomask);
      const size_t widx = ((((size_t)(q & rmask)) << s0) + lo) << (L - s - 1);
      const int e1 = (grp << k) | (int)t1, e2 = (grp << k) | (int)t2;
      Fr x1 = tile_load(sm, E, e1), x2 = tile_load(sm, E, e2);
      Fr y1, y2;
      if (widx == 0) {  // w = 1
        y1 = add(x1, x2);
        y2 = sub(x1, x2);
      } else {
        const Fr w = load_fp<FrParams>(tw + 8 * widx);
        if (DIT) {
          x2 = mul_kara(x2, w);
          y1 = add(x1, x2);
          y2 = sub(x1, x2);
        } else {
          y1 = add(x1, x2);
          y2 = mul_kara(sub(x1, x2), w);
        }
      }
      tile_store(sm, E, e1, y1);
      tile_store(sm, E, e2, y2);
    }
    __syncthreads();
  }

  for (int idx = threadIdx.x; idx < E; idx += blockDim.x) {
    int grp, t;
    if (s0 == 0) {
      grp = idx >> k;
      t = idx & kmask;
    } else {
      grp = idx % G;
      t = idx / G;
    }
    const size_t gid = gid0 + grp;
    const size_t j = (s0 == 0) ? ((gid << k) | (size_t)t)
                               : (((gid >> s0) << (s0 + k)) | ((size_t)t << s0) | (gid & lomask));
    Fr x = tile_load(sm, E, (grp << k) | t);
    if (post_mode != SC_NONE) x = mul(x, scale_factor(post_mode, j, L, sc));
    store_fp(data + 8 * j, x);
  }
}

// out[i] = lo[i & (2^bits - 1)] * hi[i >> bits]
__global__ void k_table_expand(uint32_t* __restrict__ out, const uint32_t* __restrict__ lo,
                               const uint32_t* __restrict__ hi, int bits, size_t n) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const Fr a = load_fp<FrParams>(lo + 8 * (i & ((size_t(1) << bits) - 1)));
  const Fr b = load_fp<FrParams>(hi + 8 * (i >> bits));
  store_fp(out + 8 * i, mul(a, b));
}

// out[bitrev_L(i)] = in[i]
__global__ void k_bitrev(const uint32_t* __restrict__ in, uint32_t* __restrict__ out, int L, size_t n) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const size_t j = L ? (__brevll((unsigned long long)i) >> (64 - L)) : 0;
  store_fp(out + 8 * j, load_fp<FrParams>(in + 8 * i));
}

// a[i] = (a[i] * b[i] - c[i]) * zinv
__global__ void k_qap_pointwise(uint32_t* __restrict__ a, const uint32_t* __restrict__ b,
                                const uint32_t* __restrict__ c, const uint32_t* __restrict__ zinv, size_t n) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const Fr x = load_fp<FrParams>(a + 8 * i), y = load_fp<FrParams>(b + 8 * i), z = load_fp<FrParams>(c + 8 * i);
  store_fp(a + 8 * i, mul(sub(mul(x, y), z), load_fp<FrParams>(zinv)));
}

// ---------------------------------------------------------------- host side
using bgh::Fe;
using bgh::FR;

// 2-adic root of unity of order 2^28 (canonical; bend2/gen/gen_ntt.py:11)
static const Fe kRootCanonical{{0x9bd61b6e725b19f0ull, 0x402d111e41112ed4ull, 0x00e0a7eb8ef62abcull,
                                0x2a3c09f0a58a7e85ull}};

static Fe fr_mont_u64(uint64_t x) { return bgh::fe_to_mont(FR, bgh::fe_raw(x)); }

static Fe omega_mont(int L) {
  Fe w = bgh::fe_to_mont(FR, kRootCanonical);
  for (int i = L; i < 28; i++) w = bgh::fe_sqr(FR, w);
  return w;
}

static void upload_fes(Ctx& ctx, uint32_t* d, const std::vector<Fe>& v) {
  std::vector<uint32_t> words(v.size() * 8);
  for (size_t i = 0; i < v.size(); i++) bgh::fe_to_words32(words.data() + 8 * i, v[i]);
  BG_CUDA(cudaMemcpyAsync(d, words.data(), words.size() * 4, cudaMemcpyHostToDevice, ctx.stream));
  ctx.h2d_bytes += words.size() * 4;
  BG_CUDA(cudaStreamSynchronize(ctx.stream));
}

static std::vector<Fe> powers(const Fe& base, size_t n, const Fe& first) {
  std::vector<Fe> out(n);
  Fe x = first;
  for (size_t i = 0; i < n; i++) {
    out[i] = x;
    x = bgh::fe_mul(FR, x, base);
  }
  return out;
}

NttTables& ntt_tables(Ctx& ctx, int L) {
  NttTables& slot = ctx.ntt_tabs[L];
  if (slot.ready) return slot;
  const size_t n = size_t(1) << L;
  const size_t half = n > 1 ? n / 2 : 1;
  const std::string tag = "ntt" + std::to_string(L);
  slot.tw_fwd = ctx.ws.get_t<uint32_t>(tag + ".tw_fwd", half * 8);
  slot.tw_inv = ctx.ws.get_t<uint32_t>(tag + ".tw_inv", half * 8);
  const Fe one = bgh::fe_one(FR);
  const Fe w = omega_mont(L);
  const Fe winv = bgh::fe_inv(FR, w);
  // twiddles: two-level expansion lo (2^10) x hi
  const int tb = 10;
  const size_t nlo = std::min(half, size_t(1) << tb);
  const size_t nhi = (half + nlo - 1) / nlo;
  uint32_t* tmp_lo = ctx.ws.get_t<uint32_t>(tag + ".tmp_lo", nlo * 8);
  uint32_t* tmp_hi = ctx.ws.get_t<uint32_t>(tag + ".tmp_hi", nhi * 8);
  const int lo_bits = (nlo == 1) ? 0 : tb;
  for (int dir = 0; dir < 2; dir++) {
    const Fe base = dir == 0 ? w : winv;
    Fe step = base;
    for (int i = 0; i < lo_bits; i++) step = bgh::fe_sqr(FR, step);
    upload_fes(ctx, tmp_lo, powers(base, nlo, one));
    upload_fes(ctx, tmp_hi, powers(step, nhi, one));
    k_table_expand<<<ceil_div(half, 256), 256, 0, ctx.stream>>>(dir == 0 ? slot.tw_fwd : slot.tw_inv, tmp_lo,
                                                                  tmp_hi, lo_bits, half);
    BG_CHECK_LAUNCH();
  }
  // coset tables: g^i, g^-i (lo), and n^-1 * g^(i 2^a), n^-1 * g^(-i 2^a) (hi), plain g^(i 2^a) for
  // the natural-order coset NTT
  const int a = (L + 1) / 2;
  const size_t clo = size_t(1) << a, chi = size_t(1) << (L - a);
  const Fe g = fr_mont_u64(5);
  const Fe ginv = bgh::fe_inv(FR, g);
  const Fe ninv = bgh::fe_inv(FR, fr_mont_u64(n));
  Fe ga = g, gia = ginv;
  for (int i = 0; i < a; i++) {
    ga = bgh::fe_sqr(FR, ga);
    gia = bgh::fe_sqr(FR, gia);
  }
  slot.coset_bits = a;
  slot.g_lo = ctx.ws.get_t<uint32_t>(tag + ".g_lo", clo * 8);
  slot.gi_lo = ctx.ws.get_t<uint32_t>(tag + ".gi_lo", clo * 8);
  slot.g_hi = ctx.ws.get_t<uint32_t>(tag + ".g_hi", chi * 8);
  slot.g_hi_ninv = ctx.ws.get_t<uint32_t>(tag + ".g_hi_ninv", chi * 8);
  slot.gi_hi_ninv = ctx.ws.get_t<uint32_t>(tag + ".gi_hi_ninv", chi * 8);
  slot.ninv = ctx.ws.get_t<uint32_t>(tag + ".ninv", 8);
  slot.zinv = ctx.ws.get_t<uint32_t>(tag + ".zinv", 8);
  upload_fes(ctx, slot.g_lo, powers(g, clo, one));
  upload_fes(ctx, slot.gi_lo, powers(ginv, clo, one));
  upload_fes(ctx, slot.g_hi, powers(ga, chi, one));
  upload_fes(ctx, slot.g_hi_ninv, powers(ga, chi, ninv));
  upload_fes(ctx, slot.gi_hi_ninv, powers(gia, chi, ninv));
  upload_fes(ctx, slot.ninv, {ninv});
  // Z(g x) on the coset is the constant g^n - 1
  const Fe zc = bgh::fe_sub(FR, bgh::fe_pow_u64(FR, g, n), one);
  upload_fes(ctx, slot.zinv, {bgh::fe_inv(FR, zc)});
  slot.ready = true;
  return slot;
}

struct PassPlan {
  int s0, k, G;
  int nt = kNttThreads;  // threads per CTA
};

// Small domains (at most 2^kSmallMaxL elements, a small proof's QAP) are a chain of
// latency-bound transforms: they take 128-element tiles of 64 threads, one butterfly per thread
// per stage and at most 7 stages per pass, so a pass spreads over many SMs.  The 1024-element
// tiles give a 2^11 transform two passes of two CTAs each, every thread doing two butterflies
// per stage; one CTA of 1024 threads over the whole vector measured 60-70 us per transform,
// the SM's issue rate spread over 1024 butterflies a stage.
constexpr int kSmallMaxL = 14;
constexpr int kSmallTile = 128;

static std::vector<PassPlan> plan_passes(int L) {
  const bool small = L <= kSmallMaxL;
  const int tile = small ? kSmallTile : kNttTile;
  const int kmax = small ? 7 : kContigMax;
  std::vector<PassPlan> out;
  auto add = [&](int s0, int k, int G) {
    PassPlan p{s0, k, G};
    p.nt = small ? std::max(32, (G << k) / 2) : kNttThreads;
    out.push_back(p);
  };
  const int k0 = std::min(L, kmax);
  {
    int G = tile >> k0;
    const int groups = 1 << (L - k0);
    if (G > groups) G = groups;
    if (G < 1) G = 1;
    add(0, k0, G);
  }
  int rest = L - k0;
  int s0 = k0;
  const int npass = (rest + kmax - 1) / kmax;
  for (int p = 0; p < npass; p++) {
    const int k = (rest + (npass - p) - 1) / (npass - p);
    int G = tile >> k;
    const int lo_count = 1 << s0;
    if (G > lo_count) G = lo_count;
    add(s0, k, G);
    s0 += k;
    rest -= k;
  }
  return out;
}

static void launch_pass(Ctx& ctx, cudaStream_t st, bool dit, const NttVecs& v, int nvec, const uint32_t* tw, int L,
                        const PassPlan& p, int pre, int post, const ScaleTab& sc) {
  const size_t n = size_t(1) << L;
  const int E = p.G << p.k;
  const dim3 grid((unsigned)(n / E), (unsigned)nvec);
  const size_t smem = (size_t)E * 32;
  KernelTimer kt(ctx, "ntt_pass", st);
  if (dit) k_ntt_pass<true, kNttThreads><<<grid, p.nt, smem, st>>>(v, tw, L, p.s0, p.k, p.G, pre, post, sc);
  else k_ntt_pass<false, kNttThreads><<<grid, p.nt, smem, st>>>(v, tw, L, p.s0, p.k, p.G, pre, post, sc);
  BG_CHECK_LAUNCH();
}

// the opt-in to 32 KiB of dynamic shared memory holds for the device current when it is set:
// once per device, safely from several host threads (batch lanes, server threads)
void ntt_init_kernels() {
  constexpr int kMaxDevices = 64;
  static std::once_flag once[kMaxDevices];
  int dev = 0;
  BG_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) throw Error(BG_E_ARG, "ntt: device index out of range");
  std::call_once(once[dev], [] {
    BG_CUDA(cudaFuncSetAttribute(k_ntt_pass<true, kNttThreads>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 kNttTile * 32));
    BG_CUDA(cudaFuncSetAttribute(k_ntt_pass<false, kNttThreads>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 kNttTile * 32));
  });
}

// DIF passes (natural -> bit-reversed).  `first_pre` scales on load in the first pass;
// `last_post` scales on store in the last (contiguous) pass.
static void dif(Ctx& ctx, cudaStream_t st, const NttVecs& v, int nvec, const uint32_t* tw, int L, int first_pre,
                const ScaleTab& pre_sc, int last_post, const ScaleTab& post_sc) {
  auto plan = plan_passes(L);
  for (int i = (int)plan.size() - 1; i >= 0; i--) {
    const bool first = i == (int)plan.size() - 1, last = i == 0;
    if (first && last) {
      // one pass: both scalings come from different tables; apply pre separately if needed
      if (first_pre != SC_NONE && last_post != SC_NONE)
        throw Error(BG_E_ARG, "ntt: pre and post scaling in a single-pass transform");
      launch_pass(ctx, st, false, v, nvec, tw, L, plan[i], first_pre, last_post, first_pre ? pre_sc : post_sc);
    } else {
      launch_pass(ctx, st, false, v, nvec, tw, L, plan[i], first ? first_pre : SC_NONE, last ? last_post : SC_NONE,
                  first ? pre_sc : post_sc);
    }
  }
}

static void dit(Ctx& ctx, cudaStream_t st, const NttVecs& v, int nvec, const uint32_t* tw, int L) {
  auto plan = plan_passes(L);
  for (size_t i = 0; i < plan.size(); i++)
    launch_pass(ctx, st, true, v, nvec, tw, L, plan[i], SC_NONE, SC_NONE, ScaleTab{});
}

void ntt_run(Ctx& ctx, cudaStream_t st, uint32_t* d_data, int L, int mode) {
  if (L == 0) return;
  ntt_init_kernels();
  NttTables& T = ntt_tables(ctx, L);
  const size_t n = size_t(1) << L;
  uint32_t* tmp = ctx.ws.get_t<uint32_t>("ntt.tmp", n * 8);
  ScaleTab none;
  const NttVecs v{{d_data, d_data, d_data}};
  switch (mode) {
    case BG_NTT_FORWARD:
      dif(ctx, st, v, 1, T.tw_fwd, L, SC_NONE, none, SC_NONE, none);
      break;
    case BG_NTT_INVERSE: {
      ScaleTab c;
      c.hi = T.ninv;
      dif(ctx, st, v, 1, T.tw_inv, L, SC_NONE, none, SC_CONST, c);
      break;
    }
    case BG_NTT_COSET_FORWARD: {
      ScaleTab c{T.g_lo, T.g_hi, T.coset_bits};
      dif(ctx, st, v, 1, T.tw_fwd, L, SC_NATURAL, c, SC_NONE, none);
      break;
    }
    case BG_NTT_COSET_INVERSE: {
      ScaleTab c{T.gi_lo, T.gi_hi_ninv, T.coset_bits};
      dif(ctx, st, v, 1, T.tw_inv, L, SC_NONE, none, SC_BITREV, c);
      break;
    }
    default:
      throw Error(BG_E_ARG, "ntt: unknown mode");
  }
  k_bitrev<<<ceil_div(n, 256), 256, 0, st>>>(d_data, tmp, L, n);
  BG_CHECK_LAUNCH();
  BG_CUDA(cudaMemcpyAsync(d_data, tmp, n * 32, cudaMemcpyDeviceToDevice, st));
}

// h from the three evaluation vectors (all natural order, packed Montgomery, n = 2^L each).
// a, b, c are overwritten; h receives n elements (h[n-1] = 0 for a satisfied R1CS).
void qap_h_run(Ctx& ctx, cudaStream_t st, uint32_t* d_a, uint32_t* d_b, uint32_t* d_c, uint32_t* d_h, int L) {
  ntt_init_kernels();
  NttTables& T = ntt_tables(ctx, L);
  const size_t n = size_t(1) << L;
  ScaleTab none;
  ScaleTab to_coset{T.g_lo, T.g_hi_ninv, T.coset_bits};
  ScaleTab from_coset{T.gi_lo, T.gi_hi_ninv, T.coset_bits};
  // a, b and c are transformed by the same launches (grid y = 3): each pass fills three times
  // the CTAs, and a small proof's QAP is 8 launches instead of 16
  const NttVecs abc{{d_a, d_b, d_c}};
  dif(ctx, st, abc, 3, T.tw_inv, L, SC_NONE, none, SC_BITREV, to_coset);  // iNTT, then * n^-1 g^j
  dit(ctx, st, abc, 3, T.tw_fwd, L);                                      // NTT on the coset
  k_qap_pointwise<<<ceil_div(n, 256), 256, 0, st>>>(d_a, d_b, d_c, T.zinv, n);
  BG_CHECK_LAUNCH();
  const NttVecs a{{d_a, d_a, d_a}};
  dif(ctx, st, a, 1, T.tw_inv, L, SC_NONE, none, SC_BITREV, from_coset);  // coset iNTT
  k_bitrev<<<ceil_div(n, 256), 256, 0, st>>>(d_a, d_h, L, n);
  BG_CHECK_LAUNCH();
}

}  // namespace bg
