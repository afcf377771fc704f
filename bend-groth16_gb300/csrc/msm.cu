// Pippenger multi-scalar multiplication sum_i s_i * P_i over BN254 G1 (Fq) and G2 (Fq2).
//
// Reference semantics: Msm.g1 / Msm.g2 (bend2/src/msm.bend:297, :529) take n affine
// Montgomery points and n canonical scalars and return the sum as a Jacobian point; the
// caller normalises it (bend2/src/groth16.bend:281-295).  The reference runs unsigned c-bit
// windows (msm.bend:34-58), private per-leaf bucket arrays joined element-wise (:158-173),
// a running-sum reduction per window (:192-205) and a Horner window combine (:225-239).
//
// This implementation (one device, all phases on the device except the final Horner):
//   1. k_digits_hist  signed c-bit digits (|d| <= 2^(c-1)), one thread per scalar; a global
//                     histogram of (window, |d|-1) bucket keys
//   2. exclusive scan of the histogram -> bucket offsets
//   3. k_scatter      (point index | sign << 31) written into bucket order
//   4. k_bucket_acc   one thread per bucket: XYZZ accumulator += +-P (mixed add)
//   5. k_reduce_level hierarchical running sums: sum_b (b+1) B_b per window, segments of
//                     L buckets per thread, log_L(2^(c-1)) levels
//   6. host: W window sums -> Horner with c doublings per window -> affine.
// Window sums and the final point are exact group elements, so the affine result equals the
// reference's for the same inputs regardless of bucket order inside a window.
#include "common.cuh"
#include "ec.cuh"
#include "host_ff.hpp"
#include "msm.h"

namespace bg {

// ---------------------------------------------------------------- scan (exclusive, u32)
constexpr int kScanThreads = 256;
constexpr int kScanItems = 8;
constexpr int kScanTile = kScanThreads * kScanItems;

__global__ void k_scan_tile(const uint32_t* __restrict__ in, uint32_t* __restrict__ out,
                            uint32_t* __restrict__ tile_sums, size_t n) {
  __shared__ uint32_t warp_tot[kScanThreads / 32];
  const size_t base = (size_t)blockIdx.x * kScanTile + (size_t)threadIdx.x * kScanItems;
  uint32_t v[kScanItems];
  uint32_t sum = 0;
#pragma unroll
  for (int k = 0; k < kScanItems; k++) {
    v[k] = (base + k < n) ? in[base + k] : 0u;
    sum += v[k];
  }
  // inclusive warp scan of per-thread sums
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  uint32_t x = sum;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) warp_tot[wid] = x;
  __syncthreads();
  if (wid == 0) {
    uint32_t t = lane < kScanThreads / 32 ? warp_tot[lane] : 0u;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      uint32_t y = __shfl_up_sync(0xffffffffu, t, o);
      if (lane >= o) t += y;
    }
    if (lane < kScanThreads / 32) warp_tot[lane] = t;  // inclusive
  }
  __syncthreads();
  uint32_t excl = x - sum + (wid > 0 ? warp_tot[wid - 1] : 0u);
#pragma unroll
  for (int k = 0; k < kScanItems; k++) {
    if (base + k < n) out[base + k] = excl;
    excl += v[k];
  }
  if (threadIdx.x == kScanThreads - 1 && tile_sums) tile_sums[blockIdx.x] = excl;
}

__global__ void k_scan_add(uint32_t* __restrict__ out, const uint32_t* __restrict__ tile_off, size_t n) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] += tile_off[i / kScanTile];
}

// exclusive scan of n u32 (n >= 1); recursion depth log_2048(n)
void exclusive_scan(Workspace& ws, const std::string& tag, const uint32_t* d_in, uint32_t* d_out, size_t n,
                    cudaStream_t st, int depth) {
  const unsigned tiles = ceil_div(n, kScanTile);
  if (tiles == 1) {
    k_scan_tile<<<1, kScanThreads, 0, st>>>(d_in, d_out, nullptr, n);
    BG_CHECK_LAUNCH();
    return;
  }
  uint32_t* sums = ws.get_t<uint32_t>(tag + ".scan_sums" + std::to_string(depth), tiles);
  uint32_t* offs = ws.get_t<uint32_t>(tag + ".scan_offs" + std::to_string(depth), tiles);
  k_scan_tile<<<tiles, kScanThreads, 0, st>>>(d_in, d_out, sums, n);
  BG_CHECK_LAUNCH();
  exclusive_scan(ws, tag, sums, offs, tiles, st, depth + 1);
  k_scan_add<<<ceil_div(n, 256), 256, 0, st>>>(d_out, offs, n);
  BG_CHECK_LAUNCH();
}

// ---------------------------------------------------------------- digits
BG_DEV uint32_t window_bits(const uint32_t* s, int bit, int c) {
  const int limb = bit >> 5, sh = bit & 31;
  if (limb >= 8) return 0u;
  uint64_t v = s[limb];
  if (limb + 1 < 8) v |= (uint64_t)s[limb + 1] << 32;
  return (uint32_t)(v >> sh) & ((1u << c) - 1u);
}

BG_DEV void load_scalar(uint32_t* s, const uint32_t* __restrict__ scalars, size_t i) {
  const uint4 a = reinterpret_cast<const uint4*>(scalars + 8 * i)[0];
  const uint4 b = reinterpret_cast<const uint4*>(scalars + 8 * i)[1];
  s[0] = a.x; s[1] = a.y; s[2] = a.z; s[3] = a.w;
  s[4] = b.x; s[5] = b.y; s[6] = b.z; s[7] = b.w;
}

// signed digit of window w: returns magnitude (0 = no bucket) and updates carry; *neg set
// when the digit is negative.  Digits lie in [-(2^(c-1) - 1), 2^(c-1)].
BG_DEV uint32_t signed_digit(const uint32_t* s, int w, int c, uint32_t& carry, bool& negd) {
  const uint32_t half = 1u << (c - 1);
  const uint32_t d = window_bits(s, w * c, c) + carry;
  if (d > half) {
    carry = 1u;
    negd = true;
    return (1u << c) - d;
  }
  carry = 0u;
  negd = false;
  return d;
}

__global__ void k_digits_hist(const uint32_t* __restrict__ scalars, size_t n, int c, int W,
                              uint32_t* __restrict__ counts, uint32_t* __restrict__ status) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  uint32_t s[8];
  load_scalar(s, scalars, i);
  if (s[7] >> 30) {  // scalars must be below 2^254 (every canonical Fr element is)
    atomicOr(status, BG_DSTATUS_SCALAR_RANGE);
    return;
  }
  const uint32_t nb = 1u << (c - 1);
  uint32_t carry = 0;
  for (int w = 0; w < W; w++) {
    bool ng;
    const uint32_t mag = signed_digit(s, w, c, carry, ng);
    if (mag) atomicAdd(&counts[(size_t)w * nb + mag - 1], 1u);
  }
}

__global__ void k_scatter(const uint32_t* __restrict__ scalars, size_t n, int c, int W,
                          uint32_t* __restrict__ cursor, uint32_t* __restrict__ sorted) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  uint32_t s[8];
  load_scalar(s, scalars, i);
  if (s[7] >> 30) return;
  const uint32_t nb = 1u << (c - 1);
  uint32_t carry = 0;
  for (int w = 0; w < W; w++) {
    bool ng;
    const uint32_t mag = signed_digit(s, w, c, carry, ng);
    if (mag) {
      const uint32_t slot = atomicAdd(&cursor[(size_t)w * nb + mag - 1], 1u);
      sorted[slot] = (uint32_t)i | (ng ? 0x80000000u : 0u);
    }
  }
}

// ---------------------------------------------------------------- buckets
template <class F>
__global__ void __launch_bounds__(128) k_bucket_acc(const uint32_t* __restrict__ points,
                                                    const uint32_t* __restrict__ offsets,
                                                    const uint32_t* __restrict__ sorted, uint32_t nbuckets,
                                                    uint32_t* __restrict__ buckets) {
  constexpr int FW = FieldWords<F>::value;
  const uint32_t g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= nbuckets) return;
  const uint32_t beg = offsets[g], end = offsets[g + 1];
  XYZZ<F> acc = xyzz_inf<F>();
  for (uint32_t e = beg; e < end; e++) {
    const uint32_t code = sorted[e];
    Affine<F> p = load_affine<F>(points + (size_t)(code & 0x7fffffffu) * 2 * FW);
    if (code >> 31) p = affine_neg(p);
    acc = xyzz_madd(acc, p);
  }
  store_xyzz(buckets + (size_t)g * 4 * FW, acc);
}

// One level of the bucket reduction.  Input per window: M pairs (R_e, Q_e) representing
// sum_e [Q_e + lam * e * R_e] (level 1: Q absent, R = buckets, weights b + 1).  Thread (w, u)
// folds elements [uL, uL + L) into R'_u = sum R_e and
// Q'_u = sum Q_e + lam * sum_e (e - uL) R_e   (level 1: Q'_u = sum_k (k + 1) B_{uL+k}),
// so the window sum is sum_u [Q'_u + (lam L) u R'_u].  One segment left => window sum = Q'_0.
template <class F>
__global__ void __launch_bounds__(128) k_reduce_level(const uint32_t* __restrict__ R, const uint32_t* __restrict__ Q,
                                                      uint32_t M, uint32_t L, int lam_log2, uint32_t S,
                                                      uint32_t W, uint32_t* __restrict__ Rout,
                                                      uint32_t* __restrict__ Qout) {
  constexpr int FW = FieldWords<F>::value;
  constexpr int PW = 4 * FW;
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= S * W) return;
  const uint32_t w = t / S, u = t % S;
  const uint32_t beg = u * L;
  const uint32_t len = (M - beg) < L ? (M - beg) : L;
  const uint32_t* Rw = R + ((size_t)w * M + beg) * PW;
  XYZZ<F> run = xyzz_inf<F>(), acc = xyzz_inf<F>();
  if (Q == nullptr) {
    for (int k = (int)len - 1; k >= 0; k--) {
      run = xyzz_add(run, load_xyzz<F>(Rw + (size_t)k * PW));
      acc = xyzz_add(acc, run);
    }
  } else {
    for (int k = (int)len - 1; k >= 1; k--) {
      run = xyzz_add(run, load_xyzz<F>(Rw + (size_t)k * PW));
      acc = xyzz_add(acc, run);
    }
    run = xyzz_add(run, load_xyzz<F>(Rw));
    for (int d = 0; d < lam_log2; d++) acc = xyzz_dbl(acc);
    const uint32_t* Qw = Q + ((size_t)w * M + beg) * PW;
    for (uint32_t k = 0; k < len; k++) acc = xyzz_add(acc, load_xyzz<F>(Qw + (size_t)k * PW));
  }
  store_xyzz(Rout + (size_t)t * PW, run);
  store_xyzz(Qout + (size_t)t * PW, acc);
}

// ---------------------------------------------------------------- host driver
int msm_pick_c(size_t n) {
  int lg = 0;
  while ((size_t(1) << (lg + 1)) <= n) lg++;
  int c = lg - 3;
  if (c < 3) c = 3;
  if (c > 16) c = 16;
  return c;
}

template <class F>
struct HostField;
template <>
struct HostField<Fq> {
  typedef bgh::FqOps T;
};
template <>
struct HostField<Fq2> {
  typedef bgh::Fq2Ops T;
};

template <class F>
void msm_launch(Ctx& ctx, cudaStream_t st, const std::string& tag, const uint32_t* d_points,
                const uint32_t* d_scalars, size_t n, MsmPlan& plan) {
  constexpr int FW = FieldWords<F>::value;
  constexpr int PW = 4 * FW;
  if (n == 0) {
    plan.W = 0;
    return;
  }
  if (n >= 0x80000000ull) throw Error(BG_E_ARG, "msm: n must be below 2^31");
  const int c = plan.c > 0 ? plan.c : msm_pick_c(n);
  const int W = 254 / c + 1;
  const uint32_t nb = 1u << (c - 1);
  const size_t nkeys = (size_t)W * nb;
  plan.c = c;
  plan.W = W;

  Workspace& ws = ctx.ws;
  uint32_t* counts = ws.get_t<uint32_t>(tag + ".counts", nkeys + 1);
  uint32_t* offsets = ws.get_t<uint32_t>(tag + ".offsets", nkeys + 1);
  uint32_t* cursor = ws.get_t<uint32_t>(tag + ".cursor", nkeys + 1);
  uint32_t* sorted = ws.get_t<uint32_t>(tag + ".sorted", n * (size_t)W);
  uint32_t* buckets = ws.get_t<uint32_t>(tag + ".buckets", nkeys * PW);

  BG_CUDA(cudaMemsetAsync(counts, 0, (nkeys + 1) * sizeof(uint32_t), st));
  {
    KernelTimer kt(ctx, "msm_digits", st);
    k_digits_hist<<<ceil_div(n, 256), 256, 0, st>>>(d_scalars, n, c, W, counts, ctx.d_status);
    BG_CHECK_LAUNCH();
  }
  exclusive_scan(ws, tag, counts, offsets, nkeys + 1, st, 0);
  BG_CUDA(cudaMemcpyAsync(cursor, offsets, (nkeys + 1) * sizeof(uint32_t), cudaMemcpyDeviceToDevice, st));
  {
    KernelTimer kt(ctx, "msm_scatter", st);
    k_scatter<<<ceil_div(n, 256), 256, 0, st>>>(d_scalars, n, c, W, cursor, sorted);
    BG_CHECK_LAUNCH();
  }
  {
    KernelTimer kt(ctx, FieldWords<F>::value == 8 ? "msm_bucket_acc_g1" : "msm_bucket_acc_g2", st);
    k_bucket_acc<F><<<ceil_div(nkeys, 128), 128, 0, st>>>(d_points, offsets, sorted, (uint32_t)nkeys, buckets);
    BG_CHECK_LAUNCH();
  }
  plan.entries = n * (size_t)W;

  // hierarchical reduction, L = 8 elements per thread and level
  const uint32_t L = 8;
  uint32_t M = nb;
  const uint32_t* R = buckets;
  const uint32_t* Q = nullptr;
  int lam_log2 = 0;
  int level = 0;
  uint32_t* out_q = nullptr;
  while (true) {
    const uint32_t S = (M + L - 1) / L;
    uint32_t* Rout = ws.get_t<uint32_t>(tag + ".red_r" + std::to_string(level & 1), (size_t)S * W * PW);
    uint32_t* Qout = ws.get_t<uint32_t>(tag + ".red_q" + std::to_string(level & 1), (size_t)S * W * PW);
    {
      KernelTimer kt(ctx, FieldWords<F>::value == 8 ? "msm_reduce_g1" : "msm_reduce_g2", st);
      k_reduce_level<F><<<ceil_div((size_t)S * W, 128), 128, 0, st>>>(R, Q, M, L, lam_log2, S, W, Rout, Qout);
      BG_CHECK_LAUNCH();
    }
    lam_log2 = (Q == nullptr) ? 3 : lam_log2 + 3;
    R = Rout;
    Q = Qout;
    out_q = Qout;
    M = S;
    level++;
    if (S == 1) break;
  }
  plan.d_window_sums = out_q;
  plan.host_window_sums.resize((size_t)W * PW);
}

template <class F>
void msm_fetch(cudaStream_t st, MsmPlan& plan) {
  constexpr int PW = 4 * FieldWords<F>::value;
  if (plan.W == 0) return;
  BG_CUDA(cudaMemcpyAsync(plan.host_window_sums.data(), plan.d_window_sums, (size_t)plan.W * PW * sizeof(uint32_t),
                          cudaMemcpyDeviceToHost, st));
}

// sum_w 2^(c w) S_w on the host (Horner, c doublings per window)
template <class F>
void msm_finish(const MsmPlan& plan, uint32_t* out_affine_words32) {
  typedef typename HostField<F>::T H;
  constexpr int PW = 4 * H::WORDS;
  bgh::Xyzz<H> acc = bgh::xyzz_inf<H>();
  for (int w = plan.W - 1; w >= 0; w--) {
    for (int d = 0; d < plan.c; d++) acc = bgh::xyzz_dbl(acc);
    acc = bgh::xyzz_add(acc, bgh::xyzz_from_words32<H>(plan.host_window_sums.data() + (size_t)w * PW));
  }
  bgh::aff_to_words32<H>(out_affine_words32, bgh::xyzz_to_affine(acc));
}

template void msm_launch<Fq>(Ctx&, cudaStream_t, const std::string&, const uint32_t*, const uint32_t*, size_t,
                             MsmPlan&);
template void msm_launch<Fq2>(Ctx&, cudaStream_t, const std::string&, const uint32_t*, const uint32_t*, size_t,
                              MsmPlan&);
template void msm_fetch<Fq>(cudaStream_t, MsmPlan&);
template void msm_fetch<Fq2>(cudaStream_t, MsmPlan&);
template void msm_finish<Fq>(const MsmPlan&, uint32_t*);
template void msm_finish<Fq2>(const MsmPlan&, uint32_t*);

}  // namespace bg
