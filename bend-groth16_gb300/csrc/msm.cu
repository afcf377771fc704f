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
//   4. k_bucket_acc   load-balanced slices of K entries per thread: XYZZ accumulator += +-P
//                     (mixed add); a bucket cut by slice boundaries leaves pieces, joined
//                     where the reduction reads it (k_bucket_heavy first joins the rare
//                     buckets of very many pieces)
//   5. k_window_reduce one CTA per window part: running sums over M buckets per thread, an
//                     in-CTA suffix scan and tree sum give sum_b (b+1) B_b for the part
//   6. host: parts -> window sums -> Horner (a window's width of doublings per window) ->
//      affine.  Windows have balanced widths of at most c bits (window_width).
// Window sums and the final point are exact group elements, so the affine result equals the
// reference's for the same inputs regardless of bucket order inside a window.
#include "common.cuh"
#include "ec.cuh"
#include "host_ff.hpp"
#include "host_pool.hpp"
#include "msm.h"
#include "msm_tune.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <memory>
#include <mutex>
#include <vector>

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

// Window layout: W windows cover bits [0, 255) (254 scalar bits and room for the last carry)
// with balanced widths -- the first 255 mod W windows one bit wider -- so that no window is
// much narrower than the others (a narrow top window would pile its entries into a few huge
// buckets).  W = floor(254 / c) + 1 keeps every width at most c.
__host__ __device__ inline int window_width(int w, int W) { return 255 / W + (w < 255 % W ? 1 : 0); }
__host__ __device__ inline int window_offset(int w, int W) { return w * (255 / W) + (w < 255 % W ? w : 255 % W); }

// signed digit of window w of W: returns magnitude (0 = no bucket) and updates carry; *neg set
// when the digit is negative.  Digits lie in [-(2^(b-1) - 1), 2^(b-1)] for a window of b bits;
// scalars below 2^254 leave no carry out of the top window.
BG_DEV uint32_t signed_digit(const uint32_t* s, int w, int W, uint32_t& carry, bool& negd) {
  const int b = window_width(w, W);
  const uint32_t half = 1u << (b - 1);
  const uint32_t d = window_bits(s, window_offset(w, W), b) + carry;
  if (d > half) {
    carry = 1u;
    negd = true;
    return (1u << b) - d;
  }
  carry = 0u;
  negd = false;
  return d;
}

// Bucket key of window w's digit: w * key_stride + |d| - 1 (key_stride = 2^(c-1): one bucket
// set per window; 0: all windows share one set).  Point index stored with it:
// i + w * idx_stride (0: the point itself; n: row w of a table of 2^(o_w)-multiples).
__global__ void k_digits_hist(const uint32_t* __restrict__ scalars, size_t n, int c, int W, uint32_t key_stride,
                              uint32_t* __restrict__ counts, uint32_t* __restrict__ status) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  uint32_t s[8];
  load_scalar(s, scalars, i);
  if (s[7] >> 30) {  // scalars must be below 2^254 (every canonical Fr element is)
    atomicOr(status, BG_DSTATUS_SCALAR_RANGE);
    return;
  }
  uint32_t carry = 0;
  for (int w = 0; w < W; w++) {
    bool ng;
    const uint32_t mag = signed_digit(s, w, W, carry, ng);
    if (mag) atomicAdd(&counts[(size_t)w * key_stride + mag - 1], 1u);
  }
}

__global__ void k_scatter(const uint32_t* __restrict__ scalars, size_t n, int c, int W, uint32_t key_stride,
                          uint32_t idx_stride, uint32_t* __restrict__ cursor, uint32_t* __restrict__ sorted) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  uint32_t s[8];
  load_scalar(s, scalars, i);
  if (s[7] >> 30) return;
  uint32_t carry = 0;
  for (int w = 0; w < W; w++) {
    bool ng;
    const uint32_t mag = signed_digit(s, w, W, carry, ng);
    if (mag) {
      const uint32_t slot = atomicAdd(&cursor[(size_t)w * key_stride + mag - 1], 1u);
      sorted[slot] = ((uint32_t)i + (uint32_t)w * idx_stride) | (ng ? 0x80000000u : 0u);
    }
  }
}

// Window table of a fixed point set: row w holds 2^(o_w) P_i, o_w the offset of window w
// (affine, row-major, n points per row); computed once per proving key, one thread per point
// (a window's width of doublings per row, one inversion per entry).
template <class F>
__global__ void __launch_bounds__(128) k_build_table(const uint32_t* __restrict__ pts, size_t n, int c, int W,
                                                     uint32_t* __restrict__ table) {
  constexpr int PW = 2 * FieldWords<F>::value;
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const Affine<F> p = load_affine<F>(pts + i * PW);
  store_affine(table + i * PW, p);
  XYZZ<F> q = xyzz_from_affine(p);
  for (int w = 1; w < W; w++) {
    for (int d = 0; d < window_width(w - 1, W); d++) q = xyzz_dbl(q);
    Affine<F> a;
    if (is_inf(q)) {
      a.x = field_zero<F>();
      a.y = field_zero<F>();
    } else {
      const F t = field_inv_any(fmul(q.zz, q.zzz));
      a.x = fmul(q.x, fmul(t, q.zzz));
      a.y = fmul(q.y, fmul(t, q.zz));
    }
    store_affine(table + ((size_t)w * n + i) * PW, a);
  }
}


// ---------------------------------------------------------------- buckets
// Segmented accumulation: the bucket-ordered entry list (T entries) is cut into slices of K
// entries, one per thread, so every thread runs exactly K mixed additions whatever the bucket
// sizes are (one thread per bucket would idle most lanes of a warp on Poisson-sized buckets).
// A run of entries that covers a whole bucket is written to that bucket; a run cut by a slice
// boundary becomes a piece: entry 2t of the piece list if the run started in an earlier slice,
// entry 2t+1 if the bucket starts in slice t and continues into a later one.  So a bucket with
// entries [o, o') cut into slices t0 = o / K .. t1 = (o' - 1) / K has its pieces at 2 t0 + 1
// and 2 u for t0 < u <= t1; the window reduction adds them where it reads the bucket
// (bucket_value), which costs the same additions as a separate join pass without its launch
// and its mostly idle lanes.  A bucket of more than kPieceLimit + 1 pieces (a scalar value
// repeated thousands of times) is joined beforehand by k_bucket_heavy: the thread that owns its
// first piece lists it in heavy[1 + i] (heavy[0] counts, cleared before the accumulation).
constexpr uint32_t kPieceLimit = 24;
// G2's accumulation stages the next entry's point in shared memory (cp.async) instead of
// registers, where a prefetched Fq2 point held 32 registers across the whole addition: 222
// registers instead of 242, the G2 accumulation of a 2^18 MSM 2.96 -> 2.93 ms,
// SquareChain(2^18) 9.88 -> 9.75-9.79 ms, 2^20 34.8 -> 34.4-34.5 ms.  The registers saved do
// not buy more warps: capped at 200 (10 warps per SM in 64-thread CTAs, a few spills) or 216
// (9 warps in 32-thread CTAs) the same kernel measured 3.14 / 3.12 ms.  G1 keeps its register
// prefetch (126 registers, four 128-thread CTAs per SM either way).
template <class F>
constexpr bool kAccStaged = FieldWords<F>::value == 16;
// CTA size of the accumulation
template <class F>
constexpr int kAccThreads = 128;

// 16-byte asynchronous copy global -> shared (cached in L2 only), and the wait for a thread's
// own copies
BG_DEV void cp_async16(void* smem, const void* gmem) {
  const uint32_t s = (uint32_t)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem) : "memory");
}
BG_DEV void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
BG_DEV void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;\n" ::: "memory"); }

// the affine point held in 16-byte chunks c[0 .. 2 FW / 4)
BG_DEV Fq fp_of(const uint4& a, const uint4& b) {
  Fq r;
  r.v[0] = a.x; r.v[1] = a.y; r.v[2] = a.z; r.v[3] = a.w;
  r.v[4] = b.x; r.v[5] = b.y; r.v[6] = b.z; r.v[7] = b.w;
  return r;
}
template <class F>
BG_DEV Affine<F> affine_of_chunks(const uint4* c, size_t stride) {
  Affine<F> p;
  if constexpr (FieldWords<F>::value == 16) {
    p.x.c0 = fp_of(c[0], c[stride]);
    p.x.c1 = fp_of(c[2 * stride], c[3 * stride]);
    p.y.c0 = fp_of(c[4 * stride], c[5 * stride]);
    p.y.c1 = fp_of(c[6 * stride], c[7 * stride]);
  } else {
    p.x = fp_of(c[0], c[stride]);
    p.y = fp_of(c[2 * stride], c[3 * stride]);
  }
  return p;
}

template <class F>
__global__ void __launch_bounds__(kAccThreads<F>) k_bucket_acc(const uint32_t* __restrict__ points,
                                                               const uint32_t* __restrict__ offsets,
                                                               const uint32_t* __restrict__ sorted, uint32_t nbuckets,
                                                               uint32_t K, uint32_t* __restrict__ buckets,
                                                               uint32_t* __restrict__ parts, uint32_t* __restrict__ heavy) {
  constexpr int FW = FieldWords<F>::value;
  constexpr int PW = 4 * FW;
  const uint32_t total = offsets[nbuckets];
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  const uint64_t beg64 = (uint64_t)t * K;
  if (beg64 >= total) return;
  const uint32_t beg = (uint32_t)beg64;
  const uint32_t end = (total - beg) < K ? total : beg + K;
  // bucket holding entry `beg`: the last b with offsets[b] <= beg
  uint32_t lo = 0, hi = nbuckets;  // offsets[lo] <= beg < offsets[hi]
  while (hi - lo > 1) {
    const uint32_t mid = (lo + hi) >> 1;
    if (offsets[mid] <= beg) lo = mid;
    else hi = mid;
  }
  // One flat loop of exactly (end - beg) mixed additions, so the lanes of a warp stay in
  // step; a bucket boundary only costs a short divergent flush.
  uint32_t b = lo;
  uint32_t bstart = offsets[b], bend = offsets[b + 1];
  XYZZ<F> acc = xyzz_inf<F>();
  // The next entry's point is gathered before this entry's addition, so the gather's latency
  // hides behind the arithmetic (G1 accumulation 2^20 3.88 -> 3.82 ms; 126 registers, still
  // four CTAs per SM): into registers for G1, into one of two shared-memory slots for G2 (the
  // slot read in this iteration is refilled two iterations later, after the addition that
  // consumed it).
  // sorted == nullptr: the entries are the points themselves (the output of the pair rounds)
  constexpr int CH = 2 * FW / 4;  // 16-byte chunks of an affine point
  constexpr int kSlots = kAccStaged<F> ? 2 : 1, kChunks = kAccStaged<F> ? CH : 1;
  __shared__ uint4 stage[kSlots][kChunks][kAccThreads<F>];
  auto gather = [&](uint32_t c, int slot) {
    if constexpr (kAccStaged<F>) {
      const uint4* src = reinterpret_cast<const uint4*>(points + (size_t)(c & 0x7fffffffu) * 2 * FW);
#pragma unroll
      for (int j = 0; j < CH; j++) cp_async16(&stage[slot][j][threadIdx.x], src + j);
      cp_async_commit();
    }
  };
  uint32_t code = sorted ? sorted[beg] : beg;
  Affine<F> p;
  if constexpr (kAccStaged<F>) gather(code, 0);
  else p = load_affine<F>(points + (size_t)(code & 0x7fffffffu) * 2 * FW);
  int slot = 0;
  for (uint32_t e = beg; e < end; e++) {
    uint32_t code_n = 0;
    Affine<F> pn;
    if constexpr (kAccStaged<F>) {
      cp_async_wait_all();
      p = affine_of_chunks<F>(&stage[slot][0][threadIdx.x], kAccThreads<F>);
      if (e + 1 < end) {
        code_n = sorted ? sorted[e + 1] : e + 1;
        gather(code_n, slot ^ 1);
      }
      slot ^= 1;
    } else if (e + 1 < end) {
      code_n = sorted ? sorted[e + 1] : e + 1;
      pn = load_affine<F>(points + (size_t)(code_n & 0x7fffffffu) * 2 * FW);
    }
    if (code >> 31) p = affine_neg(p);
    acc = xyzz_madd(acc, p);
    if constexpr (!kAccStaged<F>) p = pn;
    code = code_n;
    if (e + 1 == bend || e + 1 == end) {
      if (bstart < beg || bend > end) {
        const size_t slot = 2 * (size_t)t + (bstart < beg ? 0 : 1);
        store_xyzz(parts + slot * PW, acc);
        if (bstart >= beg && (bend - 1) / K - t > kPieceLimit) heavy[1 + atomicAdd(heavy, 1u)] = b;
      } else {
        store_xyzz(buckets + (size_t)b * PW, acc);
      }
      acc = xyzz_inf<F>();
      if (e + 1 < end) {
        do {
          b++;
        } while (offsets[b + 1] <= e + 1);  // skip empty buckets
        bstart = offsets[b];
        bend = offsets[b + 1];
      }
    }
  }
}

// Heavy buckets: one CTA per bucket, a strided sum of its pieces per thread and a tree over the
// CTA; the sum goes to the bucket.  The grid is fixed; CTAs loop over however many the
// accumulation listed (none for uniformly spread scalars).
template <class F>
__global__ void __launch_bounds__(128) k_bucket_heavy(const uint32_t* __restrict__ offsets,
                                                      const uint32_t* __restrict__ parts, uint32_t K,
                                                      const uint32_t* __restrict__ heavy,
                                                      uint32_t* __restrict__ buckets) {
  constexpr int PW = 4 * FieldWords<F>::value;
  extern __shared__ uint32_t sm[];
  const uint32_t nh = heavy[0];
  for (uint32_t h = blockIdx.x; h < nh; h += gridDim.x) {
    const uint32_t b = heavy[1 + h];
    const uint32_t t0 = offsets[b] / K;
    const uint32_t np = (offsets[b + 1] - 1) / K - t0 + 1;
    XYZZ<F> acc = xyzz_inf<F>();
    for (uint32_t i = threadIdx.x; i < np; i += blockDim.x) {
      const size_t slot = i == 0 ? 2 * (size_t)t0 + 1 : 2 * ((size_t)t0 + i);
      acc = xyzz_add(acc, load_xyzz<F>(parts + slot * PW));
    }
    store_xyzz(sm + (size_t)threadIdx.x * PW, acc);
    __syncthreads();
    for (uint32_t d = blockDim.x >> 1; d >= 1; d >>= 1) {
      if (threadIdx.x < d) {
        acc = xyzz_add(acc, load_xyzz<F>(sm + (size_t)(threadIdx.x + d) * PW));
        store_xyzz(sm + (size_t)threadIdx.x * PW, acc);
      }
      __syncthreads();
    }
    if (threadIdx.x == 0) store_xyzz(buckets + (size_t)b * PW, acc);
    __syncthreads();
  }
}
constexpr uint32_t kHeavyThreads = 128;
constexpr uint32_t kHeavyGrid = 152;

#include "msm_pairs.cuh"

// acc += value of bucket `key` (entries [offsets[key], offsets[key+1])): nothing when empty, the
// stored bucket when it lies in one slice or is heavy, else its pieces.
template <class F>
BG_DEV XYZZ<F> add_bucket(XYZZ<F> acc, const uint32_t* __restrict__ offsets, const uint32_t* __restrict__ buckets,
                          const uint32_t* __restrict__ parts, uint32_t K, size_t key) {
  constexpr int PW = 4 * FieldWords<F>::value;
  const uint32_t o0 = offsets[key], o1 = offsets[key + 1];
  if (o1 == o0) return acc;
  const uint32_t t0 = o0 / K, t1 = (o1 - 1) / K;
  if (t0 == t1 || t1 - t0 > kPieceLimit) return xyzz_add(acc, load_xyzz<F>(buckets + key * PW));
  acc = xyzz_add(acc, load_xyzz<F>(parts + (2 * (size_t)t0 + 1) * PW));
  for (uint32_t u = t0 + 1; u <= t1; u++) acc = xyzz_add(acc, load_xyzz<F>(parts + 2 * (size_t)u * PW));
  return acc;
}

// Entries per accumulation thread, from a latency model with constants measured on GB300 (G1;
// G2 scales them alike): a thread's K mixed additions take K x 6.6 us at low occupancy, the
// whole accumulation cannot beat its throughput (4.58 entries per ns), and a bucket of e
// entries leaves about e / K + 1 pieces for the reduction (4.5 us each: a 9 us addition, of
// which half is hidden under other work, fitted to SquareChain(2^12..2^16) proofs).  Large MSMs
// get 32-entry slices (throughput-bound, fewest pieces); small ones 8 (SquareChain(2^12) proof
// 2.06 -> 1.69 ms, 2^14 2.44 -> 2.34 ms).
inline uint32_t slice_entries(size_t max_entries, size_t nkeys, double piece_us = 4.5) {
  const double e = (double)max_entries / (double)(nkeys ? nkeys : 1);
  const double floor_us = (double)max_entries / 4580.0;
  uint32_t best = 32;
  double best_us = 1e300;
  for (uint32_t k = 4; k <= 32; k <<= 1) {
    const double t = std::max(k * 6.6, floor_us) + (e / k + 2.0) * piece_us;
    if (t < best_us - 1e-9 || (t <= best_us + 1e-9 && k > best)) {
      best_us = t;
      best = k;
    }
  }
  return best;
}

// Resident threads of a pair round on the whole GPU (SMs x CTAs per SM x CTA size).
template <class F>
double pair_slots() {
  static std::atomic<double> slots{0.0};
  double s = slots.load();
  if (s == 0.0) {
    int dev = 0, sms = 0, occ = 0;
    BG_CUDA(cudaGetDevice(&dev));
    BG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    BG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_pair_round<F, true>, kPairThreads<F>, 0));
    s = (double)sms * (occ > 0 ? occ : 1) * kPairThreads<F>;
    slots.store(s);
  }
  return s;
}

// Scratch of the bucket phase for at most max_entries entries (words): pieces and the heavy list.
struct BucketScratch {
  uint32_t K = 32;            // entries per accumulation thread
  uint32_t* parts = nullptr;  // 2 x slices XYZZ points
  uint32_t* heavy = nullptr;  // 1 + slices / kPieceLimit + 1
};
inline size_t bucket_slices(size_t max_entries, uint32_t K) { return (max_entries + K - 1) / K; }

// Accumulation threads resident on the whole GPU at once (SMs x CTAs per SM x CTA size).
template <class F>
double acc_slots() {
  static double slots = 0;
  if (slots == 0) {
    int dev = 0, sms = 0, occ = 0;
    BG_CUDA(cudaGetDevice(&dev));
    BG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    BG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_bucket_acc<F>, kAccThreads<F>, 0));
    slots = (double)sms * (occ > 0 ? occ : 1) * kAccThreads<F>;
  }
  return slots;
}

// Every slice costs the same K additions, so an accumulation grid of 1.6 waves takes as long
// as 2.  When the model's slices need more than one wave, K is rounded so that the grid is a
// whole number of waves (the nearest, at least one): SquareChain(2^18) proof 11.05 -> 10.7 ms,
// G2 accumulation 2^18 3.25 -> 2.95 ms.  Slices then hold at least 3/4 of the model's K
// (rounding 1.5 waves up to 2 at worst); the model picks K = 32 for every MSM that needs more
// than a wave and at least 2^21 entries.
template <class F>
uint32_t whole_wave_slices(size_t max_entries, uint32_t K) {
  const double slots = acc_slots<F>();
  const double waves = std::ceil((double)max_entries / K) / slots;
  if (waves <= 1.0) return K;
  const double rounded = std::max(1.0, std::round(waves));
  return (uint32_t)std::ceil((double)max_entries / (rounded * slots));
}

template <class F, class Get>
BucketScratch bucket_scratch(size_t max_entries, size_t nkeys, Get get, uint32_t K = 0) {
  constexpr int PW = 4 * FieldWords<F>::value;
  BucketScratch b;
  // a G2 piece costs a G2 addition in the reduction: about twice a G1 one relative to the
  // accumulation's mixed additions (SquareChain(2^12): G2 slices of 16 instead of 8)
  const double piece_us = FieldWords<F>::value == 16 ? 9.0 : 4.5;
  b.K = K ? K : whole_wave_slices<F>(max_entries, slice_entries(max_entries, nkeys, piece_us));
  const size_t s = bucket_slices(max_entries, b.K);
  b.parts = get("parts", 2 * s * PW);
  b.heavy = get("heavy", s / kPieceLimit + 2);
  return b;
}

// Accumulation on `st`: buckets of single-slice runs are final, cut buckets leave pieces.
template <class F>
void bucket_accumulate(Ctx* prof, cudaStream_t st, const uint32_t* points, const uint32_t* offsets,
                       const uint32_t* sorted, uint32_t nkeys, size_t max_entries, uint32_t* buckets,
                       const BucketScratch& s) {
  constexpr int FW = FieldWords<F>::value;
  const size_t slices = bucket_slices(max_entries, s.K);
  BG_CUDA(cudaMemsetAsync(s.heavy, 0, sizeof(uint32_t), st));
  std::unique_ptr<KernelTimer> kt(prof ? new KernelTimer(*prof, FW == 8 ? "msm_bucket_acc_g1" : "msm_bucket_acc_g2", st)
                                       : nullptr);
  k_bucket_acc<F><<<ceil_div(slices, kAccThreads<F>), kAccThreads<F>, 0, st>>>(points, offsets, sorted, nkeys, s.K, buckets, s.parts,
                                                         s.heavy);
  BG_CHECK_LAUNCH();
}

// Heavy buckets on `st` (a pass that exits at once when there are none).
template <class F>
void bucket_heavy(Ctx* prof, cudaStream_t st, const uint32_t* offsets, uint32_t* buckets, const BucketScratch& s) {
  constexpr int FW = FieldWords<F>::value;
  constexpr int PW = 4 * FW;
  std::unique_ptr<KernelTimer> kt(prof ? new KernelTimer(*prof, FW == 8 ? "msm_heavy_g1" : "msm_heavy_g2", st)
                                       : nullptr);
  k_bucket_heavy<F><<<kHeavyGrid, kHeavyThreads, kHeavyThreads * PW * sizeof(uint32_t), st>>>(
      offsets, s.parts, s.K, s.heavy, buckets);
  BG_CHECK_LAUNCH();
}

// Window reduction, one CTA per (window, part).  Part j of window w covers buckets
// [j RT M, (j+1) RT M); thread t folds M consecutive buckets into R_t = sum B and
// T_t = sum_k (k+1) B_{tM+k} (running sums).  The part's weighted sum
//   S_j = sum_{local b} (b+1) B_b = sum_t T_t + M sum_{t>=1} Suf_t,   Suf_t = sum_{t'>=t} R_t'
// comes from an in-CTA suffix scan of R and a tree sum; the part also reports R_j = Suf_0.
// The host finishes window w as sum_j S_j + (RT M) sum_j j R_j.
// Bucket values are read through add_bucket (stored bucket or its pieces).
template <class F>
__global__ void k_window_reduce(const uint32_t* __restrict__ offsets, const uint32_t* __restrict__ buckets,
                                const uint32_t* __restrict__ pieces, uint32_t K, uint32_t nb, uint32_t M, uint32_t J,
                                uint32_t* __restrict__ out) {
  constexpr int PW = 4 * FieldWords<F>::value;
  extern __shared__ uint32_t sm[];
  const uint32_t RT = blockDim.x;
  const uint32_t w = blockIdx.x / J, j = blockIdx.x % J, t = threadIdx.x;
  const size_t key0 = (size_t)w * nb + ((size_t)j * RT + t) * M;
  XYZZ<F> run = xyzz_inf<F>(), acc = xyzz_inf<F>();
  for (int k = (int)M - 1; k >= 0; k--) {
    run = add_bucket(run, offsets, buckets, pieces, K, key0 + k);
    acc = xyzz_add(acc, run);
  }
  // inclusive suffix scan of R over the CTA (Hillis-Steele)
  store_xyzz(sm + (size_t)t * PW, run);
  __syncthreads();
  for (uint32_t d = 1; d < RT; d <<= 1) {
    XYZZ<F> v = xyzz_inf<F>();
    if (t + d < RT) v = load_xyzz<F>(sm + (size_t)(t + d) * PW);
    __syncthreads();
    run = xyzz_add(run, v);
    store_xyzz(sm + (size_t)t * PW, run);
    __syncthreads();
  }
  // R_j, written at once so that it holds no registers through the tree below
  if (t == 0) store_xyzz(out + ((size_t)blockIdx.x * 2 + 1) * PW, run);
  // Y_t = T_t + M Suf_t (t >= 1), Y_0 = T_0
  if (t >= 1) {
    for (uint32_t m = M; m > 1; m >>= 1) run = xyzz_dbl(run);
    acc = xyzz_add(acc, run);
  }
  __syncthreads();
  store_xyzz(sm + (size_t)t * PW, acc);
  __syncthreads();
  for (uint32_t d = RT >> 1; d >= 1; d >>= 1) {
    if (t < d) {
      acc = xyzz_add(acc, load_xyzz<F>(sm + (size_t)(t + d) * PW));
      store_xyzz(sm + (size_t)t * PW, acc);
    }
    __syncthreads();
  }
  if (t == 0) store_xyzz(out + (size_t)blockIdx.x * 2 * PW, acc);
}

// The same reduction with the points a thread owns in shared memory (word i of thread t's
// point at base[i * RT + t]): R, T and a staging column for the scan.  One out-of-line body
// adds a point into another (and one doubles in place), so no point is live in registers
// across a call.  The register-resident form above spills in G2 (R, T and the addend are
// 3 x 64 words across inlined Fq2 additions: 2.4 KB of spill stores per thread); this one
// leaves 0.4 KB, and an addition's latency falls with it (G2 MSM 2^18 5.59 -> 5.33 ms,
// SquareChain(2^10) proof 1.24 -> 1.11 ms, 2^12 1.66 -> 1.46 ms, 2^18 10.74 -> 10.62 ms).  For
// G1 (no spills either way) it was measured level, so G1 keeps the register form.
BG_DEV void elem_load(Fq& e, const uint32_t* src, uint32_t stride) {
#pragma unroll
  for (int l = 0; l < 8; l++) e.v[l] = src[l * stride];
}
BG_DEV void elem_load(Fq2& e, const uint32_t* src, uint32_t stride) {
  elem_load(e.c0, src, stride);
  elem_load(e.c1, src + 8 * stride, stride);
}
BG_DEV void elem_store(uint32_t* dst, uint32_t stride, const Fq& e) {
#pragma unroll
  for (int l = 0; l < 8; l++) dst[l * stride] = e.v[l];
}
BG_DEV void elem_store(uint32_t* dst, uint32_t stride, const Fq2& e) {
  elem_store(dst, stride, e.c0);
  elem_store(dst + 8 * stride, stride, e.c1);
}
template <class F>
BG_DEV void pt_load(XYZZ<F>& p, const uint32_t* src, uint32_t stride) {
  constexpr int FW = FieldWords<F>::value;
  elem_load(p.x, src, stride);
  elem_load(p.y, src + FW * stride, stride);
  elem_load(p.zz, src + 2 * FW * stride, stride);
  elem_load(p.zzz, src + 3 * FW * stride, stride);
}
template <class F>
BG_DEV void pt_store(uint32_t* dst, uint32_t stride, const XYZZ<F>& p) {
  constexpr int FW = FieldWords<F>::value;
  elem_store(dst, stride, p.x);
  elem_store(dst + FW * stride, stride, p.y);
  elem_store(dst + 2 * FW * stride, stride, p.zz);
  elem_store(dst + 3 * FW * stride, stride, p.zzz);
}
// dst (stride) += src: shared memory with stride sstride, or a contiguous point in global
// memory (sstride 1)
template <class F>
static __device__ __noinline__ void pt_add_into(uint32_t* dst, uint32_t stride, const uint32_t* src,
                                                uint32_t sstride) {
  XYZZ<F> p, q;
  pt_load(p, dst, stride);
  if (sstride == 1) q = load_xyzz<F>(src);
  else pt_load(q, src, sstride);
  pt_store(dst, stride, xyzz_add(p, q));
}
template <class F>
static __device__ __noinline__ void pt_dbl_in(uint32_t* dst, uint32_t stride) {
  XYZZ<F> p;
  pt_load(p, dst, stride);
  pt_store(dst, stride, xyzz_dbl(p));
}
// shared memory of k_window_reduce_sm: R, T and the scan's staging column
template <class F>
constexpr size_t reduce_sm_bytes(uint32_t RT) {
  return 3 * (size_t)RT * 4 * FieldWords<F>::value * sizeof(uint32_t);
}

template <class F>
__global__ void k_window_reduce_sm(const uint32_t* __restrict__ offsets, const uint32_t* __restrict__ buckets,
                                   const uint32_t* __restrict__ pieces, uint32_t K, uint32_t nb, uint32_t M,
                                   uint32_t J, uint32_t* __restrict__ out) {
  constexpr int PW = 4 * FieldWords<F>::value;
  extern __shared__ uint32_t sm[];
  const uint32_t RT = blockDim.x;
  const uint32_t w = blockIdx.x / J, j = blockIdx.x % J, t = threadIdx.x;
  const size_t key0 = (size_t)w * nb + ((size_t)j * RT + t) * M;
  uint32_t* R = sm + t;                        // running sum R_t
  uint32_t* T = sm + (size_t)PW * RT + t;      // weighted sum T_t
  uint32_t* S = sm + (size_t)2 * PW * RT + t;  // staging for the scan
  pt_store(R, RT, xyzz_inf<F>());
  pt_store(T, RT, xyzz_inf<F>());
  for (int k = (int)M - 1; k >= 0; k--) {
    const size_t key = key0 + k;
    const uint32_t o0 = offsets[key], o1 = offsets[key + 1];
    if (o1 != o0) {
      const uint32_t t0 = o0 / K, t1 = (o1 - 1) / K;
      if (t0 == t1 || t1 - t0 > kPieceLimit) {
        pt_add_into<F>(R, RT, buckets + key * PW, 1);
      } else {
        pt_add_into<F>(R, RT, pieces + (2 * (size_t)t0 + 1) * PW, 1);
        for (uint32_t u = t0 + 1; u <= t1; u++) pt_add_into<F>(R, RT, pieces + 2 * (size_t)u * PW, 1);
      }
    }
    pt_add_into<F>(T, RT, R, RT);
  }
  __syncthreads();
  // inclusive suffix scan of R over the CTA (Hillis-Steele), through the staging column
  for (uint32_t d = 1; d < RT; d <<= 1) {
    if (t + d < RT) {
#pragma unroll 8
      for (int i = 0; i < PW; i++) S[i * RT] = R[i * RT + d];
    } else {
      pt_store(S, RT, xyzz_inf<F>());
    }
    __syncthreads();
    pt_add_into<F>(R, RT, S, RT);
    __syncthreads();
  }
  // R_j = Suf_0
  if (t == 0) {
#pragma unroll 8
    for (int i = 0; i < PW; i++) out[((size_t)blockIdx.x * 2 + 1) * PW + i] = R[i * RT];
  }
  // Y_t = T_t + M Suf_t (t >= 1), Y_0 = T_0
  if (t >= 1) {
    for (uint32_t m = M; m > 1; m >>= 1) pt_dbl_in<F>(R, RT);
    pt_add_into<F>(T, RT, R, RT);
  }
  __syncthreads();
  for (uint32_t d = RT >> 1; d >= 1; d >>= 1) {
    if (t < d) pt_add_into<F>(T, RT, T + d, RT);
    __syncthreads();
  }
  if (t == 0) {
#pragma unroll 8
    for (int i = 0; i < PW; i++) out[(size_t)blockIdx.x * 2 * PW + i] = T[i * RT];
  }
}

// which form reduces a field's windows (G1's register-resident form does not spill: 200
// registers)
template <class F>
constexpr bool kReduceInSmem = FieldWords<F>::value == 16;

// Shape of the window reduction: RT threads x M buckets per thread x J parts per window, picked
// by a latency model.  A thread's dependent chain is M (2 + e / K) additions (each bucket
// costs its pieces, about 1 + e / K for e entries per bucket, plus the running-sum addition),
// two log2(RT) trees and log2(M) doublings, times the number of waves the sets x J CTAs need
// at the kernel's occupancy; the host then adds 3 J points per bucket set, at about 1/16 of a
// device addition's latency each (a single dependent chain is ~20x faster on a CPU core than
// on one GPU thread).
struct ReduceShape {
  uint32_t RT, M, J;
  double cost = 0;     // the model's latency, in dependent additions
  bool coop = false;   // k_window_reduce_coop: RT groups of 8 lanes
};
template <class F>
int reduce_blocks_per_sm(uint32_t RT) {
  static int cache[9] = {};
  int lrt = 0;
  while ((1u << lrt) < RT) lrt++;
  if (!cache[lrt]) {
    int n = 0;
    if constexpr (kReduceInSmem<F>)
      BG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_window_reduce_sm<F>, (int)RT,
                                                            reduce_sm_bytes<F>(RT)));
    else
      BG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_window_reduce<F>, (int)RT,
                                                            RT * 4 * FieldWords<F>::value * sizeof(uint32_t)));
    cache[lrt] = n > 0 ? n : 1;
  }
  return cache[lrt];
}
// The host's part of a reduction, in device additions: J parts per bucket set, 3 host additions
// each at about 1/16 of a device addition's latency.  With `pooled`, a single bucket set of a
// power-of-two J >= 32 (window tables) counts as msm_finish sums it: in chunks on the host pool,
// so its latency is a chunk's parts plus the chunks' join.
inline double host_parts_cost(uint32_t J, int sets, bool pooled) {
  if (pooled && sets == 1 && J >= 32 && (J & (J - 1)) == 0) {
    const uint32_t chunks = std::min<uint32_t>(16, J / 8), C = J / chunks;
    return 3.0 * (C + chunks) / 16.0;
  }
  return 3.0 * J * sets / 16.0;
}

template <class F>
ReduceShape reduce_shape(uint32_t nb, int sets, size_t entries, uint32_t K, int sm_count, uint32_t max_rt,
                         bool pooled_host = false) {
  const double e = (double)entries / ((double)nb * sets);
  const double per_bucket = 2.0 + e / K;
  ReduceShape best{nb < 32 ? nb : 32, 1, 1};
  best.J = nb / best.RT;
  double best_cost = 1e300;
  for (uint32_t RT = 32; RT <= max_rt; RT <<= 1) {
    for (uint32_t M = 1; M <= 16; M <<= 1) {
      if ((uint64_t)RT * M > nb) continue;
      const uint32_t J = nb / (RT * M);
      int lrt = 0, lm = 0;
      while ((1u << lrt) < RT) lrt++;
      while ((1u << lm) < M) lm++;
      const double slots = (double)sm_count * reduce_blocks_per_sm<F>(RT);
      const double waves = std::ceil((double)J * sets / slots);
      const double cost = waves * (M * per_bucket + 2.0 * lrt + lm) + host_parts_cost(J, sets, pooled_host);
      if (cost < best_cost) {
        best_cost = cost;
        best = {RT, M, J, cost, false};
      }
    }
  }
  best.cost = best_cost;
  return best;
}

// A hidden reduction's shape by work instead of latency: the one with the fewest warp-additions
// per bucket (the running sums, plus the scan, doublings and tree that a CTA of RT threads adds
// on top, counted per warp as a warp issues them) whose latency by reduce_shape's model stays
// within `max_cost` dependent additions; {0, 0, 0} when none does.
template <class F>
ReduceShape reduce_shape_work(uint32_t nb, int sets, size_t entries, uint32_t K, int sm_count, uint32_t max_rt,
                              double max_cost) {
  const double e = (double)entries / ((double)nb * sets);
  const double per_bucket = 2.0 + e / K;
  ReduceShape best{0, 0, 0, 1e300, false};
  double best_work = 1e300;
  for (uint32_t RT = 32; RT <= max_rt; RT <<= 1) {
    for (uint32_t M = 1; M <= 16; M <<= 1) {
      if ((uint64_t)RT * M > nb) continue;
      const uint32_t J = nb / (RT * M);
      int lrt = 0, lm = 0;
      while ((1u << lrt) < RT) lrt++;
      while ((1u << lm) < M) lm++;
      const double slots = (double)sm_count * reduce_blocks_per_sm<F>(RT);
      const double waves = std::ceil((double)J * sets / slots);
      const double cost = waves * (M * per_bucket + 2.0 * lrt + lm) + host_parts_cost(J, sets, false);
      if (cost > max_cost) continue;
      const double warps = RT / 32.0;
      double scan = 0, tree = 0;
      for (uint32_t d = 1; d < RT; d <<= 1) scan += std::ceil((RT - d) / 32.0);
      for (uint32_t d = RT >> 1; d >= 1; d >>= 1) tree += std::ceil(d / 32.0);
      const double work = (warps * M * per_bucket + scan + warps * (lm + 1) + tree) / ((double)RT * M);
      if (work < best_work - 1e-12) {
        best_work = work;
        best = {RT, M, J, cost, false};
      }
    }
  }
  return best;
}

#include "msm_coop.cuh"

// The cooperative form's shape by the same model: RT groups (of 8 lanes) per CTA, each addition
// about kCoopAddCost of a thread's addition (dependency depth 4.6 of 14 products, plus the
// group's exchanges), the log2 M doublings on one lane at full cost.
constexpr double kCoopAddCost = 0.45;
template <class F>
int reduce_coop_blocks_per_sm(uint32_t RT) {
  static int cache[6] = {};
  int lrt = 0;
  while ((1u << lrt) < RT) lrt++;
  if (!cache[lrt]) {
    int n = 0;
    BG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_window_reduce_coop<F>, (int)RT * kCoopLanes,
                                                          RT * coop_group_words<F>() * sizeof(uint32_t)));
    cache[lrt] = n > 0 ? n : 1;
  }
  return cache[lrt];
}
template <class F>
ReduceShape reduce_shape_coop(uint32_t nb, int sets, size_t entries, uint32_t K, int sm_count, bool pooled_host) {
  const double e = (double)entries / ((double)nb * sets);
  const double per_bucket = 2.0 + e / K;
  ReduceShape best{0, 0, 0, 1e300, true};
  for (uint32_t RT = 4; RT <= 32; RT <<= 1) {
    for (uint32_t M = 1; M <= 16; M <<= 1) {
      if ((uint64_t)RT * M > nb) continue;
      const uint32_t J = nb / (RT * M);
      int lrt = 0, lm = 0;
      while ((1u << lrt) < RT) lrt++;
      while ((1u << lm) < M) lm++;
      const double slots = (double)sm_count * reduce_coop_blocks_per_sm<F>(RT);
      const double waves = std::ceil((double)J * sets / slots);
      const double cost =
          waves * (kCoopAddCost * (M * per_bucket + 2.0 * lrt) + lm) + host_parts_cost(J, sets, pooled_host);
      if (cost < best.cost) best = {RT, M, J, cost, true};
    }
  }
  return best;
}

// ---------------------------------------------------------------- host driver
static int floor_log2(size_t n) {
  int lg = 0;
  while ((size_t(1) << (lg + 1)) <= n) lg++;
  return lg;
}
static int tuned(const signed char (*tab)[kTuneMaxLog2 - kTuneMinLog2 + 1], size_t n, bool g2) {
  const int lg = floor_log2(n);
  return lg >= kTuneMinLog2 && lg <= kTuneMaxLog2 ? tab[g2 ? 1 : 0][lg - kTuneMinLog2] : 0;
}

int msm_pick_c(size_t n, bool g2) {
  if (const int t = tuned(kTuneSets, n, g2)) return t;
  int c = floor_log2(n) - 3;
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

void msm_sort(Ctx& ctx, cudaStream_t st, const std::string& tag, const uint32_t* d_scalars, size_t n, int c,
              bool shared_set, MsmSort& out) {
  out = MsmSort();
  out.n = n;
  if (n == 0) return;
  if (n >= 0x80000000ull) throw Error(BG_E_ARG, "msm: n must be below 2^31");
  if (c < 2 || c > 24) throw Error(BG_E_ARG, "msm: window width out of range");
  const int W = 254 / c + 1;
  const uint32_t nb = 1u << (c - 1);
  const int sets = shared_set ? 1 : W;
  const size_t nkeys = (size_t)sets * nb;
  const uint32_t key_stride = shared_set ? 0u : nb;
  const uint32_t idx_stride = shared_set ? (uint32_t)n : 0u;
  const size_t max_entries = n * (size_t)W;
  if (max_entries >= 0x80000000ull) throw Error(BG_E_ARG, "msm: n x windows must be below 2^31");
  out.c = c;
  out.W = W;
  out.sets = sets;
  out.nb = nb;
  out.nkeys = nkeys;
  out.max_entries = max_entries;

  Workspace& ws = ctx.ws;
  uint32_t* counts = ws.get_t<uint32_t>(tag + ".counts", nkeys + 1);
  uint32_t* cursor = ws.get_t<uint32_t>(tag + ".cursor", nkeys + 1);
  out.offsets = ws.get_t<uint32_t>(tag + ".offsets", nkeys + 1);
  out.sorted = ws.get_t<uint32_t>(tag + ".sorted", max_entries);
  BG_CUDA(cudaMemsetAsync(counts, 0, (nkeys + 1) * sizeof(uint32_t), st));
  {
    KernelTimer kt(ctx, "msm_digits", st);
    k_digits_hist<<<ceil_div(n, 256), 256, 0, st>>>(d_scalars, n, c, W, key_stride, counts, ctx.d_status);
    BG_CHECK_LAUNCH();
  }
  exclusive_scan(ws, tag, counts, out.offsets, nkeys + 1, st, 0);
  BG_CUDA(cudaMemcpyAsync(cursor, out.offsets, (nkeys + 1) * sizeof(uint32_t), cudaMemcpyDeviceToDevice, st));
  {
    KernelTimer kt(ctx, "msm_scatter", st);
    k_scatter<<<ceil_div(n, 256), 256, 0, st>>>(d_scalars, n, c, W, key_stride, idx_stride, cursor, out.sorted);
    BG_CHECK_LAUNCH();
  }
  out.done = ctx.event(tag + ".sorted");
  BG_CUDA(cudaEventRecord(out.done, st));
}

template <class F>
void msm_accumulate(Ctx& ctx, cudaStream_t st, const std::string& tag, const uint32_t* d_points, const MsmSort& so,
                    MsmPlan& plan, cudaStream_t st_reduce, const MsmTable* table) {
  constexpr int FW = FieldWords<F>::value;
  constexpr int PW = 4 * FW;
  if (so.n == 0) {
    plan.W = 0;
    return;
  }
  if (table && (table->n != so.n || table->c != so.c || so.sets != 1))
    throw Error(BG_E_ARG, "msm: window table and bucket order disagree");
  if (!table && so.sets == 1) throw Error(BG_E_ARG, "msm: a shared bucket set needs a window table");
  msm_init_kernels();
  if (table) d_points = table->d;
  plan.c = so.c;
  plan.W = so.sets;
  Workspace& ws = ctx.ws;
  if (so.done) BG_CUDA(cudaStreamWaitEvent(st, so.done, 0));
  Ctx* prof = (ctx.profile || ctx.timeline) ? &ctx : nullptr;

  // Batch-affine pair rounds, where the cost model (or the tuning override) takes them, halve
  // every bucket in affine coordinates first (msm_pairs.cuh); the XYZZ accumulation, the heavy
  // pass and the reduction then read the last level's points directly, with its offsets.
  const uint32_t* acc_points = d_points;
  const uint32_t* acc_sorted = so.sorted;
  const uint32_t* acc_offsets = so.offsets;
  size_t acc_entries = so.max_entries;
  const int rounds = ctx.pair_rounds_override >= 0 ? ctx.pair_rounds_override
                                                   : pair_rounds_model(so.max_entries, so.nkeys, FW == 16);
  if (rounds > 0) {
    constexpr int NT = kPairThreads<F>;
    const double pslots = pair_slots<F>();
    const uint32_t me = (uint32_t)so.max_entries;
    const uint32_t nk = (uint32_t)so.nkeys;
    uint32_t* lvl[2] = {ws.get_t<uint32_t>(tag + ".pairs0", level_start(me, nk, 1) * 2 * FW), nullptr};
    if (rounds > 1) lvl[1] = ws.get_t<uint32_t>(tag + ".pairs1", level_start(me, nk, 2) * 2 * FW);
    uint32_t* fin = ws.get_t<uint32_t>(tag + ".pair_offsets", so.nkeys + 1);
    KernelTimer kt(ctx, FW == 8 ? "msm_pair_g1" : "msm_pair_g2", st);
    for (int r = 0; r < rounds; r++) {
      // Up to 256 positions per thread, in a whole number of waves of resident threads: one
      // wave of long batches amortises each CTA's product tree and inversion best (G1 MSM 2^20
      // round 0: 1.99 ms with 32 positions per thread in 4 waves, 1.78 ms in one wave of 118).
      const double outs = (double)level_start(me, nk, r + 1);
      const double waves = std::max(1.0, std::ceil(outs / (pslots * 256.0)));
      const uint32_t per = (uint32_t)std::max(1.0, std::ceil(outs / (waves * pslots)));
      const unsigned grid = ceil_div(ceil_div((size_t)outs, per), NT);
      if (r == 0)
        k_pair_round<F, true><<<grid, NT, 0, st>>>(d_points, so.sorted, so.offsets, nk, 0, per, lvl[0], rounds, fin);
      else
        k_pair_round<F, false><<<grid, NT, 0, st>>>(lvl[(r - 1) & 1], nullptr, so.offsets, nk, r, per, lvl[r & 1],
                                                    rounds, nullptr);
      BG_CHECK_LAUNCH();
    }
    acc_points = lvl[(rounds - 1) & 1];
    acc_sorted = nullptr;
    acc_offsets = fin;
    acc_entries = level_start(me, nk, rounds);
  }
  plan.entries = acc_entries;
  uint32_t* buckets = ws.get_t<uint32_t>(tag + ".buckets", so.nkeys * PW);
  const BucketScratch bs = bucket_scratch<F>(acc_entries, so.nkeys, [&](const char* name, size_t words) {
    return ws.get_t<uint32_t>(tag + ".slice_" + name, words);
  });
  bucket_accumulate<F>(prof, st, acc_points, acc_offsets, acc_sorted, (uint32_t)so.nkeys, acc_entries, buckets, bs);

  cudaStream_t rs = st;
  if (st_reduce && st_reduce != st) {
    // the latency-bound heavy-bucket pass and reduction run on their own stream and overlap
    // whatever `st` does next (the next MSM's accumulation)
    cudaEvent_t ev = ctx.event(tag + ".acc_done");
    BG_CUDA(cudaEventRecord(ev, st));
    BG_CUDA(cudaStreamWaitEvent(st_reduce, ev, 0));
    rs = st_reduce;
  }
  bucket_heavy<F>(prof, rs, acc_offsets, buckets, bs);

  // A reduction hidden under a later accumulation keeps its CTAs at 128 threads: a 256-thread
  // CTA of ~210 registers leaves no room for an accumulation CTA on its SM for its whole
  // (latency-bound) life (K = 18 proof: caps 64 / 128 / 256 measured 11.0 / 10.8 / 10.8 ms
  // with the reductions' streams first, 10.12 / 9.87 / 9.94 ms with the accumulations first).
  ReduceShape rsh =
      reduce_shape<F>(so.nb, so.sets, acc_entries, bs.K, ctx.sm_count, plan.latency_critical ? 256u : 128u);
  // A reduction meant to run under later accumulations that the latency model says outlasts
  // them (a mid-size proof's G2 MSM: SquareChain(2^14)'s took 1.02 ms after 0.39 ms of
  // remaining accumulations) is critical after all.  Latency of one dependent addition at a
  // reduction's occupancy: about 11 us (G1), 29 us (G2), measured on GB300.
  // It takes the critical shapes only when it would outlast its budget twice over (by one time,
  // SquareChain(2^15) and 2^16 proofs measured 1-4% slower: reductions near their budget are
  // hidden well enough; by four times, 2^14 measured 1.59 -> 1.95 ms).  A critical reduction that ends while the host pool is otherwise idle
  // (not one of a small proof's reductions, which end together and share the pool with the
  // combine's products) has its host part sums priced as the pool runs them.  Interleaved on
  // one GB300 against the fixed rule (only the last MSM critical): SquareChain(2^13) 2.12 ->
  // 1.24 ms, 2^14 2.09 -> 1.68 ms, 2^16 3.75 -> 3.70 ms, 2^10 / 2^12 / 2^18 level.
  bool critical = plan.latency_critical;
  const double add_us = FW == 16 ? 29.0 : 11.0;
  if (!critical && plan.hidden_us > 0 && rsh.cost * add_us > 2.0 * plan.hidden_us) critical = true;
  // A hidden G1 reduction takes the shape with the least work per bucket (longer chains, fewer
  // scan, doubling and tree additions per bucket) whose modelled latency stays within a quarter
  // of its budget (the model underestimates a reduction running beside accumulations by 1.3-2x).
  // Interleaved against the shortest-chain shapes on one GB300: SquareChain(2^16) 3.69 ->
  // 3.46 ms, 2^17 6.14 -> 5.96 ms, 2^18 10.55 -> 10.48 ms, 2^14 and 2^20 level; with the
  // accumulations first, half or all of the budget instead of a quarter measured level to 6%
  // slower (2^16 3.46 -> 3.51 / 3.69 ms).  For G2 it
  // measured level to 1% slower at 2^20 (the G2 reduction stretched 2.9 -> 5.1 ms and crowded
  // the last accumulations), so G2 keeps the shortest chain.
  if (!critical && plan.hidden_us > 0 && FW == 8) {
    const ReduceShape wsh =
        reduce_shape_work<F>(so.nb, so.sets, acc_entries, bs.K, ctx.sm_count, 128u, 0.25 * plan.hidden_us / add_us);
    if (wsh.RT) rsh = wsh;
  }
  const bool pooled = critical && plan.host_pool_free;
  if (pooled) rsh = reduce_shape<F>(so.nb, so.sets, acc_entries, bs.K, ctx.sm_count, 256u, true);
  // a reduction that ends a critical path may take the cooperative form (8 lanes per addition)
  if (critical && ctx.coop_reduce != 0) {
    const ReduceShape csh = reduce_shape_coop<F>(so.nb, so.sets, acc_entries, bs.K, ctx.sm_count, pooled);
    if (ctx.coop_reduce > 0 || csh.cost < rsh.cost) rsh = csh;
  }
  const uint32_t RT = rsh.RT, M = rsh.M, J = rsh.J;
  uint32_t* parts = ws.get_t<uint32_t>(tag + ".parts", (size_t)so.sets * J * 2 * PW);
  {
    KernelTimer kt(ctx, FW == 8 ? "msm_reduce_g1" : "msm_reduce_g2", rs);
    if (rsh.coop)
      k_window_reduce_coop<F><<<so.sets * J, RT * kCoopLanes, RT * coop_group_words<F>() * sizeof(uint32_t), rs>>>(
          acc_offsets, buckets, bs.parts, bs.K, so.nb, M, J, parts);
    else if constexpr (kReduceInSmem<F>)
      k_window_reduce_sm<F><<<so.sets * J, RT, reduce_sm_bytes<F>(RT), rs>>>(acc_offsets, buckets, bs.parts, bs.K,
                                                                             so.nb, M, J, parts);
    else
      k_window_reduce<F><<<so.sets * J, RT, RT * PW * sizeof(uint32_t), rs>>>(acc_offsets, buckets, bs.parts, bs.K,
                                                                               so.nb, M, J, parts);
    BG_CHECK_LAUNCH();
  }
  plan.fetch_stream = rs;
  plan.J = J;
  plan.part_span = RT * M;
  plan.d_window_sums = parts;
  plan.host_window_sums = ctx.host_cache.get_t<uint32_t>(tag + ".window_sums", (size_t)so.sets * J * 2 * PW);
}

template <class F>
void msm_launch(Ctx& ctx, cudaStream_t st, const std::string& tag, const uint32_t* d_points,
                const uint32_t* d_scalars, size_t n, MsmPlan& plan, cudaStream_t st_reduce, const MsmTable* table) {
  if (table && table->n != n) throw Error(BG_E_ARG, "msm: window table built for another size");
  const int c = table ? table->c : (plan.c > 0 ? plan.c : msm_pick_c(n, FieldWords<F>::value == 16));
  MsmSort so;
  msm_sort(ctx, st, tag, d_scalars, n, c, table != nullptr, so);
  so.done = nullptr;  // same stream: already ordered
  msm_accumulate<F>(ctx, st, tag, d_points, so, plan, st_reduce, table);
}

int msm_pair_rounds_entries(size_t max_entries, size_t nkeys, bool g2) {
  return pair_rounds_model(max_entries, nkeys, g2);
}

int msm_pair_rounds(size_t n, bool g2) {
  if (n == 0) return 0;
  const int c = msm_pick_c(n, g2);
  const size_t W = 254 / c + 1;
  return pair_rounds_model(n * W, W << (c - 1), g2);
}

int msm_pick_c_proof(size_t n, bool g2) {
  if (const int t = tuned(kTuneProofSets, n, g2)) return t;
  return msm_pick_c(n, g2);
}

int msm_pick_c_table(size_t n, bool g2) {
  // one shared bucket set: wider windows (fewer additions) at the price of 2^(c-1) buckets
  if (const int t = tuned(kTuneTables, n, g2)) return t;
  int c = floor_log2(n) - 1;
  if (c < 6) c = 6;
  if (c > 18) c = 18;
  return c;
}

template <class F>
void msm_build_table(cudaStream_t st, const uint32_t* d_points, size_t n, MsmTable& t, int c) {
  constexpr int PW = 2 * FieldWords<F>::value;
  if (c != 0 && (c < 2 || c > 22)) throw Error(BG_E_ARG, "msm table: window width out of range");
  t.n = n;
  t.c = c ? c : msm_pick_c_table(n, FieldWords<F>::value == 16);
  t.W = 254 / t.c + 1;
  if (n == 0) return;
  if (n * (size_t)t.W >= 0x80000000ull) throw Error(BG_E_ARG, "msm table: n x windows must be below 2^31");
  void* p = nullptr;
  const size_t bytes = n * (size_t)t.W * PW * sizeof(uint32_t);
  cudaError_t e = cudaMalloc(&p, bytes);
  if (e != cudaSuccess) {
    cudaGetLastError();
    throw Error(BG_E_OOM, "window table allocation of " + std::to_string(bytes) + " bytes failed");
  }
  t.d = static_cast<uint32_t*>(p);
  k_build_table<F><<<ceil_div(n, 128), 128, 0, st>>>(d_points, n, t.c, t.W, t.d);
  BG_CHECK_LAUNCH();
}

template void msm_build_table<Fq>(cudaStream_t, const uint32_t*, size_t, MsmTable&, int);
template void msm_build_table<Fq2>(cudaStream_t, const uint32_t*, size_t, MsmTable&, int);

template <class F>
void msm_fetch(Ctx& ctx, cudaStream_t st, MsmPlan& plan) {
  constexpr int PW = 4 * FieldWords<F>::value;
  if (plan.W == 0) return;
  if (plan.fetch_stream) st = plan.fetch_stream;
  BG_CUDA(cudaMemcpyAsync(plan.host_window_sums, plan.d_window_sums,
                          (size_t)plan.W * plan.J * 2 * PW * sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
  ctx.d2h_bytes += (uint64_t)plan.W * plan.J * 2 * PW * sizeof(uint32_t);
}

// Window w = sum_j S_j + span * sum_j j R_j; total = sum_w 2^(o_w) window_w (Horner).
template <class F>
void msm_finish(const MsmPlan& plan, uint32_t* out_affine_words32) {
  typedef typename HostField<F>::T H;
  constexpr int PW = 4 * H::WORDS;
  // window w's sum from its J parts: sum_j S_j + span sum_{j>=1} j R_j (independent per window)
  std::vector<bgh::Xyzz<H>> wsum(plan.W);
  auto window_sum = [&](int w) {
    const uint32_t* pw = plan.host_window_sums + (size_t)w * plan.J * 2 * PW;
    bgh::Xyzz<H> s = bgh::xyzz_inf<H>(), run = bgh::xyzz_inf<H>(), jr = bgh::xyzz_inf<H>();
    for (int j = (int)plan.J - 1; j >= 0; j--) {
      s = bgh::xyzz_add(s, bgh::xyzz_from_words32<H>(pw + (size_t)(2 * j) * PW));
      if (j >= 1) {
        run = bgh::xyzz_add(run, bgh::xyzz_from_words32<H>(pw + (size_t)(2 * j + 1) * PW));
        jr = bgh::xyzz_add(jr, run);  // sum_{j>=1} j R_j
      }
    }
    for (uint32_t m = plan.part_span; m > 1; m >>= 1) jr = bgh::xyzz_dbl(jr);
    wsum[w] = bgh::xyzz_add(s, jr);
  };
  // One window of many parts (the shared bucket set of a key's window tables, e.g. J = 128 for
  // msm_h of a SquareChain(2^18) proof: ~390 host additions after the proof's last kernel) is
  // split into power-of-two chunks of parts on the host pool.  Chunk c covers parts [lo, lo + C)
  // with lo = c C and gives s_c = sum S_j, t_c = sum R_j, u_c = sum (j - lo) R_j; then
  // sum_j j R_j = sum_c u_c + C sum_{c>=1} c t_c, the last sum by a running sum over chunks.
  auto single_window_chunked = [&]() {
    const uint32_t J = plan.J;
    const uint32_t chunks = std::min<uint32_t>(16, J / 8), C = J / chunks;
    const uint32_t* pw = plan.host_window_sums;
    std::vector<bgh::Xyzz<H>> cs(chunks), ct(chunks), cu(chunks);
    HostPool::get().parallel_for((int)chunks, [&](int c) {
      const uint32_t lo = (uint32_t)c * C;
      bgh::Xyzz<H> s = bgh::xyzz_inf<H>(), run = bgh::xyzz_inf<H>(), u = bgh::xyzz_inf<H>();
      for (int j = (int)(lo + C) - 1; j >= (int)lo; j--) {
        s = bgh::xyzz_add(s, bgh::xyzz_from_words32<H>(pw + (size_t)(2 * j) * PW));
        run = bgh::xyzz_add(run, bgh::xyzz_from_words32<H>(pw + (size_t)(2 * j + 1) * PW));
        if (j > (int)lo) u = bgh::xyzz_add(u, run);
      }
      cs[c] = s;
      ct[c] = run;
      cu[c] = u;
    });
    bgh::Xyzz<H> s = bgh::xyzz_inf<H>(), jr = bgh::xyzz_inf<H>(), run = bgh::xyzz_inf<H>(),
                 ctop = bgh::xyzz_inf<H>();
    for (int c = (int)chunks - 1; c >= 0; c--) {
      s = bgh::xyzz_add(s, cs[c]);
      jr = bgh::xyzz_add(jr, cu[c]);
      if (c >= 1) {
        run = bgh::xyzz_add(run, ct[c]);
        ctop = bgh::xyzz_add(ctop, run);  // sum_{c>=1} c t_c
      }
    }
    for (uint32_t m = C; m > 1; m >>= 1) ctop = bgh::xyzz_dbl(ctop);
    jr = bgh::xyzz_add(jr, ctop);  // sum_{j>=1} j R_j
    for (uint32_t m = plan.part_span; m > 1; m >>= 1) jr = bgh::xyzz_dbl(jr);
    wsum[0] = bgh::xyzz_add(s, jr);
  };
  // The window sums of a bucket-set-per-window MSM are about two thirds of its host work
  // (17 windows x 8 parts: ~550 of ~850 point operations); they run on the host pool, the
  // Horner chain after them stays serial.  SquareChain(2^18) one-shot proof: the G2 finish is
  // the tail of the proof.
  const bool pow2_parts = plan.J >= 32 && (plan.J & (plan.J - 1)) == 0;
  if (plan.W == 1 && pow2_parts && HostPool::get().workers() > 0) single_window_chunked();
  else if (plan.W >= 4 && (size_t)plan.W * plan.J >= 32) HostPool::get().parallel_for(plan.W, window_sum);
  else
    for (int w = 0; w < plan.W; w++) window_sum(w);
  bgh::Xyzz<H> acc = bgh::xyzz_inf<H>();
  for (int w = plan.W - 1; w >= 0; w--) {
    for (int d = 0; d < window_width(w, plan.W); d++) acc = bgh::xyzz_dbl(acc);
    acc = bgh::xyzz_add(acc, wsum[w]);
  }
  bgh::aff_to_words32<H>(out_affine_words32, bgh::xyzz_to_affine(acc));
}

// Kernel attributes (the opt-in to large dynamic shared memory) apply to the device that is
// current when they are set, so they are set once per device; batch lanes and server threads
// may get here at the same time, hence the per-device once flags.
constexpr int kInitMaxDevices = 64;
void msm_init_kernels() {
  static std::once_flag once[kInitMaxDevices];
  static_assert(!kReduceInSmem<Fq> && kReduceInSmem<Fq2>, "reduction forms: G1 in registers, G2 in shared memory");
  int dev = 0;
  BG_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kInitMaxDevices) throw Error(BG_E_ARG, "msm: device index out of range");
  std::call_once(once[dev], [] {
    BG_CUDA(cudaFuncSetAttribute(k_window_reduce<Fq>, cudaFuncAttributeMaxDynamicSharedMemorySize, 256 * 32 * 4));
    BG_CUDA(cudaFuncSetAttribute(k_window_reduce_sm<Fq2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)reduce_sm_bytes<Fq2>(256)));
  });
}

template void msm_launch<Fq>(Ctx&, cudaStream_t, const std::string&, const uint32_t*, const uint32_t*, size_t,
                             MsmPlan&, cudaStream_t, const MsmTable*);
template void msm_accumulate<Fq>(Ctx&, cudaStream_t, const std::string&, const uint32_t*, const MsmSort&, MsmPlan&,
                                 cudaStream_t, const MsmTable*);
template void msm_accumulate<Fq2>(Ctx&, cudaStream_t, const std::string&, const uint32_t*, const MsmSort&, MsmPlan&,
                                  cudaStream_t, const MsmTable*);
template void msm_launch<Fq2>(Ctx&, cudaStream_t, const std::string&, const uint32_t*, const uint32_t*, size_t,
                              MsmPlan&, cudaStream_t, const MsmTable*);
template void msm_fetch<Fq>(Ctx&, cudaStream_t, MsmPlan&);
template void msm_fetch<Fq2>(Ctx&, cudaStream_t, MsmPlan&);
template void msm_finish<Fq>(const MsmPlan&, uint32_t*);
template void msm_finish<Fq2>(const MsmPlan&, uint32_t*);

}  // namespace bg

// ---------------------------------------------------------------- allocation-free G1 MSM
// bg_msm_g1_noalloc serves callers that must not allocate device memory at all: a host
// program that has handed the whole GPU to its own memory pool and forbids any further
// cudaMalloc, or a latency-critical loop in which the device-wide synchronisation that
// cudaMalloc/cudaFree imply is not acceptable.  It runs the same kernels as the other MSM
// entry points, but every scratch buffer is carved out of one fixed array that lives in the
// library's own device image, so the call allocates nothing (no cudaMalloc, cudaFree,
// pinned-host allocation or context).  The price is a hard size limit and shared state:
//   * at most kNoAllocMaxPoints points (larger requests fail with BG_E_ARG);
//   * every GPU that loads the library holds the kNoAllocScratchBytes array until the process
//     exits;
//   * all calls use the same array, which keeps the previous call's contents (the bucket
//     counters are cleared at the start of each call); calls that overlap on the GPU race, so
//     this entry point serialises calls made from one process and returns only when its work
//     is complete;
//   * the first call on a device looks up the array's device address on that device (the
//     device current at the call);
//   * every call ends with a synchronisation of its stream and copies to pageable host memory,
//     so it must not be called on a stream that is being captured.
namespace bg {
namespace {

constexpr size_t kNoAllocMaxPoints = size_t(1) << 14;
constexpr size_t kNoAllocScratchBytes = size_t(9) << 20;  // the worst case up to 2^14 points needs 6.6 MiB
constexpr size_t kNoAllocHostWords = 8192;                // window parts copied back for the Horner
constexpr int kNoAllocMaxDevices = 64;

static __device__ __align__(256) uint8_t g_noalloc_scratch[kNoAllocScratchBytes];
static uint32_t g_noalloc_host_parts[kNoAllocHostWords];
static uint32_t g_noalloc_host_status;
static void* g_noalloc_dev_ptr[kNoAllocMaxDevices];
static std::mutex g_noalloc_mu;

// device address of the scratch array on the current device (looked up once per device)
uint8_t* noalloc_scratch() {
  int dev = 0;
  BG_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kNoAllocMaxDevices) throw Error(BG_E_ARG, "bg_msm_g1_noalloc: device index out of range");
  if (!g_noalloc_dev_ptr[dev]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p)
      throw Error(BG_E_DEVICE, std::string("bg_msm_g1_noalloc: cudaGetSymbolAddress failed: ") + cudaGetErrorString(e));
    g_noalloc_dev_ptr[dev] = p;
  }
  return static_cast<uint8_t*>(g_noalloc_dev_ptr[dev]);
}

void msm_g1_noalloc(const uint32_t* d_points, const uint32_t* d_scalars, size_t n, cudaStream_t st,
                    uint32_t* out_aff32) {
  constexpr int PW = 32;  // packed words of a G1 XYZZ point
  if (n == 0) {
    memset(out_aff32, 0, 16 * sizeof(uint32_t));
    return;
  }
  if (n > kNoAllocMaxPoints)
    throw Error(BG_E_ARG, "bg_msm_g1_noalloc: " + std::to_string(n) + " points exceed the fixed maximum of " +
                              std::to_string(kNoAllocMaxPoints));
  uint8_t* base = noalloc_scratch();
  const int c = msm_pick_c(n);
  const int W = 254 / c + 1;
  const uint32_t nb = 1u << (c - 1);
  const size_t nkeys = (size_t)W * nb;
  const size_t max_entries = n * (size_t)W;
  int dev = 0, sms = 0;
  BG_CUDA(cudaGetDevice(&dev));
  BG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  msm_init_kernels();
  const ReduceShape rsh = reduce_shape<Fq>(nb, W, max_entries, 32, sms, 256u);
  const uint32_t RT = rsh.RT, M = rsh.M, J = rsh.J;
  const unsigned tiles = ceil_div(nkeys + 1, kScanTile);

  size_t off = 0;
  auto carve = [&](size_t words) {
    uint32_t* p = reinterpret_cast<uint32_t*>(base + off);
    off += (words * sizeof(uint32_t) + 255) & ~size_t(255);
    return p;
  };
  uint32_t* status = carve(1);
  uint32_t* counts = carve(nkeys + 1);
  uint32_t* offsets = carve(nkeys + 1);
  uint32_t* cursor = carve(nkeys + 1);
  uint32_t* tile_sums = carve(tiles);
  uint32_t* tile_offs = carve(tiles);
  uint32_t* sorted = carve(max_entries);
  uint32_t* buckets = carve(nkeys * PW);
  // 32-entry slices: the fixed array is sized for them
  const BucketScratch bs =
      bucket_scratch<Fq>(max_entries, nkeys, [&](const char*, size_t words) { return carve(words); }, 32);
  uint32_t* parts = carve((size_t)W * J * 2 * PW);
  const size_t host_words = (size_t)W * J * 2 * PW;
  if (off > kNoAllocScratchBytes || host_words > kNoAllocHostWords || tiles > (unsigned)kScanTile)
    throw Error(BG_E_ARG, "bg_msm_g1_noalloc: scratch layout exceeds the fixed array");

  // what must start at zero: the status word and the bucket counters
  BG_CUDA(cudaMemsetAsync(status, 0, sizeof(uint32_t), st));
  BG_CUDA(cudaMemsetAsync(counts, 0, (nkeys + 1) * sizeof(uint32_t), st));
  k_digits_hist<<<ceil_div(n, 256), 256, 0, st>>>(d_scalars, n, c, W, nb, counts, status);
  BG_CHECK_LAUNCH();
  if (tiles == 1) {
    k_scan_tile<<<1, kScanThreads, 0, st>>>(counts, offsets, nullptr, nkeys + 1);
    BG_CHECK_LAUNCH();
  } else {
    k_scan_tile<<<tiles, kScanThreads, 0, st>>>(counts, offsets, tile_sums, nkeys + 1);
    BG_CHECK_LAUNCH();
    k_scan_tile<<<1, kScanThreads, 0, st>>>(tile_sums, tile_offs, nullptr, tiles);
    BG_CHECK_LAUNCH();
    k_scan_add<<<ceil_div(nkeys + 1, 256), 256, 0, st>>>(offsets, tile_offs, nkeys + 1);
    BG_CHECK_LAUNCH();
  }
  BG_CUDA(cudaMemcpyAsync(cursor, offsets, (nkeys + 1) * sizeof(uint32_t), cudaMemcpyDeviceToDevice, st));
  k_scatter<<<ceil_div(n, 256), 256, 0, st>>>(d_scalars, n, c, W, nb, 0, cursor, sorted);
  BG_CHECK_LAUNCH();
  bucket_accumulate<Fq>(nullptr, st, d_points, offsets, sorted, (uint32_t)nkeys, max_entries, buckets, bs);
  bucket_heavy<Fq>(nullptr, st, offsets, buckets, bs);
  k_window_reduce<Fq><<<W * J, RT, RT * PW * sizeof(uint32_t), st>>>(offsets, buckets, bs.parts, bs.K, nb, M, J,
                                                                     parts);
  BG_CHECK_LAUNCH();
  BG_CUDA(cudaMemcpyAsync(g_noalloc_host_parts, parts, host_words * sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
  BG_CUDA(cudaMemcpyAsync(&g_noalloc_host_status, status, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
  BG_CUDA(cudaStreamSynchronize(st));
  if (g_noalloc_host_status & BG_DSTATUS_SCALAR_RANGE)
    throw Error(BG_E_ARG, "bg_msm_g1_noalloc: a scalar is not below 2^254 (not a canonical Fr)");
  MsmPlan plan;
  plan.c = c;
  plan.W = W;
  plan.J = J;
  plan.part_span = RT * M;
  plan.host_window_sums = g_noalloc_host_parts;
  msm_finish<Fq>(plan, out_aff32);
}

}  // namespace
}  // namespace bg

extern "C" int bg_msm_g1_noalloc(const uint32_t* d_points, const uint32_t* d_scalars, size_t n, void* stream,
                                 uint32_t* out_aff32) {
  if (!out_aff32 || (n && (!d_points || !d_scalars))) {
    bg::set_noctx_error("bg_msm_g1_noalloc: invalid argument (a null pointer)");
    return BG_E_ARG;
  }
  // points and scalars are read in 16-byte vectors: refuse a pointer off that boundary here
  // rather than let the device fault on it
  if ((reinterpret_cast<uintptr_t>(d_points) | reinterpret_cast<uintptr_t>(d_scalars)) & 15u) {
    bg::set_noctx_error("bg_msm_g1_noalloc: invalid argument (a device pointer not 16-byte aligned)");
    return BG_E_ARG;
  }
  std::lock_guard<std::mutex> lock(bg::g_noalloc_mu);
  try {
    bg::msm_g1_noalloc(d_points, d_scalars, n, static_cast<cudaStream_t>(stream), out_aff32);
    return BG_OK;
  } catch (const bg::Error& e) {
    bg::set_noctx_error(e.what());
    if (e.status == BG_E_DEVICE) cudaGetLastError();
    return e.status;
  } catch (const std::bad_alloc&) {
    bg::set_noctx_error("bg_msm_g1_noalloc: host allocation failed");
    return BG_E_OOM;
  } catch (const std::exception& e) {
    bg::set_noctx_error(std::string("bg_msm_g1_noalloc: ") + e.what());
    return BG_E_DEVICE;
  }
}
