// Batch-affine pair rounds of the MSM bucket accumulation (included by msm.cu).
//
// The bucket phase of Msm.g1 / Msm.g2 (bend2/src/msm.bend:120-158 adds every point of a
// window into its bucket with a Jacobian mixed addition) may be preceded by rounds that halve
// every bucket: round r adds the points of each bucket in pairs, in affine coordinates, and
// writes the sums (plus the odd point out) as the bucket's points for round r + 1.  The
// additions of a round are independent, so they share their field inversions: each thread
// multiplies its denominators into a running product, the CTA multiplies the threads'
// products in a tree in shared memory, one thread inverts the root (binary Euclid,
// inv_binary), and the tree and the running products are walked back to give every
// addition 1 / d (Montgomery's simultaneous inversion).  An addition then costs 5 products
// and a square (3 of them for the shared inversion) against madd-2008-s's 8 products and 2
// squares; the XYZZ accumulation that follows adds what the rounds left, and the window
// reduction is unchanged.
//
// Layout.  The entry list of the sort holds bucket b's m_b entries at [o_b, o_b + m_b).  After
// L rounds bucket b holds ceil(m_b / 2^L) points starting at
//     start_L(b) = floor((o_b + (2^(L+1) - 2) b) / 2^L),
// a closed form of the sort's offsets (start_{L+1}(b) = floor(start_L(b) / 2) + b), so no
// round needs a scan.  A bucket's region [start_L(b), start_L(b + 1)) is at least its point
// count (start_{L+1}(b) + ceil(m / 2) <= floor(start_L(b + 1) / 2) + b + 1 because
// start_L(b + 1) >= start_L(b) + m), every region of a level L >= 1 has at least one slot, and
// the slots past the points -- at most two per bucket after a few rounds -- hold the affine
// infinity (0, 0), so the XYZZ accumulation reads level L's regions as ordinary buckets with
// start_L as their offsets.
//
// Round r writes every position j of level r + 1: j in bucket b at index i = j - start_{r+1}(b)
// is the sum of level-r points 2i and 2i + 1 when both exist, point 2i when only it does, and
// infinity otherwise.  Round 0 reads its points through the sort's entries (index | sign << 31)
// from the MSM's point set or window table; later rounds read the previous level directly.

// start_L(b) for the sort's offset o = o_b; b = nkeys gives the level's size
__host__ __device__ inline uint64_t level_start(uint32_t o, uint64_t b, int level) {
  return ((uint64_t)o + (((uint64_t)2 << level) - 2) * b) >> level;
}
// ceil(m / 2^L): points of a bucket of m entries after L rounds
__host__ __device__ inline uint32_t level_count(uint32_t m, int level) {
  return (uint32_t)(((uint64_t)m + (1ull << level) - 1) >> level);
}

// CTA size (the batch of one shared inversion is CTA size x positions per thread); two CTAs per
// SM (G1: 124 registers, G2: 228)
template <class F>
constexpr int kPairThreads = FieldWords<F>::value == 8 ? 256 : 128;

// Input point k of a round: round 0 reads it through the sort's entry (index | sign << 31) from
// the MSM's point set or window table, later rounds read the previous level directly.  The
// entry code is loaded apart from the point so that it can be fetched a position ahead.
template <bool kFirst>
BG_DEV uint32_t pair_code(const uint32_t* __restrict__ sorted, uint64_t k) {
  if constexpr (kFirst) return sorted[k];
  else return (uint32_t)k;
}
template <class F, bool kFirst>
BG_DEV Affine<F> pair_point(const uint32_t* __restrict__ src, uint32_t code) {
  constexpr int FW = FieldWords<F>::value;
  const Affine<F> a = load_affine<F>(src + (size_t)(code & 0x7fffffffu) * 2 * FW);
  return (kFirst && (code >> 31)) ? affine_neg(a) : a;
}
template <class F>
BG_DEV F pair_x(const uint32_t* __restrict__ src, uint32_t code) {
  constexpr int FW = FieldWords<F>::value;
  F x;
  load_elem(x, src + (size_t)(code & 0x7fffffffu) * 2 * FW);
  return x;
}

// A bucket of the output level: its output region [out_lo, out_hi), its input points at
// [in_lo, in_lo + m_in).
struct PairBucket {
  uint32_t b;
  uint64_t out_lo, out_hi, in_lo;
  uint32_t m_in;
};
BG_DEV void pair_bucket_set(PairBucket& k, const uint32_t* __restrict__ offsets, uint32_t b, int level) {
  const uint32_t o0 = offsets[b], o1 = offsets[b + 1];
  k.b = b;
  k.out_lo = level_start(o0, b, level + 1);
  k.out_hi = level_start(o1, (uint64_t)b + 1, level + 1);
  k.in_lo = level_start(o0, b, level);
  k.m_in = level_count(o1 - o0, level);
}

// What output position j of a round reads: the input pair (in, in + 1), the single input in
// (the odd point of a bucket), or nothing (a slot past the bucket's points: infinity).  The
// bucket cursor k moves forward or backward to the bucket holding j.
enum : uint32_t { kSrcPair = 0, kSrcCopy = 1, kSrcNone = 2 };
template <bool kForward>
BG_DEV uint32_t pair_source(PairBucket& k, const uint32_t* __restrict__ offsets, uint64_t j, int level,
                            uint64_t& in) {
  if (kForward) {
    while (j >= k.out_hi) pair_bucket_set(k, offsets, k.b + 1, level);
  } else {
    while (j < k.out_lo) pair_bucket_set(k, offsets, k.b - 1, level);
  }
  const uint64_t i = j - k.out_lo;
  in = k.in_lo + 2 * i;
  return 2 * i + 1 < k.m_in ? kSrcPair : (2 * i < k.m_in ? kSrcCopy : kSrcNone);
}

// One round: input level `level` (src), output level + 1 (dst), `per_thread` consecutive output
// positions per thread.  dst's x field of each position first holds the running product of the
// thread's denominators up to it (read back by the backward pass) and is then overwritten by
// the sum.  Round 0 also writes the offsets of level `final_level` (the accumulation's).
template <class F, bool kFirst>
__global__ void __launch_bounds__(kPairThreads<F>, 2)
    k_pair_round(const uint32_t* __restrict__ src, const uint32_t* __restrict__ sorted,
                 const uint32_t* __restrict__ offsets, uint32_t nkeys, int level, uint32_t per_thread,
                 uint32_t* __restrict__ dst, int final_level, uint32_t* __restrict__ final_offsets) {
  constexpr int FW = FieldWords<F>::value;
  constexpr int PW = 2 * FW;
  constexpr int NT = kPairThreads<F>;
  __shared__ __align__(16) uint32_t tree[2 * NT * FW];
  const uint32_t tid = threadIdx.x;
  if (final_offsets) {
    for (size_t g = (size_t)blockIdx.x * NT + tid; g <= nkeys; g += (size_t)gridDim.x * NT)
      final_offsets[g] = (uint32_t)level_start(offsets[g], g, final_level);
  }
  const uint64_t total = level_start(offsets[nkeys], nkeys, level + 1);
  const uint64_t beg = ((uint64_t)blockIdx.x * NT + tid) * per_thread;
  const uint32_t cnt = beg >= total ? 0u : (total - beg < per_thread ? (uint32_t)(total - beg) : per_thread);

  // ---- forward: classify each position, multiply the denominators into acc
  F acc = field_one<F>();
  PairBucket k{};
  if (cnt) {
    uint32_t lo = 0, hi = nkeys;  // start_{level+1}(lo) <= beg < start_{level+1}(hi)
    while (hi - lo > 1) {
      const uint32_t mid = (lo + hi) >> 1;
      if (level_start(offsets[mid], mid, level + 1) <= beg) lo = mid;
      else hi = mid;
    }
    pair_bucket_set(k, offsets, lo, level);
    // The denominator of a pair is x_Q - x_P unless the x coordinates agree or one is zero (a
    // point at infinity, or a rare point with x = 0): only then are the full points read.  The
    // next pair's entry codes and x coordinates are fetched during this pair's product.
    uint64_t in_n;
    uint32_t src_n = pair_source<true>(k, offsets, beg, level, in_n);
    uint32_t cp_n = 0, cq_n = 0;
    F xp_n = field_zero<F>(), xq_n = field_zero<F>();
    if (src_n == kSrcPair) {
      cp_n = pair_code<kFirst>(sorted, in_n);
      cq_n = pair_code<kFirst>(sorted, in_n + 1);
      xp_n = pair_x<F>(src, cp_n);
      xq_n = pair_x<F>(src, cq_n);
    }
    for (uint32_t t = 0; t < cnt; t++) {
      const uint64_t j = beg + t;
      const uint32_t kind_src = src_n, cp = cp_n, cq = cq_n;
      const F xp = xp_n, xq = xq_n;
      if (t + 1 < cnt) {
        src_n = pair_source<true>(k, offsets, j + 1, level, in_n);
        if (src_n == kSrcPair) {
          cp_n = pair_code<kFirst>(sorted, in_n);
          cq_n = pair_code<kFirst>(sorted, in_n + 1);
          xp_n = pair_x<F>(src, cp_n);
          xq_n = pair_x<F>(src, cq_n);
        }
      }
      if (kind_src == kSrcPair) {
        F d = sub(xq, xp);
        bool inverted = true;
        if (is_zero(d) || is_zero(xp) || is_zero(xq)) {
          const Affine<F> p = pair_point<F, kFirst>(src, cp), q = pair_point<F, kFirst>(src, cq);
          inverted = pair_kind(p, q, d) <= kPairTangent;
        }
        if (inverted) acc = fmul(acc, d);
      }
      store_elem(dst + j * PW, acc);
    }
  }

  // ---- the CTA's product tree (leaves NT..2NT-1, node i = node 2i * node 2i+1), one
  // inversion of the root, and the tree walked back: leaf t ends as 1 / (thread t's product)
  store_elem(tree + (size_t)(NT + tid) * FW, acc);
  __syncthreads();
  for (uint32_t half = NT / 2; half >= 1; half >>= 1) {
    if (tid < half) {
      const uint32_t i = half + tid;
      F a, b;
      load_elem(a, tree + (size_t)(2 * i) * FW);
      load_elem(b, tree + (size_t)(2 * i + 1) * FW);
      store_elem(tree + (size_t)i * FW, fmul(a, b));
    }
    __syncthreads();
  }
  if (tid == 0) {
    F root;
    load_elem(root, tree + FW);
    store_elem(tree + FW, field_inv_fast(root));
  }
  __syncthreads();
  for (uint32_t half = 1; half < NT; half <<= 1) {
    if (tid < half) {
      const uint32_t i = half + tid;
      F iv, a, b;
      load_elem(iv, tree + (size_t)i * FW);
      load_elem(a, tree + (size_t)(2 * i) * FW);
      load_elem(b, tree + (size_t)(2 * i + 1) * FW);
      store_elem(tree + (size_t)(2 * i) * FW, fmul(iv, b));
      store_elem(tree + (size_t)(2 * i + 1) * FW, fmul(iv, a));
    }
    __syncthreads();
  }
  if (!cnt) return;
  F inv;
  load_elem(inv, tree + (size_t)(NT + tid) * FW);

  // ---- backward: 1 / d_t = inv * (product up to t - 1), inv *= d_t, and the sums; the next
  // position's entry codes are fetched a position ahead
  uint64_t in_n;
  uint32_t src_n = pair_source<false>(k, offsets, beg + cnt - 1, level, in_n);
  uint32_t cp_n = 0, cq_n = 0;
  if (src_n != kSrcNone) cp_n = pair_code<kFirst>(sorted, in_n);
  if (src_n == kSrcPair) cq_n = pair_code<kFirst>(sorted, in_n + 1);
  for (uint32_t t = cnt; t-- > 0;) {
    const uint64_t j = beg + t;
    const uint32_t kind_src = src_n, cp = cp_n, cq = cq_n;
    if (t > 0) {
      src_n = pair_source<false>(k, offsets, j - 1, level, in_n);
      if (src_n != kSrcNone) cp_n = pair_code<kFirst>(sorted, in_n);
      if (src_n == kSrcPair) cq_n = pair_code<kFirst>(sorted, in_n + 1);
    }
    Affine<F> r;
    if (kind_src == kSrcPair) {
      const Affine<F> p = pair_point<F, kFirst>(src, cp), q = pair_point<F, kFirst>(src, cq);
      F d = field_zero<F>(), dinv = field_zero<F>();
      const uint32_t kind = pair_kind(p, q, d);
      if (kind <= kPairTangent) {
        if (t > 0) {
          F prev;
          load_elem(prev, dst + (j - 1) * PW);
          dinv = fmul(inv, prev);
        } else {
          dinv = inv;
        }
        inv = fmul(inv, d);
      }
      r = pair_finish(p, q, kind, dinv);
    } else if (kind_src == kSrcCopy) {
      r = pair_point<F, kFirst>(src, cp);
    } else {
      r.x = field_zero<F>();
      r.y = field_zero<F>();
    }
    store_affine(dst + j * PW, r);
  }
}

// Rounds before the XYZZ accumulation.  Measured on GB300 (G1 MSM 2^20 with one bucket set per
// window, 17.8 M entries, 64 per bucket): a pair round costs 0.90 of the mixed additions it
// replaces (the pair kernel issues 76% of their instructions but loses more of its cycles to
// gathers and to the CTA's inversion: issue active 50% against 60%), and fewer entries per
// bucket make the window reduction cheaper: two rounds take the MSM from 5.13 to 4.90 ms, more
// rounds cost more than they save.  G2 pair rounds measured 0.95 of the mixed additions and
// slower MSMs (G2 MSM 2^18: 5.32 ms without, 5.44 / 5.69 ms with one / two rounds), and proofs
// over window tables (one bucket set, 3.9 M entries per SquareChain(2^18) G1 MSM, reductions
// hidden under later accumulations) measured slower with any rounds (10.45 -> 10.73 ms with
// one), so the model takes two rounds for large G1 MSMs only (SquareChain(2^20) proof, whose G1
// table MSMs have 14.7 M entries: 36.85 -> 36.19 ms).
inline int pair_rounds_model(size_t max_entries, size_t nkeys, bool g2) {
  if (g2 || max_entries < (size_t(1) << 23) || max_entries < 32 * nkeys) return 0;
  return 2;
}
