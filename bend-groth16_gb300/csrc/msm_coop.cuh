// Cooperative XYZZ additions and the window reduction built on them (included by msm.cu).
//
// A window reduction that ends a critical path (a small proof's MSMs, the last MSM of a large
// one) is a chain of dependent point additions per thread: a bucket's slice pieces, the
// running sums, the scan and the tree.  One add-2008-s addition is 14 field products, but its
// dependency depth is about 4.6: six independent products (u1, u2, s1, s2, zz1 zz2,
// zzz1 zzz2), two squares, three products (ppp, qq, zz3), and zzz3 beside
// y3 = r (qq - x3) - s1 ppp.  Here the 8 lanes of a group share one addition: each level's
// products run on different lanes at once, on the same code path (operands picked by selects,
// so the lanes do not diverge), and the group exchanges them through its shared-memory scratch
// with __syncwarp.  A chain of additions then runs about three times faster, at the price of
// idle lanes, which only pays where latency, not throughput, bounds the reduction.
//
// Points in shared memory are 4 consecutive field elements (x, y, zz, zzz); infinity is zz = 0.

constexpr int kCoopLanes = 8;
constexpr int kCoopTmp = 10;  // scratch field elements of one group's addition

template <class F>
BG_DEV F coop_ld(const uint32_t* p) {
  F x;
  load_elem(x, p);
  return x;
}

// point dst (shared) = point src (global or shared), element gl copied by lane gl < 4
template <class F>
BG_DEV void coop_copy(uint32_t* dst, const uint32_t* src, int gl, unsigned gmask) {
  constexpr int FW = FieldWords<F>::value;
  __syncwarp(gmask);
  if (gl < 4) store_elem(dst + gl * FW, coop_ld<F>(src + gl * FW));
  __syncwarp(gmask);
}
template <class F>
BG_DEV void coop_set_inf(uint32_t* dst, int gl, unsigned gmask) {
  constexpr int FW = FieldWords<F>::value;
  __syncwarp(gmask);
  if (gl < 4) store_elem(dst + gl * FW, gl < 2 ? field_one<F>() : field_zero<F>());
  __syncwarp(gmask);
}

// d += s for points in shared memory, by the 8 lanes of a group (gl: lane in the group, gmask:
// the group's lanes); tmp: kCoopTmp elements of the group's scratch.  Every lane of the group
// calls it with the same arguments, so every branch below is taken by the whole group.
template <class F>
BG_DEV void coop_add(uint32_t* d, const uint32_t* s, uint32_t* tmp, int gl, unsigned gmask) {
  constexpr int FW = FieldWords<F>::value;
  __syncwarp(gmask);
  if (is_zero(coop_ld<F>(s + 2 * FW))) return;  // s at infinity
  if (is_zero(coop_ld<F>(d + 2 * FW))) {         // d at infinity: d = s
    coop_copy<F>(d, s, gl, gmask);
    return;
  }
  // level 1 (lanes 0-5): u1 = x_d zz_s, u2 = x_s zz_d, s1 = y_d zzz_s, s2 = y_s zzz_d,
  // zz12 = zz_d zz_s, zzz12 = zzz_d zzz_s  ->  tmp[0..5]
  {
    const uint32_t* a = gl == 0 ? d : gl == 1 ? s : gl == 2 ? d + FW : gl == 3 ? s + FW : gl == 4 ? d + 2 * FW
                                                                                                   : d + 3 * FW;
    const uint32_t* b = gl == 0 ? s + 2 * FW : gl == 1 ? d + 2 * FW : gl == 2 ? s + 3 * FW : gl == 3 ? d + 3 * FW
                        : gl == 4 ? s + 2 * FW : s + 3 * FW;
    if (gl < 6) store_elem(tmp + gl * FW, fmul(coop_ld<F>(a), coop_ld<F>(b)));
  }
  __syncwarp(gmask);
  const F p_ = sub(coop_ld<F>(tmp + FW), coop_ld<F>(tmp));        // u2 - u1
  const F r_ = sub(coop_ld<F>(tmp + 3 * FW), coop_ld<F>(tmp + 2 * FW));  // s2 - s1
  if (is_zero(p_)) {  // equal x: d = s (double) or d = -s (infinity); rare, one lane
    __syncwarp(gmask);
    if (gl == 0) {
      XYZZ<F> r = xyzz_inf<F>();
      if (is_zero(r_)) {
        XYZZ<F> q;
        q.x = coop_ld<F>(tmp);
        q.y = coop_ld<F>(tmp + 2 * FW);
        q.zz = coop_ld<F>(tmp + 4 * FW);
        q.zzz = coop_ld<F>(tmp + 5 * FW);
        r = xyzz_dbl(q);
      }
      store_xyzz(d, r);
    }
    __syncwarp(gmask);
    return;
  }
  // level 2 (lanes 0-1): pp = p_^2, rr = r_^2  ->  tmp[6], tmp[7]
  if (gl < 2) store_elem(tmp + (6 + gl) * FW, fsqr(gl == 0 ? p_ : r_));
  __syncwarp(gmask);
  // level 3 (lanes 0-2): ppp = p_ pp -> tmp[8], qq = u1 pp -> tmp[9], zz3 = zz12 pp -> d.zz
  {
    const F pp = coop_ld<F>(tmp + 6 * FW);
    const F a = gl == 0 ? p_ : coop_ld<F>(tmp + (gl == 1 ? 0 : 4) * FW);
    if (gl < 3) store_elem(gl == 2 ? d + 2 * FW : tmp + (8 + gl) * FW, fmul(a, pp));
  }
  __syncwarp(gmask);
  // level 4: x3 = rr - ppp - 2 qq (every lane), y3 = r_ (qq - x3) - s1 ppp (lane 0),
  // zzz3 = zzz12 ppp - 0 (lane 1, the same multiply-subtract body), x3 stored by lane 2
  {
    const F ppp = coop_ld<F>(tmp + 8 * FW), qq = coop_ld<F>(tmp + 9 * FW);
    const F x3 = sub(sub(coop_ld<F>(tmp + 7 * FW), ppp), dbl(qq));
    const F a = gl == 0 ? r_ : coop_ld<F>(tmp + 5 * FW);
    const F b = gl == 0 ? sub(qq, x3) : ppp;
    const F c = gl == 0 ? coop_ld<F>(tmp + 2 * FW) : field_zero<F>();
    const F e = gl == 0 ? ppp : field_zero<F>();
    if (gl < 2) store_elem(gl == 0 ? d + FW : d + 3 * FW, fmul_sub(a, b, c, e));
    if (gl == 2) store_elem(d, x3);
  }
  __syncwarp(gmask);
}

// scratch words of one group: R, T, S (one point each) and the addition's scratch
template <class F>
constexpr size_t coop_group_words() {
  return (size_t)(12 + kCoopTmp) * FieldWords<F>::value;
}

// k_window_reduce with one group of 8 lanes in place of each thread (RT groups per CTA, M
// buckets per group, J parts per bucket set): the same running sums, suffix scan and tree, on
// cooperative additions; the part's two points out as k_window_reduce writes them.
template <class F>
__global__ void __launch_bounds__(256) k_window_reduce_coop(const uint32_t* __restrict__ offsets,
                                                            const uint32_t* __restrict__ buckets,
                                                            const uint32_t* __restrict__ pieces, uint32_t K,
                                                            uint32_t nb, uint32_t M, uint32_t J,
                                                            uint32_t* __restrict__ out) {
  constexpr int FW = FieldWords<F>::value;
  constexpr int PW = 4 * FW;
  extern __shared__ __align__(16) uint32_t sm[];
  const uint32_t RT = blockDim.x / kCoopLanes;
  const uint32_t g = threadIdx.x / kCoopLanes;
  const int gl = (int)(threadIdx.x % kCoopLanes);
  const unsigned gmask = 0xffu << (kCoopLanes * (g & 3u));
  uint32_t* const R = sm + (size_t)g * coop_group_words<F>();
  uint32_t* const T = R + PW;
  uint32_t* const S = R + 2 * PW;
  uint32_t* const tmp = R + 3 * PW;
  const uint32_t w = blockIdx.x / J, j = blockIdx.x % J;
  const size_t key0 = (size_t)w * nb + ((size_t)j * RT + g) * M;
  coop_set_inf<F>(R, gl, gmask);
  coop_set_inf<F>(T, gl, gmask);
  for (int k = (int)M - 1; k >= 0; k--) {
    const size_t key = key0 + k;
    const uint32_t o0 = offsets[key], o1 = offsets[key + 1];
    if (o1 != o0) {
      const uint32_t t0 = o0 / K, t1 = (o1 - 1) / K;
      if (t0 == t1 || t1 - t0 > kPieceLimit) {
        coop_copy<F>(S, buckets + key * PW, gl, gmask);
        coop_add<F>(R, S, tmp, gl, gmask);
      } else {
        coop_copy<F>(S, pieces + (2 * (size_t)t0 + 1) * PW, gl, gmask);
        coop_add<F>(R, S, tmp, gl, gmask);
        for (uint32_t u = t0 + 1; u <= t1; u++) {
          coop_copy<F>(S, pieces + 2 * (size_t)u * PW, gl, gmask);
          coop_add<F>(R, S, tmp, gl, gmask);
        }
      }
    }
    coop_add<F>(T, R, tmp, gl, gmask);
  }
  __syncthreads();
  // inclusive suffix scan of R over the groups (Hillis-Steele), through S
  for (uint32_t dd = 1; dd < RT; dd <<= 1) {
    if (g + dd < RT) coop_copy<F>(S, R + (size_t)dd * coop_group_words<F>(), gl, gmask);
    else coop_set_inf<F>(S, gl, gmask);
    __syncthreads();
    coop_add<F>(R, S, tmp, gl, gmask);
    __syncthreads();
  }
  // R_j = Suf_0
  if (g == 0 && gl < 4) store_elem(out + ((size_t)blockIdx.x * 2 + 1) * PW + gl * FW, coop_ld<F>(R + gl * FW));
  // Y_g = T_g + M Suf_g (g >= 1), Y_0 = T_0; the log2 M doublings on one lane
  if (g >= 1) {
    __syncwarp(gmask);
    if (gl == 0 && M > 1) {
      XYZZ<F> r = load_xyzz<F>(R);
      for (uint32_t m = M; m > 1; m >>= 1) r = xyzz_dbl(r);
      store_xyzz(R, r);
    }
    coop_add<F>(T, R, tmp, gl, gmask);
  }
  __syncthreads();
  for (uint32_t dd = RT >> 1; dd >= 1; dd >>= 1) {
    if (g < dd) coop_add<F>(T, T + (size_t)dd * coop_group_words<F>(), tmp, gl, gmask);
    __syncthreads();
  }
  if (g == 0 && gl < 4) store_elem(out + (size_t)blockIdx.x * 2 * PW + gl * FW, coop_ld<F>(T + gl * FW));
}
