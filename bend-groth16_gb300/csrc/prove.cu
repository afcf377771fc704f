// The Groth16 prove pipeline on one device.
//
// Mirrors Pr.run (bend2/prove.bend:129-162): load (bend2/src/groth16.bend:238-254), evals
// (Ev.matrix / matrix_a, groth16.bend:162-188, then Sc.canon, :214), qap (Pr.qap,
// prove.bend:52-56), the five MSMs (prove.bend:64-117) and Groth.combine (groth16.bend:298-308).
//
// Device schedule (one context, the main stream + seven side streams + a copy stream):
//   main:   witness H2D + repack -> z canonical -> evals (3 CSR SpMV) -> qap_h -> h canonical
//           -> msm_h's sort
//   side6:  the sorts of msm_a / msm_b1 / msm_b2 (shared) and msm_l, once z canonical exists
//   side0:  accumulations back to back (each fills the GPU): msm_a, msm_b1, msm_b2 (G2),
//           msm_l (scalars z[ni..]), then msm_h once h is sorted
//   side1..5: each MSM's heavy-bucket pass, window reduction and result copy, overlapping the
//           next accumulation (small proofs: each MSM's whole chain on its side stream)
//   copy:   one-shot keys only: query sets and R1CS matrices in the order they are needed
// The QAP runs concurrently with the first accumulations.  The host finishes every MSM as soon
// as its stream drains and assembles A, B and most of C (r delta, s delta, s A + r B1, ...)
// while msm_h is still running, so only msm_h's finish is left at the end.
#include <algorithm>
#include <chrono>
#include <cstring>
#include <memory>
#include <thread>

#include "common.cuh"
#include "ec.cuh"
#include "host_ff.hpp"
#include "host_pool.hpp"
#include "msm.h"
#include "ntt.h"
#include "prims.h"
#include "prove.h"

namespace bg {

using bgh::Aff;
using bgh::Fe;
using bgh::Fq2Ops;
using bgh::FqOps;
using bgh::Xyzz;

// ---------------------------------------------------------------- evaluation vectors
// Row i < N: sum_e coeff_e * z[col_e] over the CSR row (a coefficient equal to Montgomery one
// skips the product, as Ev.ent.s2 does, groth16.bend:108-113).  Rows N .. N+ni-1 of A carry the
// libsnark input-consistency entries a[N+i] = z[i] (groth16.bend:182-188); all other rows are 0.
__global__ void k_evals(const uint32_t* __restrict__ offs, const uint32_t* __restrict__ cols,
                        const uint32_t* __restrict__ coeffs, const uint32_t* __restrict__ z, uint32_t nz,
                        uint32_t nrows, uint32_t ni_rows, size_t d, uint32_t* __restrict__ out,
                        uint32_t* __restrict__ status) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= d) return;
  Fr acc = fp_zero<FrParams>();
  if (i < nrows) {
    const Fr one = fp_one<FrParams>();
    for (uint32_t e = offs[i]; e < offs[i + 1]; e++) {
      const uint32_t col = cols[e];
      if (col >= nz) {
        atomicOr(status, BG_DSTATUS_COLUMN);
        continue;
      }
      const Fr zv = load_fp<FrParams>(z + 8 * (size_t)col);
      const Fr cf = load_fp<FrParams>(coeffs + 8 * (size_t)e);
      acc = add(acc, eq(cf, one) ? zv : mul(cf, zv));
    }
  } else if (i - nrows < ni_rows) {
    acc = load_fp<FrParams>(z + 8 * (i - nrows));
  }
  store_fp(out + 8 * i, acc);
}

// split raw CSR entries (u32 col, 16 wire words) into cols[] and packed coefficients
__global__ void k_csr_split(const uint32_t* __restrict__ raw, size_t nnz, uint32_t* __restrict__ cols,
                            uint32_t* __restrict__ coeffs, uint32_t* __restrict__ status) {
  const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= nnz) return;
  const uint32_t* src = raw + 17 * e;
  cols[e] = src[0];
  uint32_t hi = 0;
  uint32_t w[8];
#pragma unroll
  for (int j = 0; j < 8; j++) {
    const uint32_t lo = src[1 + 2 * j], up = src[2 + 2 * j];
    hi |= (lo | up) >> 16;
    w[j] = (lo & 0xffffu) | (up << 16);
  }
  if (hi) atomicOr(status, BG_DSTATUS_FORMAT);
#pragma unroll
  for (int j = 0; j < 8; j++) coeffs[8 * e + j] = w[j];
}

// ---------------------------------------------------------------- input validation (host)
static const uint32_t* words(const void* p) { return static_cast<const uint32_t*>(p); }

Header parse_header(const bg_inputs& in) {
  if (!in.header || in.header_bytes != 32) throw Error(BG_E_FORMAT, "header.bin must hold 8 u32 words");
  const uint32_t* w = words(in.header);
  Header h{w[0], w[1], w[2], w[3], w[4], w[5], w[6], w[7]};
  const uint64_t d = 1ull << h.lg;
  if (h.lg > 27) throw Error(BG_E_FORMAT, "header: domain_log2 above the 2-adic limit");
  if ((uint64_t)h.nc + h.ni > d) throw Error(BG_E_FORMAT, "header: constraints + instance exceed the domain");
  if (h.na != h.ni + h.nw || h.nb != h.ni + h.nw) throw Error(BG_E_FORMAT, "header: n_a/n_b must equal num_instance + num_witness");
  if (h.nh > d) throw Error(BG_E_FORMAT, "header: n_h exceeds the domain");
  if (h.nl > h.nw) throw Error(BG_E_FORMAT, "header: n_l exceeds num_witness");
  if (h.ni < 1) throw Error(BG_E_FORMAT, "header: num_instance must be >= 1");
  return h;
}

static void need(size_t got, size_t want, const char* what) {
  if (got != want)
    throw Error(BG_E_FORMAT, std::string(what) + ": " + std::to_string(got) + " bytes, header implies " +
                                 std::to_string(want));
}

static void check_csr(const void* p, size_t bytes, uint32_t nc, const char* what, uint32_t& nnz) {
  if (!p || bytes < 4) throw Error(BG_E_FORMAT, std::string(what) + ": missing");
  const uint32_t* w = words(p);
  nnz = w[0];
  need(bytes, 4ull * (1 + (size_t)nc + 1 + 17ull * nnz), what);
  const uint32_t* offs = w + 1;
  if (offs[0] != 0 || offs[nc] != nnz) throw Error(BG_E_FORMAT, std::string(what) + ": offsets do not span nnz");
  for (uint32_t i = 0; i < nc; i++)
    if (offs[i + 1] < offs[i]) throw Error(BG_E_FORMAT, std::string(what) + ": offsets decrease");
}

void validate_inputs(const bg_inputs& in, const Header& h, bool need_witness) {
  need(in.pk_g1_bytes, 3 * 128, "pk_g1.bin");
  need(in.pk_g2_bytes, 2 * 256, "pk_g2.bin");
  need(in.pk_a_bytes, (size_t)h.na * 128, "pk_a.bin");
  need(in.pk_b1_bytes, (size_t)h.nb * 128, "pk_b1.bin");
  need(in.pk_b2_bytes, (size_t)h.nb * 256, "pk_b2.bin");
  need(in.pk_h_bytes, (size_t)h.nh * 128, "pk_h.bin");
  need(in.pk_l_bytes, (size_t)h.nl * 128, "pk_l.bin");
  if (need_witness) {
    need(in.witness_bytes, (size_t)(h.ni + h.nw) * 64, "witness.bin");
    need(in.rs_bytes, 2 * 64, "rs.bin");
  }
  uint32_t nnz;
  check_csr(in.r1cs_a, in.r1cs_a_bytes, h.nc, "r1cs_a.bin", nnz);
  check_csr(in.r1cs_b, in.r1cs_b_bytes, h.nc, "r1cs_b.bin", nnz);
  check_csr(in.r1cs_c, in.r1cs_c_bytes, h.nc, "r1cs_c.bin", nnz);
}

// ---------------------------------------------------------------- proving key upload
template <class H>
static Aff<H> host_affine_from_wire(const uint32_t* w16) {
  Aff<H> a;
  uint32_t packed[2 * H::WORDS];
  for (int i = 0; i < 2 * H::WORDS; i++) {
    packed[i] = (w16[2 * i] & 0xffffu) | (w16[2 * i + 1] << 16);
  }
  return bgh::aff_from_words32<H>(packed);
}

static void* dmalloc(size_t bytes) {
  void* p = nullptr;
  cudaError_t e = cudaMalloc(&p, bytes < 256 ? 256 : bytes);
  if (e != cudaSuccess) {
    cudaGetLastError();
    throw Error(BG_E_OOM, "device allocation of " + std::to_string(bytes) + " bytes failed");
  }
  return p;
}

// copy `bytes` of host memory to a device buffer through the context's pinned staging
static void h2d(Ctx& ctx, int slot, void* dst, const void* src, size_t bytes, cudaStream_t st) {
  if (bytes == 0) return;
  cudaPointerAttributes attr;
  if (cudaPointerGetAttributes(&attr, src) == cudaSuccess) {
    if (attr.type == cudaMemoryTypeHost) {
      BG_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, st));
      ctx.h2d_bytes += bytes;
      return;
    }
    if (attr.type == cudaMemoryTypeDevice || attr.type == cudaMemoryTypeManaged) {
      BG_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToDevice, st));
      return;
    }
  }
  cudaGetLastError();
  ctx.h2d_bytes += bytes;
  // pageable source: stage in chunks through pinned memory
  const size_t chunk = 64ull << 20;
  char* pin = static_cast<char*>(ctx.pinned[slot].get(std::min(bytes, chunk) * 2));
  const char* s = static_cast<const char*>(src);
  char* d = static_cast<char*>(dst);
  size_t off = 0;
  int half = 0;
  cudaEvent_t done[2];
  BG_CUDA(cudaEventCreateWithFlags(&done[0], cudaEventDisableTiming));
  BG_CUDA(cudaEventCreateWithFlags(&done[1], cudaEventDisableTiming));
  bool used[2] = {false, false};
  while (off < bytes) {
    const size_t len = std::min(chunk, bytes - off);
    char* buf = pin + (size_t)half * std::min(bytes, chunk);
    if (used[half]) BG_CUDA(cudaEventSynchronize(done[half]));
    memcpy(buf, s + off, len);
    BG_CUDA(cudaMemcpyAsync(d + off, buf, len, cudaMemcpyHostToDevice, st));
    BG_CUDA(cudaEventRecord(done[half], st));
    used[half] = true;
    off += len;
    half ^= 1;
  }
  BG_CUDA(cudaEventSynchronize(done[0]));
  BG_CUDA(cudaEventSynchronize(done[1]));
  cudaEventDestroy(done[0]);
  cudaEventDestroy(done[1]);
}

// device buffer: cudaMalloc'd (owned by the key) or, for pooled one-shot keys, the context's
// workspace slot `tag` (kept for the next proof)
static void* key_alloc(Ctx& ctx, bool pooled, const std::string& tag, size_t bytes) {
  if (pooled) return ctx.ws.get_t<uint32_t>("oneshot." + tag, (bytes + 3) / 4);
  return dmalloc(bytes);
}

static void upload_points(Ctx& ctx, const void* src, size_t n, int words_per_point, uint32_t*& d_out,
                          cudaStream_t st, bool pooled = false, const std::string& tag = "") {
  // wire words -> staging on device -> packed
  const size_t wire_words = n * words_per_point;
  d_out = static_cast<uint32_t*>(key_alloc(ctx, pooled, tag, wire_words / 2 * 4));
  uint32_t* stage = ctx.ws.get_t<uint32_t>(pooled ? "oneshot.stage." + tag : "upload.stage", wire_words);
  h2d(ctx, 0, stage, src, wire_words * 4, st);
  wire_to_packed(st, stage, d_out, wire_words / 16, ctx.d_status);
}

static void upload_csr(Ctx& ctx, const void* src, uint32_t nc, CsrDev& out, cudaStream_t st, bool pooled = false,
                       const std::string& tag = "") {
  const uint32_t* w = words(src);
  out.nnz = w[0];
  out.offs = static_cast<uint32_t*>(key_alloc(ctx, pooled, tag + ".offs", ((size_t)nc + 1) * 4));
  out.cols = static_cast<uint32_t*>(key_alloc(ctx, pooled, tag + ".cols", (size_t)out.nnz * 4));
  out.coeffs = static_cast<uint32_t*>(key_alloc(ctx, pooled, tag + ".coeffs", (size_t)out.nnz * 32));
  h2d(ctx, 0, out.offs, w + 1, ((size_t)nc + 1) * 4, st);
  if (out.nnz) {
    uint32_t* stage = ctx.ws.get_t<uint32_t>("upload.csr", 17ull * out.nnz);
    h2d(ctx, 0, stage, w + 2 + nc, 17ull * out.nnz * 4, st);
    k_csr_split<<<ceil_div(out.nnz, 256), 256, 0, st>>>(stage, out.nnz, out.cols, out.coeffs, ctx.d_status);
    BG_CHECK_LAUNCH();
  }
}

void check_status(Ctx& ctx, cudaStream_t st) {
  uint32_t s = 0;
  BG_CUDA(cudaMemcpyAsync(&s, ctx.d_status, 4, cudaMemcpyDeviceToHost, st));
  ctx.d2h_bytes += 4;
  BG_CUDA(cudaStreamSynchronize(st));
  if (s) {
    BG_CUDA(cudaMemsetAsync(ctx.d_status, 0, 4, st));
    BG_CUDA(cudaStreamSynchronize(st));
    if (s & BG_DSTATUS_SCALAR_RANGE) throw Error(BG_E_ARG, "an MSM scalar is not below 2^254 (not a canonical Fr)");
    if (s & BG_DSTATUS_FORMAT) throw Error(BG_E_FORMAT, "a wire word has bits above its 16-bit limb");
    if (s & BG_DSTATUS_COLUMN) throw Error(BG_E_FORMAT, "an R1CS column index is outside the assignment");
    throw Error(BG_E_DEVICE, "device status flag " + std::to_string(s));
  }
}

PkDev* pk_upload(Ctx& ctx, const bg_inputs& in, bool build_tables) {
  const Header h = parse_header(in);
  validate_inputs(in, h, false);
  PkDev* pk = new PkDev();
  pk->h = h;
  try {
    cudaStream_t st = ctx.stream;
    upload_points(ctx, in.pk_a, h.na, 32, pk->pa, st);
    upload_points(ctx, in.pk_b1, h.nb, 32, pk->pb1, st);
    upload_points(ctx, in.pk_b2, h.nb, 64, pk->pb2, st);
    upload_points(ctx, in.pk_h, h.nh, 32, pk->ph, st);
    upload_points(ctx, in.pk_l, h.nl, 32, pk->pl, st);
    upload_csr(ctx, in.r1cs_a, h.nc, pk->ca, st);
    upload_csr(ctx, in.r1cs_b, h.nc, pk->cb, st);
    upload_csr(ctx, in.r1cs_c, h.nc, pk->cc, st);
    const uint32_t* g1 = words(in.pk_g1);
    const uint32_t* g2 = words(in.pk_g2);
    pk->alpha = host_affine_from_wire<FqOps>(g1);
    pk->beta = host_affine_from_wire<FqOps>(g1 + 32);
    pk->delta = host_affine_from_wire<FqOps>(g1 + 64);
    pk->beta2 = host_affine_from_wire<Fq2Ops>(g2);
    pk->delta2 = host_affine_from_wire<Fq2Ops>(g2 + 64);
    HostPool::get().parallel_for(2, [&](int i) {
      if (i == 0) {
        pk->delta_pow[0] = bgh::xyzz_from(pk->delta);
        for (int j = 1; j < 4; j++) {
          pk->delta_pow[j] = pk->delta_pow[j - 1];
          for (int b = 0; b < 64; b++) pk->delta_pow[j] = bgh::xyzz_dbl(pk->delta_pow[j]);
        }
      } else {
        pk->delta2_pow[0] = bgh::xyzz_from(pk->delta2);
        for (int j = 1; j < 4; j++) {
          pk->delta2_pow[j] = pk->delta2_pow[j - 1];
          for (int b = 0; b < 64; b++) pk->delta2_pow[j] = bgh::xyzz_dbl(pk->delta2_pow[j]);
        }
      }
    });
    pk->delta_pow_ready = true;
    if (build_tables) {
      msm_build_table<Fq>(st, pk->pa, h.na, pk->tab[0], ctx.c_override[1][0]);
      msm_build_table<Fq>(st, pk->pb1, h.nb, pk->tab[1], ctx.c_override[1][0]);
      msm_build_table<Fq2>(st, pk->pb2, h.nb, pk->tab[2], ctx.c_override[1][1]);
      msm_build_table<Fq>(st, pk->ph, h.nh, pk->tab[3], ctx.c_override[1][0]);
      msm_build_table<Fq>(st, pk->pl, h.nl, pk->tab[4], ctx.c_override[1][0]);
      pk->tables = true;
    }
    check_status(ctx, st);
  } catch (...) {
    pk_free(pk);
    throw;
  }
  return pk;
}

PkDev* pk_stage_oneshot(Ctx& ctx, const bg_inputs& in) {
  const Header h = parse_header(in);
  validate_inputs(in, h, false);
  PkDev* pk = new PkDev();
  pk->h = h;
  pk->pooled = true;
  try {
    const uint32_t* g1 = words(in.pk_g1);
    const uint32_t* g2 = words(in.pk_g2);
    pk->alpha = host_affine_from_wire<FqOps>(g1);
    pk->beta = host_affine_from_wire<FqOps>(g1 + 32);
    pk->delta = host_affine_from_wire<FqOps>(g1 + 64);
    pk->beta2 = host_affine_from_wire<Fq2Ops>(g2);
    pk->delta2 = host_affine_from_wire<Fq2Ops>(g2 + 64);
    // Everything goes up on the copy stream, in the order the proof needs it: the query sets
    // of the first two accumulations (a, b1), then the R1CS matrices (the evaluations and the
    // QAP, which feed only msm_h, the last accumulation), then b2, l and h.  The witness
    // travels on the main stream meanwhile, so the shared sort of a, b1 and b2 starts as
    // soon as the canonical scalars exist.  Each set has its own staging buffer, so no
    // transfer waits for an earlier repack.
    cudaStream_t cs = ctx.copy;
    struct Set {
      int idx;
      const void* src;
      size_t n;
      int words;
      uint32_t** dst;
      const char* tag;
    };
    const Set sets[5] = {{0, in.pk_a, h.na, 32, &pk->pa, "pa"}, {1, in.pk_b1, h.nb, 32, &pk->pb1, "pb1"},
                         {2, in.pk_b2, h.nb, 64, &pk->pb2, "pb2"}, {4, in.pk_l, h.nl, 32, &pk->pl, "pl"},
                         {3, in.pk_h, h.nh, 32, &pk->ph, "ph"}};
    for (const Set& q : sets) {
      upload_points(ctx, q.src, q.n, q.words, *q.dst, cs, true, q.tag);
      pk->ready[q.idx] = ctx.event(std::string("oneshot.ready.") + q.tag);
      BG_CUDA(cudaEventRecord(pk->ready[q.idx], cs));
      if (q.idx == 1) {
        upload_csr(ctx, in.r1cs_a, h.nc, pk->ca, cs, true, "ca");
        upload_csr(ctx, in.r1cs_b, h.nc, pk->cb, cs, true, "cb");
        upload_csr(ctx, in.r1cs_c, h.nc, pk->cc, cs, true, "cc");
        pk->csr_ready = ctx.event("oneshot.csr");
        BG_CUDA(cudaEventRecord(pk->csr_ready, cs));
      }
    }
  } catch (...) {
    pk_free(pk);
    throw;
  }
  return pk;
}

void pk_free(PkDev* pk) {
  if (!pk) return;
  if (pk->pooled) {  // workspace buffers and context events stay with the context
    delete pk;
    return;
  }
  for (uint32_t* p : {pk->pa, pk->pb1, pk->pb2, pk->ph, pk->pl, pk->ca.offs, pk->ca.cols, pk->ca.coeffs,
                      pk->cb.offs, pk->cb.cols, pk->cb.coeffs, pk->cc.offs, pk->cc.cols, pk->cc.coeffs})
    if (p) cudaFree(p);
  for (MsmTable& t : pk->tab)
    if (t.d) cudaFree(t.d);
  delete pk;
}

// ---------------------------------------------------------------- combine (host)
static void scalar_from_mont_wire(const uint32_t* w16, uint64_t out[4]) {
  const Fe m = bgh::fe_from_words16(w16);
  const Fe c = bgh::fe_from_mont(bgh::FR, m);
  for (int i = 0; i < 4; i++) out[i] = c.v[i];
}

template <class H>
static void wire_from_affine(uint32_t* w16, const Aff<H>& a) {
  uint32_t packed[2 * H::WORDS];
  bgh::aff_to_words32<H>(packed, a);
  for (int i = 0; i < 2 * H::WORDS; i++) {
    w16[2 * i] = packed[i] & 0xffffu;
    w16[2 * i + 1] = packed[i] >> 16;
  }
}

struct Timer {
  cudaEvent_t a = nullptr, b = nullptr;
  void start(cudaStream_t st) {
    BG_CUDA(cudaEventCreate(&a));
    BG_CUDA(cudaEventCreate(&b));
    BG_CUDA(cudaEventRecord(a, st));
  }
  void stop(cudaStream_t st) { BG_CUDA(cudaEventRecord(b, st)); }
  double ms() {
    float t = 0;
    if (a && b) cudaEventElapsedTime(&t, a, b);
    return t;
  }
  ~Timer() {
    if (a) cudaEventDestroy(a);
    if (b) cudaEventDestroy(b);
  }
};

void prove_resident(Ctx& ctx, PkDev& pk, const uint32_t* witness16, const uint32_t* rs16, bg_proof* out,
                    bg_phase_ms* times, double load_ms_before) {
  const auto t_wall0 = std::chrono::steady_clock::now();
  const Header& h = pk.h;
  const size_t d = size_t(1) << h.lg;
  const size_t nz = (size_t)h.ni + h.nw;
  cudaStream_t st = ctx.stream;
  Workspace& ws = ctx.ws;

  // ---- load: witness to the device
  Timer t_load, t_evals, t_qap, t_msm[5];
  t_load.start(st);
  uint32_t* z_wire = ws.get_t<uint32_t>("prove.z_wire", nz * 16);
  uint32_t* z = ws.get_t<uint32_t>("prove.z", nz * 8);
  uint32_t* zc = ws.get_t<uint32_t>("prove.zc", nz * 8);
  h2d(ctx, 1, z_wire, witness16, nz * 64, st);
  wire_to_packed(st, z_wire, z, nz, ctx.d_status);
  t_load.stop(st);
  // the MSM scalars (canonical z) first: the sorts need nothing else
  fr_from_mont(st, z, zc, nz);
  cudaEvent_t ev_scalars = ctx.event("prove.scalars");
  BG_CUDA(cudaEventRecord(ev_scalars, st));

  // ---- the MSMs whose scalars are the assignment go first (host launch order matters for
  // small proofs, whose kernels are shorter than the host's launches): msm_a, msm_b1, msm_b2,
  // msm_l; msm_h follows the QAP
  uint32_t* hh = ws.get_t<uint32_t>("prove.h", d * 8);
  uint32_t* hc = ws.get_t<uint32_t>("prove.hc", d * 8);
  MsmPlan plan[5];  // a, b1, b2, h, l
  struct Job {
    int idx;
    const char* tag;
    bool g2;
    const uint32_t* pts;
    const uint32_t* sc;
    size_t n;
    const MsmTable* tab;  // the query set's window table (resident keys), else null
  };
  auto tab = [&](int k) -> const MsmTable* { return pk.tables && pk.tab[k].d ? &pk.tab[k] : nullptr; };
  const Job jobs[5] = {{0, "msm_a", false, pk.pa, zc, h.na, tab(0)},
                       {1, "msm_b1", false, pk.pb1, zc, h.nb, tab(1)},
                       {2, "msm_b2", true, pk.pb2, zc, h.nb, tab(2)},
                       {4, "msm_l", false, pk.pl, zc + 8 * (size_t)h.ni, h.nl, tab(4)},
                       {3, "msm_h", false, pk.ph, hc, h.nh, tab(3)}};
  auto width = [&](const Job& jb) {
    if (jb.tab) return jb.tab->c;
    const int forced = ctx.c_override[0][jb.g2 ? 1 : 0];
    return forced ? forced : msm_pick_c_proof(jb.n, jb.g2);
  };
  // Bucket orders on their own stream: a, b1 and b2 take the same scalars (the whole
  // assignment) and, with equal lengths, the same window layout, so they share one sort; l's
  // follows; h's is made on the main stream once the QAP is done.  The accumulation stream then
  // runs the five accumulations back to back, each waiting only for its own sort.
  cudaStream_t acc_st = ctx.side[0];
  cudaStream_t sort_st = ctx.side[kSortStream];
  BG_CUDA(cudaStreamWaitEvent(sort_st, ev_scalars, 0));
  struct SortKey {
    const uint32_t* sc;
    size_t n;
    int c;
    bool shared;
  };
  std::vector<std::pair<SortKey, MsmSort>> sorts;
  sorts.reserve(5);
  auto sort_for = [&](const Job& jb, cudaStream_t s) -> const MsmSort& {
    const SortKey k{jb.sc, jb.n, width(jb), jb.tab != nullptr};
    for (auto& e : sorts)
      if (e.first.sc == k.sc && e.first.n == k.n && e.first.c == k.c && e.first.shared == k.shared) return e.second;
    sorts.emplace_back(k, MsmSort());
    msm_sort(ctx, s, std::string(jb.tag) + ".sort", jb.sc, jb.n, k.c, k.shared, sorts.back().second);
    return sorts.back().second;
  };
  BG_CUDA(cudaStreamWaitEvent(acc_st, ev_scalars, 0));
  // A small proof's accumulations together fill less than one wave of the GPU (short slices:
  // about entries / 8 threads each), so queueing them on one stream would leave it mostly
  // idle: each MSM then runs its whole chain -- accumulation, heavy pass, reduction -- on its
  // own stream, and the five overlap.  Not in a batch or server lane, where other proofs
  // fill the GPU and the one-stream schedule's lighter reductions give more proofs per second.
  size_t acc_threads = 0;
  for (const Job& jb : jobs) acc_threads += jb.n * (size_t)(254 / width(jb) + 1) / 8 + 1;
  const bool overlap = !ctx.shared_gpu && acc_threads <= (size_t)ctx.sm_count * 4 * 128;
  auto launch = [&](int j, const MsmSort& so) {
    const Job& jb = jobs[j];
    cudaStream_t red = ctx.side[1 + j];
    cudaStream_t ast = overlap ? red : acc_st;
    MsmPlan& p = plan[jb.idx];
    // only msm_h's reduction is not hidden under a later accumulation; overlapped, none is.  The
    // others get the accumulation time queued after them (entries x about 0.3 ns for G1 and
    // 0.9 ns for G2 inside a proof), which the reduction should not outlast.
    p.latency_critical = overlap || j == 4;
    p.host_pool_free = !overlap && !ctx.shared_gpu;
    // (Batch and server lanes keep the fixed rule: other proofs fill the GPU there.)
    p.hidden_us = 0;
    if (!ctx.shared_gpu)
      for (int k = j + 1; k < 5; k++)
        p.hidden_us += (double)jobs[k].n * (254 / width(jobs[k]) + 1) * (jobs[k].g2 ? 0.9e-3 : 0.3e-3);
    if (overlap) BG_CUDA(cudaStreamWaitEvent(ast, ev_scalars, 0));
    if (pk.ready[jb.idx]) BG_CUDA(cudaStreamWaitEvent(ast, pk.ready[jb.idx], 0));
    t_msm[jb.idx].start(ast);
    if (jb.g2) {
      msm_accumulate<Fq2>(ctx, ast, jb.tag, jb.pts, so, p, red, jb.tab);
      msm_fetch<Fq2>(ctx, ast, p);
    } else {
      msm_accumulate<Fq>(ctx, ast, jb.tag, jb.pts, so, p, red, jb.tab);
      msm_fetch<Fq>(ctx, ast, p);
    }
    t_msm[jb.idx].stop(red);
  };
  const MsmSort* so[4];
  for (int j = 0; j < 4; j++) so[j] = &sort_for(jobs[j], sort_st);
  for (int j = 0; j < 4; j++) launch(j, *so[j]);

  // ---- evals
  t_evals.start(st);
  uint32_t* ea = ws.get_t<uint32_t>("prove.ea", d * 8);
  uint32_t* eb = ws.get_t<uint32_t>("prove.eb", d * 8);
  uint32_t* ec = ws.get_t<uint32_t>("prove.ec", d * 8);
  const CsrDev* m[3] = {&pk.ca, &pk.cb, &pk.cc};
  uint32_t* ev[3] = {ea, eb, ec};
  if (pk.csr_ready) BG_CUDA(cudaStreamWaitEvent(st, pk.csr_ready, 0));
  std::unique_ptr<KernelTimer> kt_evals(new KernelTimer(ctx, "evals", st));
  for (int k = 0; k < 3; k++) {
    k_evals<<<ceil_div(d, 128), 128, 0, st>>>(m[k]->offs, m[k]->cols, m[k]->coeffs, z, (uint32_t)nz, h.nc,
                                              k == 0 ? h.ni : 0, d, ev[k], ctx.d_status);
    BG_CHECK_LAUNCH();
  }
  kt_evals.reset();
  t_evals.stop(st);

  // ---- QAP on the main stream; it needs only the evaluation vectors
  t_qap.start(st);
  {
    KernelTimer kt(ctx, "qap", st);
    qap_h_run(ctx, st, ea, eb, ec, hh, h.lg);
    fr_from_mont(st, hh, hc, h.nh);
  }
  t_qap.stop(st);

  // ---- msm_h: its sort on the main stream after the QAP, then its accumulation last
  launch(4, sort_for(jobs[4], st));

  // ---- host work that needs no MSM result, overlapped with the device
  uint64_t r[4], s[4], rs[4];
  scalar_from_mont_wire(rs16, r);
  scalar_from_mont_wire(rs16 + 16, s);
  {
    const Fe rm = bgh::fe_from_words16(rs16), sm = bgh::fe_from_words16(rs16 + 16);
    const Fe prod = bgh::fe_from_mont(bgh::FR, bgh::fe_mul(bgh::FR, rm, sm));
    for (int i = 0; i < 4; i++) rs[i] = prod.v[i];
  }
  // The four products of the key's delta points by r, s and r s are independent chains of
  // about 320 host point operations (146 us in G1, 404 us in G2 on one core): they run at once
  // on the host pool, and with a resident key each splits into four 64-bit pieces over
  // precomputed 2^(64 j) delta.  A small proof's device work is shorter than them one after
  // another (SquareChain(2^10): kernels end about 0.63 ms into the proof).
  const Xyzz<FqOps> dj = bgh::xyzz_from(pk.delta);
  const Xyzz<Fq2Ops> dj2 = bgh::xyzz_from(pk.delta2);
  Xyzz<FqOps> r_delta, s_delta, rs_delta;
  Xyzz<Fq2Ops> s_delta2;
  if (pk.delta_pow_ready) {
    // resident key: each product is four 64-bit pieces k_j (2^(64 j) delta), 16 tasks
    Xyzz<FqOps> piece[3][4];
    Xyzz<Fq2Ops> piece2[4];
    const uint64_t* ks[3] = {r, s, rs};
    HostPool::get().parallel_for(16, [&](int t) {
      const int j = t & 3, m = t >> 2;  // the four G2 pieces first: they are the longest
      if (m == 0) piece2[j] = bgh::xyzz_mul64(pk.delta2_pow[j], s[j]);
      else piece[m - 1][j] = bgh::xyzz_mul64(pk.delta_pow[j], ks[m - 1][j]);
    });
    Xyzz<FqOps>* out[3] = {&r_delta, &s_delta, &rs_delta};
    for (int m = 0; m < 3; m++)
      *out[m] = bgh::xyzz_add(bgh::xyzz_add(piece[m][0], piece[m][1]), bgh::xyzz_add(piece[m][2], piece[m][3]));
    s_delta2 = bgh::xyzz_add(bgh::xyzz_add(piece2[0], piece2[1]), bgh::xyzz_add(piece2[2], piece2[3]));
  } else {
    HostPool::get().parallel_for(4, [&](int i) {
      if (i == 0) s_delta2 = bgh::xyzz_mul(dj2, s);
      else if (i == 1) r_delta = bgh::xyzz_mul(dj, r);
      else if (i == 2) s_delta = bgh::xyzz_mul(dj, s);
      else rs_delta = bgh::xyzz_mul(dj, rs);
    });
  }

  // ---- finish each MSM on the host as soon as its reduction stream drains (accumulation order
  // a, b1, b2, l, h); everything that does not need msm_h -- A, B1, B2 and s A + r B1 - r s delta
  // + mL -- is computed while msm_h is still on the device.  Combine (groth16.bend:298-308):
  // A = alpha + mA + r delta; B1 = beta + mB1 + s delta; B2 = beta2 + mB2 + s delta2;
  // C = s A + r B1 - r s delta + (mL + mH)
  auto g1 = [](const uint32_t* w) { return bgh::xyzz_from(bgh::aff_from_words32<FqOps>(w)); };
  uint32_t res[5][32];
  // an MSM's window parts are on the host once its reduction stream drains (an empty MSM has
  // no stream: nothing to wait for)
  auto drain = [](const MsmPlan& p) {
    if (p.fetch_stream) BG_CUDA(cudaStreamSynchronize(p.fetch_stream));
  };
  drain(plan[0]);
  msm_finish<Fq>(plan[0], res[0]);
  const Xyzz<FqOps> A = bgh::xyzz_add(bgh::xyzz_add(g1(res[0]), r_delta), bgh::xyzz_from(pk.alpha));
  drain(plan[1]);
  msm_finish<Fq>(plan[1], res[1]);
  const Xyzz<FqOps> B1 = bgh::xyzz_add(bgh::xyzz_add(g1(res[1]), s_delta), bgh::xyzz_from(pk.beta));
  Xyzz<FqOps> sA, rB1;
  HostPool::get().parallel_for(2, [&](int i) {
    if (i == 0) sA = bgh::xyzz_mul(A, s);
    else rB1 = bgh::xyzz_mul(B1, r);
  });
  Xyzz<FqOps> c_part = bgh::xyzz_add(bgh::xyzz_add(sA, rB1), bgh::xyzz_neg(rs_delta));
  drain(plan[2]);
  msm_finish<Fq2>(plan[2], res[2]);
  const Xyzz<Fq2Ops> B2 = bgh::xyzz_add(
      bgh::xyzz_add(bgh::xyzz_from(bgh::aff_from_words32<Fq2Ops>(res[2])), s_delta2), bgh::xyzz_from(pk.beta2));
  // A and B are final here: their inversions to affine run while msm_h is still on the device
  const auto a_aff = bgh::xyzz_to_affine(A);
  const auto b_aff = bgh::xyzz_to_affine(B2);
  drain(plan[4]);
  msm_finish<Fq>(plan[4], res[4]);
  c_part = bgh::xyzz_add(c_part, g1(res[4]));
  for (int j = 0; j < kStreams; j++) BG_CUDA(cudaStreamSynchronize(ctx.side[j]));
  BG_CUDA(cudaStreamSynchronize(st));
  check_status(ctx, st);
  msm_finish<Fq>(plan[3], res[3]);
  const Xyzz<FqOps> C = bgh::xyzz_add(c_part, g1(res[3]));
  wire_from_affine<FqOps>(out->a, a_aff);
  wire_from_affine<Fq2Ops>(out->b, b_aff);
  wire_from_affine<FqOps>(out->c, bgh::xyzz_to_affine(C));

  if (times) {
    times->load = load_ms_before + t_load.ms();
    times->evals = t_evals.ms();
    times->qap = t_qap.ms();
    times->msm_a = t_msm[0].ms();
    times->msm_b1 = t_msm[1].ms();
    times->msm_b2 = t_msm[2].ms();
    times->msm_h = t_msm[3].ms();
    times->msm_l = t_msm[4].ms();
    times->total =
        load_ms_before +
        std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t_wall0).count();
  }
}

// ---------------------------------------------------------------- scratch footprint
// Device bytes one proof's workspace needs (the buffers msm_launch, qap_h_run and
// prove_resident request), used for admission control; a 10% margin covers rounding.
static size_t msm_footprint_c(size_t n, bool g2, int c) {
  const size_t W = 254 / c + 1, nb = size_t(1) << (c - 1), nkeys = W * nb;
  const size_t PW = g2 ? 64 : 32;
  const size_t entries = n * W;
  // shortest slices: 3/4 of 32 after whole-wave rounding, 4 in the latency regime
  const size_t K = entries >= (size_t(1) << 21) ? 24 : 4;
  const size_t threads = (entries + K - 1) / K;
  const size_t J = nb < 32 ? 1 : nb / 32;  // most parts a reduction shape can have (RT >= 32)
  // counters, offsets, cursors, entry list, buckets, slice pieces + heavy list, window parts,
  // scan sums
  // batch-affine pair rounds where the model takes them: levels 1 and 2 (affine points, half
  // an XYZZ point each) and their offsets
  const size_t pairs = msm_pair_rounds_entries(entries, nkeys, g2) == 0
                           ? 0
                           : (entries / 2 + nkeys) * PW / 2 + (entries / 4 + 2 * nkeys) * PW / 2 + nkeys + 1;
  const size_t words = 3 * (nkeys + 1) + entries + nkeys * PW + 2 * threads * PW + threads / 8 + 2 +
                       W * J * 2 * PW + 2 * ((nkeys + 1) / 2048 + 1) + pairs;
  return words * 4;
}
static size_t msm_footprint(size_t n, bool g2) {
  if (n == 0) return 0;
  return std::max(msm_footprint_c(n, g2, msm_pick_c(n, g2)), msm_footprint_c(n, g2, msm_pick_c_proof(n, g2)));
}

size_t prove_footprint(const Header& h) {
  const size_t d = size_t(1) << h.lg, nz = (size_t)h.ni + h.nw;
  size_t b = nz * (64 + 32 + 32)          // witness wire, packed, canonical
             + 5 * d * 32                 // ea, eb, ec, h, h canonical
             + d * 32 + 4096 * 32;        // twiddle tables (w^i and w^-i, n/2 each) + coset tables
  b += msm_footprint(h.na, false) + msm_footprint(h.nb, false) + msm_footprint(h.nb, true) +
       msm_footprint(h.nh, false) + msm_footprint(h.nl, false);
  return b + b / 10 + (4u << 20);
}

// ---------------------------------------------------------------- proof text
int format_proof(const bg_proof* p, char* buf, size_t cap) {
  auto hex = [](const uint32_t* w16, bool mont_fq, char* o) {
    Fe v = bgh::fe_from_words16(w16);
    if (mont_fq) v = bgh::fe_from_mont(bgh::FQ, v);
    o += sprintf(o, "0x");
    for (int i = 3; i >= 0; i--) o += sprintf(o, "%016llx", (unsigned long long)v.v[i]);
    return o;
  };
  if (cap < 600) return BG_E_ARG;
  char* o = buf;
  o += sprintf(o, "A ");
  o = hex(p->a, true, o);
  *o++ = ' ';
  o = hex(p->a + 16, true, o);
  o += sprintf(o, "\nB ");
  for (int i = 0; i < 4; i++) {
    o = hex(p->b + 16 * i, true, o);
    *o++ = i < 3 ? ' ' : '\n';
  }
  o += sprintf(o, "C ");
  o = hex(p->c, true, o);
  *o++ = ' ';
  o = hex(p->c + 16, true, o);
  *o++ = '\n';
  *o = 0;
  return BG_OK;
}

}  // namespace bg
