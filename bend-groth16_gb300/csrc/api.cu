// extern "C" entry points of include/bg.h: argument checks, host <-> device staging in the
// wire layout of bend2/FORMAT.md, and the mapping of exceptions to BG_E_* statuses.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cstdio>
#include <cstring>
#include <memory>
#include <string>
#include <thread>
#include <vector>

#include <fcntl.h>
#include <sys/stat.h>
#include <unistd.h>

#include "common.cuh"
#include "host_pool.hpp"
#include "pairing.hpp"
#include "ec.cuh"
#include "host_ff.hpp"
#include "msm.h"
#include "ntt.h"
#include "prims.h"
#include "prove.h"

namespace bg {
std::atomic<uint64_t> g_launches{0};
void synth_square_chain(Ctx& c, uint32_t log2n, uint64_t seed, const std::string& dir);
}

struct bg_ctx {
  bg::Ctx c;
  // lanes of bg_prove_batch: each a context of its own (streams, workspace), created on demand
  std::vector<std::unique_ptr<bg::Ctx>> lanes;
};
struct bg_pk {
  bg::PkDev* pk;
  bg_ctx* owner;
};
struct bg_server {
  bg::Server* s;
  bg_ctx* owner;
};

using namespace bg;

namespace {

thread_local std::string g_err_noctx;

template <class Fn>
int guard(bg_ctx* ctx, Fn&& fn) {
  try {
    fn();
    if (ctx) ctx->c.last_error.clear();
    return BG_OK;
  } catch (const Error& e) {
    if (ctx) ctx->c.last_error = e.what();
    else g_err_noctx = e.what();
    if (ctx && e.status == BG_E_DEVICE) cudaGetLastError();
    return e.status;
  } catch (const std::bad_alloc&) {
    if (ctx) ctx->c.last_error = "host allocation failed";
    else g_err_noctx = "host allocation failed";
    return BG_E_OOM;
  } catch (const std::exception& e) {
    if (ctx) ctx->c.last_error = e.what();
    else g_err_noctx = e.what();
    return BG_E_DEVICE;
  }
}

// a failed argument check of an entry point: BG_E_ARG, with the failed condition in the message
int arg_error(bg_ctx* ctx, const char* fn, const char* condition) {
  const std::string m = std::string(fn) + ": invalid argument (" + condition + ")";
  if (ctx) ctx->c.last_error = m;
  else g_err_noctx = m;
  return BG_E_ARG;
}

#define BG_ARG_CHECK(ctx, bad)                              \
  do {                                                      \
    if (bad) return arg_error((ctx), __func__, #bad);       \
  } while (0)

// Device buffers handed to the _dev entry points are read and written in 16-byte vectors (and
// gathered by 16-byte asynchronous copies): a pointer off that boundary is refused here rather
// than left to fault on the device.  cudaMalloc returns 256-byte aligned memory.
inline bool misaligned16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15u) != 0; }

void require(bool ok, const char* msg) {
  if (!ok) throw Error(BG_E_ARG, msg);
}

// copy n wire elements (16 words each) from the host and repack them on the device
uint32_t* stage_in(Ctx& c, const std::string& name, const uint32_t* host16, size_t n_elems) {
  uint32_t* wire = c.ws.get_t<uint32_t>(name + ".wire", n_elems * 16);
  uint32_t* packed = c.ws.get_t<uint32_t>(name, n_elems * 8);
  BG_CUDA(cudaMemcpyAsync(wire, host16, n_elems * 64, cudaMemcpyHostToDevice, c.stream));
  c.h2d_bytes += n_elems * 64;
  wire_to_packed(c.stream, wire, packed, n_elems, c.d_status);
  return packed;
}

void stage_out(Ctx& c, const std::string& name, const uint32_t* d_packed, uint32_t* host16, size_t n_elems) {
  uint32_t* wire = c.ws.get_t<uint32_t>(name + ".wire_out", n_elems * 16);
  packed_to_wire(c.stream, d_packed, wire, n_elems);
  BG_CUDA(cudaMemcpyAsync(host16, wire, n_elems * 64, cudaMemcpyDeviceToHost, c.stream));
  c.d2h_bytes += n_elems * 64;
}

// affine packed result -> Jacobian wire words (x, y, z) with z = 1, infinity = (0, 1, 0)
template <class H>
void affine_to_jacobian_wire(const uint32_t* aff32, uint32_t* jac16) {
  constexpr int W = H::WORDS;  // packed words per field element
  bool inf = true;
  for (int i = 0; i < 2 * W; i++) inf &= aff32[i] == 0;
  uint32_t packed[3 * W];
  memset(packed, 0, sizeof(packed));
  const bgh::Fe one = bgh::fe_one(bgh::FQ);
  if (inf) {
    bgh::fe_to_words32(packed + W, one);  // y = 1 (c0 of Fq2), x = z = 0
  } else {
    memcpy(packed, aff32, sizeof(uint32_t) * 2 * W);
    bgh::fe_to_words32(packed + 2 * W, one);
  }
  for (int i = 0; i < 3 * W; i++) {
    jac16[2 * i] = packed[i] & 0xffffu;
    jac16[2 * i + 1] = packed[i] >> 16;
  }
}

template <class F, class H>
void msm_host(Ctx& c, const uint32_t* points16, const uint32_t* scalars16, size_t n, uint32_t* out_jac16) {
  constexpr int PW = 2 * H::WORDS;  // packed words per affine point
  uint32_t aff[2 * 16];
  if (n == 0) {
    memset(aff, 0, sizeof(aff));
  } else {
    const uint32_t* pts = stage_in(c, "api.msm_pts", points16, n * (PW / 8));
    // scalars are canonical: repack without a Montgomery conversion
    const uint32_t* sc = stage_in(c, "api.msm_sc", scalars16, n);
    MsmPlan plan;
    plan.c = c.c_override[0][FieldWords<F>::value == 16 ? 1 : 0];
    msm_launch<F>(c, c.stream, "api.msm", pts, sc, n, plan);
    msm_fetch<F>(c, c.stream, plan);
    BG_CUDA(cudaStreamSynchronize(c.stream));
    check_status(c, c.stream);
    msm_finish<F>(plan, aff);
  }
  affine_to_jacobian_wire<H>(aff, out_jac16);
}

template <class F>
void msm_dev(Ctx& c, const uint32_t* d_points, const uint32_t* d_scalars, size_t n, uint32_t* out_aff32) {
  constexpr int PW = 2 * FieldWords<F>::value;
  if (n == 0) {
    memset(out_aff32, 0, PW * 4);
    return;
  }
  MsmPlan plan;
  plan.c = c.c_override[0][FieldWords<F>::value == 16 ? 1 : 0];
  msm_launch<F>(c, c.stream, "api.msm", d_points, d_scalars, n, plan);
  msm_fetch<F>(c, c.stream, plan);
  BG_CUDA(cudaStreamSynchronize(c.stream));
  check_status(c, c.stream);
  msm_finish<F>(plan, out_aff32);
}

}  // namespace

namespace bg {

// streams, events and the status word of one context on `device`
void ctx_init(Ctx& c, int device) {
  int ndev = 0;
  BG_CUDA(cudaGetDeviceCount(&ndev));
  require(device >= 0 && device < ndev, "bg_ctx_create: no such CUDA device");
  BG_CUDA(cudaSetDevice(device));
  c.device = device;
  BG_CUDA(cudaDeviceGetAttribute(&c.sm_count, cudaDevAttrMultiProcessorCount, device));
  // Priorities: side[0] carries the throughput-bound accumulations of a proof's five MSMs
  // back to back, the path that sets a large proof's time; the main stream (evaluations, QAP),
  // the sort stream and the reduction streams carry work that runs beside it.  When an SM frees
  // a slot, pending blocks of the higher-priority stream are dispatched first, so the next
  // accumulation's CTAs take it and the NTT passes and hidden reductions fill what is left
  // (measured on one GB300 against the reverse order: SquareChain(2^18) 10.37-10.47 ->
  // 9.86-9.90 ms, 2^20 36.4 -> 34.6-34.9 ms, 2^10 to 2^16 level).
  int least = 0, greatest = 0;
  BG_CUDA(cudaDeviceGetStreamPriorityRange(&least, &greatest));
  BG_CUDA(cudaStreamCreateWithPriority(&c.stream, cudaStreamNonBlocking, least));
  BG_CUDA(cudaStreamCreateWithPriority(&c.copy, cudaStreamNonBlocking, least));
  for (int i = 0; i < kStreams; i++) {
    BG_CUDA(cudaStreamCreateWithPriority(&c.side[i], cudaStreamNonBlocking, i == 0 ? greatest : least));
  }
  c.d_status = c.ws.get_t<uint32_t>("status", 1);
  BG_CUDA(cudaMemsetAsync(c.d_status, 0, 4, c.stream));
  BG_CUDA(cudaStreamSynchronize(c.stream));
}

void ctx_release(Ctx& c) {
  cudaSetDevice(c.device);
  if (c.stream) cudaStreamSynchronize(c.stream);
  if (c.copy) {
    cudaStreamSynchronize(c.copy);
    cudaStreamDestroy(c.copy);
    c.copy = nullptr;
  }
  for (int i = 0; i < kStreams; i++) {
    if (c.side[i]) {
      cudaStreamSynchronize(c.side[i]);
      cudaStreamDestroy(c.side[i]);
      c.side[i] = nullptr;
    }
  }
  for (auto& kv : c.events) cudaEventDestroy(kv.second);
  c.events.clear();
  for (const Ctx::Span& sp : c.spans) {
    cudaEventDestroy(sp.a);
    cudaEventDestroy(sp.b);
  }
  c.spans.clear();
  c.ws.clear();
  if (c.stream) cudaStreamDestroy(c.stream);
  c.stream = nullptr;
}

}  // namespace bg

namespace {

// The .bin files of one directory, opened and sized up front, then read in parallel.
struct DirFiles {
  static constexpr size_t kChunk = size_t(16) << 20;
  std::vector<int> fd;
  std::vector<size_t> size;
  std::vector<std::string> path;
  DirFiles(const char* dir, const char* const* names, int n) : fd(n, -1), size(n, 0), path(n) {
    for (int i = 0; i < n; i++) {
      path[i] = std::string(dir) + "/" + names[i] + ".bin";
      fd[i] = open(path[i].c_str(), O_RDONLY);
      struct stat st;
      if (fd[i] < 0 || fstat(fd[i], &st) != 0 || st.st_size < 0) throw Error(BG_E_IO, "cannot read " + path[i]);
      size[i] = (size_t)st.st_size;
    }
  }
  ~DirFiles() {
    for (int f : fd)
      if (f >= 0) close(f);
  }
  // every file into its buffer: chunks of kChunk bytes on the host pool and the calling thread
  void read_all(char* const* buf) {
    std::vector<std::pair<int, size_t>> chunks;  // (file, offset)
    for (size_t i = 0; i < fd.size(); i++)
      for (size_t off = 0; off < size[i]; off += kChunk) chunks.emplace_back((int)i, off);
    std::atomic<int> bad{-1};
    HostPool::get().parallel_for((int)chunks.size(), [&](int c) {
      const int i = chunks[c].first;
      const size_t off = chunks[c].second, len = std::min(kChunk, size[i] - off);
      size_t got = 0;
      while (got < len) {
        const ssize_t r = pread(fd[i], buf[i] + off + got, len - got, (off_t)(off + got));
        if (r <= 0) {
          bad.store(i);
          return;
        }
        got += (size_t)r;
      }
    });
    if (bad.load() >= 0) throw Error(BG_E_IO, "cannot read " + path[bad.load()]);
  }
};

}  // namespace

extern "C" {

int bg_ctx_create(int device, bg_ctx** out) {
  BG_ARG_CHECK(nullptr, !out);
  *out = nullptr;
  bg_ctx* ctx = new bg_ctx();
  int st = guard(nullptr, [&] { ctx_init(ctx->c, device); });
  if (st != BG_OK) {
    delete ctx;
    return st;
  }
  *out = ctx;
  return BG_OK;
}

void bg_ctx_destroy(bg_ctx* ctx) {
  if (!ctx) return;
  for (auto& lane : ctx->lanes) ctx_release(*lane);
  ctx->lanes.clear();
  ctx_release(ctx->c);
  delete ctx;
}

const char* bg_strerror(int status) {
  switch (status) {
    case BG_OK: return "ok";
    case BG_E_ARG: return "invalid argument";
    case BG_E_OOM: return "out of memory";
    case BG_E_FORMAT: return "input does not match bend2/FORMAT.md";
    case BG_E_TIMEOUT: return "device wait timed out";
    case BG_E_DEVICE: return "CUDA error";
    case BG_E_IO: return "file read error";
    default: return "unknown status";
  }
}

const char* bg_last_error(const bg_ctx* ctx) { return ctx ? ctx->c.last_error.c_str() : g_err_noctx.c_str(); }

}  // extern "C"

// message of the last failure of an entry point that takes no context (read with bg_last_error(NULL))
void bg::set_noctx_error(const std::string& msg) { g_err_noctx = msg; }

extern "C" {

void* bg_ctx_stream(bg_ctx* ctx) { return ctx ? (void*)ctx->c.stream : nullptr; }

uint64_t bg_ctx_launches(const bg_ctx*) { return g_launches.load(); }

int bg_host_alloc(size_t bytes, void** out) {
  BG_ARG_CHECK(nullptr, !out);
  cudaError_t e = cudaMallocHost(out, bytes);
  if (e != cudaSuccess) {
    cudaGetLastError();
    *out = nullptr;
    return BG_E_OOM;
  }
  return BG_OK;
}

void bg_host_free(void* p) {
  if (p) cudaFreeHost(p);
}

int bg_msm_window_bits(size_t n, int curve) { return msm_pick_c(n, curve == BG_CURVE_G2); }
int bg_msm_table_window_bits(size_t n, int curve) { return msm_pick_c_table(n, curve == BG_CURVE_G2); }
int bg_msm_proof_window_bits(size_t n, int curve) { return msm_pick_c_proof(n, curve == BG_CURVE_G2); }
int bg_msm_pair_rounds(size_t n, int curve) { return msm_pair_rounds(n, curve == BG_CURVE_G2); }

int bg_msm_window_override(bg_ctx* ctx, int layout, int curve, int c) {
  BG_ARG_CHECK(ctx, !ctx || (layout != 0 && layout != 1) || (curve != BG_CURVE_G1 && curve != BG_CURVE_G2) ||
                        (c != 0 && (c < 2 || c > 22)));
  ctx->c.c_override[layout][curve == BG_CURVE_G2 ? 1 : 0] = c;
  return BG_OK;
}

int bg_msm_coop_reduce_override(bg_ctx* ctx, int mode) {
  BG_ARG_CHECK(ctx, !ctx || mode < -1 || mode > 1);
  ctx->c.coop_reduce = mode;
  for (auto& lane : ctx->lanes) lane->coop_reduce = mode;
  return BG_OK;
}

int bg_msm_pair_rounds_override(bg_ctx* ctx, int rounds) {
  BG_ARG_CHECK(ctx, !ctx || rounds < -1 || rounds > 12);
  ctx->c.pair_rounds_override = rounds;
  for (auto& lane : ctx->lanes) lane->pair_rounds_override = rounds;
  return BG_OK;
}

int bg_msm_g1(bg_ctx* ctx, const uint32_t* points16, const uint32_t* scalars16, size_t n, uint32_t* out_jac16) {
  BG_ARG_CHECK(ctx, !ctx || !out_jac16 || (n && (!points16 || !scalars16)));
  return guard(ctx, [&] {
    cudaSetDevice(ctx->c.device);
    msm_host<Fq, bgh::FqOps>(ctx->c, points16, scalars16, n, out_jac16);
  });
}

int bg_msm_g2(bg_ctx* ctx, const uint32_t* points16, const uint32_t* scalars16, size_t n, uint32_t* out_jac16) {
  BG_ARG_CHECK(ctx, !ctx || !out_jac16 || (n && (!points16 || !scalars16)));
  return guard(ctx, [&] {
    cudaSetDevice(ctx->c.device);
    msm_host<Fq2, bgh::Fq2Ops>(ctx->c, points16, scalars16, n, out_jac16);
  });
}

int bg_msm_g1_dev(bg_ctx* ctx, const uint32_t* d_points, const uint32_t* d_scalars, size_t n, uint32_t* out_aff32) {
  BG_ARG_CHECK(ctx, misaligned16(d_points) || misaligned16(d_scalars));
  BG_ARG_CHECK(ctx, !ctx || !out_aff32 || (n && (!d_points || !d_scalars)));
  return guard(ctx, [&] {
    cudaSetDevice(ctx->c.device);
    msm_dev<Fq>(ctx->c, d_points, d_scalars, n, out_aff32);
  });
}

int bg_msm_g2_dev(bg_ctx* ctx, const uint32_t* d_points, const uint32_t* d_scalars, size_t n, uint32_t* out_aff32) {
  BG_ARG_CHECK(ctx, misaligned16(d_points) || misaligned16(d_scalars));
  BG_ARG_CHECK(ctx, !ctx || !out_aff32 || (n && (!d_points || !d_scalars)));
  return guard(ctx, [&] {
    cudaSetDevice(ctx->c.device);
    msm_dev<Fq2>(ctx->c, d_points, d_scalars, n, out_aff32);
  });
}

int bg_qap_h(bg_ctx* ctx, const uint32_t* a16, const uint32_t* b16, const uint32_t* c16, uint32_t log2d,
             uint32_t* h16) {
  BG_ARG_CHECK(ctx, !ctx || !a16 || !b16 || !c16 || !h16 || log2d > 27);
  return guard(ctx, [&] {
    Ctx& c = ctx->c;
    cudaSetDevice(c.device);
    const size_t d = size_t(1) << log2d;
    uint32_t* a = stage_in(c, "api.qa", a16, d);
    uint32_t* b = stage_in(c, "api.qb", b16, d);
    uint32_t* cc = stage_in(c, "api.qc", c16, d);
    uint32_t* h = c.ws.get_t<uint32_t>("api.qh", d * 8);
    if (log2d == 0) {
      // d = 1: h = (a b - c) / (g - 1) on the one-point coset; handled by the general path
    }
    qap_h_run(c, c.stream, a, b, cc, h, (int)log2d);
    stage_out(c, "api.qh", h, h16, d);
    BG_CUDA(cudaStreamSynchronize(c.stream));
    check_status(c, c.stream);
  });
}

int bg_ntt(bg_ctx* ctx, uint32_t* data16, uint32_t log2n, int mode) {
  BG_ARG_CHECK(ctx, !ctx || !data16 || log2n > 27 || mode < 0 || mode > 3);
  return guard(ctx, [&] {
    Ctx& c = ctx->c;
    cudaSetDevice(c.device);
    const size_t n = size_t(1) << log2n;
    uint32_t* d = stage_in(c, "api.ntt", data16, n);
    ntt_run(c, c.stream, d, (int)log2n, mode);
    stage_out(c, "api.ntt", d, data16, n);
    BG_CUDA(cudaStreamSynchronize(c.stream));
    check_status(c, c.stream);
  });
}

int bg_ntt_dev(bg_ctx* ctx, uint32_t* d_data, uint32_t log2n, int mode) {
  BG_ARG_CHECK(ctx, misaligned16(d_data));
  BG_ARG_CHECK(ctx, !ctx || !d_data || log2n > 27 || mode < 0 || mode > 3);
  return guard(ctx, [&] {
    cudaSetDevice(ctx->c.device);
    ntt_run(ctx->c, ctx->c.stream, d_data, (int)log2n, mode);
  });
}

int bg_repack_to_packed_dev(bg_ctx* ctx, const uint32_t* d_wire, uint32_t* d_packed, size_t n) {
  BG_ARG_CHECK(ctx, misaligned16(d_wire) || misaligned16(d_packed));
  BG_ARG_CHECK(ctx, !ctx || (n && (!d_wire || !d_packed)));
  return guard(ctx, [&] { wire_to_packed(ctx->c.stream, d_wire, d_packed, n, ctx->c.d_status); });
}

int bg_repack_to_wire_dev(bg_ctx* ctx, const uint32_t* d_packed, uint32_t* d_wire, size_t n) {
  BG_ARG_CHECK(ctx, misaligned16(d_wire) || misaligned16(d_packed));
  BG_ARG_CHECK(ctx, !ctx || (n && (!d_wire || !d_packed)));
  return guard(ctx, [&] { packed_to_wire(ctx->c.stream, d_packed, d_wire, n); });
}

int bg_field_op(bg_ctx* ctx, int field, int op, const uint32_t* a16, const uint32_t* b16, uint32_t* out16,
                size_t n) {
  const bool binary = op == BG_FOP_ADD || op == BG_FOP_SUB || op == BG_FOP_MUL;
  BG_ARG_CHECK(ctx, !ctx || (field != BG_FIELD_FR && field != BG_FIELD_FQ) || op < 0 || op > BG_FOP_FROM_MONT);
  BG_ARG_CHECK(ctx, n && (!a16 || !out16 || (binary && !b16)));
  return guard(ctx, [&] {
    Ctx& c = ctx->c;
    cudaSetDevice(c.device);
    if (n == 0) return;
    uint32_t* a = stage_in(c, "api.fa", a16, n);
    uint32_t* b = binary ? stage_in(c, "api.fb", b16, n) : nullptr;
    uint32_t* o = c.ws.get_t<uint32_t>("api.fo", n * 8);
    field_op(c.stream, field, op, a, b, o, n);
    stage_out(c, "api.fo", o, out16, n);
    BG_CUDA(cudaStreamSynchronize(c.stream));
    check_status(c, c.stream);
  });
}

int bg_curve_op(bg_ctx* ctx, int curve, int op, const uint32_t* p16, const uint32_t* q16, const uint32_t* k16,
                uint32_t* out16, size_t n) {
  BG_ARG_CHECK(ctx, !ctx || (curve != BG_CURVE_G1 && curve != BG_CURVE_G2) || op < 0 || op > BG_COP_MUL);
  BG_ARG_CHECK(ctx, n && (!p16 || !out16 || (op == BG_COP_ADD && !q16) || (op == BG_COP_MUL && !k16)));
  return guard(ctx, [&] {
    Ctx& c = ctx->c;
    cudaSetDevice(c.device);
    if (n == 0) return;
    const size_t fe = curve == BG_CURVE_G1 ? 2 : 4;  // field elements per affine point
    uint32_t* p = stage_in(c, "api.cp", p16, n * fe);
    uint32_t* q = op == BG_COP_ADD ? stage_in(c, "api.cq", q16, n * fe) : nullptr;
    uint32_t* k = op == BG_COP_MUL ? stage_in(c, "api.ck", k16, n) : nullptr;
    uint32_t* o = c.ws.get_t<uint32_t>("api.co", n * fe * 8);
    curve_op(c.stream, curve, op, p, q, k, o, n);
    stage_out(c, "api.co", o, out16, n * fe);
    BG_CUDA(cudaStreamSynchronize(c.stream));
    check_status(c, c.stream);
  });
}

int bg_pk_upload(bg_ctx* ctx, const bg_inputs* in, bg_pk** out) {
  BG_ARG_CHECK(ctx, !ctx || !in || !out);
  *out = nullptr;
  return guard(ctx, [&] {
    cudaSetDevice(ctx->c.device);
    PkDev* pk = pk_upload(ctx->c, *in, true);
    *out = new bg_pk{pk, ctx};
  });
}

void bg_pk_release(bg_pk* pk) {
  if (!pk) return;
  cudaSetDevice(pk->owner->c.device);
  cudaStreamSynchronize(pk->owner->c.stream);
  pk_free(pk->pk);
  delete pk;
}

int bg_prove_resident(bg_ctx* ctx, bg_pk* pk, const uint32_t* witness16, const uint32_t* rs16, bg_proof* out,
                      bg_phase_ms* times) {
  BG_ARG_CHECK(ctx, !ctx || !pk || !witness16 || !rs16 || !out);
  return guard(ctx, [&] {
    cudaSetDevice(ctx->c.device);
    prove_resident(ctx->c, *pk->pk, witness16, rs16, out, times, 0.0);
  });
}

int bg_prove_batch(bg_ctx* ctx, bg_pk* const* pks, const uint32_t* const* witnesses, const uint32_t* const* rs,
                   size_t count, int lanes, bg_proof* out, bg_phase_ms* times, int* statuses) {
  BG_ARG_CHECK(ctx, !ctx || (count && (!pks || !witnesses || !rs || !out || !statuses)) || lanes < 1 || lanes > 32);
  for (size_t i = 0; i < count; i++)
    BG_ARG_CHECK(ctx, !pks[i] || !witnesses[i] || !rs[i] || pks[i]->owner != ctx);
  return guard(ctx, [&] {
    cudaSetDevice(ctx->c.device);
    while ((int)ctx->lanes.size() < lanes) {
      std::unique_ptr<Ctx> lane(new Ctx());
      ctx_init(*lane, ctx->c.device);
      lane->shared_gpu = true;
      lane->pair_rounds_override = ctx->c.pair_rounds_override;
      lane->coop_reduce = ctx->c.coop_reduce;
      ctx->lanes.push_back(std::move(lane));
    }
    // largest domains first (longest-processing-time order) so the tail is made of small proofs
    std::vector<size_t> order(count);
    for (size_t i = 0; i < count; i++) order[i] = i;
    std::stable_sort(order.begin(), order.end(),
                     [&](size_t a, size_t b) { return pks[a]->pk->h.lg > pks[b]->pk->h.lg; });
    std::atomic<size_t> next{0};
    auto work = [&](Ctx* lane) {
      cudaSetDevice(lane->device);
      for (;;) {
        const size_t k = next.fetch_add(1);
        if (k >= count) return;
        const size_t i = order[k];
        try {
          prove_resident(*lane, *pks[i]->pk, witnesses[i], rs[i], &out[i], times ? &times[i] : nullptr, 0.0);
          statuses[i] = BG_OK;
        } catch (const Error& e) {
          statuses[i] = e.status;
          if (e.status == BG_E_DEVICE) cudaGetLastError();
        } catch (...) {
          statuses[i] = BG_E_DEVICE;
        }
      }
    };
    std::vector<std::thread> threads;
    for (int l = 0; l < lanes; l++) threads.emplace_back(work, ctx->lanes[l].get());
    for (auto& t : threads) t.join();
  });
}

size_t bg_prove_footprint(const bg_pk* pk) { return pk ? prove_footprint(pk->pk->h) : 0; }

int bg_server_create(bg_ctx* ctx, int lanes, size_t hbm_budget_bytes, bg_server** out) {
  BG_ARG_CHECK(ctx, !ctx || !out || lanes < 1 || lanes > 32 || hbm_budget_bytes == 0);
  *out = nullptr;
  return guard(ctx, [&] {
    cudaSetDevice(ctx->c.device);
    *out = new bg_server{server_create(ctx->c.device, lanes, hbm_budget_bytes), ctx};
  });
}

int bg_server_submit(bg_server* s, bg_pk* pk, const uint32_t* witness16, const uint32_t* rs16, uint64_t tag) {
  BG_ARG_CHECK(s ? s->owner : nullptr, !s || !pk || !witness16 || !rs16 || pk->owner != s->owner);
  return guard(s->owner, [&] { server_submit(s->s, pk->pk, witness16, rs16, tag); });
}

int bg_server_wait(bg_server* s, int timeout_ms, uint64_t* tag, bg_proof* out, bg_phase_ms* times,
                   double* latency_ms, double* queue_ms, int* status) {
  BG_ARG_CHECK(s ? s->owner : nullptr, !s || !tag || !status || timeout_ms < 0);
  return server_wait(s->s, timeout_ms, tag, out, times, latency_ms, queue_ms, status) ? BG_OK : BG_E_TIMEOUT;
}

size_t bg_server_reserved_bytes(bg_server* s) { return s ? server_reserved(s->s) : 0; }

void bg_server_destroy(bg_server* s) {
  if (!s) return;
  server_destroy(s->s);
  delete s;
}

int bg_prove_host(bg_ctx* ctx, const bg_inputs* in, bg_proof* out, bg_phase_ms* times) {
  BG_ARG_CHECK(ctx, !ctx || !in || !out);
  return guard(ctx, [&] {
    cudaSetDevice(ctx->c.device);
    const auto t0 = std::chrono::steady_clock::now();
    const Header h = parse_header(*in);
    validate_inputs(*in, h, true);
    PkDev* pk = pk_stage_oneshot(ctx->c, *in);
    const double up_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    try {
      prove_resident(ctx->c, *pk, static_cast<const uint32_t*>(in->witness), static_cast<const uint32_t*>(in->rs),
                     out, times, up_ms);
    } catch (...) {
      pk_free(pk);
      throw;
    }
    pk_free(pk);
  });
}

int bg_prove_dir(bg_ctx* ctx, const char* dir, bg_proof* out, bg_phase_ms* times) {
  BG_ARG_CHECK(ctx, !ctx || !dir || !out);
  return guard(ctx, [&] {
    const auto t0 = std::chrono::steady_clock::now();
    static const char* names[13] = {"header", "witness", "r1cs_a", "r1cs_b", "r1cs_c", "pk_g1", "pk_g2",
                                    "pk_a",   "pk_b1",   "pk_b2",  "pk_h",   "pk_l",   "rs"};
    // The files go straight into pinned host buffers cached by the context (no zero-filled
    // pageable copy, no staging on the way to the device): the 13 files are cut into 16 MiB
    // chunks read with pread on the host pool, and every upload of the proof is then an
    // asynchronous copy from pinned memory that overlaps the proof (load_u32 of
    // bend2/src/bin_io.bend:73-78 reads them one after another).
    cudaSetDevice(ctx->c.device);
    DirFiles files(dir, names, 13);
    char* buf[13];
    for (int i = 0; i < 13; i++)
      buf[i] = ctx->c.host_cache.get_t<char>(std::string("dir.") + names[i], std::max<size_t>(files.size[i], 1));
    files.read_all(buf);
    bg_inputs in;
    const void** ptrs[13] = {&in.header, &in.witness, &in.r1cs_a, &in.r1cs_b, &in.r1cs_c, &in.pk_g1, &in.pk_g2,
                             &in.pk_a,   &in.pk_b1,   &in.pk_b2,  &in.pk_h,   &in.pk_l,   &in.rs};
    size_t* sizes[13] = {&in.header_bytes, &in.witness_bytes, &in.r1cs_a_bytes, &in.r1cs_b_bytes,
                         &in.r1cs_c_bytes, &in.pk_g1_bytes,   &in.pk_g2_bytes,  &in.pk_a_bytes,
                         &in.pk_b1_bytes,  &in.pk_b2_bytes,   &in.pk_h_bytes,   &in.pk_l_bytes,
                         &in.rs_bytes};
    for (int i = 0; i < 13; i++) {
      *ptrs[i] = buf[i];
      *sizes[i] = files.size[i];
    }
    const Header h = parse_header(in);
    validate_inputs(in, h, true);
    PkDev* pk = pk_stage_oneshot(ctx->c, in);
    const double load_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    try {
      prove_resident(ctx->c, *pk, static_cast<const uint32_t*>(in.witness), static_cast<const uint32_t*>(in.rs),
                     out, times, load_ms);
    } catch (...) {
      pk_free(pk);
      throw;
    }
    pk_free(pk);
  });
}

int bg_synth_square_chain(bg_ctx* ctx, uint32_t log2n, uint64_t seed, const char* dir) {
  BG_ARG_CHECK(ctx, !ctx || !dir);
  return guard(ctx, [&] {
    cudaSetDevice(ctx->c.device);
    synth_square_chain(ctx->c, log2n, seed, dir);
  });
}

int bg_ctx_profile(bg_ctx* ctx, int enable) {
  BG_ARG_CHECK(ctx, !ctx);
  return guard(ctx, [&] {
    cudaSetDevice(ctx->c.device);
    for (int i = 0; i < kStreams; i++) BG_CUDA(cudaStreamSynchronize(ctx->c.side[i]));
    BG_CUDA(cudaStreamSynchronize(ctx->c.stream));
    for (auto& kv : ctx->c.ktimes)
      for (auto& ev : kv.second.pending) {
        cudaEventDestroy(ev.first);
        cudaEventDestroy(ev.second);
      }
    ctx->c.ktimes.clear();
    ctx->c.profile = enable != 0;
  });
}

int bg_ctx_timeline(bg_ctx* ctx, int enable, char* buf, size_t cap) {
  BG_ARG_CHECK(ctx, !ctx || (!enable && (!buf || cap == 0)));
  return guard(ctx, [&] {
    Ctx& c = ctx->c;
    cudaSetDevice(c.device);
    for (int i = 0; i < kStreams; i++) BG_CUDA(cudaStreamSynchronize(c.side[i]));
    BG_CUDA(cudaStreamSynchronize(c.stream));
    std::string text;
    if (!enable && !c.spans.empty()) {
      char line[160];
      for (const Ctx::Span& sp : c.spans) {
        float t0 = 0, t1 = 0;
        BG_CUDA(cudaEventElapsedTime(&t0, c.spans[0].a, sp.a));
        BG_CUDA(cudaEventElapsedTime(&t1, c.spans[0].a, sp.b));
        snprintf(line, sizeof line, "%s %.4f %.4f\n", sp.name.c_str(), t0, t1);
        text += line;
      }
    }
    for (const Ctx::Span& sp : c.spans) {
      cudaEventDestroy(sp.a);
      cudaEventDestroy(sp.b);
    }
    c.spans.clear();
    c.timeline = enable != 0;
    if (!enable) {
      require(text.size() < cap, "bg_ctx_timeline: buffer too small for the recorded spans");
      memcpy(buf, text.c_str(), text.size() + 1);
    }
  });
}

int bg_ctx_transfer_bytes(bg_ctx* ctx, uint64_t* h2d, uint64_t* d2h) {
  BG_ARG_CHECK(ctx, !ctx || !h2d || !d2h);
  return guard(ctx, [&] {
    *h2d = ctx->c.h2d_bytes;
    *d2h = ctx->c.d2h_bytes;
    for (auto& l : ctx->lanes) {
      *h2d += l->h2d_bytes;
      *d2h += l->d2h_bytes;
    }
  });
}

int bg_ctx_kernel_stats(bg_ctx* ctx, const char* name, uint64_t* launches, double* total_ms) {
  BG_ARG_CHECK(ctx, !ctx || !name || !launches || !total_ms);
  return guard(ctx, [&] {
    *launches = 0;
    *total_ms = 0;
    auto it = ctx->c.ktimes.find(name);
    if (it == ctx->c.ktimes.end()) return;
    Ctx::KernelTimes& kt = it->second;
    for (auto& ev : kt.pending) {
      BG_CUDA(cudaEventSynchronize(ev.second));
      float ms = 0;
      BG_CUDA(cudaEventElapsedTime(&ms, ev.first, ev.second));
      kt.total_ms += ms;
      cudaEventDestroy(ev.first);
      cudaEventDestroy(ev.second);
    }
    kt.pending.clear();
    *launches = kt.launches;
    *total_ms = kt.total_ms;
  });
}

int bg_probe_imad(bg_ctx* ctx, int which, uint32_t iters, double* ops, double* ms) {
  BG_ARG_CHECK(ctx, !ctx || !ops || !ms || which < 0 || which > 4 || iters == 0);
  return guard(ctx, [&] {
    Ctx& c = ctx->c;
    cudaSetDevice(c.device);
    const int threads = 256, blocks = c.sm_count * 8;
    uint32_t* sink = c.ws.get_t<uint32_t>("probe.sink", 1);
    cudaEvent_t a, b;
    BG_CUDA(cudaEventCreate(&a));
    BG_CUDA(cudaEventCreate(&b));
    imad_probe(c.stream, blocks, threads, 1, sink, which);  // warm-up
    BG_CUDA(cudaEventRecord(a, c.stream));
    imad_probe(c.stream, blocks, threads, iters, sink, which);
    BG_CUDA(cudaEventRecord(b, c.stream));
    BG_CUDA(cudaEventSynchronize(b));
    float t = 0;
    BG_CUDA(cudaEventElapsedTime(&t, a, b));
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    const double per_thread = which == 1 ? 4.0 * iters : 16.0 * iters;
    *ops = per_thread * threads * blocks;
    *ms = t;
  });
}

int bg_proof_format(const bg_proof* proof, char* buf, size_t buf_bytes) {
  BG_ARG_CHECK(nullptr, !proof || !buf);
  return format_proof(proof, buf, buf_bytes);
}

int bg_verify(const bg_vk* vk, const uint32_t* public16, size_t n_public, const bg_proof* proof, int* valid) {
  BG_ARG_CHECK(nullptr, !vk || !proof || !valid);
  try {
    const bgh::VkWire w{vk->alpha_g1, vk->beta_g2, vk->gamma_g2, vk->delta_g2, vk->gamma_abc_g1, vk->n_ic};
    *valid = bgh::groth16_verify(w, public16, n_public, proof->a, proof->b, proof->c);
    return BG_OK;
  } catch (const bgh::MalformedInput& e) {
    *valid = 0;
    bg::set_noctx_error(e.what());
    return BG_E_FORMAT;
  } catch (const std::exception& e) {
    bg::set_noctx_error(e.what());
    return BG_E_ARG;
  }
}

int bg_pairing(const uint32_t* p32, const uint32_t* q64, uint32_t* out192) {
  BG_ARG_CHECK(nullptr, !p32 || !q64 || !out192);
  try {
    bgh::pairing_wire(p32, q64, out192);
    return BG_OK;
  } catch (const std::exception& e) {
    bg::set_noctx_error(e.what());
    return BG_E_ARG;
  }
}

}  // extern "C"
