// Shared host-side plumbing for the CUDA translation units: error handling, the per-context
// workspace cache and the context record behind the C ABI handle.
#pragma once
#include <cuda_runtime.h>

#include <atomic>
#include <cstdint>
#include <cstdio>
#include <map>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/bg.h"

namespace bg {

struct Error : std::runtime_error {
  int status;
  Error(int s, const std::string& m) : std::runtime_error(m), status(s) {}
};

#define BG_CUDA(call)                                                                       \
  do {                                                                                      \
    cudaError_t e_ = (call);                                                                \
    if (e_ != cudaSuccess) {                                                                \
      throw ::bg::Error(e_ == cudaErrorMemoryAllocation ? BG_E_OOM : BG_E_DEVICE,           \
                        std::string(#call) + ": " + cudaGetErrorString(e_) + " at " +        \
                            __FILE__ + ":" + std::to_string(__LINE__));                      \
    }                                                                                       \
  } while (0)

// kernels launched by this library in this process (every launch site is followed by this check)
extern std::atomic<uint64_t> g_launches;
#define BG_CHECK_LAUNCH()      \
  do {                         \
    ::bg::g_launches++;        \
    BG_CUDA(cudaGetLastError()); \
  } while (0)

// Device buffers cached per context by name: a call asks for `bytes` and gets a buffer of at
// least that size, reused across calls (grown, never shrunk, until the context is freed).
class Workspace {
 public:
  void* get(const std::string& name, size_t bytes) {
    auto it = bufs_.find(name);
    if (it != bufs_.end() && it->second.bytes >= bytes) return it->second.ptr;
    if (it != bufs_.end()) {
      cudaFree(it->second.ptr);
      bufs_.erase(it);
    }
    void* p = nullptr;
    size_t want = bytes < 256 ? 256 : bytes;
    cudaError_t e = cudaMalloc(&p, want);
    if (e != cudaSuccess) {
      cudaGetLastError();
      throw Error(BG_E_OOM, "device allocation of " + std::to_string(want) + " bytes for " + name + " failed: " +
                                cudaGetErrorString(e));
    }
    bufs_[name] = {p, want};
    return p;
  }
  template <class T>
  T* get_t(const std::string& name, size_t count) {
    return static_cast<T*>(get(name, count * sizeof(T)));
  }
  size_t bytes() const {
    size_t s = 0;
    for (auto& kv : bufs_) s += kv.second.bytes;
    return s;
  }
  void clear() {
    for (auto& kv : bufs_) cudaFree(kv.second.ptr);
    bufs_.clear();
  }
  ~Workspace() { clear(); }

 private:
  struct Buf {
    void* ptr;
    size_t bytes;
  };
  std::map<std::string, Buf> bufs_;
};

// Pinned host staging buffer, grown on demand
class PinnedBuf {
 public:
  void* get(size_t bytes) {
    if (bytes > cap_) {
      if (ptr_) cudaFreeHost(ptr_);
      ptr_ = nullptr;
      BG_CUDA(cudaMallocHost(&ptr_, bytes));
      cap_ = bytes;
    }
    return ptr_;
  }
  ~PinnedBuf() {
    if (ptr_) cudaFreeHost(ptr_);
  }

 private:
  void* ptr_ = nullptr;
  size_t cap_ = 0;
};

// Pinned host buffers cached by name (allocation synchronises the device, so it happens once)
class PinnedCache {
 public:
  template <class T>
  T* get_t(const std::string& name, size_t count) {
    auto& b = bufs_[name];
    return static_cast<T*>(b.get(count * sizeof(T)));
  }

 private:
  std::map<std::string, PinnedBuf> bufs_;
};

constexpr int kStreams = 7;
constexpr int kSortStream = 6;  // side stream of a proof's bucket sorts

// NTT tables for one domain size 2^L (device pointers into the context workspace)
struct NttTables {
  bool ready = false;
  uint32_t* tw_fwd = nullptr;      // w^i, i < 2^(L-1), w of order 2^L (Montgomery)
  uint32_t* tw_inv = nullptr;      // w^-i
  int coset_bits = 0;              // a: coset powers split as lo[i & (2^a-1)] * hi[i >> a]
  uint32_t* g_lo = nullptr;        // g^i, i < 2^a
  uint32_t* gi_lo = nullptr;       // g^-i
  uint32_t* g_hi = nullptr;        // g^(i 2^a)
  uint32_t* g_hi_ninv = nullptr;   // n^-1 g^(i 2^a)
  uint32_t* gi_hi_ninv = nullptr;  // n^-1 g^(-i 2^a)
  uint32_t* ninv = nullptr;        // n^-1
  uint32_t* zinv = nullptr;        // (g^n - 1)^-1
};

struct Ctx {
  int device = 0;
  int sm_count = 0;
  // a lane of bg_prove_batch or of the server: other lanes' proofs share the GPU, so a proof
  // keeps the throughput-oriented schedule even when it is small
  bool shared_gpu = false;
  cudaStream_t stream = nullptr;          // main stream: every public call is ordered on it
  cudaStream_t side[kStreams] = {};       // concurrent MSMs inside a proof
  cudaStream_t copy = nullptr;            // uploads that overlap a proof (one-shot keys)
  Workspace ws;
  PinnedBuf pinned[4];
  PinnedCache host_cache;
  std::string last_error;
  uint32_t* d_status = nullptr;           // device-side error flags (see BG_DSTATUS_*)
  uint64_t h2d_bytes = 0, d2h_bytes = 0;  // host <-> device bytes this context has copied
  // window widths forced for tuning (bg_msm_window_override): [0] per-window bucket sets,
  // [1] window tables of keys uploaded afterwards; [curve]; 0 = the library's choice
  int c_override[2][2] = {{0, 0}, {0, 0}};
  // batch-affine pair rounds before each MSM's accumulation (bg_msm_pair_rounds_override):
  // -1 = the library's cost model, 0 = none
  int pair_rounds_override = -1;
  // cooperative window reductions for latency-critical MSMs (bg_msm_coop_reduce_override):
  // -1 = the library's model, 0 = never, 1 = always
  int coop_reduce = -1;
  std::map<int, NttTables> ntt_tabs;      // per domain size, built on first use
  // optional per-kernel timing: CUDA events recorded around selected launches on their
  // own stream, resolved when the statistics are read
  bool profile = false;
  struct KernelTimes {
    std::vector<std::pair<cudaEvent_t, cudaEvent_t>> pending;
    uint64_t launches = 0;
    double total_ms = 0;
  };
  std::map<std::string, KernelTimes> ktimes;
  // optional launch timeline: (family, start, end) events of every timed launch, in order
  bool timeline = false;
  struct Span {
    std::string name;
    cudaEvent_t a, b;
  };
  std::vector<Span> spans;
  // named events for cross-stream ordering, created on first use
  std::map<std::string, cudaEvent_t> events;
  cudaEvent_t event(const std::string& name) {
    auto it = events.find(name);
    if (it != events.end()) return it->second;
    cudaEvent_t e = nullptr;
    BG_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    events[name] = e;
    return e;
  }
};

// Brackets one kernel launch with events when the context profiles (see bg_ctx_profile).
class KernelTimer {
 public:
  KernelTimer(Ctx& c, const char* name, cudaStream_t st) : c_(c), st_(st) {
    if (c.timeline) {
      span_ = true;
      name_ = name;
      cudaEventCreate(&ta_);
      cudaEventCreate(&tb_);
      cudaEventRecord(ta_, st);
    }
    if (!c.profile) return;
    kt_ = &c.ktimes[name];
    cudaEventCreate(&a_);
    cudaEventCreate(&b_);
    cudaEventRecord(a_, st);
  }
  ~KernelTimer() {
    if (span_) {
      cudaEventRecord(tb_, st_);
      c_.spans.push_back({name_, ta_, tb_});
    }
    if (!kt_) return;
    cudaEventRecord(b_, st_);
    kt_->pending.push_back({a_, b_});
    kt_->launches++;
  }

 private:
  Ctx& c_;
  cudaStream_t st_;
  Ctx::KernelTimes* kt_ = nullptr;
  cudaEvent_t a_ = nullptr, b_ = nullptr;
  bool span_ = false;
  const char* name_ = nullptr;
  cudaEvent_t ta_ = nullptr, tb_ = nullptr;
};

// device status flag bits
enum : uint32_t {
  BG_DSTATUS_SCALAR_RANGE = 1u,  // an MSM scalar had bit 254 or 255 set
  BG_DSTATUS_CAPACITY = 2u,      // a bucket list overflowed its capacity
  BG_DSTATUS_FORMAT = 4u,        // a wire word had bits above its 16-bit limb
  BG_DSTATUS_COLUMN = 8u,        // an R1CS column index was outside the assignment
};

inline unsigned ceil_div(size_t a, size_t b) { return (unsigned)((a + b - 1) / b); }

void set_noctx_error(const std::string& msg);
// create / destroy the streams, events and workspace of a context on `device`
void ctx_init(Ctx& c, int device);
void ctx_release(Ctx& c);

}  // namespace bg
