// MSM engine interface (see msm.cu)
#pragma once
#include <string>
#include <vector>

#include "common.cuh"

namespace bg {

struct MsmPlan {
  int c = 0;                              // window bits (0: pick from n)
  int W = 0;                              // windows
  size_t entries = 0;                     // bucket entries (n * W upper bound)
  uint32_t J = 1;                         // reduction parts per window
  uint32_t part_span = 1;                 // buckets per part
  const uint32_t* d_window_sums = nullptr;  // W x J x 2 XYZZ points on the device
  cudaStream_t fetch_stream = nullptr;      // stream the reduction (and the copy) run on
  // W XYZZ points after msm_fetch, in the context's pinned cache (a pageable destination
  // would make the copy block the host and serialise the streams of a proof)
  uint32_t* host_window_sums = nullptr;
  // false: the reduction runs underneath later work (another MSM's accumulation) and takes
  // small CTAs; true: it is the tail of the caller's critical path and takes the shape with
  // the shortest dependent chain
  bool latency_critical = true;
  // for a reduction that is not latency-critical: the accumulation work (us) queued after it
  // on the accumulation stream, which it should finish under; a longer reduction by the latency
  // model is treated as critical (0 = no budget known: trust latency_critical)
  double hidden_us = 0;
  // the host pool is otherwise idle when this reduction ends (not one of a small proof's
  // reductions that end together), so its part sums are priced as the pool runs them
  bool host_pool_free = false;
};

// Window table of a fixed point set: row w (w < W) holds 2^(o_w) P_i for all i (o_w the bit
// offset of window w in the balanced layout of msm.cu), so every
// window's digits index one shared bucket set (no window combination afterwards).
struct MsmTable {
  uint32_t* d = nullptr;  // W rows of n packed affine points (device, owned by the key)
  size_t n = 0;
  int c = 0, W = 0;
};

// Bucket order of one scalar vector for one window layout (c-bit signed digits; one bucket set
// per window, or one set shared by all windows for window tables).  It depends on the scalars
// and the layout only, so MSMs over the same scalars and layout share it.
struct MsmSort {
  size_t n = 0;
  int c = 0, W = 0, sets = 0;
  uint32_t nb = 0;
  size_t nkeys = 0, max_entries = 0;
  uint32_t* offsets = nullptr;  // nkeys + 1 bucket offsets into sorted
  uint32_t* sorted = nullptr;   // entries: point index (+ w n for tables) | sign << 31
  cudaEvent_t done = nullptr;   // recorded after the scatter (null: ordered by the stream)
};

// window width for n points (the committed table of msm_tune.h, else a size rule)
int msm_pick_c(size_t n, bool g2 = false);
int msm_pick_c_table(size_t n, bool g2 = false);
// window width of a bucket-set-per-window MSM inside a proof (one-shot proofs)
int msm_pick_c_proof(size_t n, bool g2 = false);
// batch-affine pair rounds the cost model takes for a standalone MSM of n points
int msm_pair_rounds(size_t n, bool g2 = false);
// the same for an MSM of at most max_entries bucket entries over nkeys buckets
int msm_pair_rounds_entries(size_t max_entries, size_t nkeys, bool g2);
void msm_init_kernels();
// allocate t.d (cudaMalloc) and fill it from n packed affine points on `st`; c = 0 picks the
// window width from n
template <class F>
void msm_build_table(cudaStream_t st, const uint32_t* d_points, size_t n, MsmTable& t, int c = 0);
void exclusive_scan(Workspace& ws, const std::string& tag, const uint32_t* d_in, uint32_t* d_out, size_t n,
                    cudaStream_t st, int depth);

// Enqueue every device phase of one MSM on `st` (the window reduction on `st_reduce` when
// given, after an event); scratch buffers are named by `tag` so that MSMs in flight at the
// same time use different memory.
// With `table`, d_points is ignored and the table's rows are used (one bucket set).
template <class F>
void msm_launch(Ctx& ctx, cudaStream_t st, const std::string& tag, const uint32_t* d_points,
                const uint32_t* d_scalars, size_t n, MsmPlan& plan, cudaStream_t st_reduce = nullptr,
                const MsmTable* table = nullptr);
// The two halves of msm_launch: the sort on `st` (records so.done), and everything after it
// on `st` (waits for so.done) with the fixup and reduction on `st_reduce`.
void msm_sort(Ctx& ctx, cudaStream_t st, const std::string& tag, const uint32_t* d_scalars, size_t n, int c,
              bool shared_set, MsmSort& out);
template <class F>
void msm_accumulate(Ctx& ctx, cudaStream_t st, const std::string& tag, const uint32_t* d_points, const MsmSort& so,
                    MsmPlan& plan, cudaStream_t st_reduce = nullptr, const MsmTable* table = nullptr);
// Enqueue the copy of the window sums to the host.
template <class F>
void msm_fetch(Ctx& ctx, cudaStream_t st, MsmPlan& plan);
// After the stream is synchronised: Horner over windows, affine result (packed words,
// 16 for G1, 32 for G2; all zero = infinity).
template <class F>
void msm_finish(const MsmPlan& plan, uint32_t* out_affine_words32);

}  // namespace bg
