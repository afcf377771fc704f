// Serving loop: continuous batching of prove requests against device-resident proving keys.
//
// The reference proves one proof per process (bend2/prove.bend:164-168); this is the serving
// configuration of the benchmark plan (requests of different K arriving over time).  A fixed
// pool of lanes -- each a context with its own streams and cached workspace -- takes requests
// from one FIFO queue.  The head request is admitted as soon as a lane is free and the lanes'
// reserved scratch (the largest per-proof footprint each lane has served) stays within the
// HBM budget after admitting it; admitted requests run concurrently on the device, so a request
// that arrives while others are proving starts as soon as a lane and memory free up.  Every
// result is the proof prove_resident makes for the same inputs alone.
#include <chrono>
#include <condition_variable>
#include <deque>
#include <memory>
#include <mutex>
#include <thread>
#include <vector>

#include "common.cuh"
#include "msm.h"
#include "prove.h"

namespace bg {

using Clock = std::chrono::steady_clock;

struct ServerRequest {
  uint64_t tag;
  PkDev* pk;
  const uint32_t* witness16;
  const uint32_t* rs16;
  size_t footprint;
  Clock::time_point t_submit;
};

struct ServerDone {
  uint64_t tag;
  bg_proof proof;
  bg_phase_ms times;
  int status;
  double latency_ms;  // submit -> result ready
  double queue_ms;    // submit -> start on a lane
};

class Server {
 public:
  Server(int device, int lanes, size_t budget) : device_(device), budget_(budget) {
    for (int i = 0; i < lanes; i++) {
      std::unique_ptr<Ctx> c(new Ctx());
      ctx_init(*c, device);
      c->shared_gpu = lanes > 1;
      lanes_.push_back(std::move(c));
      reserved_.push_back(0);
      busy_.push_back(false);
    }
    for (int i = 0; i < lanes; i++) workers_.emplace_back(&Server::worker, this, i);
  }

  ~Server() {
    {
      std::lock_guard<std::mutex> lk(mu_);
      stop_ = true;
      queue_.clear();
    }
    cv_work_.notify_all();
    for (auto& t : workers_) t.join();
    for (auto& c : lanes_) ctx_release(*c);
  }

  void submit(const ServerRequest& r) {
    if (r.footprint > budget_)
      throw Error(BG_E_OOM, "bg_server_submit: the request needs " + std::to_string(r.footprint) +
                                " bytes of scratch, above the server's HBM budget of " + std::to_string(budget_));
    {
      std::lock_guard<std::mutex> lk(mu_);
      queue_.push_back(r);
    }
    cv_work_.notify_all();
  }

  bool wait(int timeout_ms, ServerDone& out) {
    std::unique_lock<std::mutex> lk(mu_);
    if (!cv_done_.wait_for(lk, std::chrono::milliseconds(timeout_ms), [&] { return !done_.empty(); })) return false;
    out = done_.front();
    done_.pop_front();
    return true;
  }

  size_t reserved_bytes() {
    std::lock_guard<std::mutex> lk(mu_);
    size_t s = 0;
    for (size_t v : reserved_) s += v;
    return s;
  }

 private:
  // called with mu_ held: can lane i take the head request?
  bool admissible(int i) const {
    if (busy_[i] || queue_.empty()) return false;
    const size_t fp = queue_.front().footprint;
    if (reserved_[i] >= fp) return true;
    size_t total = 0;
    for (size_t v : reserved_) total += v;
    return total - reserved_[i] + fp <= budget_;
  }

  void worker(int i) {
    cudaSetDevice(device_);
    Ctx& lane = *lanes_[i];
    for (;;) {
      ServerRequest r;
      {
        std::unique_lock<std::mutex> lk(mu_);
        cv_work_.wait(lk, [&] { return stop_ || admissible(i); });
        if (stop_) return;
        r = queue_.front();
        queue_.pop_front();
        busy_[i] = true;
        if (reserved_[i] < r.footprint) reserved_[i] = r.footprint;
      }
      cv_work_.notify_all();  // the next head request may fit another lane
      ServerDone d;
      d.tag = r.tag;
      const auto t_start = Clock::now();
      try {
        prove_resident(lane, *r.pk, r.witness16, r.rs16, &d.proof, &d.times, 0.0);
        d.status = BG_OK;
      } catch (const Error& e) {
        d.status = e.status;
        if (e.status == BG_E_DEVICE) cudaGetLastError();
      } catch (...) {
        d.status = BG_E_DEVICE;
      }
      const auto t_end = Clock::now();
      d.queue_ms = std::chrono::duration<double, std::milli>(t_start - r.t_submit).count();
      d.latency_ms = std::chrono::duration<double, std::milli>(t_end - r.t_submit).count();
      {
        std::lock_guard<std::mutex> lk(mu_);
        busy_[i] = false;
        done_.push_back(d);
      }
      cv_done_.notify_all();
      cv_work_.notify_all();
    }
  }

  int device_;
  size_t budget_;
  std::vector<std::unique_ptr<Ctx>> lanes_;
  std::vector<size_t> reserved_;
  std::vector<bool> busy_;
  std::vector<std::thread> workers_;
  std::mutex mu_;
  std::condition_variable cv_work_, cv_done_;
  std::deque<ServerRequest> queue_;
  std::deque<ServerDone> done_;
  bool stop_ = false;
};

Server* server_create(int device, int lanes, size_t budget) { return new Server(device, lanes, budget); }
void server_destroy(Server* s) { delete s; }
void server_submit(Server* s, PkDev* pk, const uint32_t* w, const uint32_t* rs, uint64_t tag) {
  s->submit(ServerRequest{tag, pk, w, rs, prove_footprint(pk->h), Clock::now()});
}
bool server_wait(Server* s, int timeout_ms, uint64_t* tag, bg_proof* out, bg_phase_ms* times, double* latency_ms,
                 double* queue_ms, int* status) {
  ServerDone d;
  if (!s->wait(timeout_ms, d)) return false;
  *tag = d.tag;
  if (out) *out = d.proof;
  if (times) *times = d.times;
  if (latency_ms) *latency_ms = d.latency_ms;
  if (queue_ms) *queue_ms = d.queue_ms;
  *status = d.status;
  return true;
}
size_t server_reserved(Server* s) { return s->reserved_bytes(); }

}  // namespace bg
