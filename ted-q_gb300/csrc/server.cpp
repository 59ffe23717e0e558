// server.cpp -- continuous-batching server for circuit evaluations
// (tedq_server_* in include/tedq_gb300.h).
//
// A server owns a device-memory arena (the admission budget, allocated
// once), a pinned host staging arena and a set of streams, served by one
// worker thread per size-class lane.  Each turn a worker (1) retires its
// lane's batches whose completion event has fired, copying
// results to their requests and returning the memory; (2) forms new batches
// from the queue: the oldest queued request selects the program, queued
// requests of that program (same gradient flag) join it up to max_batch, the
// batch shrinks until its buffers fit in the free part of the arena, and it is
// launched on a free stream (H2D, forward, adjoint, D2H, event).  A partially
// filled batch waits up to max_wait_us for more requests while other batches
// of its lane are in flight.  Batches of different programs overlap on the
// device.
//
// Size-class lanes keep small circuits fast while large ones saturate the
// GPU: requests of states with at most lane_qubits qubits form the small
// lane, the rest the large lane.  Each lane has its own streams (the small
// lane's at the device's highest stream priority, so their CTAs are scheduled
// ahead of the large lane's as SMs free up), its own share of the memory
// budget (the small lane's region is reserved, large batches cannot take it)
// and forms batches from its own queue in arrival order.  A large circuit
// therefore never holds a stream or memory a small one is waiting for, and
// the small lane's worker never waits while the large lane's launches a
// batch.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "tedq_gb300.h"

int32_t tedq_record_error(int32_t status, const char* msg);

namespace {

using Clock = std::chrono::steady_clock;

double us_between(Clock::time_point a, Clock::time_point b) {
  return std::chrono::duration<double, std::micro>(b - a).count();
}

int64_t align256(int64_t v) { return (v + 255) & ~int64_t(255); }

// First-fit allocator over [0, size) with coalescing free list.
class Arena {
 public:
  void reset(int64_t size) {
    free_.clear();
    if (size > 0) free_[0] = size;
  }
  // moves the whole (still free) range to start at `base`
  void shift(int64_t base) {
    std::map<int64_t, int64_t> moved;
    for (auto& kv : free_) moved[kv.first + base] = kv.second;
    free_.swap(moved);
  }
  bool alloc(int64_t n, int64_t& off) {
    n = align256(n);
    for (auto it = free_.begin(); it != free_.end(); ++it) {
      if (it->second < n) continue;
      off = it->first;
      const int64_t rest = it->second - n;
      free_.erase(it);
      if (rest > 0) free_[off + n] = rest;
      return true;
    }
    return false;
  }
  void release(int64_t off, int64_t n) {
    n = align256(n);
    auto it = free_.emplace(off, n).first;
    auto nx = std::next(it);
    if (nx != free_.end() && it->first + it->second == nx->first) {
      it->second += nx->second;
      free_.erase(nx);
    }
    if (it != free_.begin()) {
      auto pv = std::prev(it);
      if (pv->first + pv->second == it->first) {
        pv->second += it->second;
        free_.erase(it);
      }
    }
  }

 private:
  std::map<int64_t, int64_t> free_;
};

enum ReqState { RQ_QUEUED = 0, RQ_LAUNCHED = 1, RQ_DONE = 2, RQ_CANCELLED = 3 };

struct ProgInfo {
  int32_t n_params = 0, n_real = 0, ns = 0, rbytes = 4, cbytes = 8;
};

struct Request {
  int64_t ticket = 0;
  tedq_program_t* prog = nullptr;
  ProgInfo info;
  int lane = 0;  // 0 small, 1 large
  bool grad = false;
  std::vector<char> params, dy, out, gout;
  int state = RQ_QUEUED;
  int32_t status = TEDQ_OK;
  int32_t batch = 0;
  Clock::time_point t_submit, t_launch, t_done;
};

struct Batch {
  std::vector<std::shared_ptr<Request>> reqs;
  tedq_program_t* prog = nullptr;
  ProgInfo info;
  bool grad = false;
  int lane = 0;
  int stream = -1;
  cudaEvent_t done = nullptr;
  int64_t dev_off = 0, dev_bytes = 0, host_off = 0, host_bytes = 0;
  int64_t h_out = 0, h_grad = 0;  // offsets of the results in the host slice
  int32_t status = TEDQ_OK;
};

}  // namespace

struct tedq_server {
  tedq_server_options_t opt{};
  char* dev_arena = nullptr;
  char* host_arena = nullptr;
  int64_t host_size = 0;
  // per lane: device arena over its region of the budget (offsets relative
  // to dev_arena), host staging arena
  Arena dA[2], hA[2];
  int lane_qubits = 16;  // states of at most this many qubits: small lane
  int n_lanes = 2;
  std::vector<cudaStream_t> streams;
  std::vector<int> stream_lane;
  std::vector<bool> stream_busy;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<std::shared_ptr<Request>> queue[2];
  std::unordered_map<int64_t, std::shared_ptr<Request>> all;
  std::vector<Batch> inflight;
  std::thread workers[2];
  bool stop = false;
  bool paused = false;
  int64_t next_ticket = 1;
  tedq_server_stats_t stats{};
  std::string worker_error;
};

namespace {

ProgInfo prog_info(tedq_program_t* p) {
  ProgInfo r;
  tedq_program_info_t i;
  if (tedq_program_info(p, &i) != TEDQ_OK) return r;
  r.n_params = i.n_params;
  r.n_real = i.n_real_outputs;
  r.ns = i.state_qubits;
  r.rbytes = i.precision == TEDQ_PREC_C128 ? 8 : 4;
  r.cbytes = 2 * r.rbytes;
  return r;
}

struct Layout {
  int64_t psi, lam, params, dy, out, grad, ws, wsb, dev_total;
  int64_t hp, hdy, hout, hgrad, host_total;
};

Layout layout(const ProgInfo& in, tedq_program_t* prog, int64_t B, bool grad) {
  Layout L{};
  const int64_t state = align256((B << in.ns) * in.cbytes);
  int64_t o = 0;
  L.psi = o, o += state;
  L.lam = o, o += grad ? state : 0;
  L.params = o, o += align256(B * in.n_params * in.rbytes);
  L.dy = o, o += align256(B * in.n_real * in.rbytes);
  L.out = o, o += align256(B * in.n_real * in.rbytes);
  L.grad = o, o += grad ? align256(B * in.n_params * in.rbytes) : 0;
  L.wsb = tedq_program_workspace_bytes(prog, B);
  L.ws = o, o += align256(L.wsb);
  L.dev_total = o;
  int64_t h = 0;
  L.hp = h, h += align256(B * in.n_params * in.rbytes);
  L.hdy = h, h += align256(B * in.n_real * in.rbytes);
  L.hout = h, h += align256(B * in.n_real * in.rbytes);
  L.hgrad = h, h += align256(B * in.n_params * in.rbytes);
  L.host_total = h;
  return L;
}

void CUDART_CB on_batch_done(void* user) {
  auto* S = static_cast<tedq_server*>(user);
  S->cv_work.notify_all();
}

// Packs the batch's inputs, launches its work on its stream and records the
// completion event (also after a failure, so the batch always retires).
int32_t launch(tedq_server* S, Batch& b) {
  const ProgInfo& in = b.info;
  const int64_t B = (int64_t)b.reqs.size();
  const Layout L = layout(in, b.prog, B, b.grad);
  cudaStream_t s = S->streams[b.stream];
  char* d = S->dev_arena + b.dev_off;
  char* h = S->host_arena + b.host_off;
  const size_t pbytes = (size_t)in.n_params * in.rbytes, rbytes = (size_t)in.n_real * in.rbytes;
  for (int64_t i = 0; i < B; ++i) {
    const Request& r = *b.reqs[i];
    if (pbytes) std::memcpy(h + L.hp + i * pbytes, r.params.data(), pbytes);
    if (b.grad && rbytes) {
      if (!r.dy.empty()) {
        std::memcpy(h + L.hdy + i * rbytes, r.dy.data(), rbytes);
      } else {
        for (int k = 0; k < in.n_real; ++k) {
          if (in.rbytes == 8) reinterpret_cast<double*>(h + L.hdy + i * rbytes)[k] = 1.0;
          else reinterpret_cast<float*>(h + L.hdy + i * rbytes)[k] = 1.0f;
        }
      }
    }
  }
  int32_t st = TEDQ_OK;
  cudaError_t e = cudaSuccess;
  if (pbytes) e = cudaMemcpyAsync(d + L.params, h + L.hp, B * pbytes, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess && b.grad && rbytes) e = cudaMemcpyAsync(d + L.dy, h + L.hdy, B * rbytes, cudaMemcpyHostToDevice, s);
  if (e != cudaSuccess) st = TEDQ_ERR_CUDA;
  if (st == TEDQ_OK)
    st = tedq_run(b.prog, d + L.params, B, d + L.psi, rbytes ? d + L.out : nullptr, nullptr, d + L.ws, (size_t)L.wsb, s);
  if (st == TEDQ_OK && b.grad && pbytes)
    st = tedq_run_adjoint(b.prog, d + L.params, B, rbytes ? d + L.dy : nullptr, nullptr, d + L.psi, d + L.lam,
                          d + L.grad, d + L.ws, (size_t)L.wsb, s);
  if (st == TEDQ_OK && rbytes) e = cudaMemcpyAsync(h + L.hout, d + L.out, B * rbytes, cudaMemcpyDeviceToHost, s);
  if (st == TEDQ_OK && e == cudaSuccess && b.grad && pbytes)
    e = cudaMemcpyAsync(h + L.hgrad, d + L.grad, B * pbytes, cudaMemcpyDeviceToHost, s);
  if (e != cudaSuccess && st == TEDQ_OK) st = TEDQ_ERR_CUDA;
  cudaLaunchHostFunc(s, on_batch_done, S);
  cudaEventRecord(b.done, s);
  b.h_out = L.hout;
  b.h_grad = L.hgrad;
  return st;
}

// Forms the next batch from the queue (lock held).  Returns false when nothing
// should launch now.
bool form_batch(tedq_server* S, Batch& b, Clock::time_point now, int lane) {
  auto& q = S->queue[lane];
  while (!q.empty() && q.front()->state != RQ_QUEUED) q.pop_front();
  if (q.empty()) return false;
  const std::shared_ptr<Request> r0 = q.front();
  std::vector<std::shared_ptr<Request>> cand;
  for (auto& r : q) {
    if (r->state != RQ_QUEUED || r->prog != r0->prog || r->grad != r0->grad) continue;
    cand.push_back(r);
    if ((int)cand.size() == S->opt.max_batch) break;
  }
  bool lane_busy = false;
  for (const Batch& f : S->inflight) lane_busy |= f.lane == lane;
  if ((int)cand.size() < S->opt.max_batch && lane_busy &&
      us_between(r0->t_submit, now) < (double)S->opt.max_wait_us)
    return false;
  int64_t B = (int64_t)cand.size();
  int64_t doff = 0, hoff = 0;
  Layout L{};
  for (; B > 0; B /= 2) {
    L = layout(r0->info, r0->prog, B, r0->grad);
    if (!S->dA[lane].alloc(L.dev_total, doff)) continue;
    if (!S->hA[lane].alloc(L.host_total, hoff)) {
      S->dA[lane].release(doff, L.dev_total);
      continue;
    }
    break;
  }
  if (B == 0) {
    if (!lane_busy) {  // can never fit: fail the request
      r0->state = RQ_DONE;
      r0->status = TEDQ_ERR_OOM;
      r0->t_done = now;
      S->stats.failed++;
      S->cv_done.notify_all();
    }
    return false;
  }
  b.reqs.assign(cand.begin(), cand.begin() + B);
  b.prog = r0->prog;
  b.info = r0->info;
  b.grad = r0->grad;
  b.lane = lane;
  b.dev_off = doff;
  b.dev_bytes = L.dev_total;
  b.host_off = hoff;
  b.host_bytes = L.host_total;
  for (auto& r : b.reqs) {
    r->state = RQ_LAUNCHED;
    r->t_launch = now;
    r->batch = (int32_t)B;
  }
  std::deque<std::shared_ptr<Request>> rest;
  for (auto& r : q)
    if (r->state == RQ_QUEUED) rest.push_back(r);
  q.swap(rest);
  S->stats.in_flight_bytes += L.dev_total;
  S->stats.peak_in_flight_bytes = std::max(S->stats.peak_in_flight_bytes, S->stats.in_flight_bytes);
  S->stats.batches++;
  return true;
}

// Retires finished batches (lock held); returns true if any finished.
bool retire(tedq_server* S, int lane) {
  bool any = false;
  for (size_t i = 0; i < S->inflight.size();) {
    Batch& b = S->inflight[i];
    if (b.lane != lane) {
      ++i;
      continue;
    }
    const cudaError_t q = cudaEventQuery(b.done);
    if (q == cudaErrorNotReady) {
      ++i;
      continue;
    }
    const int32_t st = q == cudaSuccess ? b.status : TEDQ_ERR_CUDA;
    const Clock::time_point now = Clock::now();
    const size_t pbytes = (size_t)b.info.n_params * b.info.rbytes, rbytes = (size_t)b.info.n_real * b.info.rbytes;
    const char* h = S->host_arena + b.host_off;
    for (size_t k = 0; k < b.reqs.size(); ++k) {
      Request& r = *b.reqs[k];
      r.status = st;
      if (st == TEDQ_OK) {
        r.out.assign(h + b.h_out + k * rbytes, h + b.h_out + (k + 1) * rbytes);
        if (b.grad) r.gout.assign(h + b.h_grad + k * pbytes, h + b.h_grad + (k + 1) * pbytes);
      }
      r.state = RQ_DONE;
      r.t_done = now;
      if (st == TEDQ_OK) S->stats.completed++;
      else S->stats.failed++;
    }
    cudaEventDestroy(b.done);
    S->dA[b.lane].release(b.dev_off, b.dev_bytes);
    S->hA[b.lane].release(b.host_off, b.host_bytes);
    S->stats.in_flight_bytes -= b.dev_bytes;
    S->stream_busy[b.stream] = false;
    S->inflight.erase(S->inflight.begin() + i);
    any = true;
  }
  return any;
}

void fail_queued(tedq_server* S, int32_t status) {
  for (auto& q : S->queue) {
    for (auto& r : q)
      if (r->state == RQ_QUEUED) {
        r->state = RQ_DONE;
        r->status = status;
        r->t_done = Clock::now();
        S->stats.failed++;
      }
    q.clear();
  }
  S->cv_done.notify_all();
}

// The worker of one lane: retires the lane's finished batches and launches
// new ones on the lane's free streams (the lock is released while a batch is
// packed and launched).
void worker_main(tedq_server* S, int lane) {
  cudaSetDevice(S->opt.device);
  std::unique_lock<std::mutex> lk(S->mu);
  for (;;) {
    bool mine = false;
    for (const Batch& f : S->inflight) mine |= f.lane == lane;
    if (S->stop) {
      fail_queued(S, TEDQ_ERR_STATE);
      if (!mine) break;
    }
    bool progress = retire(S, lane);
    if (progress) S->cv_done.notify_all();
    if (!S->paused && !S->stop) {
      for (size_t si = 0; si < S->streams.size(); ++si) {
        if (S->stream_busy[si] || S->stream_lane[si] != lane) continue;
        Batch b;
        b.stream = (int)si;
        b.done = nullptr;
        if (!form_batch(S, b, Clock::now(), S->stream_lane[si])) continue;
        S->stream_busy[si] = true;
        cudaEventCreateWithFlags(&b.done, cudaEventDisableTiming);
        lk.unlock();
        b.status = launch(S, b);
        lk.lock();
        S->inflight.push_back(b);
        progress = true;
      }
    }
    if (!progress) S->cv_work.wait_for(lk, std::chrono::microseconds(mine ? 50 : 2000));
  }
}

}  // namespace

// ---------------------------------------------------------------- public API

extern "C" {

int32_t tedq_server_create(const tedq_server_options_t* opts, tedq_server_t** out) {
  if (!out) return tedq_record_error(TEDQ_ERR_ARG, "tedq_server_create: out is null");
  *out = nullptr;
  std::unique_ptr<tedq_server> S(new tedq_server());
  if (opts) S->opt = *opts;
  if (S->opt.n_streams <= 0) S->opt.n_streams = 4;
  if (S->opt.max_batch <= 0) S->opt.max_batch = 256;
  if (S->opt.max_wait_us < 0) S->opt.max_wait_us = 0;
  if (opts == nullptr) S->opt.max_wait_us = 200;
  if (S->opt.memory_budget_bytes <= 0) S->opt.memory_budget_bytes = int64_t(1) << 30;
  S->paused = S->opt.paused != 0;
  int prev = 0;
  cudaGetDevice(&prev);
  cudaError_t e = cudaSetDevice(S->opt.device);
  if (e != cudaSuccess)
    return tedq_record_error(TEDQ_ERR_CUDA, (std::string("tedq_server_create: ") + cudaGetErrorString(e)).c_str());
  e = cudaMalloc(&S->dev_arena, (size_t)S->opt.memory_budget_bytes);
  if (e != cudaSuccess) {
    cudaGetLastError();
    cudaSetDevice(prev);
    return tedq_record_error(TEDQ_ERR_OOM, "tedq_server_create: device memory budget cannot be allocated");
  }
  S->host_size = std::min<int64_t>(int64_t(256) << 20, std::max<int64_t>(int64_t(64) << 20, S->opt.memory_budget_bytes / 8));
  e = cudaMallocHost(&S->host_arena, (size_t)S->host_size);
  if (e != cudaSuccess) {
    cudaFree(S->dev_arena);
    cudaSetDevice(prev);
    return tedq_record_error(TEDQ_ERR_OOM, "tedq_server_create: pinned host staging cannot be allocated");
  }
  // lanes: lane_qubits < 0 or a single stream puts every request in one lane
  S->lane_qubits = S->opt.lane_qubits == 0 ? 16 : S->opt.lane_qubits;
  S->n_lanes = (S->lane_qubits < 0 || S->opt.n_streams < 2) ? 1 : 2;
  if (S->n_lanes == 1) {
    S->dA[1].reset(S->opt.memory_budget_bytes);  // everything in the large lane
    S->hA[1].reset(S->host_size);
  } else {
    // the small lane's reserve: 1/8 of the budget, at most 8 GiB (a batch of
    // 256 value+grad requests of 16 qubits needs 256 MiB of states)
    const int64_t small = std::min<int64_t>(int64_t(8) << 30, align256(S->opt.memory_budget_bytes / 8));
    S->dA[0].reset(small);
    S->dA[1].reset(S->opt.memory_budget_bytes - small);
    S->dA[1].shift(small);
    const int64_t hsmall = align256(S->host_size / 4);
    S->hA[0].reset(hsmall);
    S->hA[1].reset(S->host_size - hsmall);
    S->hA[1].shift(hsmall);
  }
  int prio_low = 0, prio_high = 0;
  cudaDeviceGetStreamPriorityRange(&prio_low, &prio_high);
  const int n_small = S->n_lanes == 1 ? 0 : std::max(1, S->opt.n_streams / 2);
  for (int i = 0; i < S->opt.n_streams; ++i) {
    const int lane = i < n_small ? 0 : 1;
    cudaStream_t st;
    cudaStreamCreateWithPriority(&st, cudaStreamNonBlocking, lane == 0 ? prio_high : prio_low);
    S->streams.push_back(st);
    S->stream_lane.push_back(lane);
    S->stream_busy.push_back(false);
  }
  cudaSetDevice(prev);
  tedq_server* raw = S.release();
  for (int l = 2 - raw->n_lanes; l < 2; ++l) raw->workers[l] = std::thread(worker_main, raw, l);
  *out = raw;
  return TEDQ_OK;
}

int32_t tedq_server_destroy(tedq_server_t* S) {
  if (!S) return TEDQ_OK;
  {
    std::lock_guard<std::mutex> lk(S->mu);
    S->stop = true;
  }
  S->cv_work.notify_all();
  for (auto& w : S->workers)
    if (w.joinable()) w.join();
  int prev = 0;
  cudaGetDevice(&prev);
  cudaSetDevice(S->opt.device);
  for (auto st : S->streams) cudaStreamDestroy(st);
  cudaFree(S->dev_arena);
  cudaFreeHost(S->host_arena);
  cudaSetDevice(prev);
  delete S;
  return TEDQ_OK;
}

int32_t tedq_server_submit(tedq_server_t* S, tedq_program_t* prog, const void* params, const void* dy,
                           int32_t with_grad, int64_t* ticket) {
  if (!S || !prog || !ticket) return tedq_record_error(TEDQ_ERR_ARG, "tedq_server_submit: null argument");
  auto r = std::make_shared<Request>();
  r->prog = prog;
  r->info = prog_info(prog);
  if (r->info.ns == 0) return tedq_record_error(TEDQ_ERR_ARG, "tedq_server_submit: invalid program");
  if (r->info.n_params > 0 && !params) return tedq_record_error(TEDQ_ERR_ARG, "tedq_server_submit: params is null");
  r->grad = with_grad != 0;
  r->lane = (S->n_lanes == 2 && r->info.ns <= S->lane_qubits) ? 0 : 1;
  const size_t pbytes = (size_t)r->info.n_params * r->info.rbytes, rbytes = (size_t)r->info.n_real * r->info.rbytes;
  if (pbytes) r->params.assign((const char*)params, (const char*)params + pbytes);
  if (dy && rbytes) r->dy.assign((const char*)dy, (const char*)dy + rbytes);
  r->t_submit = Clock::now();
  {
    std::lock_guard<std::mutex> lk(S->mu);
    if (S->stop) return tedq_record_error(TEDQ_ERR_STATE, "tedq_server_submit: server is stopping");
    r->ticket = S->next_ticket++;
    S->all[r->ticket] = r;
    S->queue[r->lane].push_back(r);
    S->stats.submitted++;
    *ticket = r->ticket;
  }
  S->cv_work.notify_all();
  return TEDQ_OK;
}

int32_t tedq_server_wait(tedq_server_t* S, int64_t ticket, int64_t timeout_us, void* out_real, void* grad,
                         tedq_request_result_t* result) {
  if (!S) return tedq_record_error(TEDQ_ERR_ARG, "tedq_server_wait: server is null");
  std::unique_lock<std::mutex> lk(S->mu);
  auto it = S->all.find(ticket);
  if (it == S->all.end()) return tedq_record_error(TEDQ_ERR_ARG, "tedq_server_wait: unknown ticket");
  std::shared_ptr<Request> r = it->second;
  auto ready = [&] { return r->state == RQ_DONE || r->state == RQ_CANCELLED; };
  if (timeout_us < 0) {
    S->cv_done.wait(lk, ready);
  } else if (!S->cv_done.wait_for(lk, std::chrono::microseconds(timeout_us), ready)) {
    return tedq_record_error(TEDQ_ERR_TIMEOUT, "tedq_server_wait: request not finished within the timeout");
  }
  S->all.erase(it);
  if (result) {
    result->status = r->state == RQ_CANCELLED ? TEDQ_ERR_STATE : r->status;
    result->batch_size = r->batch;
    result->queue_us = r->batch ? us_between(r->t_submit, r->t_launch) : 0.0;
    result->total_us = us_between(r->t_submit, r->t_done);
  }
  if (r->state == RQ_CANCELLED) return tedq_record_error(TEDQ_ERR_STATE, "tedq_server_wait: request was cancelled");
  if (r->status != TEDQ_OK) return tedq_record_error(r->status, "tedq_server_wait: request failed");
  if (out_real && !r->out.empty()) std::memcpy(out_real, r->out.data(), r->out.size());
  if (grad && !r->gout.empty()) std::memcpy(grad, r->gout.data(), r->gout.size());
  return TEDQ_OK;
}

int32_t tedq_server_cancel(tedq_server_t* S, int64_t ticket) {
  if (!S) return tedq_record_error(TEDQ_ERR_ARG, "tedq_server_cancel: server is null");
  std::lock_guard<std::mutex> lk(S->mu);
  auto it = S->all.find(ticket);
  if (it == S->all.end()) return tedq_record_error(TEDQ_ERR_ARG, "tedq_server_cancel: unknown ticket");
  Request& r = *it->second;
  if (r.state != RQ_QUEUED) return tedq_record_error(TEDQ_ERR_STATE, "tedq_server_cancel: request already launched");
  r.state = RQ_CANCELLED;
  r.t_done = Clock::now();
  S->stats.cancelled++;
  S->cv_done.notify_all();
  return TEDQ_OK;
}

int32_t tedq_server_stats(tedq_server_t* S, tedq_server_stats_t* out) {
  if (!S || !out) return tedq_record_error(TEDQ_ERR_ARG, "tedq_server_stats: null argument");
  std::lock_guard<std::mutex> lk(S->mu);
  *out = S->stats;
  return TEDQ_OK;
}

int32_t tedq_server_resume(tedq_server_t* S) {
  if (!S) return tedq_record_error(TEDQ_ERR_ARG, "tedq_server_resume: server is null");
  {
    std::lock_guard<std::mutex> lk(S->mu);
    S->paused = false;
  }
  S->cv_work.notify_all();
  return TEDQ_OK;
}

}  // extern "C"
