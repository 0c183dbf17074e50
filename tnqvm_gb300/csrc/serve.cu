// Continuous-batching request loop of the GB300 MPS engine.
//
// A worker thread owns several lanes (stream + scratch).  Requests (programs
// with recorded gates, an optional observable and a shot count) queue up in
// arrival order; whenever a lane is free the worker admits as many queued
// requests as the in-flight request cap and the HBM footprint budget allow,
// launches them as one persistent batch on that lane, enqueues the batch's
// expectation and sampling work behind it, and records an event.  Batches on
// different lanes overlap on the device, so requests that arrive while others
// run start as soon as a lane is free instead of waiting for the running
// batch to drain.  Completed requests are finished out of order.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cstring>

#include "../../include/gb300mps.h"
#include "engine_internal.hpp"

namespace gbmps {

// Lanes whose batches overlap on the device.  One circuit runs per CTA, so
// a batch fills the GPU only with ~150 circuits; more lanes let the small
// batches that steady arrivals produce run side by side instead of queueing.
constexpr int kServeLanes = 16;
// Workers of the wide lane: a wide split's cooperative launches use at most
// one CTA per eight rows, so two requests of caps up to 512 run side by side.
constexpr int kWideLanes = 2;
// Per-lane host-mapped arena for fused requests: 16 B of flags plus
// 2 (n_terms + 1) doubles each (848 B for a 50-term Hamiltonian).
constexpr size_t kArenaBytes = 2u << 20;

static double now_ms() {
  return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

static int grow_pinned(void** p, size_t* cap, size_t need) {
  if (*cap >= need) return MPS_OK;
  if (*p) cudaFreeHost(*p);
  *p = nullptr;
  *cap = 0;
  const size_t n = need + need / 2 + 256;
  if (cudaMallocHost(p, n) != cudaSuccess) {
    cudaGetLastError();
    return fail(MPS_ERR_OOM, "pinned host allocation failed");
  }
  *cap = n;
  return MPS_OK;
}

static int status_of(int herr) {
  return (herr & ERR_NAN)       ? fail(MPS_ERR_NUMERIC, "non-finite value in a two-site split")
         : (herr & ERR_DIMS)    ? fail(MPS_ERR_UNSUPPORTED, "bond dimension beyond the kernel limit")
         : (herr & ERR_TIMEOUT) ? fail(MPS_ERR_TIMEOUT, "a site-parallel update waited past its bound")
                                : MPS_OK;
}

// Completion bookkeeping of one request (S->mu held).
static void complete(ServeState* S, ServeReq* r, double t) {
  r->t_done = t;
  r->done = true;
  S->inflight_bytes -= r->prog->bytes;
  S->inflight_reqs -= 1;
}

// A fused request whose flag is up (S->mu held): energy from the mapped
// observables, status from the error word the kernel copied next to the flag.
static void complete_fused(ServeState* S, ServeReq* r, double t) {
  r->status = status_of(((volatile int*)r->flag)[1]);
  r->energy = observable_value(r->prog, r->obs);
  complete(S, r, t);
}

// Requests of a running batch whose own CTA has finished (flag in mapped
// host memory) complete now, before the rest of the batch.
static void reap_fused(ServeState* S, ServeBatch& B) {
  bool any = false;
  for (ServeReq* r : B.reqs)
    if (r->fused && !r->done && *(volatile int*)r->flag == 1) {
      if (!any) std::atomic_thread_fence(std::memory_order_acquire);
      if (!any) S->mu.lock();
      any = true;
      complete_fused(S, r, now_ms());
    }
  if (any) {
    S->mu.unlock();
    S->cv_done.notify_all();
  }
}

static void finish_batch(ServeState* S, ServeBatch& B) {
  const double t = now_ms();
  std::atomic_thread_fence(std::memory_order_acquire);
  std::lock_guard<std::mutex> lk(S->mu);
  size_t ri = 0;
  for (ServeReq* r : B.reqs) {
    mps_prog* p = r->prog;
    const int herr = B.h_err[ri++];
    if (r->fused) {
      if (!r->done) complete_fused(S, r, t);
      continue;
    }
    r->status = status_of(herr);
    if (p->d_obs) r->energy = observable_value(p, B.h_exp + 2 * r->exp_off);
  }
  for (auto& bd : B.bit_dst) {
    ServeReq* r = bd.first;
    select_measured(r->prog, bd.second, r->shots, r->bits.data());
  }
  for (ServeReq* r : B.reqs) {
    if (!r->fused) complete(S, r, t);
    r->in_batch = false;
    if (r->reaped) delete r;
  }
  B.reqs.clear();
  B.bit_dst.clear();
  S->cv_done.notify_all();
}

static int launch_batch(mps_ctx* c, ServeState* S, int li, std::vector<ServeReq*>& reqs) {
  Lane& L = S->lanes[li];
  ServeBatch& B = S->batches[li];
  B.reqs = reqs;
  B.footprint = 0;
  std::vector<mps_prog*> progs;
  progs.reserve(reqs.size());
  // requests with an observable and no shots complete on their own: the
  // update kernel evaluates the observable on the program's CTA and raises a
  // flag in the lane's mapped arena
  size_t aoff = 0;
  for (ServeReq* r : reqs) {
    mps_prog* p = r->prog;
    progs.push_back(p);
    B.footprint += p->bytes;
    r->in_batch = true;
    r->fused = false;
    if (r->shots == 0 && p->d_obs && !prog_is_wide(p)) {
      const size_t need = 16 + 16 * ((size_t)p->n_terms + 1);
      if (aoff + need <= B.arena_cap) {
        r->fused = true;
        r->flag = reinterpret_cast<int*>(B.arena + aoff);
        r->obs = reinterpret_cast<double*>(B.arena + aoff + 16);
        ((volatile int*)r->flag)[0] = 0;
        ((volatile int*)r->flag)[1] = 0;
        p->serve_flag = r->flag;
        p->serve_obs = r->obs;
        aoff += need;
      }
    }
  }
  int rc = launch_programs(c, L, progs.data(), (int)progs.size(), false);
  for (mps_prog* p : progs) {
    p->serve_flag = nullptr;
    p->serve_obs = nullptr;
  }
  if (rc) return rc;
  // observables of the requests that do not complete on their own CTA: one
  // expectation launch per precision (a batch may mix complex64 and
  // complex128 programs), results packed complex128 tasks first
  std::vector<ExpTask> tasks[2];
  for (ServeReq* r : reqs)
    if (!r->fused && r->prog->d_obs) {
      r->exp_off = tasks[r->prog->prec].size();
      observable_tasks(r->prog, tasks[r->prog->prec]);
    }
  const size_t n_tasks = tasks[0].size() + tasks[1].size();
  if (n_tasks > 0) {
    rc = grow_pinned((void**)&B.h_exp, &B.h_exp_cap, 2 * n_tasks * sizeof(double));
    if (rc) return rc;
    for (int pr = 0; pr < 2; ++pr) {
      if (tasks[pr].empty()) continue;
      rc = enqueue_expect(L, tasks[pr], pr, B.h_exp + (pr == 1 ? 2 * tasks[0].size() : 0));
      if (rc) return rc;
    }
    for (ServeReq* r : reqs)
      if (!r->fused && r->prog->d_obs && r->prog->prec == 1) r->exp_off += tasks[0].size();
  }
  size_t bit_total = 0;
  for (ServeReq* r : reqs) bit_total += (size_t)r->shots * r->prog->n;
  if (bit_total) {
    rc = grow_pinned((void**)&B.h_bits, &B.h_bits_cap, bit_total);
    if (rc) return rc;
    size_t off = 0;
    for (ServeReq* r : reqs) {
      if (r->shots <= 0) continue;
      rc = enqueue_sample(L, r->prog, r->shots, r->seed, B.h_bits + off);
      if (rc) return rc;
      B.bit_dst.push_back({r, B.h_bits + off});
      off += (size_t)r->shots * r->prog->n;
    }
  }
  // error words of the batch's programs, read by finish_batch without a sync
  rc = grow_pinned((void**)&B.h_err, &B.h_err_cap, std::max<size_t>(reqs.size(), 1024) * sizeof(int));
  if (rc) return rc;
  for (size_t i = 0; i < reqs.size(); ++i) {
    cudaError_t e = cudaMemcpyAsync(B.h_err + i, reqs[i]->prog->d_err, sizeof(int), cudaMemcpyDeviceToHost, L.stream);
    if (e != cudaSuccess) return fail(MPS_ERR_CUDA, cudaGetErrorString(e));
  }
  cudaError_t e = cudaEventRecord(B.ev, L.stream);
  if (e != cudaSuccess) return fail(MPS_ERR_CUDA, cudaGetErrorString(e));
  return MPS_OK;
}

static void serve_loop(mps_ctx* c) {
  cudaSetDevice(c->device);
  ServeState* S = c->serve;
  for (;;) {
    bool any_busy = false;
    for (int l = 0; l < kServeLanes; ++l) {
      if (!S->lane_busy[l]) continue;
      const cudaError_t e = cudaEventQuery(S->batches[l].ev);
      if (e == cudaErrorNotReady) {
        reap_fused(S, S->batches[l]);
        any_busy = true;
        continue;
      }
      finish_batch(S, S->batches[l]);
      S->lane_busy[l] = 0;
    }
    int free_lane = -1;
    for (int l = 0; l < kServeLanes; ++l)
      if (!S->lane_busy[l]) {
        free_lane = l;
        break;
      }
    std::vector<ServeReq*> take;
    {
      std::unique_lock<std::mutex> lk(S->mu);
      if (S->stop && S->queue.empty() && !any_busy) break;
      if (free_lane >= 0 && !S->queue.empty()) {
        // the fused kernel runs each program in its own precision, so a
        // batch takes every queued request in arrival order
        size_t bytes = S->inflight_bytes;
        while (!S->queue.empty()) {
          ServeReq* r = S->queue.front();
          if (S->inflight_reqs + (int)take.size() >= S->max_inflight) break;
          if (!take.empty() && bytes + r->prog->bytes > c->budget) break;
          bytes += r->prog->bytes;
          take.push_back(r);
          S->queue.pop_front();
        }
        S->inflight_bytes = bytes;
        S->inflight_reqs += (int)take.size();
      } else if (!any_busy && S->queue.empty()) {
        S->cv_work.wait_for(lk, std::chrono::milliseconds(5));
        continue;
      }
    }
    if (!take.empty()) {
      const int rc = launch_batch(c, S, free_lane, take);
      if (rc) {
        std::lock_guard<std::mutex> lk(S->mu);
        for (ServeReq* r : take) {
          r->status = rc;
          r->fused = false;
          complete(S, r, now_ms());
          r->in_batch = false;
          if (r->reaped) delete r;
        }
        S->batches[free_lane].reqs.clear();
        S->cv_done.notify_all();
      } else {
        S->lane_busy[free_lane] = 1;
      }
      continue;
    }
    std::this_thread::sleep_for(std::chrono::microseconds(50));
  }
}

// Wide requests: each wide worker takes one at a time (host-driven splits on
// its own lane and workspace), admitted under the same HBM footprint budget
// as the batches.
static void serve_wide_loop(mps_ctx* c, int w) {
  cudaSetDevice(c->device);
  ServeState* S = c->serve;
  Lane& lane = S->wide_lanes[w];
  void** ws = &S->wide_ws[w];
  for (;;) {
    ServeReq* r = nullptr;
    {
      std::unique_lock<std::mutex> lk(S->mu);
      S->cv_wide.wait_for(lk, std::chrono::milliseconds(5), [&] { return S->stop || !S->wide_queue.empty(); });
      if (S->wide_queue.empty()) {
        if (S->stop) break;
        continue;
      }
      ServeReq* head = S->wide_queue.front();
      if (S->inflight_reqs > 0 && S->inflight_bytes + head->prog->bytes > c->budget) continue;
      r = head;
      S->wide_queue.pop_front();
      S->inflight_bytes += r->prog->bytes;
      S->inflight_reqs += 1;
    }
    mps_prog* p = r->prog;
    int rc = wide_run(c, lane, p, ws);
    double energy = 0.0;
    std::vector<uint8_t> all;
    if (!rc && p->d_obs) {
      std::vector<double> res(2 * ((size_t)p->n_terms + 1));
      rc = wide_expect(p, p->obs_codes.data(), p->n_terms + 1, res.data(), &lane, ws);
      if (!rc) energy = observable_value(p, res.data());
    }
    if (!rc && r->shots > 0) {
      all.resize((size_t)r->shots * p->n);
      rc = wide_sample(p, r->shots, r->seed, all.data(), &lane, ws);
    }
    if (!rc) rc = prog_check_err(p);
    {
      std::lock_guard<std::mutex> lk(S->mu);
      r->status = rc;
      r->energy = energy;
      if (!rc && r->shots > 0) select_measured(p, all.data(), r->shots, r->bits.data());
      r->t_done = now_ms();
      r->done = true;
      S->inflight_bytes -= p->bytes;
      S->inflight_reqs -= 1;
      S->cv_done.notify_all();
    }
  }
}

}  // namespace gbmps

using namespace gbmps;

extern "C" {

int mps_serve_start(mps_ctx* c, int max_inflight) {
  if (!c) return fail(MPS_ERR_ARG, "ctx is NULL");
  if (c->serve) return MPS_OK;
  cudaError_t e = cudaSetDevice(c->device);
  if (e != cudaSuccess) return fail(MPS_ERR_CUDA, cudaGetErrorString(e));
  ServeState* S = new ServeState();
  S->max_inflight = max_inflight > 0 ? max_inflight : 256;
  S->lanes.resize(kServeLanes);
  S->batches.resize(kServeLanes);
  S->lane_busy.assign(kServeLanes, 0);
  for (int l = 0; l < kServeLanes; ++l) {
    // batch lanes at the highest stream priority: their CTAs go first when
    // SMs free up between the wide lane's cooperative launches
    int rc = lane_init(S->lanes[l], 1);
    if (rc) return rc;
    e = cudaEventCreateWithFlags(&S->batches[l].ev, cudaEventDisableTiming);
    if (e != cudaSuccess) return fail(MPS_ERR_CUDA, cudaGetErrorString(e));
    S->batches[l].lane = l;
    e = cudaHostAlloc((void**)&S->batches[l].arena, kArenaBytes, cudaHostAllocMapped);
    if (e != cudaSuccess) return fail(MPS_ERR_OOM, cudaGetErrorString(e));
    S->batches[l].arena_cap = kArenaBytes;
  }
  S->wide_lanes.resize(kWideLanes);
  S->wide_ws.assign(kWideLanes, nullptr);
  for (int w = 0; w < kWideLanes; ++w) {
    const int rc = lane_init(S->wide_lanes[w], -1);
    if (rc) return rc;
  }
  S->running = true;
  c->serve = S;
  S->worker = std::thread(serve_loop, c);
  for (int w = 0; w < kWideLanes; ++w) S->wide_workers.emplace_back(serve_wide_loop, c, w);
  return MPS_OK;
}

int mps_serve_submit(mps_ctx* c, mps_prog* p, int shots, uint64_t seed, uint64_t* ticket) {
  if (!c || !p || !ticket || shots < 0) return fail(MPS_ERR_ARG, "bad argument");
  if (!c->serve) return fail(MPS_ERR_STATE, "serve loop not started");
  if (p->ctx != c) return fail(MPS_ERR_ARG, "program from another context");
  if (p->density) return fail(MPS_ERR_UNSUPPORTED, "the serve loop runs state programs");
  ServeState* S = c->serve;
  ServeReq* r = new ServeReq();
  r->prog = p;
  r->shots = shots;
  r->seed = seed;
  r->t_submit = now_ms();
  r->t_done = 0.0;
  r->status = MPS_OK;
  r->energy = 0.0;
  r->done = false;
  int nm = p->measured.empty() ? p->n : (int)p->measured.size();
  r->bits.assign((size_t)shots * nm, 0);
  {
    std::lock_guard<std::mutex> lk(S->mu);
    if (S->stop) {
      delete r;
      return fail(MPS_ERR_STATE, "serve loop stopping");
    }
    r->ticket = S->next_ticket++;
    S->all[r->ticket] = r;
    if (prog_is_wide(p))
      S->wide_queue.push_back(r);
    else
      S->queue.push_back(r);
  }
  if (prog_is_wide(p)) S->cv_wide.notify_all();
  S->cv_work.notify_one();
  *ticket = r->ticket;
  return MPS_OK;
}

int mps_serve_poll(mps_ctx* c, uint64_t ticket, int timeout_ms, double* energy, uint8_t* bits, double* latency_ms) {
  if (!c) return fail(MPS_ERR_ARG, "ctx is NULL");
  if (!c->serve) return fail(MPS_ERR_STATE, "serve loop not started");
  ServeState* S = c->serve;
  std::unique_lock<std::mutex> lk(S->mu);
  auto it = S->all.find(ticket);
  if (it == S->all.end()) return fail(MPS_ERR_ARG, "unknown ticket");
  ServeReq* r = it->second;
  const auto pred = [&] { return r->done; };
  if (timeout_ms < 0)
    S->cv_done.wait(lk, pred);
  else if (!S->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), pred))
    return fail(MPS_ERR_TIMEOUT, "request not finished");
  const int status = r->status;
  if (energy) *energy = r->energy;
  if (bits && !r->bits.empty()) std::memcpy(bits, r->bits.data(), r->bits.size());
  if (latency_ms) *latency_ms = r->t_done - r->t_submit;
  S->all.erase(it);
  if (r->in_batch)
    r->reaped = true;  // the running batch still holds it; finish_batch frees it
  else
    delete r;
  return status;
}

int mps_serve_stop(mps_ctx* c) {
  if (!c || !c->serve) return MPS_OK;
  ServeState* S = c->serve;
  {
    std::lock_guard<std::mutex> lk(S->mu);
    S->stop = true;
  }
  S->cv_work.notify_all();
  S->cv_wide.notify_all();
  if (S->worker.joinable()) S->worker.join();
  for (std::thread& t : S->wide_workers)
    if (t.joinable()) t.join();
  cudaSetDevice(c->device);
  for (Lane& l : S->wide_lanes) lane_free(l);
  for (void*& w : S->wide_ws) wide_ws_free(&w);
  for (int l = 0; l < kServeLanes; ++l) {
    lane_free(S->lanes[l]);
    if (S->batches[l].ev) cudaEventDestroy(S->batches[l].ev);
    if (S->batches[l].h_exp) cudaFreeHost(S->batches[l].h_exp);
    if (S->batches[l].h_bits) cudaFreeHost(S->batches[l].h_bits);
    if (S->batches[l].h_err) cudaFreeHost(S->batches[l].h_err);
    if (S->batches[l].arena) cudaFreeHost(S->batches[l].arena);
  }
  for (auto& kv : S->all) delete kv.second;
  delete S;
  c->serve = nullptr;
  return MPS_OK;
}

}  // extern "C"
