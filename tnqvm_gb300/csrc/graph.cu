// Captured batches: one CUDA graph per batch of programs, replayed for every
// parameter update (the batched-VQE loop).  Body: reset every program to
// |0...0> on the device, one persistent launch of the fused op kernel over
// all programs (each CTA evaluates its program's attached observable right
// after the program's gates), and the copy of the raw expectation values to
// pinned host memory.
#include <algorithm>
#include <cstring>

#include "../../include/gb300mps.h"
#include "engine_internal.hpp"

struct mps_graph {
  mps_ctx* c = nullptr;
  gbmps::Lane L;
  std::vector<mps_prog*> progs;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  std::vector<gbmps::DevOp> flat;
  std::vector<size_t> first, count;
  std::vector<gbmps::ExpTask> tasks;
  std::vector<size_t> task_first;
  double* h_out = nullptr;
  cudaEvent_t ev[3] = {nullptr, nullptr, nullptr};
  // measured cost: each program's cycles in the last replay (copied to
  // pinned memory by the graph), and the descriptors by program, so that the
  // next replay takes the programs longest-measured first
  double* d_cycles = nullptr;
  double* h_cycles = nullptr;
  std::vector<gbmps::ProgDesc> desc_of;
  std::vector<int> order;
  // pinned staging of the op table for mps_graph_update (the host-to-device
  // copy runs at full bus speed and asynchronously); copied_ev marks the end
  // of the last copy out of it
  gbmps::DevOp* h_ops = nullptr;
  cudaEvent_t copied_ev = nullptr;
};

namespace gbmps {

static int build_ops(mps_graph* g, std::vector<DevOp>& flat, std::vector<size_t>& first, std::vector<size_t>& count) {
  flat.clear();
  first.assign(g->progs.size(), 0);
  count.assign(g->progs.size(), 0);
  std::vector<DevOp> ops;
  for (size_t i = 0; i < g->progs.size(); ++i) {
    mps_prog* p = g->progs[i];
    p->center = 0;  // every replay starts from |0...0>
    compile_program(p, ops);
    first[i] = flat.size();
    count[i] = ops.size();
    flat.insert(flat.end(), ops.begin(), ops.end());
  }
  return MPS_OK;
}

}  // namespace gbmps

using namespace gbmps;

#define GCK(call)                                                             \
  do {                                                                        \
    cudaError_t e_ = (call);                                                  \
    if (e_ != cudaSuccess) return fail(MPS_ERR_CUDA, cudaGetErrorString(e_)); \
  } while (0)

extern "C" {

int mps_graph_destroy(mps_graph* g) {
  if (!g) return MPS_OK;
  cudaSetDevice(g->c->device);
  if (g->L.stream) cudaStreamSynchronize(g->L.stream);
  if (g->exec) cudaGraphExecDestroy(g->exec);
  if (g->graph) cudaGraphDestroy(g->graph);
  if (g->h_out) cudaFreeHost(g->h_out);
  if (g->h_cycles) cudaFreeHost(g->h_cycles);
  if (g->h_ops) cudaFreeHost(g->h_ops);
  if (g->copied_ev) cudaEventDestroy(g->copied_ev);
  if (g->d_cycles) cudaFree(g->d_cycles);
  for (int i = 0; i < 3; ++i)
    if (g->ev[i]) cudaEventDestroy(g->ev[i]);
  lane_free(g->L);
  delete g;
  return MPS_OK;
}

int mps_graph_create(mps_ctx* c, mps_prog* const* progs, int n, mps_graph** out) {
  if (!c || !out || n <= 0 || !progs) return fail(MPS_ERR_ARG, "bad argument");
  *out = nullptr;
  for (int i = 0; i < n; ++i) {
    if (!progs[i] || progs[i]->ctx != c) return fail(MPS_ERR_ARG, "program from another context");
    if (prog_is_wide(progs[i]))
      return fail(MPS_ERR_UNSUPPORTED, "captured batches hold single-CTA programs (bond cap <= 64)");
    if (progs[i]->density) return fail(MPS_ERR_UNSUPPORTED, "captured batches hold state programs");
  }
  std::lock_guard<std::mutex> lk(c->mu);
  GCK(cudaSetDevice(c->device));
  mps_graph* g = new mps_graph();
  g->c = c;
  g->progs.assign(progs, progs + n);
  int rc = lane_init(g->L);
  if (rc) {
    delete g;
    return rc;
  }
  auto bail = [&](int code) {
    mps_graph_destroy(g);
    return code;
  };
  build_ops(g, g->flat, g->first, g->count);
  // descriptors for every program (empty ones too: they still get reset),
  // longest first
  std::vector<int> order(n);
  std::vector<double> cost(n, 0.0);
  for (int i = 0; i < n; ++i) {
    order[i] = i;
    cost[i] = program_cost(progs[i], g->flat.data() + g->first[i], g->count[i], progs[i]->d_obs != nullptr);
  }
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return cost[a] > cost[b]; });
  Lane& L = g->L;
  if (cudaMalloc(&L.d_ops, std::max<size_t>(g->flat.size(), 1) * sizeof(DevOp)) != cudaSuccess ||
      cudaMalloc(&L.d_desc, (size_t)n * sizeof(ProgDesc)) != cudaSuccess) {
    cudaGetLastError();
    return bail(fail(MPS_ERR_OOM, "graph op table allocation failed"));
  }
  L.d_ops_cap = std::max<size_t>(g->flat.size(), 1);
  L.d_desc_cap = n;
  g->task_first.assign(n, (size_t)-1);
  for (int i = 0; i < n; ++i)
    if (progs[i]->d_obs) {
      g->task_first[i] = g->tasks.size();
      observable_tasks(progs[i], g->tasks);
    }
  const int nt = (int)g->tasks.size();
  if (nt > 0 && (cudaMalloc(&L.d_exp_out, 2 * (size_t)nt * sizeof(double)) != cudaSuccess ||
                 cudaMallocHost(&g->h_out, 2 * (size_t)nt * sizeof(double)) != cudaSuccess)) {
    cudaGetLastError();
    return bail(fail(MPS_ERR_OOM, "graph expectation buffers failed"));
  }
  L.d_exp_out_cap = 2 * (size_t)nt;
  if (cudaMalloc(&g->d_cycles, (size_t)n * sizeof(double)) != cudaSuccess ||
      cudaMallocHost(&g->h_cycles, (size_t)n * sizeof(double)) != cudaSuccess) {
    cudaGetLastError();
    return bail(fail(MPS_ERR_OOM, "graph cost buffers failed"));
  }
  std::memset(g->h_cycles, 0, (size_t)n * sizeof(double));
  std::vector<ProgDesc> descs;
  g->desc_of.assign(n, ProgDesc());
  for (int i : order) {
    mps_prog* p = progs[i];
    ProgDesc d;
    std::memset(&d, 0, sizeof(d));
    d.sites = p->d_sites;
    d.site_off = p->d_off;
    d.bond = p->d_bond;
    d.ops = L.d_ops + g->first[i];
    d.n_ops = (int)g->count[i];
    d.n = p->n;
    d.chi_cap = p->chi_cap;
    d.mode = p->mode;
    d.flags = p->flags;
    d.prec = p->prec;
    d.cutoff = p->cutoff;
    d.stats = p->d_stats;
    d.err = p->d_err;
    if (p->d_obs) {  // observable evaluated by the program's CTA after its gates
      d.obs_codes = p->d_obs;
      d.n_obs = p->n_terms + 1;
      d.obs_out = L.d_exp_out + 2 * g->task_first[i];
    }
    d.cycles_out = g->d_cycles + i;
    g->desc_of[i] = d;
    descs.push_back(d);
  }
  g->order = order;
  if (!g->flat.empty())
    GCK(cudaMemcpy(L.d_ops, g->flat.data(), g->flat.size() * sizeof(DevOp), cudaMemcpyHostToDevice));
  GCK(cudaMemcpy(L.d_desc, descs.data(), descs.size() * sizeof(ProgDesc), cudaMemcpyHostToDevice));
  const int grid = std::min(n, c->num_sms);
  if (cudaMalloc(&L.op_scratch, op_scratch_bytes() * (size_t)grid) != cudaSuccess) {
    cudaGetLastError();
    return bail(fail(MPS_ERR_OOM, "graph scratch allocation failed"));
  }
  L.op_scratch_ctas = grid;
  cudaStream_t st = L.stream;
  for (int i = 0; i < 3; ++i)
    if (cudaEventCreate(&g->ev[i]) != cudaSuccess) return bail(fail(MPS_ERR_CUDA, "event creation failed"));
  GCK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
  cudaError_t e = cudaEventRecordWithFlags(g->ev[0], st, cudaEventRecordExternal);
  if (e == cudaSuccess) e = launch_reset(L.d_desc, n, st);
  if (e == cudaSuccess) e = cudaMemsetAsync(L.d_queue, 0, sizeof(int), st);
  if (e == cudaSuccess) e = launch_ops(L.d_desc, n, grid, n > 1 ? L.d_queue : nullptr, L.op_scratch, st);
  if (e == cudaSuccess) e = cudaEventRecordWithFlags(g->ev[1], st, cudaEventRecordExternal);
  if (e == cudaSuccess && nt > 0)
    e = cudaMemcpyAsync(g->h_out, L.d_exp_out, 2 * (size_t)nt * sizeof(double), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(g->h_cycles, g->d_cycles, (size_t)n * sizeof(double), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaEventRecordWithFlags(g->ev[2], st, cudaEventRecordExternal);
  cudaGraph_t graph = nullptr;
  const cudaError_t e2 = cudaStreamEndCapture(st, &graph);
  if (e != cudaSuccess || e2 != cudaSuccess) {
    if (graph) cudaGraphDestroy(graph);
    return bail(fail(MPS_ERR_CUDA, cudaGetErrorString(e != cudaSuccess ? e : e2)));
  }
  g->graph = graph;
  e = cudaGraphInstantiate(&g->exec, graph, 0);
  if (e != cudaSuccess) return bail(fail(MPS_ERR_CUDA, cudaGetErrorString(e)));
  *out = g;
  return MPS_OK;
}

// Programs compile independently, so an update compiles them on host
// threads, checks that each keeps its op structure (kind, site, orientation
// of every op: the captured launch depends on it) and writes its ops straight
// into the pinned staging buffer, from which one copy goes to the device.
int mps_graph_update(mps_graph* g) {
  if (!g) return fail(MPS_ERR_ARG, "NULL graph");
  GCK(cudaSetDevice(g->c->device));
  const size_t np = g->progs.size();
  const size_t total = g->flat.size();
  const size_t bytes = total * sizeof(DevOp);
  if (total > 0) {
    if (!g->h_ops) {
      if (cudaMallocHost(&g->h_ops, bytes) != cudaSuccess ||
          cudaEventCreateWithFlags(&g->copied_ev, cudaEventDisableTiming) != cudaSuccess) {
        cudaGetLastError();
        return fail(MPS_ERR_OOM, "pinned op-table staging failed");
      }
    } else {
      GCK(cudaEventSynchronize(g->copied_ev));  // the previous copy has left the staging buffer
    }
  }
  std::atomic<size_t> next{0};
  std::atomic<int> changed{0};
  auto work = [&]() {
    std::vector<DevOp> ops;
    for (size_t i; (i = next.fetch_add(1)) < np;) {
      mps_prog* p = g->progs[i];
      p->center = 0;  // every replay starts from |0...0>
      compile_program(p, ops);
      if (ops.size() != g->count[i]) {
        changed.store(1);
        continue;
      }
      const DevOp* old = g->flat.data() + g->first[i];
      for (size_t k = 0; k < ops.size(); ++k)
        if (ops[k].kind != old[k].kind || ops[k].site != old[k].site || ops[k].orient != old[k].orient) {
          changed.store(1);
          break;
        }
      if (!ops.empty()) std::memcpy(g->h_ops + g->first[i], ops.data(), ops.size() * sizeof(DevOp));
    }
  };
  const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
  const int nt = (int)std::min<size_t>({(size_t)hw, (size_t)16, std::max<size_t>(np / 32, 1)});
  std::vector<std::thread> pool;
  for (int t = 1; t < nt; ++t) pool.emplace_back(work);
  work();
  for (auto& t : pool) t.join();
  if (changed.load()) return fail(MPS_ERR_ARG, "update changes the circuit structure");
  if (total == 0) return MPS_OK;
  GCK(cudaMemcpyAsync(g->L.d_ops, g->h_ops, bytes, cudaMemcpyHostToDevice, g->L.stream));
  GCK(cudaEventRecord(g->copied_ev, g->L.stream));
  return MPS_OK;
}

int mps_graph_launch_async(mps_graph* g) {
  if (!g) return fail(MPS_ERR_ARG, "NULL graph");
  GCK(cudaSetDevice(g->c->device));
  GCK(cudaGraphLaunch(g->exec, g->L.stream));
  for (mps_prog* p : g->progs) GCK(cudaEventRecord(p->ev, g->L.stream));
  return MPS_OK;
}

// Longest measured first for the next replay: the persistent kernel's
// queue order is the descriptor order, and a replay's makespan is shortest
// when the costliest programs start first.  The descriptors are rewritten on
// the graph's stream ahead of the next replay; results do not depend on the
// order (each program runs alone on one CTA).
static int reorder_by_cycles(mps_graph* g) {
  const int n = (int)g->progs.size();
  std::vector<int> order(n);
  for (int i = 0; i < n; ++i) order[i] = i;
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return g->h_cycles[a] > g->h_cycles[b]; });
  if (order == g->order) return MPS_OK;
  std::vector<ProgDesc> descs(n);
  for (int k = 0; k < n; ++k) descs[k] = g->desc_of[order[k]];
  // pageable source: the copy is staged before the call returns
  GCK(cudaMemcpyAsync(g->L.d_desc, descs.data(), (size_t)n * sizeof(ProgDesc), cudaMemcpyHostToDevice,
                      g->L.stream));
  g->order.swap(order);
  return MPS_OK;
}

int mps_graph_sync(mps_graph* g, double* energies) {
  if (!g) return fail(MPS_ERR_ARG, "NULL graph");
  GCK(cudaSetDevice(g->c->device));
  GCK(cudaStreamSynchronize(g->L.stream));
  {
    const int rc = reorder_by_cycles(g);
    if (rc) return rc;
  }
  for (size_t i = 0; i < g->progs.size(); ++i) {
    int rc = prog_check_err(g->progs[i]);
    if (rc) return rc;
    if (energies)
      energies[i] = g->task_first[i] == (size_t)-1 ? 0.0
                                                   : observable_value(g->progs[i], g->h_out + 2 * g->task_first[i]);
  }
  return MPS_OK;
}

int mps_graph_launch(mps_graph* g, double* energies) {
  int rc = mps_graph_launch_async(g);
  if (rc) return rc;
  return mps_graph_sync(g, energies);
}

int mps_graph_timing(mps_graph* g, double out[6]) {
  if (!g || !out) return fail(MPS_ERR_ARG, "NULL argument");
  GCK(cudaSetDevice(g->c->device));
  GCK(cudaStreamSynchronize(g->L.stream));
  float a = 0.f, b = 0.f;
  GCK(cudaEventElapsedTime(&a, g->ev[0], g->ev[1]));
  GCK(cudaEventElapsedTime(&b, g->ev[1], g->ev[2]));
  out[0] = a;
  out[1] = b;
  double fl = 0.0, ef = 0.0;
  for (mps_prog* p : g->progs) {
    double st[ST_COUNT];
    GCK(cudaMemcpy(st, p->d_stats, sizeof(st), cudaMemcpyDeviceToHost));
    fl += st[ST_FLOPS];
    ef += st[ST_EIG_FLOPS];
  }
  out[2] = fl;
  out[3] = ef;
  out[4] = (double)(g->flat.size() * sizeof(DevOp));
  out[5] = (double)(2 * g->tasks.size() * sizeof(double));
  return MPS_OK;
}

int mps_graph_phase_cycles(mps_graph* g, double out[5]) {
  if (!g || !out) return fail(MPS_ERR_ARG, "NULL argument");
  GCK(cudaSetDevice(g->c->device));
  GCK(cudaStreamSynchronize(g->L.stream));
  for (int i = 0; i < 5; ++i) out[i] = 0.0;
  for (mps_prog* p : g->progs) {
    double st[ST_COUNT];
    GCK(cudaMemcpy(st, p->d_stats, sizeof(st), cudaMemcpyDeviceToHost));
    for (int i = 0; i < 5; ++i) out[i] += st[ST_CYC_THETA + i];
  }
  return MPS_OK;
}

int mps_graph_stat_sums(mps_graph* g, double* out, int n) {
  if (!g || !out) return fail(MPS_ERR_ARG, "NULL argument");
  if (n < 1 || n > ST_COUNT) return fail(MPS_ERR_ARG, "n must be in 1..17");
  GCK(cudaSetDevice(g->c->device));
  GCK(cudaStreamSynchronize(g->L.stream));
  for (int i = 0; i < n; ++i) out[i] = 0.0;
  for (mps_prog* p : g->progs) {
    double st[ST_COUNT];
    GCK(cudaMemcpy(st, p->d_stats, sizeof(st), cudaMemcpyDeviceToHost));
    for (int i = 0; i < n; ++i) out[i] += st[i];
  }
  return MPS_OK;
}

int mps_graph_stream(mps_graph* g, void** s) {
  if (!g || !s) return fail(MPS_ERR_ARG, "NULL argument");
  *s = (void*)g->L.stream;
  return MPS_OK;
}

}  // extern "C"
