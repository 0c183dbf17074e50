// Host engine behind the gb300mps C ABI: contexts, programs (one MPS each),
// gate recording, routing, 1-qubit fusion, gauge planning, launches and
// result read-back.  All device work goes through the kernels in k_ops.cu and
// k_measure.cu; there is no CPU execution path.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <climits>
#include <cstdint>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <thread>
#include <string>
#include <vector>

#include "../../include/gb300mps.h"
#include "engine_internal.hpp"
#include "gates.hpp"
#include "wide.hpp"

namespace gbmps {

thread_local std::string g_err;
static std::atomic<int> g_parallel_width{0};  // mps_diag_set_parallel_width

int fail(int code, const std::string& msg) {
  g_err = msg;
  return code;
}

static size_t elem_bytes(int prec) { return prec == MPS_PREC_FP64 ? 16 : 8; }

static void bond_caps(int n, int chi, std::vector<int>& cap) {
  cap.assign(n + 1, 1);
  for (int b = 1; b < n; ++b) {
    long long c = chi;
    const int lft = b, rgt = n - b;
    if (lft < 31) c = std::min<long long>(c, 1LL << lft);
    if (rgt < 31) c = std::min<long long>(c, 1LL << rgt);
    cap[b] = (int)c;
  }
}

size_t footprint(int n, int chi, int prec) {
  std::vector<int> cap;
  bond_caps(n, chi, cap);
  size_t e = 0;
  for (int i = 0; i < n; ++i) e += (size_t)cap[i] * 2 * cap[i + 1];
  return e * elem_bytes(prec);
}

template <typename X>
static int grow(X** ptr, size_t* cap, size_t need) {
  if (*cap >= need) return MPS_OK;
  if (*ptr) cudaFree(*ptr);
  *ptr = nullptr;
  *cap = 0;
  size_t n = std::max<size_t>(need, 64);
  n = std::max(n, need + need / 2);
  if (cudaMalloc((void**)ptr, n * sizeof(X)) != cudaSuccess) {
    cudaGetLastError();
    return fail(MPS_ERR_OOM, "device allocation failed");
  }
  *cap = n;
  return MPS_OK;
}

// ------------------------------------------------------------ compilation
// Recorded gates -> routed adjacent gates -> 1-qubit gates fused into the
// next 2-qubit gate on the same site -> gauge moves (itensor semantics).
void compile_program(mps_prog* p, std::vector<DevOp>& ops) {
  ops.clear();
  std::vector<GateRec> routed;
  routed.reserve(p->pending.size() * 2);
  for (const GateRec& g : p->pending) route_append(g, routed);
  p->pending.clear();
  if (p->flags & MPS_FLAG_FUSE) cancel_swap_pairs(routed);

  struct Raw {
    int kind;
    int site;
    cd m[16];
  };
  std::vector<Raw> raw;
  raw.reserve(routed.size());
  std::vector<cd> pend(4 * p->n);
  std::vector<char> has(p->n, 0);
  auto ident = [](cd* m) {
    m[0] = 1.0;
    m[1] = 0.0;
    m[2] = 0.0;
    m[3] = 1.0;
  };
  for (int q = 0; q < p->n; ++q) ident(&pend[4 * q]);
  // MPS_FLAG_FUSE: the last raw op on each site, so that a 2-qubit gate on
  // the pair its predecessor acted on (nothing else on either site in
  // between) multiplies into that op instead of splitting again
  const bool fuse = (p->flags & MPS_FLAG_FUSE) != 0;
  std::vector<int> last(p->n, -1);
  for (const GateRec& g : routed) {
    if (g.nq == 1) {
      cd* P = &pend[4 * g.q0];
      cd r[4];
      for (int i = 0; i < 2; ++i)
        for (int j = 0; j < 2; ++j) r[i * 2 + j] = g.m[i * 2 + 0] * P[0 * 2 + j] + g.m[i * 2 + 1] * P[1 * 2 + j];
      for (int i = 0; i < 4; ++i) P[i] = r[i];
      has[g.q0] = 1;
      continue;
    }
    const int lo = std::min(g.q0, g.q1);
    cd ms[16];
    if (g.q0 < g.q1)
      for (int i = 0; i < 16; ++i) ms[i] = g.m[i];
    else
      swap_bits4(g.m, ms);
    // fold the pending 1-qubit products: M . (P_lo (x) P_hi)
    const cd* Pl = &pend[4 * lo];
    const cd* Ph = &pend[4 * (lo + 1)];
    Raw r;
    r.kind = OP_GATE2;
    r.site = lo;
    for (int row = 0; row < 4; ++row)
      for (int col = 0; col < 4; ++col) {
        cd acc = 0.0;
        const int a = col >> 1, b = col & 1;
        for (int k = 0; k < 4; ++k) {
          const int ka = k >> 1, kb = k & 1;
          acc += ms[row * 4 + k] * Pl[ka * 2 + a] * Ph[kb * 2 + b];
        }
        r.m[row * 4 + col] = acc;
      }
    ident(&pend[4 * lo]);
    ident(&pend[4 * (lo + 1)]);
    has[lo] = has[lo + 1] = 0;
    const int k = last[lo];
    if (fuse && k >= 0 && last[lo + 1] == k && raw[k].kind == OP_GATE2 && raw[k].site == lo) {
      cd prod[16];
      for (int row = 0; row < 4; ++row)
        for (int col = 0; col < 4; ++col) {
          cd acc = 0.0;
          for (int q = 0; q < 4; ++q) acc += r.m[row * 4 + q] * raw[k].m[q * 4 + col];
          prod[row * 4 + col] = acc;
        }
      for (int i = 0; i < 16; ++i) raw[k].m[i] = prod[i];
      continue;
    }
    last[lo] = last[lo + 1] = (int)raw.size();
    raw.push_back(r);
  }
  for (int q = 0; q < p->n; ++q) {
    if (!has[q]) continue;
    Raw r;
    r.kind = OP_GATE1;
    r.site = q;
    for (int i = 0; i < 4; ++i) r.m[i] = pend[4 * q + i];
    raw.push_back(r);
  }

  // Sweep scheduling (itensor semantics, opt-in): gates on disjoint qubits
  // commute, so among the gates whose predecessors on both sites are done,
  // take the one nearest the orthogonality centre (ties: the direction of
  // travel).  A brick-wall layer then costs one centre move per gate instead
  // of a sweep back across the chain after every layer.  The state is the
  // same up to the order in which truncations happen.
  if (p->mode == MPS_TRUNC_ITENSOR && (p->flags & MPS_FLAG_SWEEP) && raw.size() > 1) {
    const int n = p->n;
    std::vector<std::vector<int>> per(n);
    for (size_t i = 0; i < raw.size(); ++i) {
      per[raw[i].site].push_back((int)i);
      if (raw[i].kind == OP_GATE2) per[raw[i].site + 1].push_back((int)i);
    }
    std::vector<size_t> head(n, 0);
    auto ready = [&](int i) {
      const Raw& r = raw[i];
      if (per[r.site][head[r.site]] != i) return false;
      return r.kind != OP_GATE2 || per[r.site + 1][head[r.site + 1]] == i;
    };
    std::vector<Raw> order;
    order.reserve(raw.size());
    int c = p->center, dir = 1;
    std::vector<char> done(raw.size(), 0);
    std::vector<int> cand;
    for (size_t step = 0; step < raw.size(); ++step) {
      cand.clear();
      for (int q = 0; q < n; ++q)
        if (head[q] < per[q].size()) {
          const int i = per[q][head[q]];
          if (!done[i] && raw[i].site == q && ready(i)) cand.push_back(i);
        }
      int best = -1;
      long long bkey = 0;
      for (int i : cand) {
        const Raw& r = raw[i];
        const int lo = r.site, hi = r.kind == OP_GATE2 ? lo + 1 : lo;
        const int dist = c < lo ? lo - c : (c > hi ? c - hi : 0);
        const int side = (lo >= c) == (dir > 0) ? 0 : 1;
        const long long key = (long long)dist * 4 + side * 2 + (r.kind == OP_GATE2 ? 0 : 1);
        if (best < 0 || key < bkey || (key == bkey && i < best)) {
          best = i;
          bkey = key;
        }
      }
      const Raw& r = raw[best];
      done[best] = 1;
      ++head[r.site];
      if (r.kind == OP_GATE2) {
        ++head[r.site + 1];
        const int target = c < r.site ? r.site : (c > r.site + 1 ? r.site + 1 : c);
        if (target != c) dir = target > c ? 1 : -1;
        c = target;
      }
      order.push_back(r);
    }
    raw.swap(order);
  }

  auto emit = [&](int kind, int site, int orient, const cd* m, int nm) {
    DevOp o;
    std::memset(&o, 0, sizeof(o));
    o.kind = kind;
    o.site = site;
    o.orient = orient;
    for (int i = 0; i < nm; ++i) {
      o.m[2 * i] = m[i].real();
      o.m[2 * i + 1] = m[i].imag();
    }
    ops.push_back(o);
  };
  int center = p->center;
  for (size_t idx = 0; idx < raw.size(); ++idx) {
    const Raw& r = raw[idx];
    if (r.kind == OP_GATE1) {
      emit(OP_GATE1, r.site, 0, r.m, 4);
      continue;
    }
    const int lo = r.site;
    if (p->mode == MPS_TRUNC_EXATN) {
      emit(OP_GATE2, lo, ORIENT_SQRT, r.m, 16);
      continue;
    }
    while (center < lo) {
      emit(OP_MOVE_R, center, 0, r.m, 0);
      ++center;
    }
    while (center > lo + 1) {
      emit(OP_MOVE_L, center, 0, r.m, 0);
      --center;
    }
    int nxt = -1;
    for (size_t j = idx + 1; j < raw.size(); ++j)
      if (raw[j].kind == OP_GATE2) {
        nxt = raw[j].site;
        break;
      }
    const int orient = (nxt >= 0 && nxt < lo) ? ORIENT_TO_LO : ORIENT_TO_HI;
    emit(OP_GATE2, lo, orient, r.m, 16);
    center = orient == ORIENT_TO_HI ? lo + 1 : lo;
  }
  p->center = center;
}

int lane_init(Lane& L, int priority) {
  if (L.stream) return MPS_OK;
  // priority > 0: the device's highest stream priority, < 0: its lowest, 0: default
  int least = 0, greatest = 0;
  if (priority != 0 && cudaDeviceGetStreamPriorityRange(&least, &greatest) != cudaSuccess) {
    cudaGetLastError();
    least = greatest = 0;
  }
  const int prio = priority > 0 ? greatest : priority < 0 ? least : 0;
  cudaError_t e = cudaStreamCreateWithPriority(&L.stream, cudaStreamNonBlocking, prio);
  if (e != cudaSuccess) return fail(MPS_ERR_CUDA, cudaGetErrorString(e));
  e = cudaMalloc(&L.d_queue, 64 * sizeof(int));
  if (e != cudaSuccess) return fail(MPS_ERR_OOM, cudaGetErrorString(e));
  return MPS_OK;
}

void lane_free(Lane& L) {
  if (!L.stream) return;
  cudaStreamSynchronize(L.stream);
  if (L.op_scratch) cudaFree(L.op_scratch);
  for (int p = 0; p < 2; ++p)
    if (L.exp_scratch[p]) cudaFree(L.exp_scratch[p]);
  if (L.d_ops) cudaFree(L.d_ops);
  if (L.d_desc) cudaFree(L.d_desc);
  if (L.d_exp_tasks) cudaFree(L.d_exp_tasks);
  if (L.d_exp_out) cudaFree(L.d_exp_out);
  if (L.d_work) cudaFree(L.d_work);
  if (L.d_queue) cudaFree(L.d_queue);
  if (L.d_dag) cudaFree(L.d_dag);
  cudaStreamDestroy(L.stream);
  L = Lane();
}

static int ensure_bytes(char** ptr, int* have, int need, size_t per) {
  if (*have >= need) return MPS_OK;
  if (*ptr) cudaFree(*ptr);
  *ptr = nullptr;
  *have = 0;
  if (cudaMalloc(ptr, per * (size_t)need) != cudaSuccess) {
    cudaGetLastError();
    return fail(MPS_ERR_OOM, "scratch allocation failed");
  }
  *have = need;
  return MPS_OK;
}

// Estimated device time of a program on one CTA (arbitrary units) for the
// longest-first order of the persistent launch: each two-site split ~ m^2 (m
// + nn) at the sites' bond caps (Gram, tridiagonalisation, split; m the
// smaller side), a centre move a fifth of that, the attached observables 2
// chi_l chi_r (chi_l + chi_r) per site and term, and complex128 ~13x
// complex64 (measured per program on GB300, FP64 at 1/63 of the FP32 rate).
double program_cost(const mps_prog* p, const DevOp* ops, size_t n_ops, bool with_obs) {
  const std::vector<int>& cap = p->cap_bond;
  double c = 0.0;
  for (size_t o = 0; o < n_ops; ++o) {
    const int s = ops[o].site;
    if (ops[o].kind == OP_GATE2 && s + 2 <= p->n) {
      const double a = 2.0 * cap[s], b = 2.0 * cap[s + 2];
      const double m = std::min(a, b), nn = std::max(a, b);
      c += m * m * (m + nn);
    } else if (ops[o].kind == OP_MOVE_R || ops[o].kind == OP_MOVE_L) {
      const double d = (double)cap[s] * cap[s + 1];
      c += 0.4 * d * std::max(cap[s], cap[s + 1]);
    } else {
      c += 8.0 * cap[s] * cap[s + 1];
    }
  }
  if (with_obs) {
    double sweep = 0.0;
    for (int i = 0; i < p->n; ++i) sweep += 2.0 * cap[i] * cap[i + 1] * (double)(cap[i] + cap[i + 1]);
    c += (p->n_terms + 1) * sweep;
  }
  return p->prec == MPS_PREC_FP64 ? 13.0 * c : c;
}

// Compile, upload and launch.  Non per-gate: one persistent launch whose CTAs
// pull whole programs from an atomic queue (longest first).  Per-gate: one
// single-CTA launch per op, the plain gate-by-gate visitor path.
int launch_programs(mps_ctx* c, Lane& L, mps_prog* const* progs_in, int n_in, bool per_gate) {
  // wide programs run host-driven on this lane, one after the other
  std::vector<mps_prog*> narrow;
  narrow.reserve(n_in);
  for (int i = 0; i < n_in; ++i) {
    if (prog_is_wide(progs_in[i])) {
      const int rc = wide_run(c, L, progs_in[i]);
      if (rc) return rc;
    } else {
      narrow.push_back(progs_in[i]);
    }
  }
  mps_prog* const* progs = narrow.data();
  const int n = (int)narrow.size();
  if (n == 0) return MPS_OK;
  std::vector<std::vector<DevOp>> all(n);
  size_t total = 0;
  for (int i = 0; i < n; ++i) {
    compile_program(progs[i], all[i]);
    total += all[i].size();
  }
  bool any_fused = false;
  for (int i = 0; i < n; ++i) any_fused = any_fused || progs[i]->serve_flag != nullptr;
  cudaError_t e;
  if (total > 0 || any_fused) {
    std::vector<DevOp> flat;
    flat.reserve(total);
    std::vector<size_t> first(n);
    for (int i = 0; i < n; ++i) {
      first[i] = flat.size();
      flat.insert(flat.end(), all[i].begin(), all[i].end());
    }
    // generous first sizes: growing a buffer reallocates, and device
    // allocation synchronises the whole device (lanes of the serve loop run
    // side by side)
    int rc = grow(&L.d_ops, &L.d_ops_cap, std::max<size_t>(flat.size(), 65536));
    if (rc) return rc;
    std::vector<ProgDesc> descs;
    auto make_desc = [&](int i, size_t off, int nops) {
      mps_prog* p = progs[i];
      ProgDesc d;
      std::memset(&d, 0, sizeof(d));
      d.sites = p->d_sites;
      d.site_off = p->d_off;
      d.bond = p->d_bond;
      d.ops = L.d_ops + off;
      d.n_ops = nops;
      d.n = p->n;
      d.chi_cap = p->chi_cap;
      d.mode = p->mode;
      d.flags = p->flags;
      d.prec = p->prec;
      d.cutoff = p->cutoff;
      d.stats = p->d_stats;
      d.err = p->d_err;
      if (p->serve_flag) {
        d.obs_codes = p->d_obs;
        d.n_obs = p->d_obs ? p->n_terms + 1 : 0;
        d.obs_out = p->serve_obs;
        d.done = p->serve_flag;
      }
      return d;
    };
    if (per_gate) {
      for (int i = 0; i < n; ++i)
        for (size_t o = 0; o < all[i].size(); ++o) descs.push_back(make_desc(i, first[i] + o, 1));
    } else {
      // longest programs first (LPT) so the persistent grid drains evenly
      std::vector<int> order(n);
      std::vector<double> cost(n, 0.0);
      for (int i = 0; i < n; ++i) {
        order[i] = i;
        cost[i] = program_cost(progs[i], all[i].data(), all[i].size(),
                               progs[i]->serve_flag != nullptr && progs[i]->d_obs != nullptr);
      }
      std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return cost[a] > cost[b]; });
      for (int i : order)
        if (!all[i].empty() || progs[i]->serve_flag) descs.push_back(make_desc(i, first[i], (int)all[i].size()));
    }
    rc = grow(&L.d_desc, &L.d_desc_cap, std::max<size_t>(descs.size(), 1024));
    if (rc) return rc;
    // pageable sources: the call returns once the data is staged, so the
    // vectors may be released right after
    e = cudaMemcpyAsync(L.d_ops, flat.data(), flat.size() * sizeof(DevOp), cudaMemcpyHostToDevice, L.stream);
    if (e != cudaSuccess) return fail(MPS_ERR_CUDA, cudaGetErrorString(e));
    e = cudaMemcpyAsync(L.d_desc, descs.data(), descs.size() * sizeof(ProgDesc), cudaMemcpyHostToDevice, L.stream);
    if (e != cudaSuccess) return fail(MPS_ERR_CUDA, cudaGetErrorString(e));
    const int nd = (int)descs.size();
    if (per_gate) {
      rc = ensure_bytes(&L.op_scratch, &L.op_scratch_ctas, 1, op_scratch_bytes());
      if (rc) return rc;
      for (int i = 0; i < nd; ++i) {
        e = launch_ops(L.d_desc + i, 1, 1, nullptr, L.op_scratch, L.stream);
        if (e != cudaSuccess) return fail(MPS_ERR_CUDA, cudaGetErrorString(e));
      }
    } else if (n == 1 && nd == 1 && (progs[0]->flags & MPS_FLAG_PARALLEL) && progs[0]->serve_flag == nullptr &&
               flat.size() > 1) {
      // site-parallel: the ops by dependency level, with per-op counts of
      // earlier ops on their sites, then the op counter and per-site counts
      const mps_prog* p = progs[0];
      const size_t nops = flat.size();
      std::vector<DevOp> sorted;
      std::vector<int> host;
      site_schedule(flat, p->n, sorted, host);
      host.resize(nops * 2 + 1 + p->n, 0);
      // pageable source: staged before the call returns; lands over the
      // program-order table uploaded above
      e = cudaMemcpyAsync(L.d_ops, sorted.data(), nops * sizeof(DevOp), cudaMemcpyHostToDevice, L.stream);
      if (e != cudaSuccess) return fail(MPS_ERR_CUDA, cudaGetErrorString(e));
      int width = std::max(1, p->n / 2);  // two-site ops that can run at once
      const int cap = g_parallel_width.load();
      if (cap > 0) width = std::min(width, cap);
      rc = grow(&L.d_dag, &L.d_dag_cap, host.size());
      if (rc) return rc;
      e = cudaMemcpyAsync(L.d_dag, host.data(), host.size() * sizeof(int), cudaMemcpyHostToDevice, L.stream);
      if (e != cudaSuccess) return fail(MPS_ERR_CUDA, cudaGetErrorString(e));
      const int grid = std::min<int>({(int)nops, c->num_sms, width});
      rc = ensure_bytes(&L.op_scratch, &L.op_scratch_ctas, c->num_sms, op_scratch_bytes());
      if (rc) return rc;
      e = launch_ops_sites(L.d_desc, reinterpret_cast<const int2*>(L.d_dag), L.d_dag + 2 * nops, grid,
                           L.op_scratch, L.stream);
      if (e != cudaSuccess) return fail(MPS_ERR_CUDA, cudaGetErrorString(e));
    } else {
      const int grid = std::min(nd, c->num_sms);
      rc = ensure_bytes(&L.op_scratch, &L.op_scratch_ctas, c->num_sms, op_scratch_bytes());
      if (rc) return rc;
      e = cudaMemsetAsync(L.d_queue, 0, sizeof(int), L.stream);
      if (e != cudaSuccess) return fail(MPS_ERR_CUDA, cudaGetErrorString(e));
      e = launch_ops(L.d_desc, nd, grid, nd > 1 ? L.d_queue : nullptr, L.op_scratch, L.stream);
      if (e != cudaSuccess) return fail(MPS_ERR_CUDA, cudaGetErrorString(e));
    }
  }
  for (int i = 0; i < n; ++i) {
    e = cudaEventRecord(progs[i]->ev, L.stream);
    if (e != cudaSuccess) return fail(MPS_ERR_CUDA, cudaGetErrorString(e));
    progs[i]->submitted = true;
  }
  return MPS_OK;
}

int prog_check_err(mps_prog* p) {
  int herr = 0;
  cudaError_t e = cudaMemcpy(&herr, p->d_err, sizeof(int), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return fail(MPS_ERR_CUDA, cudaGetErrorString(e));
  if (herr & ERR_NAN) return fail(MPS_ERR_NUMERIC, "non-finite value in a two-site split");
  if (herr & ERR_DIMS) return fail(MPS_ERR_UNSUPPORTED, "bond dimension beyond the kernel limit");
  if (herr & ERR_TIMEOUT) return fail(MPS_ERR_TIMEOUT, "a site-parallel update waited past its bound");
  return MPS_OK;
}

// Gates recorded since the last submit must be on the device before a measurement.
static int flush_pending(mps_prog* p) {
  if (p->pending.empty()) return MPS_OK;
  return launch_programs(p->ctx, p->ctx->lane0, &p, 1, (p->flags & MPS_FLAG_PER_GATE) != 0);
}

// Enqueue expectation tasks; results (2 doubles per task) land in h_out, which
// must be pinned for the copy to stay asynchronous.
int enqueue_expect(Lane& L, const std::vector<ExpTask>& tasks, int prec, double* h_out) {
  const int nt = (int)tasks.size();
  if (nt == 0) return MPS_OK;
  int rc = ensure_bytes(&L.exp_scratch[prec], &L.exp_scratch_ctas[prec], nt, expect_scratch_bytes(prec));
  if (rc) return rc;
  rc = grow(&L.d_exp_tasks, &L.d_exp_tasks_cap, tasks.size());
  if (rc) return rc;
  rc = grow(&L.d_exp_out, &L.d_exp_out_cap, 2 * tasks.size());
  if (rc) return rc;
  cudaError_t e = cudaMemcpyAsync(L.d_exp_tasks, tasks.data(), tasks.size() * sizeof(ExpTask),
                                  cudaMemcpyHostToDevice, L.stream);
  if (e != cudaSuccess) return fail(MPS_ERR_CUDA, cudaGetErrorString(e));
  e = launch_expect(prec, L.d_exp_tasks, nt, L.exp_scratch[prec], L.d_exp_out, L.stream);
  if (e != cudaSuccess) return fail(MPS_ERR_CUDA, cudaGetErrorString(e));
  e = cudaMemcpyAsync(h_out, L.d_exp_out, 2 * tasks.size() * sizeof(double), cudaMemcpyDeviceToHost, L.stream);
  if (e != cudaSuccess) return fail(MPS_ERR_CUDA, cudaGetErrorString(e));
  return MPS_OK;
}

// Enqueue right environments + sampling of every qubit; h_all_bits gets
// shots * n bytes (pinned for an asynchronous copy).
int enqueue_sample(Lane& L, mps_prog* p, int shots, uint64_t seed, uint8_t* h_all_bits) {
  const size_t eb = elem_bytes(p->prec);
  std::vector<int64_t> eoff(p->n + 1, 0);
  int64_t tot = 0;
  for (int i = 1; i <= p->n; ++i) {
    eoff[i] = tot;
    tot += (int64_t)p->cap_bond[i] * p->cap_bond[i];
  }
  auto al = [](size_t x) { return (x + 255) & ~(size_t)255; };
  const size_t env_bytes = al((size_t)tot * eb);
  const size_t y_bytes = al((size_t)2 * kChiLimit * kChiLimit * eb);
  const size_t off_bytes = al(sizeof(int64_t) * (p->n + 1));
  const size_t bit_bytes = al((size_t)shots * p->n);
  const size_t need = env_bytes + y_bytes + off_bytes + bit_bytes;
  if (L.d_work_cap < need) {
    if (L.d_work) cudaFree(L.d_work);
    L.d_work = nullptr;
    L.d_work_cap = 0;
    if (cudaMalloc(&L.d_work, need) != cudaSuccess) {
      cudaGetLastError();
      return fail(MPS_ERR_OOM, "sampler workspace allocation failed");
    }
    L.d_work_cap = need;
  }
  char* d_env = L.d_work;
  char* d_y = d_env + env_bytes;
  int64_t* d_eoff = reinterpret_cast<int64_t*>(d_y + y_bytes);
  uint8_t* d_bits = reinterpret_cast<uint8_t*>(d_y + y_bytes + off_bytes);
  cudaError_t e = cudaMemcpyAsync(d_eoff, eoff.data(), sizeof(int64_t) * (p->n + 1), cudaMemcpyHostToDevice, L.stream);
  if (e != cudaSuccess) return fail(MPS_ERR_CUDA, cudaGetErrorString(e));
  EnvTask et;
  et.sites = p->d_sites;
  et.site_off = p->d_off;
  et.bond = p->d_bond;
  et.env = d_env;
  et.env_off = d_eoff;
  et.n = p->n;
  et.pad = 0;
  e = launch_right_env(p->prec, et, d_y, L.stream);
  if (e != cudaSuccess) return fail(MPS_ERR_CUDA, cudaGetErrorString(e));
  SampleTask st;
  st.sites = p->d_sites;
  st.site_off = p->d_off;
  st.bond = p->d_bond;
  st.env = d_env;
  st.env_off = d_eoff;
  st.bits = d_bits;
  st.seed = seed;
  st.n = p->n;
  st.shots = shots;
  e = launch_sample(p->prec, st, L.stream);
  if (e != cudaSuccess) return fail(MPS_ERR_CUDA, cudaGetErrorString(e));
  e = cudaMemcpyAsync(h_all_bits, d_bits, (size_t)shots * p->n, cudaMemcpyDeviceToHost, L.stream);
  if (e != cudaSuccess) return fail(MPS_ERR_CUDA, cudaGetErrorString(e));
  return MPS_OK;
}

int parse_paulis(int n, const char* paulis, int n_terms, std::vector<uint8_t>& codes) {
  codes.resize((size_t)n * n_terms);
  for (size_t i = 0; i < codes.size(); ++i) {
    switch (paulis[i]) {
      case 'I': codes[i] = 0; break;
      case 'X': codes[i] = 1; break;
      case 'Y': codes[i] = 2; break;
      case 'Z': codes[i] = 3; break;
      default: return fail(MPS_ERR_ARG, "Pauli strings must use only I, X, Y, Z");
    }
  }
  return MPS_OK;
}

void select_measured(const mps_prog* p, const uint8_t* all, int shots, uint8_t* bits) {
  std::vector<int> meas = p->measured;
  if (meas.empty())
    for (int q = 0; q < p->n; ++q) meas.push_back(q);
  for (int s = 0; s < shots; ++s)
    for (size_t i = 0; i < meas.size(); ++i) bits[(size_t)s * meas.size() + i] = all[(size_t)s * p->n + meas[i]];
}

void observable_tasks(mps_prog* p, std::vector<ExpTask>& tasks) {
  for (int t = 0; t <= p->n_terms; ++t) {
    ExpTask tk;
    tk.sites = p->d_sites;
    tk.site_off = p->d_off;
    tk.bond = p->d_bond;
    tk.codes = p->d_obs + (size_t)t * p->n;
    tk.n = p->n;
    tk.pad = 0;
    tasks.push_back(tk);
  }
}

double observable_value(const mps_prog* p, const double* r) {
  const double nrm = r[2 * (size_t)p->n_terms];
  double e = 0.0;
  for (int t = 0; t < p->n_terms; ++t) e += p->obs_coef[t] * r[2 * (size_t)t];
  return nrm > 0.0 ? e / nrm : 0.0;
}

// Schedule of a site-parallel run.  Ops are handed out by level (1 + the
// level of the previous op on each of their sites), program order within a
// level: ops of one level are independent, so the CTAs claiming them run at
// once instead of queueing behind a chain, and every site still sees its ops
// in program order (a later op on a site has a higher level).  deps holds,
// per op of the sorted list, the number of earlier ops on its first and
// second site (-1 for a one-site op).
void site_schedule(const std::vector<DevOp>& ops, int n_sites, std::vector<DevOp>& sorted, std::vector<int>& deps) {
  const size_t nops = ops.size();
  std::vector<int> level(nops), last(n_sites, 0);
  for (size_t o = 0; o < nops; ++o) {
    const DevOp& op = ops[o];
    const int s0 = op.kind == OP_MOVE_L ? op.site - 1 : op.site;
    const bool two = op.kind != OP_GATE1;
    const int l = 1 + std::max(last[s0], two ? last[s0 + 1] : 0);
    level[o] = l;
    last[s0] = l;
    if (two) last[s0 + 1] = l;
  }
  std::vector<int> order(nops);
  for (size_t o = 0; o < nops; ++o) order[o] = (int)o;
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return level[a] < level[b]; });
  sorted.resize(nops);
  deps.assign(2 * nops, 0);
  std::vector<int> seen(n_sites, 0);
  for (size_t k = 0; k < nops; ++k) {
    const DevOp& op = ops[order[k]];
    sorted[k] = op;
    const int s0 = op.kind == OP_MOVE_L ? op.site - 1 : op.site;
    deps[2 * k] = seen[s0]++;
    deps[2 * k + 1] = op.kind == OP_GATE1 ? -1 : seen[s0 + 1]++;
  }
}

// Record a gate on qubits; a density program applies U to the ket sites and
// conj(U) to the bra sites: rho -> U rho U^H.
void record_gate(mps_prog* p, const GateRec& g) {
  if (!p->density) {
    p->pending.push_back(g);
    return;
  }
  GateRec k = g, b = g;
  k.q0 = 2 * g.q0;
  b.q0 = 2 * g.q0 + 1;
  if (g.nq == 2) {
    k.q1 = 2 * g.q1;
    b.q1 = 2 * g.q1 + 1;
  }
  const int ne = g.nq == 2 ? 16 : 4;
  for (int i = 0; i < ne; ++i) b.m[i] = std::conj(g.m[i]);
  p->pending.push_back(k);
  p->pending.push_back(b);
}

}  // namespace gbmps

using namespace gbmps;

#define CK(call)                                                              \
  do {                                                                        \
    cudaError_t e_ = (call);                                                  \
    if (e_ != cudaSuccess) return fail(MPS_ERR_CUDA, cudaGetErrorString(e_)); \
  } while (0)

extern "C" {

const char* mps_last_error(void) { return g_err.c_str(); }
const char* mps_version(void) { return "gb300mps 0.1 (sm_103a)"; }

size_t mps_footprint_bytes(int n_qubits, int chi_max, int precision) {
  if (n_qubits < 1) return 0;
  if (chi_max <= 0 || chi_max > MPS_CHI_LIMIT) chi_max = MPS_CHI_LIMIT;
  return footprint(n_qubits, chi_max, precision);
}

int mps_ctx_create(const mps_cfg* cfg, mps_ctx** out) {
  if (!out) return fail(MPS_ERR_ARG, "out is NULL");
  *out = nullptr;
  const int dev = cfg ? cfg->device : 0;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= 0) {
    cudaGetLastError();
    return fail(MPS_ERR_CUDA, "no CUDA device");
  }
  if (dev < 0 || dev >= ndev) return fail(MPS_ERR_ARG, "device ordinal out of range");
  CK(cudaSetDevice(dev));
  mps_ctx* c = new mps_ctx();
  c->device = dev;
  c->budget = (cfg && cfg->hbm_budget_bytes) ? cfg->hbm_budget_bytes : (size_t)150 << 30;
  cudaDeviceProp prop;
  CK(cudaGetDeviceProperties(&prop, dev));
  c->num_sms = prop.multiProcessorCount;
  CK(configure_ops());
  CK(configure_expect());
  int rc = lane_init(c->lane0);
  if (rc) {
    delete c;
    return rc;
  }
  *out = c;
  return MPS_OK;
}

int mps_ctx_destroy(mps_ctx* c) {
  if (!c) return MPS_OK;
  mps_serve_stop(c);
  cudaSetDevice(c->device);
  lane_free(c->lane0);
  wide_free(c);
  delete c;
  return MPS_OK;
}

int mps_ctx_info(mps_ctx* c, int* num_sms, size_t* bytes_resident) {
  if (!c) return fail(MPS_ERR_ARG, "ctx is NULL");
  if (num_sms) *num_sms = c->num_sms;
  if (bytes_resident) *bytes_resident = c->resident;
  return MPS_OK;
}

static int init_state(mps_prog* p) {
  // |0...0>: every site 1x2x1 with A[0][0][0] = 1 (ExaTnMpsVisitor.cpp:281-326)
  cudaStream_t st = p->ctx->lane0.stream;
  CK(cudaMemsetAsync(p->d_sites, 0, p->bytes, st));
  const size_t eb = elem_bytes(p->prec);
  const size_t total = p->bytes / eb;
  std::vector<char> img;
  // write the unit entries with one copy per site (n small copies)
  char one[16] = {0};
  if (p->prec == MPS_PREC_FP64) {
    const double v = 1.0;
    std::memcpy(one, &v, 8);
  } else {
    const float v = 1.0f;
    std::memcpy(one, &v, 4);
  }
  (void)total;
  for (int i = 0; i < p->n; ++i)
    CK(cudaMemcpyAsync((char*)p->d_sites + p->off[i] * eb, one, eb, cudaMemcpyHostToDevice, st));
  std::vector<int> ones(p->n + 1, 1);
  CK(cudaMemcpyAsync(p->d_bond, ones.data(), ones.size() * sizeof(int), cudaMemcpyHostToDevice, st));
  CK(cudaMemsetAsync(p->d_stats, 0, ST_COUNT * sizeof(double), st));
  CK(cudaMemsetAsync(p->d_err, 0, sizeof(int), st));
  CK(cudaStreamSynchronize(st));
  p->hbond.assign(p->n + 1, 1);
  p->center = 0;
  p->pending.clear();
  p->measured.clear();
  p->submitted = false;
  return MPS_OK;
}

int mps_program_begin(mps_ctx* c, int n, int chi_max, double cutoff, int trunc_mode, int precision, int flags,
                      mps_prog** out) {
  if (!c || !out) return fail(MPS_ERR_ARG, "NULL argument");
  *out = nullptr;
  if (n < 1) return fail(MPS_ERR_ARG, "n_qubits must be >= 1");
  if (trunc_mode != MPS_TRUNC_EXATN && trunc_mode != MPS_TRUNC_ITENSOR) return fail(MPS_ERR_ARG, "bad trunc_mode");
  if (precision != MPS_PREC_FP64 && precision != MPS_PREC_FP32 && precision != MPS_PREC_AUTO &&
      precision != MPS_PREC_SPLIT_BF16)
    return fail(MPS_ERR_ARG, "bad precision");
  const int requested = precision;
  if (chi_max > MPS_WIDE_CHI_LIMIT)
    return fail(MPS_ERR_UNSUPPORTED, "max bond dimension above " + std::to_string(MPS_WIDE_CHI_LIMIT));
  if (chi_max > MPS_CHI_LIMIT && (flags & MPS_FLAG_PER_GATE))
    return fail(MPS_ERR_UNSUPPORTED, "the per-gate visitor path runs the single-CTA kernel (bond cap <= " +
                                         std::to_string(MPS_CHI_LIMIT) + ")");
  if (chi_max <= 0) chi_max = MPS_CHI_LIMIT;
  // a density program holds vec(rho) of n qubits on 2n sites
  const int nq = n;
  if (flags & MPS_FLAG_DENSITY) {
    if (n > (1 << 20)) return fail(MPS_ERR_ARG, "too many qubits");
    n = 2 * n;
  }
  if (precision == MPS_PREC_SPLIT_BF16) precision = MPS_PREC_FP32;  // complex64 storage
  if (precision == MPS_PREC_AUTO) {
    // complex128 where the register is small and exact at its cap
    const bool exact = n / 2 >= 30 || chi_max >= (1 << (n / 2));
    precision = (n <= MPS_AUTO_FP64_QUBITS && exact) ? MPS_PREC_FP64 : MPS_PREC_FP32;
  }
  std::lock_guard<std::mutex> lk(c->mu);
  CK(cudaSetDevice(c->device));
  mps_prog* p = new mps_prog();
  p->ctx = c;
  p->n = n;
  p->nq = nq;
  p->density = (flags & MPS_FLAG_DENSITY) != 0;
  p->chi_cap = chi_max;
  p->mode = trunc_mode;
  p->prec = precision;
  p->prec_mode = requested == MPS_PREC_AUTO ? precision : requested;
  p->split_bf16 = requested == MPS_PREC_SPLIT_BF16;
  p->flags = flags;
  if (cutoff < 0.0) cutoff = trunc_mode == MPS_TRUNC_EXATN ? 2.2250738585072014e-308 : 1e-6;
  p->cutoff = cutoff;
  bond_caps(n, chi_max, p->cap_bond);
  p->off.resize(n);
  int64_t e = 0;
  for (int i = 0; i < n; ++i) {
    p->off[i] = e;
    e += (int64_t)p->cap_bond[i] * 2 * p->cap_bond[i + 1];
  }
  p->bytes = (size_t)e * elem_bytes(precision);
  if (c->resident + p->bytes > c->budget) {
    delete p;
    return fail(MPS_ERR_OOM, "HBM admission budget exceeded");
  }
  if (cudaMalloc(&p->d_sites, p->bytes) != cudaSuccess) {
    cudaGetLastError();
    delete p;
    return fail(MPS_ERR_OOM, "cudaMalloc of site tensors failed");
  }
  const size_t meta = sizeof(double) * ST_COUNT + sizeof(int64_t) * n + sizeof(int) * (n + 2) + 64;
  if (cudaMalloc(&p->d_meta, meta) != cudaSuccess) {
    cudaGetLastError();
    cudaFree(p->d_sites);
    delete p;
    return fail(MPS_ERR_OOM, "cudaMalloc failed");
  }
  p->d_stats = reinterpret_cast<double*>(p->d_meta);
  p->d_off = reinterpret_cast<int64_t*>(p->d_meta + sizeof(double) * ST_COUNT);
  p->d_bond = reinterpret_cast<int*>(p->d_meta + sizeof(double) * ST_COUNT + sizeof(int64_t) * n);
  p->d_err = p->d_bond + (n + 1);
  CK(cudaMemcpyAsync(p->d_off, p->off.data(), sizeof(int64_t) * n, cudaMemcpyHostToDevice, c->lane0.stream));
  CK(cudaEventCreateWithFlags(&p->ev, cudaEventDisableTiming));
  int rc = init_state(p);
  if (rc) return rc;
  c->resident += p->bytes;
  *out = p;
  return MPS_OK;
}

int mps_program_precision(mps_prog* p, int* out) {
  if (!p || !out) return fail(MPS_ERR_ARG, "NULL argument");
  *out = p->prec_mode;
  return MPS_OK;
}

int mps_program_reset(mps_prog* p) {
  if (!p) return fail(MPS_ERR_ARG, "NULL program");
  std::lock_guard<std::mutex> lk(p->ctx->mu);
  CK(cudaSetDevice(p->ctx->device));
  CK(cudaEventSynchronize(p->ev));
  return init_state(p);
}

int mps_program_destroy(mps_prog* p) {
  if (!p) return MPS_OK;
  mps_ctx* c = p->ctx;
  std::lock_guard<std::mutex> lk(c->mu);
  cudaSetDevice(c->device);
  cudaEventSynchronize(p->ev);
  cudaStreamSynchronize(c->lane0.stream);
  cudaFree(p->d_sites);
  cudaFree(p->d_meta);
  if (p->d_obs) cudaFree(p->d_obs);
  cudaEventDestroy(p->ev);
  c->resident -= p->bytes;
  delete p;
  return MPS_OK;
}

static int check_q(mps_prog* p, int q) {
  if (q < 0 || q >= p->nq) return fail(MPS_ERR_ARG, "qubit index out of range");
  return MPS_OK;
}

int mps_gate1(mps_prog* p, int q, const double m[8]) {
  if (!p || !m) return fail(MPS_ERR_ARG, "NULL argument");
  if (check_q(p, q)) return MPS_ERR_ARG;
  GateRec g;
  g.nq = 1;
  g.q0 = q;
  g.q1 = -1;
  for (int i = 0; i < 4; ++i) g.m[i] = cd(m[2 * i], m[2 * i + 1]);
  record_gate(p, g);
  return MPS_OK;
}

int mps_gate2(mps_prog* p, int q0, int q1, const double m[32]) {
  if (!p || !m) return fail(MPS_ERR_ARG, "NULL argument");
  if (check_q(p, q0) || check_q(p, q1)) return MPS_ERR_ARG;
  if (q0 == q1) return fail(MPS_ERR_ARG, "two-qubit gate on one qubit");
  GateRec g;
  g.nq = 2;
  g.q0 = q0;
  g.q1 = q1;
  for (int i = 0; i < 16; ++i) g.m[i] = cd(m[2 * i], m[2 * i + 1]);
  record_gate(p, g);
  return MPS_OK;
}

int mps_measure(mps_prog* p, int q) {
  if (!p) return fail(MPS_ERR_ARG, "NULL program");
  if (check_q(p, q)) return MPS_ERR_ARG;
  p->measured.push_back(q);
  return MPS_OK;
}

int mps_gate_named(mps_prog* p, const char* name, const int* qubits, int nq, const double* params, int np) {
  if (!p || !name || (nq > 0 && !qubits) || (np > 0 && !params)) return fail(MPS_ERR_ARG, "NULL argument");
  GateRec g;
  const int k = gate_matrix(name, params, np, g.m);
  if (k == 0) return fail(MPS_ERR_ARG, std::string("unknown gate or bad parameter count: ") + name);
  if (k < 0) {
    if (std::strcmp(name, "Measure") == 0) {
      if (nq != 1) return fail(MPS_ERR_ARG, "Measure takes one qubit");
      return mps_measure(p, qubits[0]);
    }
    for (int i = 0; i < nq; ++i)
      if (check_q(p, qubits[i])) return MPS_ERR_ARG;
    return MPS_OK;  // identity
  }
  if (nq != k) return fail(MPS_ERR_ARG, std::string("wrong number of qubits for ") + name);
  for (int i = 0; i < nq; ++i)
    if (check_q(p, qubits[i])) return MPS_ERR_ARG;
  g.nq = k;
  g.q0 = qubits[0];
  g.q1 = k == 2 ? qubits[1] : -1;
  if (k == 2 && g.q0 == g.q1) return fail(MPS_ERR_ARG, "two-qubit gate on one qubit");
  record_gate(p, g);
  return MPS_OK;
}

int mps_gates(mps_prog* p, int n_gates, const int32_t* ids, const int32_t* qubits, const double* params) {
  static const char* kNames[MPS_G_COUNT] = {"I",  "H",   "CNOT", "Rx", "Ry",  "Rz",  "Swap",   "U",
                                            "X",  "Y",   "Z",    "Measure", "CZ", "CPhase", "S", "Sdg",
                                            "T",  "Tdg", "CY",   "CH", "CRZ", "iSwap", "fSim", "RZZ"};
  static const int kNq[MPS_G_COUNT] = {1, 1, 2, 1, 1, 1, 2, 1, 1, 1, 1, 1, 2, 2, 1, 1, 1, 1, 2, 2, 2, 2, 2, 2};
  static const int kNp[MPS_G_COUNT] = {0, 0, 0, 1, 1, 1, 0, 3, 0, 0, 0, 0, 0, 1, 0, 0, 0, 0, 0, 0, 1, 0, 2, 1};
  if (!p || n_gates < 0 || (n_gates > 0 && (!ids || !qubits || !params))) return fail(MPS_ERR_ARG, "NULL argument");
  for (int g = 0; g < n_gates; ++g) {
    const int id = ids[g];
    if (id < 0 || id >= MPS_G_COUNT) return fail(MPS_ERR_ARG, "gate id out of range");
    const int rc = mps_gate_named(p, kNames[id], qubits + 2 * g, kNq[id], params + 3 * g, kNp[id]);
    if (rc) return rc;
  }
  return MPS_OK;
}

int mps_gates_many(int n_progs, mps_prog* const* progs, const int64_t* first_gate, const int32_t* ids,
                   const int32_t* qubits, const double* params) {
  if (n_progs < 0 || (n_progs > 0 && (!progs || !first_gate || !ids || !qubits || !params)))
    return fail(MPS_ERR_ARG, "NULL argument");
  for (int i = 0; i < n_progs; ++i) {
    if (!progs[i]) return fail(MPS_ERR_ARG, "NULL program");
    if (first_gate[i + 1] < first_gate[i] || first_gate[i + 1] - first_gate[i] > INT32_MAX)
      return fail(MPS_ERR_ARG, "first_gate must be non-decreasing");
  }
  {
    // each program is recorded by one thread: a program listed twice would be
    // written by two
    std::vector<mps_prog*> sorted(progs, progs + n_progs);
    std::sort(sorted.begin(), sorted.end());
    if (std::adjacent_find(sorted.begin(), sorted.end()) != sorted.end())
      return fail(MPS_ERR_ARG, "a program is listed twice");
  }
  // programs record independently: host threads, the first failure (lowest
  // program index) is reported
  std::vector<int> rcs(n_progs, MPS_OK);
  std::vector<std::string> msgs(n_progs);
  std::atomic<int> next{0};
  auto work = [&]() {
    for (int i; (i = next.fetch_add(1)) < n_progs;) {
      const int64_t f = first_gate[i];
      rcs[i] = mps_gates(progs[i], (int)(first_gate[i + 1] - f), ids + f, qubits + 2 * f, params + 3 * f);
      if (rcs[i]) msgs[i] = g_err;
    }
  };
  const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
  const int nt = (int)std::min<long long>({(long long)hw, 16LL, std::max<long long>(n_progs / 32, 1)});
  std::vector<std::thread> pool;
  for (int t = 1; t < nt; ++t) pool.emplace_back(work);
  work();
  for (auto& t : pool) t.join();
  for (int i = 0; i < n_progs; ++i)
    if (rcs[i]) return fail(rcs[i], "program " + std::to_string(i) + ": " + msgs[i]);
  return MPS_OK;
}

int mps_submit(mps_prog* p) {
  if (!p) return fail(MPS_ERR_ARG, "NULL program");
  std::lock_guard<std::mutex> lk(p->ctx->mu);
  CK(cudaSetDevice(p->ctx->device));
  return launch_programs(p->ctx, p->ctx->lane0, &p, 1, (p->flags & MPS_FLAG_PER_GATE) != 0);
}

int mps_batch_submit(mps_ctx* c, mps_prog* const* progs, int n) {
  if (!c || (n > 0 && !progs)) return fail(MPS_ERR_ARG, "NULL argument");
  if (n <= 0) return MPS_OK;
  for (int i = 0; i < n; ++i)
    if (!progs[i] || progs[i]->ctx != c) return fail(MPS_ERR_ARG, "program from another context");
  std::lock_guard<std::mutex> lk(c->mu);
  CK(cudaSetDevice(c->device));
  return launch_programs(c, c->lane0, progs, n, false);
}

int mps_wait(mps_prog* p, int timeout_ms) {
  if (!p) return fail(MPS_ERR_ARG, "NULL program");
  CK(cudaSetDevice(p->ctx->device));
  const auto t0 = std::chrono::steady_clock::now();
  for (;;) {
    cudaError_t e = cudaEventQuery(p->ev);
    if (e == cudaSuccess) break;
    if (e != cudaErrorNotReady) return fail(MPS_ERR_CUDA, cudaGetErrorString(e));
    const double el = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    if (timeout_ms >= 0 && el > timeout_ms) return fail(MPS_ERR_TIMEOUT, "program still running");
    std::this_thread::yield();
  }
  return prog_check_err(p);
}

int mps_expect_pauli(mps_prog* p, const char* paulis, int n_terms, const double* coeffs, double* out) {
  if (!p || !paulis || !out || n_terms < 0) return fail(MPS_ERR_ARG, "NULL argument");
  mps_ctx* c = p->ctx;
  std::lock_guard<std::mutex> lk(c->mu);
  CK(cudaSetDevice(c->device));
  int rc = flush_pending(p);
  if (rc) return rc;
  std::vector<uint8_t> codes;
  rc = parse_paulis(p->nq, paulis, n_terms, codes);
  if (rc) return rc;
  if (n_terms == 0) {
    if (coeffs) out[0] = 0.0;
    return MPS_OK;
  }
  if (p->density) {
    // Tr(rho P) / Tr(rho) for every term in one walk of the doubled chain
    std::vector<cx<double>> res;
    rc = density_expect(p, codes.data(), n_terms, res);
    if (rc) return rc;
    const cx<double> tr = res[n_terms];
    const double d = tr.re * tr.re + tr.im * tr.im;
    if (!(d > 0.0)) return fail(MPS_ERR_NUMERIC, "density matrix with zero trace");
    double e = 0.0;
    for (int t = 0; t < n_terms; ++t) {
      const cx<double> v = res[t];
      out[2 * t] = (v.re * tr.re + v.im * tr.im) / d;
      out[2 * t + 1] = (v.im * tr.re - v.re * tr.im) / d;
      if (coeffs) e += coeffs[t] * out[2 * t];
    }
    if (coeffs) out[2 * n_terms] = e;
    return MPS_OK;
  }
  if (prog_is_wide(p)) {
    std::vector<double> res(2 * (size_t)n_terms);
    rc = wide_expect(p, codes.data(), n_terms, res.data());
    if (rc) return rc;
    double e = 0.0;
    for (int t = 0; t < n_terms; ++t) {
      out[2 * t] = res[2 * t];
      out[2 * t + 1] = res[2 * t + 1];
      if (coeffs) e += coeffs[t] * res[2 * t];
    }
    if (coeffs) out[2 * n_terms] = e;
    return prog_check_err(p);
  }
  uint8_t* d_codes = nullptr;
  CK(cudaMalloc(&d_codes, codes.size()));
  CK(cudaMemcpyAsync(d_codes, codes.data(), codes.size(), cudaMemcpyHostToDevice, c->lane0.stream));
  std::vector<ExpTask> tasks(n_terms);
  for (int t = 0; t < n_terms; ++t) {
    tasks[t].sites = p->d_sites;
    tasks[t].site_off = p->d_off;
    tasks[t].bond = p->d_bond;
    tasks[t].codes = d_codes + (size_t)t * p->n;
    tasks[t].n = p->n;
    tasks[t].pad = 0;
  }
  std::vector<double> res(2 * (size_t)n_terms);
  rc = enqueue_expect(c->lane0, tasks, p->prec, res.data());
  if (!rc) {
    cudaError_t e = cudaStreamSynchronize(c->lane0.stream);
    if (e != cudaSuccess) rc = fail(MPS_ERR_CUDA, cudaGetErrorString(e));
  }
  cudaFree(d_codes);
  if (rc) return rc;
  rc = prog_check_err(p);
  if (rc) return rc;
  double e = 0.0;
  for (int t = 0; t < n_terms; ++t) {
    out[2 * t] = res[2 * t];
    out[2 * t + 1] = res[2 * t + 1];
    if (coeffs) e += coeffs[t] * res[2 * t];
  }
  if (coeffs) out[2 * n_terms] = e;
  return MPS_OK;
}

int mps_norm(mps_prog* p, double* out) {
  if (!p || !out) return fail(MPS_ERR_ARG, "NULL argument");
  if (p->density) {
    // the trace of rho
    mps_ctx* c = p->ctx;
    std::lock_guard<std::mutex> lk(c->mu);
    CK(cudaSetDevice(c->device));
    int rc = flush_pending(p);
    if (rc) return rc;
    std::vector<cx<double>> res;
    rc = density_expect(p, nullptr, 0, res);
    if (rc) return rc;
    *out = res[0].re;
    return MPS_OK;
  }
  std::string ids(p->n, 'I');
  double v[2];
  int rc = mps_expect_pauli(p, ids.c_str(), 1, nullptr, v);
  if (rc) return rc;
  *out = v[0];
  return MPS_OK;
}

int mps_set_observable(mps_prog* p, const char* paulis, int n_terms, const double* coeffs) {
  if (!p || n_terms < 0 || (n_terms > 0 && (!paulis || !coeffs))) return fail(MPS_ERR_ARG, "NULL argument");
  if (p->density)
    return fail(MPS_ERR_UNSUPPORTED, "attached observables are for state programs; use mps_expect_pauli");
  std::vector<uint8_t> codes;
  int rc = parse_paulis(p->n, paulis, n_terms, codes);
  if (rc) return rc;
  codes.insert(codes.end(), p->n, 0);  // extra all-identity term: the norm
  std::lock_guard<std::mutex> lk(p->ctx->mu);
  CK(cudaSetDevice(p->ctx->device));
  if (p->d_obs) {
    CK(cudaEventSynchronize(p->ev));
    cudaFree(p->d_obs);
  }
  p->d_obs = nullptr;
  CK(cudaMalloc(&p->d_obs, codes.size()));
  CK(cudaMemcpy(p->d_obs, codes.data(), codes.size(), cudaMemcpyHostToDevice));
  p->obs_coef.assign(coeffs, coeffs + n_terms);
  p->obs_codes = codes;
  p->n_terms = n_terms;
  return MPS_OK;
}

int mps_batch_expect(mps_ctx* c, mps_prog* const* progs, int n, double* out) {
  if (!c || (n > 0 && (!progs || !out))) return fail(MPS_ERR_ARG, "NULL argument");
  std::lock_guard<std::mutex> lk(c->mu);
  CK(cudaSetDevice(c->device));
  std::vector<ExpTask> tasks[2];
  std::vector<std::pair<int, size_t>> where(n);
  for (int i = 0; i < n; ++i) {
    mps_prog* p = progs[i];
    if (!p || p->ctx != c) return fail(MPS_ERR_ARG, "program from another context");
    if (!p->d_obs) return fail(MPS_ERR_STATE, "program has no observable");
    int rc = flush_pending(p);
    if (rc) return rc;
    if (prog_is_wide(p)) continue;
    where[i] = {p->prec, tasks[p->prec].size()};
    observable_tasks(p, tasks[p->prec]);
  }
  std::vector<double> res[2];
  for (int pr = 0; pr < 2; ++pr) {
    res[pr].assign(2 * tasks[pr].size(), 0.0);
    int rc = enqueue_expect(c->lane0, tasks[pr], pr, res[pr].data());
    if (rc) return rc;
    CK(cudaStreamSynchronize(c->lane0.stream));
  }
  for (int i = 0; i < n; ++i) {
    int rc = prog_check_err(progs[i]);
    if (rc) return rc;
    if (prog_is_wide(progs[i])) {
      std::vector<double> r(2 * ((size_t)progs[i]->n_terms + 1));
      rc = wide_expect(progs[i], progs[i]->obs_codes.data(), progs[i]->n_terms + 1, r.data());
      if (rc) return rc;
      out[i] = observable_value(progs[i], r.data());
      continue;
    }
    out[i] = observable_value(progs[i], res[where[i].first].data() + 2 * where[i].second);
  }
  return MPS_OK;
}

int mps_amplitudes(mps_prog* p, double* out) {
  if (!p || !out) return fail(MPS_ERR_ARG, "NULL argument");
  if (p->density) return fail(MPS_ERR_UNSUPPORTED, "a density program has no state vector; use mps_density_matrix");
  if (p->n > MPS_AMP_QUBITS_MAX) return fail(MPS_ERR_UNSUPPORTED, "too many qubits for a full state vector");
  mps_ctx* c = p->ctx;
  std::lock_guard<std::mutex> lk(c->mu);
  CK(cudaSetDevice(c->device));
  int rc = flush_pending(p);
  if (rc) return rc;
  cudaStream_t st = c->lane0.stream;
  const size_t eb = elem_bytes(p->prec);
  const int64_t N = (int64_t)1 << p->n;
  char* buf = nullptr;
  CK(cudaMalloc(&buf, 2 * (size_t)N * eb + (size_t)N * 16));
  char* v0 = buf;
  char* v1 = buf + (size_t)N * eb;
  double* vd = reinterpret_cast<double*>(buf + 2 * (size_t)N * eb);
  std::vector<int> bond(p->n + 1);
  CK(cudaMemcpyAsync(bond.data(), p->d_bond, bond.size() * sizeof(int), cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  char one[16] = {0};
  if (p->prec == MPS_PREC_FP64) {
    const double v = 1.0;
    std::memcpy(one, &v, 8);
  } else {
    const float v = 1.0f;
    std::memcpy(one, &v, 4);
  }
  CK(cudaMemcpyAsync(v0, one, eb, cudaMemcpyHostToDevice, st));
  for (int i = 0; i < p->n; ++i) {
    const char* A = (const char*)p->d_sites + p->off[i] * eb;
    CK(launch_amp_step(p->prec, A, bond[i], bond[i + 1], i, v0, v1, st));
    std::swap(v0, v1);
  }
  CK(launch_to_f64(p->prec, v0, vd, N, st));
  CK(cudaMemcpyAsync(out, vd, (size_t)N * 16, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  cudaFree(buf);
  return prog_check_err(p);
}

int mps_amplitude(mps_prog* p, const int* bits, double out[2]) {
  if (!p || !bits || !out) return fail(MPS_ERR_ARG, "NULL argument");
  if (p->density) return fail(MPS_ERR_UNSUPPORTED, "a density program has no state vector; use mps_density_matrix");
  for (int i = 0; i < p->n; ++i)
    if (bits[i] != 0 && bits[i] != 1) return fail(MPS_ERR_ARG, "bits must be 0 or 1");
  mps_ctx* c = p->ctx;
  std::lock_guard<std::mutex> lk(c->mu);
  CK(cudaSetDevice(c->device));
  int rc = flush_pending(p);
  if (rc) return rc;
  if (prog_is_wide(p)) {
    rc = wide_amp_one(p, bits, out);
    if (rc) return rc;
    return prog_check_err(p);
  }
  cudaStream_t st = c->lane0.stream;
  char* buf = nullptr;
  CK(cudaMalloc(&buf, sizeof(int) * p->n + 16));
  double* d_out = reinterpret_cast<double*>(buf);
  int* d_bits = reinterpret_cast<int*>(buf + 16);
  CK(cudaMemcpyAsync(d_bits, bits, sizeof(int) * p->n, cudaMemcpyHostToDevice, st));
  CK(launch_amp_one(p->prec, p->d_sites, p->d_off, p->d_bond, d_bits, p->n, d_out, st));
  CK(cudaMemcpyAsync(out, d_out, 16, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  cudaFree(buf);
  return prog_check_err(p);
}

int mps_n_measured(mps_prog* p, int* out) {
  if (!p || !out) return fail(MPS_ERR_ARG, "NULL argument");
  *out = p->measured.empty() ? p->nq : (int)p->measured.size();
  return MPS_OK;
}

int mps_sample(mps_prog* p, int shots, uint64_t seed, uint8_t* bits) {
  if (!p || shots < 0 || (shots > 0 && !bits)) return fail(MPS_ERR_ARG, "bad argument");
  if (shots == 0) return MPS_OK;
  mps_ctx* c = p->ctx;
  std::lock_guard<std::mutex> lk(c->mu);
  CK(cudaSetDevice(c->device));
  int rc = flush_pending(p);
  if (rc) return rc;
  if (p->density) return density_sample(p, shots, seed, bits);
  std::vector<uint8_t> all((size_t)shots * p->n);
  if (prog_is_wide(p))
    rc = wide_sample(p, shots, seed, all.data());
  else
    rc = enqueue_sample(c->lane0, p, shots, seed, all.data());
  if (rc) return rc;
  CK(cudaStreamSynchronize(c->lane0.stream));
  rc = prog_check_err(p);
  if (rc) return rc;
  select_measured(p, all.data(), shots, bits);
  return MPS_OK;
}

int mps_stats(mps_prog* p, double out[4]) {
  if (!p || !out) return fail(MPS_ERR_ARG, "NULL argument");
  std::lock_guard<std::mutex> lk(p->ctx->mu);
  CK(cudaSetDevice(p->ctx->device));
  int rc = flush_pending(p);
  if (rc) return rc;
  double st[ST_COUNT];
  CK(cudaMemcpyAsync(st, p->d_stats, sizeof(st), cudaMemcpyDeviceToHost, p->ctx->lane0.stream));
  CK(cudaStreamSynchronize(p->ctx->lane0.stream));
  out[0] = std::exp(st[ST_LOG_FID]);
  out[1] = st[ST_MAX_DISC];
  out[2] = st[ST_N_GATE2];
  out[3] = st[ST_N_OPS];
  return prog_check_err(p);
}

int mps_truncation_fidelity(mps_prog* p, double* out) {
  if (!out) return fail(MPS_ERR_ARG, "NULL argument");
  double st[4];
  int rc = mps_stats(p, st);
  if (rc) return rc;
  *out = st[0];
  return MPS_OK;
}

int mps_diag_cgemm(mps_ctx* c, int M, int N, int K, const double* a, const double* b, double* c_tc, double* c_simt) {
  if (!c || !a || !b || !c_tc || !c_simt || M < 1 || N < 1 || K < 1 || M > 4096 || N > 4096 || K > 4096)
    return fail(MPS_ERR_ARG, "bad argument");
  std::lock_guard<std::mutex> lk(c->mu);
  CK(cudaSetDevice(c->device));
  return wide_diag_cgemm(c, M, N, K, a, b, c_tc, c_simt);
}

int mps_diag_gemm_counts(mps_ctx* c, int* tensor_core, int* cuda_core) {
  if (!c || !tensor_core || !cuda_core) return fail(MPS_ERR_ARG, "NULL argument");
  return wide_gemm_counts(c, tensor_core, cuda_core);
}

int mps_diag_cgemm_kind(mps_ctx* c, int precision, int kernel, int flags, int M, int N, int K, const double* a,
                        const double* b, double* out) {
  if (!c || !a || !b || !out || M < 1 || N < 1 || K < 1 || M > 4096 || N > 4096 || K > 4096 || kernel < 0 ||
      kernel >= MPS_GEMM_KERNELS || (precision != MPS_PREC_FP64 && precision != MPS_PREC_FP32) || flags < 0 ||
      flags > 15)
    return fail(MPS_ERR_ARG, "bad argument");
  if (precision == MPS_PREC_FP64 && kernel == MPS_GEMM_TC)
    return fail(MPS_ERR_ARG, "the tensor-core GEMM takes complex64 only");
  if ((flags & 8) && kernel != MPS_GEMM_TC) return fail(MPS_ERR_ARG, "split-BF16 applies to the tensor-core GEMM");
  std::lock_guard<std::mutex> lk(c->mu);
  CK(cudaSetDevice(c->device));
  return wide_diag_cgemm_kind(c, precision, kernel, flags, M, N, K, a, b, out);
}

int mps_autotune_set_mode(int mode) {
  if (mode < 0 || mode > 2) return fail(MPS_ERR_ARG, "autotune mode must be 0, 1 or 2");
  gemm_tune_set_mode(mode);
  return MPS_OK;
}

int mps_autotune_get_mode(int* mode) {
  if (!mode) return fail(MPS_ERR_ARG, "NULL argument");
  *mode = gemm_tune_mode();
  return MPS_OK;
}

int mps_autotune_table(int* out, int cap, int* n_entries) {
  if (!n_entries || cap < 0 || (cap > 0 && !out)) return fail(MPS_ERR_ARG, "bad argument");
  static_assert(MPS_AUTOTUNE_COLS == kTuneCols, "autotune table row width");
  *n_entries = gemm_tune_table(out, cap);
  return MPS_OK;
}

int mps_autotune_save(const char* path) {
  if (!path) return fail(MPS_ERR_ARG, "NULL argument");
  if (gemm_tune_save(path)) return fail(MPS_ERR_ARG, std::string("cannot write ") + path);
  return MPS_OK;
}

int mps_autotune_load(const char* path) {
  if (!path) return fail(MPS_ERR_ARG, "NULL argument");
  const int rc = gemm_tune_load(path);
  if (rc == 1) return fail(MPS_ERR_ARG, std::string("cannot read ") + path);
  if (rc) return fail(MPS_ERR_ARG, std::string("malformed tuning file ") + path);
  return MPS_OK;
}

int mps_autotune_clear(void) {
  gemm_tune_clear();
  return MPS_OK;
}

int mps_autotune_tunings(mps_ctx* c, int* out) {
  if (!c || !out) return fail(MPS_ERR_ARG, "NULL argument");
  std::lock_guard<std::mutex> lk(c->mu);
  *out = wide_gemm_tunings(c);
  return MPS_OK;
}

int mps_diag_set_coop_rows(int rows_per_cta) { return wide_set_coop_rows(rows_per_cta); }

int mps_diag_set_parallel_width(int max_ctas) {
  if (max_ctas < 0) return fail(MPS_ERR_ARG, "max_ctas must be >= 0");
  g_parallel_width.store(max_ctas);
  return MPS_OK;
}

int mps_bond_dims(mps_prog* p, int* out) {
  if (!p || !out) return fail(MPS_ERR_ARG, "NULL argument");
  std::lock_guard<std::mutex> lk(p->ctx->mu);
  CK(cudaSetDevice(p->ctx->device));
  int rc = flush_pending(p);
  if (rc) return rc;
  std::vector<int> b(p->n + 1);
  CK(cudaMemcpyAsync(b.data(), p->d_bond, b.size() * sizeof(int), cudaMemcpyDeviceToHost, p->ctx->lane0.stream));
  CK(cudaStreamSynchronize(p->ctx->lane0.stream));
  for (int i = 0; i + 1 < p->n; ++i) out[i] = b[i + 1];
  return prog_check_err(p);
}

}  // extern "C"
