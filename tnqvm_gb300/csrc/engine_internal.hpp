// Internal host structures of the GB300 MPS engine.
#pragma once
#include <atomic>
#include <condition_variable>
#include <deque>
#include <map>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "gates.hpp"
#include "mps_common.cuh"

namespace gbmps {

// kernels (k_ops.cu, k_measure.cu)
size_t op_scratch_bytes();
size_t op_smem_bytes();
cudaError_t launch_ops(const ProgDesc* d_progs, int n_progs, int grid, int* d_queue, char* scratch,
                       cudaStream_t st);
cudaError_t launch_ops_sites(const ProgDesc* d_prog, const int2* d_deps, int* d_ctr, int grid, char* scratch,
                             cudaStream_t st);
cudaError_t configure_ops();
cudaError_t configure_expect();
cudaError_t launch_reset(const ProgDesc* d_progs, int n_progs, cudaStream_t st);
size_t expect_smem_bytes(int prec);
size_t expect_scratch_bytes(int prec);
cudaError_t launch_expect(int prec, const ExpTask* d_tasks, int n_tasks, char* scratch, double* d_out,
                          cudaStream_t st);
cudaError_t launch_right_env(int prec, const EnvTask& tk, char* scratch, cudaStream_t st);
cudaError_t launch_sample(int prec, const SampleTask& tk, cudaStream_t st);
cudaError_t launch_amp_step(int prec, const void* A, int dl, int dr, int k, const void* vin, void* vout,
                            cudaStream_t st);
cudaError_t launch_to_f64(int prec, const void* v, double* out, int64_t n, cudaStream_t st);
cudaError_t launch_amp_one(int prec, const void* sites, const int64_t* site_off, const int* bond, const int* bits,
                           int n, double* out, cudaStream_t st);

// A lane is a stream with its own scratch and staging buffers, so work on
// different lanes can overlap on the device.
struct Lane {
  cudaStream_t stream = nullptr;
  char* op_scratch = nullptr;  // per-CTA scratch of the fused op kernel (either precision)
  int op_scratch_ctas = 0;
  char* exp_scratch[2] = {nullptr, nullptr};
  int exp_scratch_ctas[2] = {0, 0};
  DevOp* d_ops = nullptr;
  size_t d_ops_cap = 0;
  ProgDesc* d_desc = nullptr;
  size_t d_desc_cap = 0;
  ExpTask* d_exp_tasks = nullptr;
  size_t d_exp_tasks_cap = 0;
  double* d_exp_out = nullptr;
  size_t d_exp_out_cap = 0;
  char* d_work = nullptr;  // sampler environments, bits, offsets
  size_t d_work_cap = 0;
  int* d_queue = nullptr;
  int* d_dag = nullptr;  // site-parallel runs: per-op dependencies, op counter, per-site counts
  size_t d_dag_cap = 0;
  // pinned host staging
  DevOp* h_ops = nullptr;
  size_t h_ops_cap = 0;
  ProgDesc* h_desc = nullptr;
  size_t h_desc_cap = 0;
};

struct mps_prog_impl;

struct ServeReq {
  uint64_t ticket;
  struct ::mps_prog* prog;
  int shots;
  uint64_t seed;
  double t_submit;
  double t_done;
  int status;
  double energy;
  std::vector<uint8_t> bits;
  bool done;
  // fused completion: observables evaluated by the program's own CTA, results
  // and a done flag in the batch's host-mapped arena
  bool fused = false;
  int* flag = nullptr;       // [0] done, [1] error word
  double* obs = nullptr;     // 2 * (n_terms + 1) doubles
  size_t exp_off = 0;        // first of its observable results in the batch's pinned buffer
  bool in_batch = false;     // still referenced by a running batch
  bool reaped = false;       // polled by the client while in_batch
};

struct ServeBatch {
  int lane;
  std::vector<ServeReq*> reqs;
  cudaEvent_t ev;
  double* h_exp = nullptr;     // pinned, 2 doubles per task
  size_t h_exp_cap = 0;
  std::vector<std::pair<ServeReq*, uint8_t*>> bit_dst;
  uint8_t* h_bits = nullptr;   // pinned
  size_t h_bits_cap = 0;
  int* h_err = nullptr;        // pinned: each request's error word, copied behind the batch
  size_t h_err_cap = 0;
  char* arena = nullptr;       // pinned, mapped: fused requests' flags and observables
  size_t arena_cap = 0;
  size_t footprint = 0;
};

struct ServeState {
  std::thread worker;
  // wide requests (bond cap above the single-CTA limit) run on their own
  // workers, each with its lane and workspace, overlapping the batched lanes
  // and one another
  std::vector<std::thread> wide_workers;
  std::deque<ServeReq*> wide_queue;
  std::condition_variable cv_wide;
  std::vector<Lane> wide_lanes;
  std::vector<void*> wide_ws;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<ServeReq*> queue;
  std::map<uint64_t, ServeReq*> all;
  std::vector<Lane> lanes;
  std::vector<ServeBatch> batches;  // one slot per lane
  std::vector<char> lane_busy;
  uint64_t next_ticket = 1;
  bool stop = false;
  bool running = false;
  int max_inflight = 256;
  size_t inflight_bytes = 0;
  int inflight_reqs = 0;
};

}  // namespace gbmps

struct mps_ctx {
  int device = 0;
  int num_sms = 0;
  size_t budget = 0;
  size_t resident = 0;
  std::mutex mu;
  gbmps::Lane lane0;
  gbmps::ServeState* serve = nullptr;
  void* wide = nullptr;  // workspace of the wide two-site path (wide.cu)
};

struct mps_prog {
  mps_ctx* ctx = nullptr;
  int n = 0, chi_cap = 0, mode = 0, prec = 0, flags = 0;
  // qubits of the register: n for a state, n / 2 for a density program
  // (MPS_FLAG_DENSITY: ket of qubit q on site 2q, bra on site 2q + 1)
  int nq = 0;
  bool density = false;
  int prec_mode = 0;        // the precision requested at begin (MPS_PREC_*), reported back
  bool split_bf16 = false;  // wide-path tensor-core products with bf16 hi/lo operands
  double cutoff = 0.0;
  std::vector<gbmps::GateRec> pending;
  std::vector<int> measured;
  std::vector<int> cap_bond;
  std::vector<int64_t> off;
  size_t bytes = 0;
  void* d_sites = nullptr;
  char* d_meta = nullptr;
  double* d_stats = nullptr;
  int64_t* d_off = nullptr;
  int* d_bond = nullptr;
  int* d_err = nullptr;
  cudaEvent_t ev = nullptr;
  bool submitted = false;
  int center = 0;
  uint8_t* d_obs = nullptr;
  std::vector<double> obs_coef;
  std::vector<uint8_t> obs_codes;  // host copy of the observable (wide programs)
  int n_terms = 0;
  std::vector<int> hbond;  // host mirror of the bond dimensions (wide programs)
  // set by the serve loop for one launch: evaluate the observable in the
  // update kernel and signal completion through host-mapped memory
  double* serve_obs = nullptr;
  int* serve_flag = nullptr;
};

namespace gbmps {
extern thread_local std::string g_err;
int fail(int code, const std::string& msg);
size_t footprint(int n, int chi, int prec);
void compile_program(::mps_prog* p, std::vector<DevOp>& ops);
void site_schedule(const std::vector<DevOp>& ops, int n_sites, std::vector<DevOp>& sorted, std::vector<int>& deps);
int lane_init(Lane& L, int priority = 0);
void lane_free(Lane& L);
int launch_programs(mps_ctx* c, Lane& L, ::mps_prog* const* progs, int n, bool per_gate);
double program_cost(const ::mps_prog* p, const DevOp* ops, size_t n_ops, bool with_obs);
int enqueue_expect(Lane& L, const std::vector<ExpTask>& tasks, int prec, double* h_out);
int enqueue_sample(Lane& L, ::mps_prog* p, int shots, uint64_t seed, uint8_t* h_all_bits);
int prog_check_err(::mps_prog* p);
int parse_paulis(int n, const char* paulis, int n_terms, std::vector<uint8_t>& codes);
void select_measured(const ::mps_prog* p, const uint8_t* all, int shots, uint8_t* bits);
void observable_tasks(::mps_prog* p, std::vector<ExpTask>& tasks);
double observable_value(const ::mps_prog* p, const double* r);
// wide path (wide.cu): bond caps above the single-CTA limit
bool prog_is_wide(const ::mps_prog* p);
// ws: the wide workspace to use (nullptr: the context's); L: the lane whose
// stream runs the work (nullptr: the context's lane 0)
int wide_run(mps_ctx* c, Lane& L, ::mps_prog* p, void** ws = nullptr);
int wide_expect(::mps_prog* p, const uint8_t* codes, int n_terms, double* out, Lane* L = nullptr,
                void** ws = nullptr);
int wide_sample(::mps_prog* p, int shots, uint64_t seed, uint8_t* h_all_bits, Lane* L = nullptr,
                void** ws = nullptr);
void wide_ws_free(void** ws);
int wide_amp_one(::mps_prog* p, const int* bits, double* out);
int wide_gemm_counts(mps_ctx* c, int* tc, int* simt);
int wide_diag_cgemm(mps_ctx* c, int M, int N, int K, const double* a, const double* b, double* out_tc,
                    double* out_simt);
int wide_diag_cgemm_kind(mps_ctx* c, int prec, int kind, int flags, int M, int N, int K, const double* a,
                         const double* b, double* out);
int wide_gemm_tunings(mps_ctx* c);
int wide_set_coop_rows(int rows);
void wide_free(mps_ctx* c);
// density programs: a gate recorded on qubits (engine.cu), a single-qubit
// Kraus channel as the two-site superoperator on (2q, 2q+1) (density.cu)
void record_gate(::mps_prog* p, const GateRec& g);
int kraus_superop(int qubit, int n_kraus, const double* kraus, GateRec& g);
int density_expect(::mps_prog* p, const uint8_t* codes, int n_terms, std::vector<cx<double>>& res);
int density_sample(::mps_prog* p, int shots, uint64_t seed, uint8_t* bits);
}  // namespace gbmps
