/*
 * gb300mps.h - C ABI of the GB300 matrix-product-state circuit engine.
 *
 * The engine replaces the numerical layer of TNQVM's MPS visitors: the
 * per-gate loop of ExatnMpsVisitor (tnqvm/visitors/exatn-mps/ExaTnMpsVisitor.cpp)
 * and ITensorMPSVisitor (tnqvm/visitors/itensor/mps/ITensorMPSVisitor.cpp).
 * A C++ TNQVMVisitor plugin (tnqvm/visitors/TNQVMVisitor.hpp:58-82) records
 * gates through this ABI and reads results back; nothing in these signatures
 * is a C++ or torch type.  Every entry point returns an MPS_* status; on a
 * non-zero status mps_last_error() describes the failure (thread-local).
 *
 * Conventions
 *  - complex numbers are interleaved (re, im) doubles;
 *  - a 1-qubit matrix is 2x2 row-major (8 doubles);
 *  - a 2-qubit matrix is 4x4 row-major (32 doubles) and its first qubit
 *    argument is the most significant bit of the row/column index, as in
 *    tnqvm/base/Gates.hpp:238-246 (CNOT) and ExatnUtils.cpp:116-130;
 *  - amplitude index bit q is qubit q (ExaTnMpsVisitor.cpp:616-634);
 *  - sampled bit strings list qubits in Measure order
 *    (tnqvm/utils/GateMatrixAlgebra.hpp:129-137).
 */
#ifndef GB300MPS_H
#define GB300MPS_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define MPS_OK 0
#define MPS_ERR_ARG 1         /* invalid argument (xacc::error in the reference) */
#define MPS_ERR_OOM 2         /* device memory or admission budget exhausted */
#define MPS_ERR_TIMEOUT 3     /* mps_wait / serve poll ran out of time */
#define MPS_ERR_NUMERIC 4     /* NaN/Inf or a failed numerical invariant */
#define MPS_ERR_CUDA 5        /* CUDA runtime error */
#define MPS_ERR_STATE 6       /* call out of order (e.g. measuring before submit) */
#define MPS_ERR_UNSUPPORTED 7 /* size beyond what this build supports */

/* truncation semantics */
#define MPS_TRUNC_EXATN 0   /* ExaTnMpsVisitor.cpp:2366-2536: absolute per-index cut, sqrt(S) both sides */
#define MPS_TRUNC_ITENSOR 1 /* ITensor decomp.cc:307-463: relative discarded weight, canonical form */

/* arithmetic */
#define MPS_PREC_FP64 0 /* complex128 storage and arithmetic */
#define MPS_PREC_FP32 1 /* complex64 storage and arithmetic, FP64 reductions */
/* complex128 for a register of at most MPS_AUTO_FP64_QUBITS qubits whose bond
 * cap is at least 2^floor(n/2) (the state is exact at that cap), complex64
 * otherwise.  On small registers Pauli expectation values are O(1), and the
 * rounding of complex64 arithmetic over a few hundred gates reaches ~1e-6 in
 * a 50-term energy; those registers are also the cheapest to run in
 * complex128.  A batch may mix the two (one persistent launch).  No
 * counterpart in the reference (FP64 throughout). */
#define MPS_PREC_AUTO 2
#define MPS_AUTO_FP64_QUBITS 12
/* complex64 storage; the wide path's (bond caps above MPS_CHI_LIMIT)
 * tensor-core products take bf16 operands split into head and remainder
 * (three products, FP32 accumulation, ~1e-5 relative per product) at twice
 * the TF32 rate; programs with caps <= MPS_CHI_LIMIT run as MPS_PREC_FP32.
 * No counterpart in the reference. */
#define MPS_PREC_SPLIT_BF16 3

/* program flags */
#define MPS_FLAG_RENORM 1   /* rescale the kept part to the pre-truncation norm */
#define MPS_FLAG_PER_GATE 2 /* one kernel launch per gate (the plain visitor path) */
#define MPS_FLAG_SWEEP 4    /* itensor semantics: reorder gates on disjoint qubits so the
                               orthogonality centre takes the shortest path (no reference
                               counterpart; truncations then happen in another order) */
#define MPS_FLAG_FUSE 8     /* drop routed SWAP pairs that cancel (SWAP, 1-qubit gates on the
                               pair, SWAP) and multiply consecutive 2-qubit gates on the same
                               pair into one split (no reference counterpart: the reference
                               splits after every routed SWAP; exact in exact arithmetic,
                               fewer truncations otherwise) */
#define MPS_FLAG_DENSITY 16 /* noisy circuits: the program holds the density matrix rho of
                               n_qubits qubits as a vectorised MPS on 2 * n_qubits sites (ket
                               of qubit q on site 2q, bra on site 2q+1); see mps_channel1 */
#define MPS_FLAG_PARALLEL 32 /* a program submitted alone (mps_submit) runs its two-site updates
                               on disjoint sites on different SMs at once, in one launch;
                               each update computes what it computes in program order, so
                               results are unchanged.  Exatn semantics (no centre moves)
                               leaves many updates independent; itensor semantics chains
                               them through the orthogonality centre.  No counterpart in
                               the reference. */

/* largest bond dimension the single-CTA gate kernel handles */
#define MPS_CHI_LIMIT 64
/* largest bond cap of a program; caps above MPS_CHI_LIMIT run the wide
 * two-site path (tensor-core GEMMs, cooperative eigensolver and QR) */
#define MPS_WIDE_CHI_LIMIT 1024
/* largest qubit count for mps_amplitudes */
#define MPS_AMP_QUBITS_MAX 26
/* largest selections of mps_density_matrix (4^k entries) and of
 * mps_density_diag and density-program sampling (2^k entries) */
#define MPS_DM_QUBITS_MAX 13
#define MPS_DIAG_QUBITS_MAX 24

typedef struct mps_ctx mps_ctx;
typedef struct mps_prog mps_prog;

typedef struct mps_cfg {
  int device;               /* CUDA device ordinal */
  size_t hbm_budget_bytes;  /* admission budget for resident MPS state (0 = 150 GB) */
} mps_cfg;

const char* mps_last_error(void);
const char* mps_version(void);

/* Context: owns the stream, scratch and every program's device memory.
 * Replaces exatn::initialize (ExaTnMpsVisitor.cpp:187-255). */
int mps_ctx_create(const mps_cfg* cfg, mps_ctx** out);
int mps_ctx_destroy(mps_ctx* ctx);
int mps_ctx_info(mps_ctx* ctx, int* num_sms, size_t* bytes_resident);

/* Program = one MPS register plus the gates recorded on it.
 * Replaces ExatnMpsVisitor::initialize (ExaTnMpsVisitor.cpp:173-345) and
 * ITensorMPSVisitor::initialize (ITensorMPSVisitor.cpp:105-157):
 * |0...0> with every bond of dimension 1.  chi_max <= 0 means "no cap"
 * (clamped to MPS_CHI_LIMIT); caps up to MPS_WIDE_CHI_LIMIT are accepted,
 * those above MPS_CHI_LIMIT run gate by gate on the wide path (not with
 * MPS_FLAG_PER_GATE or in captured graphs).  cutoff < 0 selects
 * the visitor's default (DBL_MIN for exatn, 1e-6 for itensor). */
int mps_program_begin(mps_ctx* ctx, int n_qubits, int chi_max, double cutoff,
                      int trunc_mode, int precision, int flags, mps_prog** out);
int mps_program_reset(mps_prog* p); /* back to |0...0>, keeps the allocation */
/* the precision the program runs in (MPS_PREC_AUTO resolved at begin;
 * MPS_PREC_SPLIT_BF16 reported as such) */
int mps_program_precision(mps_prog* p, int* out);
int mps_program_destroy(mps_prog* p);

/* Gate recording.  Replaces the per-gate visit()/applyGate of
 * ExaTnMpsVisitor.cpp:1185-1292 (1 qubit) and :1387-1730 (2 qubits).
 * mps_gate2 accepts any pair of distinct qubits; non-adjacent pairs are
 * routed with SWAPs as NearestNeighborTransform.hpp:43-135 does.
 * mps_gate_named takes an XACC gate name (Gates.hpp:41-67 list, plus "CX",
 * "U3", "S", "Sdg", "RZZ") and its parameters. */
int mps_gate1(mps_prog* p, int qubit, const double m[8]);
int mps_gate2(mps_prog* p, int q0, int q1, const double m[32]);
int mps_gate_named(mps_prog* p, const char* name, const int* qubits, int n_qubits,
                   const double* params, int n_params);
int mps_measure(mps_prog* p, int qubit); /* ExaTnMpsVisitor.cpp:991-994 */
/* Bulk recording: gate ids follow tnqvm::CommonGates (Gates.hpp:41-67),
 * extended with MPS_G_RZZ; qubits holds 2 ints per gate (second ignored for
 * 1-qubit gates), params 3 doubles per gate (unused ones ignored). */
enum {
  MPS_G_I = 0, MPS_G_H, MPS_G_CNOT, MPS_G_RX, MPS_G_RY, MPS_G_RZ, MPS_G_SWAP, MPS_G_U, MPS_G_X, MPS_G_Y,
  MPS_G_Z, MPS_G_MEASURE, MPS_G_CZ, MPS_G_CPHASE, MPS_G_S, MPS_G_SDG, MPS_G_T, MPS_G_TDG, MPS_G_CY,
  MPS_G_CH, MPS_G_CRZ, MPS_G_ISWAP, MPS_G_FSIM, MPS_G_RZZ, MPS_G_COUNT
};
int mps_gates(mps_prog* p, int n_gates, const int32_t* ids, const int32_t* qubits, const double* params);
/* The same for many programs in one call (e.g. new parameters for every
 * circuit of a batch): program i records gates first_gate[i] ..
 * first_gate[i+1]-1 of the concatenated arrays (first_gate has n_progs+1
 * entries); programs are recorded on host threads, so each may appear only
 * once (MPS_ERR_ARG otherwise).  On failure the first failing program is
 * reported and the others have recorded their gates. */
int mps_gates_many(int n_progs, mps_prog* const* progs, const int64_t* first_gate, const int32_t* ids,
                   const int32_t* qubits, const double* params);

/* Execution.  mps_submit compiles the gates recorded since the previous
 * submit (routing, 1-qubit fusion, gauge moves) and enqueues them; the MPS
 * stays resident on the device across submits. */
int mps_submit(mps_prog* p);
int mps_wait(mps_prog* p, int timeout_ms);
/* One persistent launch over many programs (circuits of any size/bond cap). */
int mps_batch_submit(mps_ctx* ctx, mps_prog* const* progs, int n_progs);

/* Results.  Replace finalize (ExaTnMpsVisitor.cpp:576-681), the state-vector
 * contraction (:591-597), exp-val-z (:616-644) and ITensor's transfer-matrix
 * expectation (ITensorMPSVisitor.cpp:173-250,440-464). */
int mps_norm(mps_prog* p, double* out);                    /* <psi|psi> */
int mps_amplitudes(mps_prog* p, double* out);              /* 2 * 2^n doubles */
int mps_amplitude(mps_prog* p, const int* bits, double out[2]); /* one bit string */
/* paulis: n_terms strings of n_qubits characters from "IXYZ", character i
 * acting on qubit i, concatenated.  out: 2*n_terms doubles (<P_t> re,im,
 * unnormalised), then, if coeffs != NULL, sum_t coeffs[t]*Re<P_t>. */
int mps_expect_pauli(mps_prog* p, const char* paulis, int n_terms,
                     const double* coeffs, double* out);
/* Observable attached to a program, evaluated for many programs at once by
 * mps_batch_expect (out[i] = sum_t c_t Re<P_t>/<psi|psi> for program i). */
int mps_set_observable(mps_prog* p, const char* paulis, int n_terms, const double* coeffs);
int mps_batch_expect(mps_ctx* ctx, mps_prog* const* progs, int n_progs, double* out);
/* Shot sampling from the MPS with a counter-based RNG; bits is
 * shots * n_measured bytes (0/1); without Measure records every qubit is
 * measured in order.  Replaces getMeasureSample (ExaTnMpsVisitor.cpp:2211-2364)
 * and GenerateSamples (GateMatrixAlgebra.hpp:125-156). */
int mps_sample(mps_prog* p, int shots, uint64_t seed, uint8_t* bits);
int mps_n_measured(mps_prog* p, int* out);
/* product over 2-qubit gates of (1 - discarded weight fraction) */
int mps_truncation_fidelity(mps_prog* p, double* out);
int mps_bond_dims(mps_prog* p, int* out); /* sites-1 ints (2*n_qubits-1 for density programs) */
int mps_stats(mps_prog* p, double out[4]); /* fidelity, max discarded, #2q gates, #ops */

/* Noisy circuits (programs begun with MPS_FLAG_DENSITY).  Replace the
 * purified-MPS visitor exatn-pmps (visitors/exatn-mpo/ExaTnPmpsVisitor.cpp):
 * its gates (:820-885) are recorded with the same calls as for a state
 * (rho -> U rho U^H), and mps_channel1 replaces applyKrausOp /
 * applyLocalKrausOp (:887-1130): rho -> sum_k K_k rho K_k^H on one qubit,
 * kraus = n_kraus 2x2 matrices of interleaved (re, im) doubles, row-major
 * (like the reference, channels act on one qubit; convertNoiseChannel
 * :797-818 drops the others).  The results replace finalize (:658-795):
 *   mps_density_matrix  rho reduced to the selected qubits (the others
 *                       traced out), 2^k x 2^k complex, row-major, row =
 *                       ket, bit a of an index = qubits[a]; not normalised
 *                       (its trace is Tr rho); k <= MPS_DM_QUBITS_MAX
 *   mps_density_diag    its diagonal (2^k doubles), k <= MPS_DIAG_QUBITS_MAX
 *   mps_expect_pauli    Tr(rho P) / Tr(rho) per string (same arguments)
 *   mps_norm            Tr(rho)
 *   mps_sample          shots drawn from the diagonal of rho reduced to the
 *                       measured qubits (readout errors are the caller's)
 * State-only calls (amplitudes, attached observables, captured graphs, the
 * serve loop) return MPS_ERR_UNSUPPORTED for density programs; channels on
 * a state program return MPS_ERR_STATE. */
int mps_channel1(mps_prog* p, int qubit, int n_kraus, const double* kraus);
int mps_density_matrix(mps_prog* p, int n_sel, const int* qubits, double* out);
int mps_density_diag(mps_prog* p, int n_sel, const int* qubits, double* out);

/* Captured batch (CUDA graph).  mps_graph_create consumes the gates recorded
 * on each program and captures: reset to |0...0>, one persistent launch over
 * all programs, the attached observables, and the copy of the energies to
 * host.  mps_graph_launch replays it (energies[i] as in mps_batch_expect);
 * mps_graph_update re-reads newly recorded gates of the same structure
 * (e.g. new VQE parameters) into the captured op table. */
typedef struct mps_graph mps_graph;
int mps_graph_create(mps_ctx* ctx, mps_prog* const* progs, int n_progs, mps_graph** out);
int mps_graph_launch(mps_graph* g, double* energies);
int mps_graph_launch_async(mps_graph* g);
int mps_graph_sync(mps_graph* g, double* energies);
int mps_graph_update(mps_graph* g);
int mps_graph_stream(mps_graph* g, void** cuda_stream);
/* Device time of the last replay from CUDA events captured in the graph:
 * out[0] reset + fused op kernel (each program's observable is evaluated by
 * its CTA after its gates), out[1] copy of the results, in ms; out[2]
 * algorithmic GEMM-class flops of the op kernel (theta merge + gate + Gram +
 * split, eigensolver excluded), out[3] eigensolver (Householder) flops, out[4]
 * bytes of the op table copied to the device by mps_graph_update, out[5]
 * bytes copied back per replay. */
int mps_graph_timing(mps_graph* g, double out[6]);
/* SM clock cycles of the last replay, summed over all programs, per phase of
 * the fused update: out[0] theta, out[1] Gram, out[2] eigensolver, out[3]
 * truncation + split, out[4] centre moves. */
int mps_graph_phase_cycles(mps_graph* g, double out[5]);
/* Per-program statistics of the last replay summed over the graph's programs,
 * slots 0..n-1 (n <= 17): 0 sum log(1 - discarded fraction), 1 largest
 * discarded fraction (summed), 2 two-site splits, 3 ops, 4 GEMM-class flops,
 * 5 eigensolver flops, 6-10 the phase cycles of mps_graph_phase_cycles, 11
 * splits whose small-eigenvalue block was re-solved, 12-14 eigensolver cycles
 * in tridiagonalisation, bisection and eigenvector formation, 15 cycles of
 * orthonormalisation and the subspace step, 16 cycles of the attached
 * observables (the Pauli sweeps after the gates).  Diagnostics of this
 * engine; no counterpart in the reference. */
int mps_graph_stat_sums(mps_graph* g, double* out, int n);
int mps_graph_destroy(mps_graph* g);

/* Continuous-batching request loop (serving).  Requests are programs that
 * have recorded gates and optionally an observable and a shot count; the
 * loop admits them by projected HBM footprint, runs them in overlapping
 * persistent launches and completes them out of order.  Requests whose bond
 * cap exceeds MPS_CHI_LIMIT run one at a time on a separate wide lane that
 * overlaps the batches. */
int mps_serve_start(mps_ctx* ctx, int max_inflight);
int mps_serve_submit(mps_ctx* ctx, mps_prog* p, int shots, uint64_t seed, uint64_t* ticket);
/* Polls a ticket: returns MPS_OK when done (result written), MPS_ERR_TIMEOUT
 * if not finished within timeout_ms. energy may be NULL; bits (shots*n_meas)
 * may be NULL. */
int mps_serve_poll(mps_ctx* ctx, uint64_t ticket, int timeout_ms, double* energy,
                   uint8_t* bits, double* latency_ms);
int mps_serve_stop(mps_ctx* ctx);

/* Allocation-free two-site update.  No counterpart in the reference: TNQVM's
 * visitors always allocate through ExaTN/ITensor.  It exists for callers that
 * cannot call cudaMalloc: a plugin inside a host application whose device
 * memory belongs to that application's own pool allocator (reserved up front,
 * so a cudaMalloc fails or is forbidden), or a process under a fixed
 * device-memory cap.  It allocates nothing (no cudaMalloc/cudaFree, no
 * allocating library call); its scratch is one file-scope device array of
 * 256 B + 512 KiB that every GPU which loads this library holds until the
 * process exits.
 *
 * The caller owns all inputs and outputs, in device memory:
 *   sites      element buffer (complex128 or complex64 by precision) holding
 *              the lo site (dl x 2 x dm, row-major) at element 0 and the hi
 *              site (dm x 2 x dr) at element hi_offset; both are overwritten
 *              in place with (dl x 2 x k) and (k x 2 x dr), so each region
 *              needs room for k = min(2*dl, 2*dr, chi_max) on the new bond;
 *   d_bonds    3 ints {dl, dm, dr}; d_bonds[1] receives k;
 * and on the host: bonds (the same 3 ints, checked against the limit), the
 * 4x4 gate (row = 2*phys(lo) + phys(hi)) and the stream to run on.
 * exatn semantics split sqrt(S) onto both sites; itensor semantics leave the
 * lo site left-isometric (the caller keeps the orthogonality centre on the
 * pair).  Bonds above 64 are rejected with MPS_ERR_UNSUPPORTED, and a
 * hi_offset below 2*dl*max(dm, min(2*dl, 2*dr, chi_max)) (the hi site would
 * overlap the lo site) with MPS_ERR_ARG.  The first call on a device looks up
 * the array's device address and sets the kernel's shared-memory limit, so
 * make that first call before any stream capture.  Each call waits for its
 * kernel and reads the error word back, so it synchronises the stream.
 * Every call shares the one array, so two calls that overlap on the GPU (e.g.
 * issued from two host threads on two streams) race on it. */
int mps_gate2_apply_noalloc(int precision, int trunc_mode, int chi_max, double cutoff, void* sites,
                            int64_t hi_offset, int* d_bonds, const int* bonds, const double gate[32],
                            void* cuda_stream);

/* Diagnostics of the wide path; no counterpart in the reference.
 * mps_diag_cgemm: one complex64 product C = A B (M x K times K x N, host
 * arrays of interleaved doubles, row-major) on the tensor-core kernel (c_tc)
 * and on the CUDA-core kernel (c_simt).  mps_diag_gemm_counts: launches of
 * each GEMM kernel by the wide path of this context so far. */
int mps_diag_cgemm(mps_ctx* ctx, int M, int N, int K, const double* a, const double* b, double* c_tc,
                   double* c_simt);
int mps_diag_gemm_counts(mps_ctx* ctx, int* tensor_core, int* cuda_core);

/* GEMM autotuner of the wide path; no counterpart in the reference (its
 * contractions go through ExaTN or ITensor/LAPACK, which pick their own
 * kernels).  Every complex product of the wide path can run on one of these
 * kernels: */
#define MPS_GEMM_SIMT_64x64 0 /* CUDA cores, 64 x 64 complex outputs per CTA */
#define MPS_GEMM_SIMT_32x32 1 /* CUDA cores, 32 x 32 */
#define MPS_GEMM_SIMT_16x64 2 /* CUDA cores, 16 rows x 64 columns (short, wide outputs) */
#define MPS_GEMM_SIMT_64x16 3 /* CUDA cores, 64 rows x 16 columns (tall, thin outputs) */
#define MPS_GEMM_TC 4         /* complex64 only: tcgen05 3xTF32, 128 x 64 complex per CTA */
#define MPS_GEMM_KERNELS 5
/* Modes: 0 a static rule (tensor cores for complex64 products of at least
 * ~2M complex MACs, else 64 x 64 tiles); 1 tune: the first product of each
 * new bucket (device, precision, ceil(log2) of M, N and K, and which index
 * of A, B and C is unit-stride) times every kernel that can take it on the
 * caller's stream, writing a scratch output (the inputs are only read), then
 * uses the fastest unless the static rule is within 5 %; 2 use tuned or
 * loaded entries only.  The CUDA-core tiles give bit-identical results; the
 * tensor-core kernel differs from them by FP32 rounding (~1e-6 relative).
 * Tuning synchronises the stream and allocates a 64 MiB scratch buffer per
 * workspace once, so it is skipped inside a stream capture.  The initial
 * mode comes from the environment variable GB300MPS_AUTOTUNE (default 1).
 * The table is process-wide.  For run-to-run identical complex64 results use
 * mode 0, or mode 2 with a loaded table. */
#define MPS_AUTOTUNE_COLS 9
int mps_autotune_set_mode(int mode);
int mps_autotune_get_mode(int* mode);
/* Rows of MPS_AUTOTUNE_COLS ints: device, precision, ceil(log2) of M, N and K,
 * layout bits (1 A's rows unit-stride, 2 B's columns, 4 C's rows), chosen
 * kernel, its time per launch in ns, the static rule's time in ns.  Writes at
 * most cap rows; *n_entries receives the table size. */
int mps_autotune_table(int* out, int cap, int* n_entries);
/* Text cache of the table (one line per bucket), so a later process can
 * start from it in mode 2 without trial launches. */
int mps_autotune_save(const char* path);
int mps_autotune_load(const char* path);
int mps_autotune_clear(void);
/* Buckets tuned by this context's wide workspaces so far. */
int mps_autotune_tunings(mps_ctx* ctx, int* out);
/* One product C = A B (host arrays of interleaved doubles, row-major) on a
 * chosen kernel; flags bit 0/1/2 store A/B/C column-major on the device, bit
 * 3 runs the tensor-core kernel with split-BF16 operands. */
int mps_diag_cgemm_kind(mps_ctx* ctx, int precision, int kernel, int flags, int M, int N, int K, const double* a,
                        const double* b, double* out);

/* Diagnostic; no counterpart in the reference.  Peak fused multiply-add
 * rate of the CUDA cores of `device` in one precision (MPS_PREC_FP32 or
 * MPS_PREC_FP64), in flops/s (an FMA counts 2), from a probe kernel of
 * independent FMA chains on every SM timed with CUDA events: the roofline
 * denominator of the kernels that run on CUDA cores. */
int mps_diag_fma_rate(int device, int precision, double* flops_per_s);
/* Diagnostic: most CTAs a site-parallel run (MPS_FLAG_PARALLEL) may use,
 * process-wide (0 = as many as the program's sites allow, the default).
 * With 1 the run executes its ops one after another on the same kernel,
 * the bit-for-bit reference of a wider run.  No counterpart in the
 * reference. */
int mps_diag_set_parallel_width(int max_ctas);
/* Diagnostic: rows (eigensolver) or columns (QR) per CTA of the wide path's
 * cooperative launches, process-wide (0 = the default, 8).  More rows per
 * CTA mean fewer CTAs and cheaper grid barriers, less parallel work per
 * column.  No counterpart in the reference. */
int mps_diag_set_coop_rows(int rows_per_cta);

/* Footprint used by admission: sum over sites of chi_l * 2 * chi_r * bytes. */
size_t mps_footprint_bytes(int n_qubits, int chi_max, int precision);

#ifdef __cplusplus
}
#endif
#endif /* GB300MPS_H */
