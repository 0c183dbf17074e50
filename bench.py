"""Benchmark of the GB300 MPS engine on the batched-VQE workload.

Workload (one "step"): 1024 hardware-efficient-ansatz circuits (qubits
uniform in 8..32, layers uniform in 4..12, Ry/Rz per qubit + CNOT ladder,
max bond dimension 64, canonical truncation), each measured on its own
random 50-term Pauli Hamiltonian.  Synthetic, seeded inputs of those shapes.

``value``: circuits/s of the captured batch (reset + one persistent fused
launch that also evaluates each circuit's Hamiltonian + copy of the
energies) replayed with the op table
already in HBM, timed with CUDA events on the replay stream.
``e2e``: circuits/s through the public API from host buffers: bulk gate
recording, op-table update (host->device) and replay with the energies copied
back, wall-clock per step.

``--impl reference`` times the CPU oracle (complex128 numpy MPS with LAPACK
SVD, the reference's itensor-mps arithmetic) on a bounded sample of the
same workload with all host threads.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "circuits/s + p50/p99 latency at |dE|<=1e-6 (FP64 oracle), batched vs plain MPS"
UNIT = "circuits/s"
CHI = 64
CUTOFF = 1e-12
WORKLOAD = ("vqe-batch: 1024 HEA circuits, n~U{8..32}, layers~U{4..12}, Ry/Rz + CNOT ladder, "
            "chi<=64, 50-term Pauli Hamiltonians")


def env_int(k, d):
    try:
        return int(os.environ.get(k, d))
    except ValueError:
        return d


def replica_seed(rank):
    """Seed of a rank's shard of the batch: each rank simulates its own
    circuits (replicas; no collective on the data path)."""
    return 2024 + rank


def max_over_ranks(ms, dist, device):
    """The slowest rank's time: the whole job ends with it."""
    if dist is None:
        return ms
    import torch
    t = torch.tensor([ms], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_throughput(instances_per_rank, world, ms):
    """Whole-job circuits/s: every rank's circuits over the slowest rank's time."""
    return instances_per_rank * world / (ms / 1e3)


def build_locked():
    import fcntl
    from tnqvm_gb300 import build as B
    os.makedirs(B.OUT, exist_ok=True)
    with open(os.path.join(B.OUT, ".build.lock"), "w") as f:
        fcntl.flock(f, fcntl.LOCK_EX)
        B.build()
        fcntl.flock(f, fcntl.LOCK_UN)


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "measured"
    except (OSError, ValueError):
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0,
                "sm_max_mhz": 2070.0}, "fallback"


class Clocks:
    """nvidia-smi sampling during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        rows = []
        with open(self.path) as f:
            for line in f:
                parts = [x.strip() for x in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        os.unlink(self.path)
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower().startswith("active")})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def stratified(insts, stride):
    """Every stride-th instance in order of cost (qubits x layers): a fixed
    subset that covers the batch's cost range."""
    order = np.argsort([it["n"] * it["layers"] for it in insts], kind="stable")
    return [int(i) for i in order[::stride]]


def run_reference(args):
    """The reference arm: the CPU oracle (complex128 numpy MPS with LAPACK
    SVD, the itensor-mps arithmetic) on every host core, one circuit per
    worker process, each step the same fixed 1/8 cost-stratified subset of the
    batch the GPU arm runs."""
    rank = env_int("RANK", 0)
    if rank != 0:
        return 0
    from oracle.pool import OraclePool
    from tnqvm_gb300 import circuits
    insts = circuits.vqe_batch(args.instances, seed=replica_seed(0))
    stride = max(1, args.ref_stride)
    sub = [insts[i] for i in stratified(insts, stride)]
    times = []
    with OraclePool() as pool:
        cores = pool.workers
        for step in range(args.warmup + args.steps):
            _, wall, _ = pool.energies(sub, CHI, CUTOFF)
            if step >= args.warmup:
                times.append(wall)
    ms = 1e3 * float(np.mean(times))
    value = len(sub) / (ms / 1e3)
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "c128", "data": "synthetic",
        "config": {"workload": WORKLOAD, "instances": args.instances, "instances_per_step": len(sub),
                   "subset": "every %dth circuit of the batch in order of cost (fixed, same each step)" % stride,
                   "chi_max": CHI, "truncation": "itensor (canonical, relative cutoff %g)" % CUTOFF},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": "%d of the %d circuits (1/%d, cost-stratified) per step, one circuit per worker "
                                   "process on %d processes; numpy complex128 MPS with LAPACK SVD"
                                   % (len(sub), args.instances, stride, cores)},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


def run_ours(args):
    rank, world, local = env_int("RANK", 0), env_int("WORLD_SIZE", 1), env_int("LOCAL_RANK", 0)
    dist = None
    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    build_locked()
    import torch
    from tnqvm_gb300 import circuits
    from tnqvm_gb300 import mps as M

    ctx = M.Context(local)
    # CUDA-core FMA peaks of this GPU (the bound of the fused kernel)
    rates = {"fp32_tflops": M.fma_rate(local, M.PREC_FP32) / 1e12,
             "fp64_tflops": M.fma_rate(local, M.PREC_FP64) / 1e12}
    rates["fp32_over_fp64"] = rates["fp32_tflops"] / rates["fp64_tflops"]
    insts = circuits.vqe_batch(args.instances, seed=replica_seed(rank), qmin=args.qmin, qmax=args.qmax,
                               lmax=args.lmax)
    t_enc = time.perf_counter()
    enc = [M.encode_circuit(it["circuit"]) for it in insts]
    encode_ms = 1e3 * (time.perf_counter() - t_enc)
    progs = []
    for it, e in zip(insts, enc):
        p = M.Program(ctx, it["n"], CHI, CUTOFF, M.TRUNC_ITENSOR, M.PREC_AUTO)
        p.record(e)
        p.set_observable(it["paulis"], it["coeffs"])
        progs.append(p)
    n_c128 = sum(1 for p in progs if p.precision == M.PREC_FP64)
    g = M.Graph(ctx, progs)
    energies = None
    for _ in range(args.warmup):
        energies = g.launch()

    # ---- device-resident timing: K replays bracketed by events on the replay stream
    stream = torch.cuda.ExternalStream(g.stream)
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    if dist is not None:
        dist.barrier()
    clk = Clocks(local)
    clk.start()
    ev0.record(stream)
    for _ in range(args.steps):
        g.launch_async()
    ev1.record(stream)
    energies = g.sync()
    torch.cuda.synchronize()
    clocks = clk.stop()
    ms = ev0.elapsed_time(ev1) / args.steps
    ops_ms, exp_ms, gemm_flops, eig_flops, op_bytes, res_bytes = g.timing()
    # the fused kernel also evaluates every circuit's Hamiltonian (50 terms +
    # the norm): transfer-matrix flops sum_sites 16 chi_l^2 chi_r + 16 chi_l chi_r^2
    obs_flops = 0.0
    for p, it in zip(progs, insts):
        b = [1] + p.bond_dims() + [1]
        per = sum(16.0 * b[i] ** 2 * b[i + 1] + 16.0 * b[i] * b[i + 1] ** 2 for i in range(it["n"]))
        obs_flops += per * (len(it["paulis"]) + 1)
    cycles = g.phase_cycles()
    sums = g.stat_sums()
    cycles["observables"] = sums["cyc_obs"]
    cyc_total = sum(cycles.values()) or 1.0
    phase_share = {k: v / cyc_total for k, v in cycles.items()}
    phase_share["eigensolver_detail"] = {k: sums["cyc_" + k] / cyc_total for k in ("trid", "bisect", "vec")}
    phase_share["orthonormalise_in_split"] = sums["cyc_orth"] / cyc_total
    # mean SM busy time (phase cycles summed over programs / SMs / clock)
    # against the kernel's duration: the gap is the tail of the launch
    busy_cycles = sum(cycles[k] for k in cycles)
    phase_share["refined_splits"] = int(sums["refined"])
    phase_share["splits"] = int(sums["gate2"])
    ms = max_over_ranks(ms, dist, "cuda")
    if dist is not None:
        dist.barrier()
    value = job_throughput(args.instances, world, ms)

    # ---- end to end through the public API from host buffers: every
    # program's gates recorded by one call (the library records the programs
    # on host threads), the op table compiled and uploaded, one replay
    batch_rec = M.BatchRecord(progs, enc)
    e2e_times, rec_t, upd_t = [], [], []
    for step in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        batch_rec.record()
        t1 = time.perf_counter()
        g.update()
        t2 = time.perf_counter()
        g.launch()
        if step >= args.warmup:
            e2e_times.append(time.perf_counter() - t0)
            rec_t.append(t1 - t0)
            upd_t.append(t2 - t1)
    e2e_ms = max_over_ranks(1e3 * float(np.mean(e2e_times)), dist, "cuda")
    e2e_value = job_throughput(args.instances, world, e2e_ms)

    extras = {}
    if rank == 0 and not args.no_extras:
        extras = extra_measurements(args, ctx, insts, energies, value, world)

    if rank == 0:
        pk, pk_kind = peaks()
        fp32_flops = gemm_flops + obs_flops + eig_flops
        achieved = fp32_flops / (ops_ms / 1e3) / 1e12
        peak = rates["fp32_tflops"]
        traffic = None
        tpath = os.path.join(ROOT, "profiles", "k_run_ops_vqe_batch.json")
        if os.path.exists(tpath):
            with open(tpath) as f:
                traffic = json.load(f).get("dram_bytes_per_launch")
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "c64+c128", "data": "synthetic",
            "config": {"workload": WORKLOAD, "instances": args.instances, "chi_max": CHI,
                       "truncation": "itensor (canonical, relative cutoff %g)" % CUTOFF,
                       "precision": "MPS_PREC_AUTO: complex128 for the %d registers of <= 12 qubits (exact at "
                                    "the cap), complex64 storage and arithmetic with FP64 truncation sums for "
                                    "the other %d; one persistent launch" % (n_c128, args.instances - n_c128),
                       "parallelism": "replicas x%d" % world,
                       "l2": "inputs larger than L2 (resident MPS state of 1024 circuits > 129 MB)"},
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(op_bytes),
                    "d2h_bytes_per_step": int(res_bytes),
                    "what": "per step: bulk gate recording of every program from host arrays (one "
                            "mps_gates_many call), op-table compile and upload (mps_graph_update), replay, "
                            "energies read back; the library records and compiles the programs on host "
                            "threads; the gate lists are encoded to those arrays once, before the timed "
                            "steps, as a VQE loop re-records new parameters into the same structure",
                    "encode_ms_once": encode_ms, "record_ms": 1e3 * float(np.mean(rec_t)),
                    "compile_and_upload_ms": 1e3 * float(np.mean(upd_t))},
            "roofline": {"kernel": "k_run_ops<float> (fused 2-site update + observables)", "bound": "fp32",
                         "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                         "frac": achieved / peak, "traffic": traffic,
                         "peak_source": "measured: FP32 FMA rate of this GPU's CUDA cores (mps_diag_fma_rate)",
                         "flops_per_launch": fp32_flops, "kernel_ms": ops_ms,
                         "gemm_class_flops_per_launch": gemm_flops,
                         "observable_flops_per_launch": obs_flops,
                         "eigensolver_flops_per_launch": eig_flops,
                         "frac_of_bf16_tensor_peak": achieved / pk.get("bf16_tflops_sustained",
                                                                       pk.get("bf16_tflops")),
                         "frac_of_hbm": (traffic / (ops_ms / 1e3) / 1e9 / pk["hbm_gbs"]) if traffic else None,
                         "note": "all of the kernel's arithmetic runs on FP32 CUDA cores (no tensor-core "
                                 "instructions): theta merge, gate, Gram, split, centre moves, the observables' "
                                 "transfer matrices and the Householder eigensolver, complex MAC = 8 flops"},
            "cuda_core_rates": rates,
            "phases_ms": {"reset_ops_and_observables": ops_ms, "copy_results": exp_ms},
            "fused_kernel_cycle_share": phase_share,
            "load_balance": {"kernel_ms": ops_ms,
                             "mean_sm_busy_ms": busy_cycles / ctx.num_sms / (1e3 * ((clocks or {}).get("sm_mhz")
                                                                                   or 2070.0)),
                             "complex128_programs": n_c128},
            "gpu_launches": 2 * args.steps,
            "clocks": clocks,
        }
        line.update(extras)
        print(json.dumps(line))
    for p in progs:
        p.close()
    g.close()
    ctx.close()
    if dist is not None:
        dist.destroy_process_group()
    return 0


def extra_measurements(args, ctx, insts, energies, value, world):
    """Accuracy vs the FP64 oracle over the whole batch, the CPU baseline (the
    same oracle run timed on all host cores), the plain per-circuit FP64
    visitor, serving latency, the 48-qubit circuit and the mixed serving
    stream.  Rank 0 at N=1 only."""
    from tnqvm_gb300 import mps as M
    out = {}
    if world != 1:
        return out
    order = np.argsort([it["n"] * it["layers"] for it in insts])
    # the complex128 oracle on every circuit of the batch, one circuit per
    # host core: its energies pin the batch's accuracy, its wall time is the
    # CPU baseline on the same workload
    from oracle.pool import OraclePool
    with OraclePool() as pool:
        ref, wall, busy = pool.energies(insts, CHI, CUTOFF)
        cores = pool.workers
    errs = np.abs(np.asarray(energies) - np.asarray(ref))
    worst = int(np.argmax(errs))
    out["err_vs_oracle"] = {
        "max_abs_dE": float(errs.max()), "median_abs_dE": float(np.median(errs)),
        "p99_abs_dE": float(np.percentile(errs, 99)), "sample": len(insts),
        "worst": {"index": worst, "n": insts[worst]["n"], "layers": insts[worst]["layers"]},
        "costliest_16_max_abs_dE": float(errs[order[-16:]].max()),
        "within_1e-6": int(np.sum(errs <= 1e-6)),
        "oracle": "complex128 itensor-mode MPS (LAPACK SVD), same cap and cutoff, every circuit of the batch"}
    # the same batch with every register in complex128: the engine's mode for
    # a bound on every circuit (complex64 misses 1e-6 where a truncation cuts
    # through a nearly degenerate pair of singular values)
    if args.fp64_batch:
        progs = []
        for it in insts:
            p = M.Program(ctx, it["n"], CHI, CUTOFF, M.TRUNC_ITENSOR, M.PREC_FP64)
            p.record(M.encode_circuit(it["circuit"]))
            p.set_observable(it["paulis"], it["coeffs"])
            progs.append(p)
        g = M.Graph(ctx, progs)
        try:
            g.launch()
            tms = []
            for _ in range(2):
                e64 = np.asarray(g.launch())
                tms.append(g.timing()[0])
        finally:
            g.close()
            for p in progs:
                p.close()
        err64 = np.abs(e64 - np.asarray(ref))
        out["fp64_batch"] = {"value": len(insts) / (np.mean(tms) / 1e3), "unit": UNIT, "ms_per_step": float(np.mean(tms)),
                             "max_abs_dE": float(err64.max()), "within_1e-6": int(np.sum(err64 <= 1e-6)),
                             "what": "the same 1024 circuits, every register complex128, one captured replay, "
                                     "device time"}
    out["cpu_baseline"] = {"value": len(insts) / wall, "unit": UNIT, "cores": cores, "kind": "port",
                           "sample": "the whole %d-circuit batch in %.1f s on %d worker processes (one circuit "
                                     "per process, single-threaded BLAS; %.1f core-seconds); numpy complex128 "
                                     "MPS with LAPACK SVD (itensor-mode oracle)" % (len(insts), wall, cores, busy),
                           "per_circuit_ms_one_core": 1e3 * busy / len(insts)}
    # plain per-circuit FP64 visitor: one launch per gate, one circuit at a time
    pidx = list(order[:: max(1, len(order) // args.plain_sample)])[: args.plain_sample]
    t0 = time.perf_counter()
    done = 0
    perr = []
    for i in pidx:
        it = insts[i]
        p = M.Program(ctx, it["n"], CHI, CUTOFF, M.TRUNC_ITENSOR, M.PREC_FP64, M.FLAG_PER_GATE)
        p.run(it["circuit"])
        p.set_observable(it["paulis"], it["coeffs"])
        e = ctx.batch_expect([p])[0]
        p.close()
        perr.append(abs(e - ref[i]))
        done += 1
        if time.perf_counter() - t0 > args.plain_budget:
            break
    dt = time.perf_counter() - t0
    plain = done / dt
    out["plain_fp64"] = {"value": plain, "unit": UNIT, "sample": done,
                         "what": "per-circuit FP64 visitor path: complex128, one kernel launch per gate, no batching",
                         "per_circuit_ms": 1e3 * dt / max(1, done),
                         "batched_over_plain": value / plain,
                         "max_abs_dE_vs_oracle": float(max(perr)) if perr else None}
    out["plain_fp64_exatn"] = plain_exatn(args, ctx, [insts[i] for i in pidx[:done]], value)
    # serving latency: Poisson arrivals into the continuous-batching loop
    out["latency"] = serve_latency(args, ctx, insts, value)
    # one large circuit on the wide path, and the mixed-cap serving stream
    if args.wide:
        out["wide_48q_chi512"] = wide_single(args, ctx)
    if args.serve_stream > 0:
        out["serve_stream"] = serve_stream(args, ctx)
    out["noisy"] = noisy_circuits(ctx)
    return out


def noisy_circuits(ctx):
    """Noisy circuits (density programs, the drop-in for the exatn-pmps
    visitor): an 8-qubit brick wall of depth 8 (U3 + CNOT) with a
    depolarizing channel (p = 0.01) on both qubits after every CNOT, complex128,
    exact (bond cap 256 on the 16-site doubled chain: the wide path) and
    truncated (cap 128), each against the dense density-matrix oracle: <Z_i>
    (normalised by the trace) for every qubit, and the trace."""
    from tnqvm_gb300 import circuits
    from tnqvm_gb300 import mps as M
    from oracle import density as R
    n, depth, pdep = 8, 8, 0.01
    a, b = np.sqrt(1 - pdep), np.sqrt(pdep / 3)
    kraus = [np.array(k, dtype=np.complex128) for k in ([[a, 0], [0, a]], [[0, b], [b, 0]],
                                                         [[0, -1j * b], [1j * b, 0]], [[b, 0], [0, -b]])]
    circ = []
    for name, qs, ps in circuits.brickwall(n, depth, seed=5):
        circ.append((name, qs, ps))
        if len(qs) == 2:
            circ += [("Kraus", [qs[0]], kraus), ("Kraus", [qs[1]], kraus)]
    t0 = time.perf_counter()
    rho = R.run(n, circ)
    cpu_s = time.perf_counter() - t0
    zs = ["".join("Z" if j == i else "I" for j in range(n)) for i in range(n)]
    want = np.array([R.expect_pauli(rho, n, z).real for z in zs])
    out = {"workload": "8-qubit brick wall, depth 8, U3 + CNOT, depolarizing p=0.01 on both qubits after "
                       "every CNOT; complex128 density program (16-site doubled chain)",
           "dense_oracle_cpu_seconds": cpu_s}
    for chi in (256, 128):
        t0 = time.perf_counter()
        p = M.DensityProgram(ctx, n, chi, 1e-300, M.TRUNC_ITENSOR, M.PREC_FP64)
        for name, qs, ps in circ:
            if name == "Kraus":
                p.channel(qs[0], ps)
            else:
                p.gate(name, list(qs), list(ps))
        p.submit()
        p.wait()
        got = p.expect_pauli(zs).real
        secs = time.perf_counter() - t0
        out["chi%d" % chi] = {"seconds": secs, "max_bond": max(p.bond_dims()), "trace": p.norm(),
                              "max_abs_dZ_vs_dense": float(np.max(np.abs(got - want)))}
        p.close()
    return out


def plain_exatn(args, ctx, sample, value):
    """The per-circuit FP64 path in exatn semantics (the drop-in for the
    exatn-mps visitor and the plugin's default): one launch per gate, and the
    site-parallel single launch (MPS_FLAG_PARALLEL: the two-site updates of
    one circuit on disjoint sites run on different SMs), against the
    exatn-mode oracle on the same circuits, whose single-core time per
    circuit is the CPU figure beside them."""
    from tnqvm_gb300 import mps as M
    from oracle.pool import OraclePool
    with OraclePool(workers=1) as pool:
        ref, wall, busy = pool.energies(sample, CHI, CUTOFF, mode="exatn")
    out = {"sample": len(sample), "cpu_one_core_ms_per_circuit": 1e3 * busy / max(1, len(sample)),
           "cpu": "numpy complex128 MPS with LAPACK SVD (exatn-mode oracle), one process, single-threaded BLAS"}
    for key, flags in (("per_gate", M.FLAG_PER_GATE), ("parallel", M.FLAG_PARALLEL)):
        errs = []
        t0 = time.perf_counter()
        for it, r in zip(sample, ref):
            p = M.Program(ctx, it["n"], CHI, CUTOFF, M.TRUNC_EXATN, M.PREC_FP64, flags)
            p.run(it["circuit"])
            e = p.expect_pauli(it["paulis"], it["coeffs"])[1] / p.norm()
            p.close()
            errs.append(abs(e - r))
        dt = time.perf_counter() - t0
        out[key] = {"value": len(sample) / dt, "unit": UNIT, "per_circuit_ms": 1e3 * dt / max(1, len(sample)),
                    "max_abs_dE_vs_oracle": float(max(errs)), "batched_over_this": value / (len(sample) / dt)}
    return out


def wide_single(args, ctx):
    """48-qubit brick wall, depth 30 (U3 + CZ), bond cap 512, cutoff 1e-10:
    one circuit on the wide path in complex64 (tcgen05 3xTF32 products, FP32
    eigensolver with deflation refinement), canonical truncation with the
    gates of each layer swept in centre order (MPS_FLAG_SWEEP); outputs
    <Z_i Z_i+1> for all i and the truncation fidelity; with --wide-ref also
    the complex128 run at the same cap and the error against it."""
    from tnqvm_gb300 import circuits
    from tnqvm_gb300 import mps as M
    n, depth, chi, cut = 48, 30, 512, 1e-10
    circ = circuits.brickwall(n, depth, seed=2, entangler="CZ")
    terms = ["I" * i + "ZZ" + "I" * (n - i - 2) for i in range(n - 1)]
    out = {"workload": "brickwall n=48 depth=30 U3+CZ, chi<=512, cutoff 1e-10, itensor truncation, swept gate order"}
    vals = {}
    if args.wide_autotune >= 0:
        M.autotune_set_mode(args.wide_autotune)
    for prec in ([M.PREC_FP32, M.PREC_FP64] if args.wide_ref else [M.PREC_FP32]):
        tc0, _ = ctx.gemm_counts()
        tu0 = ctx.autotune_tunings()
        t0 = time.perf_counter()
        p = M.Program(ctx, n, chi, cut, M.TRUNC_ITENSOR, prec, M.FLAG_SWEEP)
        p.run(circ)
        p.submit()
        p.wait()
        t1 = time.perf_counter()
        v = p.expect_pauli(terms).real / p.norm()
        st = p.stats()
        tc1, _ = ctx.gemm_counts()
        key = "c64" if prec == M.PREC_FP32 else "c128"
        vals[key] = v
        out[key] = {"seconds": t1 - t0, "circuits_per_s": 1.0 / (t1 - t0), "splits": st["gate2"], "ops": st["ops"],
                    "max_bond": max(p.bond_dims()), "truncation_fidelity": float(st["fidelity"]),
                    "tensor_core_gemms": tc1 - tc0,
                    "gemm_buckets_tuned": ctx.autotune_tunings() - tu0}
        p.close()
    if args.wide_cpu_layers > 0:
        # the same circuit's first layers on the CPU oracle (complex128 numpy
        # MPS, LAPACK SVD, all BLAS threads) and on the GPU, recorded order
        from oracle import mps as omps
        from oracle import routing
        L = args.wide_cpu_layers
        pre = circuits.brickwall(n, depth, seed=2, entangler="CZ")[: L * (n + n - 1)]
        t0 = time.perf_counter()
        om = omps.run(n, routing.route(pre), mode="itensor", chi_max=chi, cutoff=cut)
        t_cpu = time.perf_counter() - t0
        zz_cpu = np.array([om.expect_pauli(s).real for s in terms]) / om.norm2()
        row = {"layers": L, "cpu_seconds": t_cpu, "cpu_threads": os.cpu_count(),
               "cpu": "numpy complex128 MPS, LAPACK SVD (itensor-mode oracle), gates in recorded order",
               "max_bond": max(om.bond_dims())}
        for prec, key in ((M.PREC_FP32, "gpu_c64_seconds"), (M.PREC_FP64, "gpu_c128_seconds")):
            t0 = time.perf_counter()
            p = M.Program(ctx, n, chi, cut, M.TRUNC_ITENSOR, prec)
            p.run(pre)
            p.submit()
            p.wait()
            row[key] = time.perf_counter() - t0
            zz = p.expect_pauli(terms).real / p.norm()
            row[key.replace("seconds", "max_abs_dZZ_vs_cpu")] = float(np.max(np.abs(zz - zz_cpu)))
            p.close()
        out["cpu_prefix"] = row
    table = M.autotune_table()
    out["gemm_autotune"] = {"mode": M.autotune_mode(), "buckets": len(table),
                            "kernels": {name: sum(1 for r in table if r["kernel"] == k)
                                        for k, name in enumerate(M.GEMM_KERNEL_NAMES)}}
    if "c128" in vals:
        d = np.abs(vals["c64"] - vals["c128"])
        out["err_c64_vs_c128"] = {"max_abs_dZZ": float(d.max()), "median_abs_dZZ": float(np.median(d))}
    return out


def qaoa_precision(args):
    """64-qubit QAOA MaxCut on a seeded random 3-regular graph (96 edges), p
    rounds, gamma and beta uniform in [0, pi], RZZ as CNOT . Rz . CNOT, bond
    cap 1024, cutoff 1e-12, itensor semantics with the routed SWAP pairs
    cancelled and same-pair gates fused (MPS_FLAG_FUSE) and the gates swept
    in centre order (MPS_FLAG_SWEEP): <H_cut> = sum over edges (1 - <Z_i
    Z_j>)/2 in split-BF16, complex64 and complex128, each mode's error
    against the complex128 run, seconds and truncation fidelity.  Off by
    default (minutes per mode); ``--leg qaoa`` runs it alone."""
    from tnqvm_gb300 import circuits
    from tnqvm_gb300 import mps as M
    n = 64
    circ, edges = circuits.qaoa_maxcut(n=n, p=args.qaoa_p, seed=7)
    terms = []
    for a, b in edges:
        s = ["I"] * n
        s[a] = s[b] = "Z"
        terms.append("".join(s))
    with M.Context(env_int("LOCAL_RANK", 0)) as ctx:
        out = {"workload": "64-qubit QAOA MaxCut, 3-regular graph (96 edges), p=%d, chi<=1024, cutoff 1e-12, "
                           "itensor, fused routing + swept order" % args.qaoa_p}
        vals = {}
        for prec, key in ((M.PREC_FP64, "c128"), (M.PREC_FP32, "c64"), (M.PREC_SPLIT_BF16, "split_bf16")):
            t0 = time.perf_counter()
            p = M.Program(ctx, n, 1024, 1e-12, M.TRUNC_ITENSOR, prec, M.FLAG_FUSE | M.FLAG_SWEEP)
            p.run(circ)
            p.submit()
            p.wait()
            secs = time.perf_counter() - t0
            zz = p.expect_pauli(terms).real / p.norm()
            st = p.stats()
            vals[key] = float(np.sum((1.0 - zz) / 2.0))
            out[key] = {"seconds": secs, "H_cut": vals[key], "splits": st["gate2"], "max_bond": max(p.bond_dims()),
                        "truncation_fidelity": float(st["fidelity"])}
            p.close()
        for key in ("c64", "split_bf16"):
            out[key]["abs_err_H_cut_vs_c128"] = abs(vals[key] - vals["c128"])
    return out


def serve_stream(args, ctx):
    """The serving stream: Poisson arrivals at each offered rate of random
    brick-wall circuits (qubits U{10..64}, depth U{10..40}, bond cap from
    {16, 64, 256, 512}), each returning 1024 shots and one Pauli expectation,
    through the continuous-batching loop (HBM admission under the 150 GB
    budget; caps above 64 on its wide lane).  Every request with a cap <= 64
    is followed by a parameter update: the same program, reset, re-recorded
    with new angles and resubmitted, its MPS allocation reused."""
    from tnqvm_gb300 import circuits
    from tnqvm_gb300 import mps as M
    out = {"mode": "qubits U{10..64}, depth U{10..40}, cap {16,64,256,512}, 1024 shots + 1 Pauli term each; "
                   "parameter updates on the resident programs of caps <= 64",
           "requests_per_rate": args.serve_stream, "rates": []}
    for ri, rate in enumerate(args.serve_rates):
        rng = np.random.default_rng(44 + ri)
        reqs = []
        for i in range(args.serve_stream):
            n = int(rng.integers(10, 65))
            depth = int(rng.integers(10, 41))
            chi = int(rng.choice([16, 64, 256, 512]))
            p = M.Program(ctx, n, chi, 1e-10, M.TRUNC_ITENSOR, M.PREC_AUTO)
            p.run(circuits.brickwall(n, depth, seed=1000 * ri + i))
            p.set_observable(["".join(rng.choice(list("IXYZ"), n))], [1.0])
            reqs.append((p, n, depth, chi))
        ctx.serve_start(256)
        lats = {16: [], 64: [], 256: [], 512: []}
        upd = []
        try:
            gaps = rng.exponential(1.0 / rate, len(reqs))
            tickets = []
            t0 = time.perf_counter()
            t_next = t0
            for (p, n, depth, chi), gap in zip(reqs, gaps):
                t_next += gap
                while time.perf_counter() < t_next:
                    pass
                tickets.append(ctx.serve_submit(p, 1024, 7))
            pending = []
            for (p, n, depth, chi), t in zip(reqs, tickets):
                _, _, lat = ctx.serve_poll(t, p, 1024)
                lats[chi].append(lat)
                if chi <= 64:  # parameter update on the resident program
                    p.reset()
                    p.run(circuits.brickwall(n, depth, seed=777 + len(pending)))
                    pending.append((p, ctx.serve_submit(p, 1024, 8)))
            for p, t in pending:
                _, _, lat = ctx.serve_poll(t, p, 1024)
                upd.append(lat)
            wall = time.perf_counter() - t0
        finally:
            ctx.serve_stop()
            for p, *_ in reqs:
                p.close()
        allv = [x for v in lats.values() for x in v] + upd
        out["rates"].append({
            "offered_rate_per_s": rate, "requests": len(allv), "wall_s": wall,
            "achieved_per_s": len(allv) / wall,
            "p50_ms": float(np.percentile(allv, 50)), "p99_ms": float(np.percentile(allv, 99)),
            "p50_ms_by_cap": {str(k): float(np.percentile(v, 50)) for k, v in lats.items() if v},
            "parameter_updates": len(upd), "update_p50_ms": float(np.percentile(upd, 50)) if upd else None})
    return out


def serve_latency(args, ctx, insts, value):
    from tnqvm_gb300 import mps as M
    n_req = min(args.serve_requests, len(insts))
    rate = max(50.0, 0.5 * value)
    rng = np.random.default_rng(11)
    sel = rng.choice(len(insts), n_req, replace=False)
    progs = []
    for i in sel:
        it = insts[i]
        p = M.Program(ctx, it["n"], CHI, CUTOFF, M.TRUNC_ITENSOR, M.PREC_AUTO)
        p.set_observable(it["paulis"], it["coeffs"])
        progs.append((p, M.encode_circuit(it["circuit"])))
    ctx.serve_start(256)
    lats = []
    try:
        gaps = rng.exponential(1.0 / rate, n_req)
        tickets = []
        t0 = time.perf_counter()
        t_next = t0
        for (p, e), gap in zip(progs, gaps):
            t_next += gap
            while time.perf_counter() < t_next:
                pass
            p.record(e)
            tickets.append(ctx.serve_submit(p, 0, 0))
        for (p, _), t in zip(progs, tickets):
            _, _, lat = ctx.serve_poll(t, p, 0)
            lats.append(lat)
        wall = time.perf_counter() - t0
    finally:
        ctx.serve_stop()
        for p, _ in progs:
            p.close()
    return {"p50_ms": float(np.percentile(lats, 50)), "p99_ms": float(np.percentile(lats, 99)),
            "requests": n_req, "offered_rate_per_s": rate, "achieved_per_s": n_req / wall,
            "mode": "continuous batching, Poisson arrivals, 1 Pauli Hamiltonian per request"}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--instances", type=int, default=1024)
    ap.add_argument("--fp64-batch", type=int, default=1, help="also time the batch all in complex128 (1/0)")
    ap.add_argument("--plain-sample", type=int, default=8)
    ap.add_argument("--plain-budget", type=float, default=60.0)
    ap.add_argument("--ref-stride", type=int, default=8,
                    help="reference arm: every n-th circuit of the batch in order of cost, each step")
    ap.add_argument("--serve-requests", type=int, default=256)
    ap.add_argument("--no-extras", action="store_true")
    ap.add_argument("--wide", type=int, default=1, help="time the 48-qubit chi=512 circuit (1/0)")
    ap.add_argument("--wide-ref", type=int, default=1,
                    help="also run it in complex128 and report the complex64 error against it (1/0)")
    ap.add_argument("--wide-cpu-layers", type=int, default=14,
                    help="layers of the 48-qubit circuit timed on the CPU oracle and on the GPU (0: off)")
    ap.add_argument("--wide-autotune", type=int, default=-1,
                    help="GEMM autotuner mode for the wide circuit (0 static, 1 tune, 2 table; -1 library default)")
    ap.add_argument("--serve-stream", type=int, default=12,
                    help="requests per offered rate of the mixed-cap serving stream (0: off)")
    ap.add_argument("--serve-rates", type=float, nargs="+", default=[1e2, 1e3, 1e4])
    ap.add_argument("--qmin", type=int, default=8, help="smallest qubit count (small profiling cases)")
    ap.add_argument("--qmax", type=int, default=32, help="largest qubit count (small profiling cases)")
    ap.add_argument("--lmax", type=int, default=12, help="largest layer count (small profiling cases)")
    ap.add_argument("--leg", default="", choices=["", "qaoa", "plain", "noisy"],
                    help="run one extra leg alone and print its JSON (qaoa: the 64-qubit precision comparison; "
                         "plain: the exatn-mode per-circuit FP64 paths on the stratified sample; noisy: the "
                         "noisy-circuit leg)")
    ap.add_argument("--qaoa-p", type=int, default=3, help="QAOA rounds of the qaoa leg")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    if args.leg == "qaoa":
        build_locked()
        print(json.dumps({"qaoa_precision": qaoa_precision(args)}))
        return 0
    if args.leg in ("plain", "noisy"):
        build_locked()
        from tnqvm_gb300 import circuits
        from tnqvm_gb300 import mps as M
        with M.Context(env_int("LOCAL_RANK", 0)) as ctx:
            if args.leg == "noisy":
                print(json.dumps({"noisy": noisy_circuits(ctx)}))
                return 0
            insts = circuits.vqe_batch(args.instances, seed=replica_seed(0), qmin=args.qmin, qmax=args.qmax,
                                       lmax=args.lmax)
            order = np.argsort([it["n"] * it["layers"] for it in insts])
            pidx = list(order[:: max(1, len(order) // args.plain_sample)])[: args.plain_sample]
            print(json.dumps({"plain_fp64_exatn": plain_exatn(args, ctx, [insts[i] for i in pidx], float("nan"))}))
        return 0
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
