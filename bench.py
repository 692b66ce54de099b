"""Benchmark: exp(-iHt)v on one GB300 (Krylov evolution, TimeEvolver algorithm).

Workload (one "step" = one full solve): open-chain Bose-Hubbard L=12, N=12,
J=1, U=3 (dim 1352078, 16871581 non-zeros), start vector a normalised complex
Gaussian (numpy default_rng(0), real then imaginary parts), evolved to t=10
with tol 1e-8, Krylov dimension m=40, <n_0> sampled every 0.5.

value: seconds per solve with H, v and the observable resident in HBM (CUDA
events on the evolver's stream).  e2e: the same solve through the C ABI with
host buffers (COO upload, start vector, results back), wall clock.
roofline: the Lanczos apply kernel (SELL-32 SpMV with the fused recurrence
epilogue): the algorithmic bytes of one complex128 CSR SpMV (20 nnz +
4 (n + 1) + 32 n) over the kernel's event-timed mean duration; the bytes of
the stored format (4 per entry with the value dictionary) and their fraction
are given beside it, and `traffic` is the DRAM bytes ncu measured per launch.

--impl reference: the CPU restatement of the reference algorithm (the oracle,
OpenMP on all host cores), every step one whole solve of the same workload,
with H, the observable and v built by the oracle's numpy model builders (the
arm loads no library of the product).

Multi-GPU: replicas only (one independent solve per rank), torchrun/NCCL for
the barrier and the max-over-ranks time.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

L_SITES, N_BOSONS, J_HOP, U_INT = 12, 12, 1.0, 3.0
T_FINAL, TOL, M_KRYLOV, SAMPLING = 10.0, 1e-8, 40, 0.5
METRIC = "exp(-iHt)v s (Bose-Hubbard L=12 N=12 U=3, t=10, tol 1e-8, m=40)"
WORKLOAD = ("Bose-Hubbard open chain L=12 N=12 J=1 U=3 (dim 1352078, nnz 16871581), complex Gaussian v seed 0, "
            "t=10, tol=1e-8, m=40, <n_0> every 0.5")


def bench_config(n, nnz):
    """The workload description printed by both arms (identical dicts)."""
    return {"workload": WORKLOAD, "n": n, "nnz": nnz,
            "l2": "inputs larger than L2 (H %.0f MB + Krylov basis %.0f MB)"
                  % (nnz * 12 / 1e6, (M_KRYLOV + 3) * 16 * n / 1e6)}


def dist_info():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def init_dist(ws, local, backend="nccl"):
    """One process per GPU (replicas); NCCL on the GPUs, gloo for host-only runs."""
    if ws <= 1:
        return None
    import torch
    import torch.distributed as dist
    if backend == "nccl":
        torch.cuda.set_device(local)
    dist.init_process_group(backend)
    return dist


def barrier(dist):
    if dist is not None:
        dist.barrier()


def max_over_ranks(dist, x):
    """The slowest rank's value (the timing rule for replicas)."""
    if dist is None:
        return x
    import torch
    device = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_seconds_per_solve(max_ms, steps, world_size):
    """Whole-job seconds per solve of N replicas, each timing `steps` solves
    (the slowest rank's time): N solves finish every max_ms / steps."""
    return max_ms / 1000.0 / steps / world_size


def load_peaks(te):
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    peaks = {"hbm_gbs": 6800.0, "source": "fallback"}
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        peaks = {"hbm_gbs": float(d["hbm_gbs"]), "source": "measured"}
    # FP64 FMA throughput of this GPU, measured live (independent FMA chains on every SM)
    peaks["fp64_tflops"] = te.probe_fp64_tflops()
    return peaks


def ncu_traffic(fixed=False):
    """Per-launch DRAM traffic of the Lanczos apply kernel in use (fixed-point
    or FP64 SpMV) from the committed ncu summary, if one exists."""
    p = os.path.join(ROOT, "profiles", "lanczos_apply_fix_bh12.json" if fixed else "lanczos_apply_bh12.json")
    if os.path.exists(p):
        with open(p) as f:
            return json.load(f).get("dram_bytes_per_launch")
    return None


class ClockSampler:
    """nvidia-smi clocks and throttle reasons every 200 ms during the timed region."""

    def __init__(self, index):
        self.index = index
        self.samples = []
        self.proc = None

    def __enter__(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 7:
                self.samples.append(parts)

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples for i in range(4) if s[3 + i].lower() == "active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


def build_problem():
    """H, <n_0> and v with the product's model builder (C++, multi-threaded)."""
    from timeevolver_gb300 import models
    B, H = models.bose_hubbard(L_SITES, N_BOSONS, J_HOP, U_INT)
    O = models.operator_matrix([models.number_operator(0, 1.0)], B)
    n = len(B)
    return n, H, O, start_vector(n)


def build_problem_oracle():
    """The same H, <n_0> and v with the oracle's numpy builders (bit-identical
    COO arrays), for the reference arm."""
    from oracle import models
    B, H = models.bose_hubbard(L_SITES, N_BOSONS, J_HOP, U_INT)
    O = models.create_matrix([models.number_operator(0, 1.0)], B)
    return len(B), H, O, start_vector(len(B))


def start_vector(n):
    rng = np.random.default_rng(0)
    v = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    v /= np.linalg.norm(v)
    return v


def spmv_option(spmv):
    """TE_OPT_FIXED_SPMV for --spmv: fixed point (the default) or FP64."""
    return {None: 1, "fixed": 1, "fp64": 0}[spmv]


def spmv_bytes(n, nnz):
    """Algorithmic bytes of one SpMV of a complex128 CSR with int32 indices:
    values and columns of every entry, the row pointers, x read once and y
    written, B = 20 nnz + 4 (n + 1) + 32 n (the count the roofline is quoted
    on, whatever the storage format)."""
    return 20 * nnz + 4 * (n + 1) + 32 * n


def whole_solve_bytes(n, nnz, iterations, vw_products, m):
    """Algorithmic bytes of a whole solve: per Lanczos iteration one SpMV plus
    the recurrence's vector traffic (u_j and w read, u_{j+1} written, u_{j-1}
    read: 64 n), per V.w product the basis read and the result written
    (16 n m + 16 n)."""
    return iterations * (spmv_bytes(n, nnz) + 64 * n) + vw_products * (16 * n * m + 16 * n)


def apply_kernel_bytes(n, nnz, real=True, fixed=False, packed=False):
    """Algorithmic bytes of one Lanczos apply launch: the matrix (values +
    int32 columns; with the value dictionary one 4-byte word per entry), the
    SELL chunk offsets, x = u_j read once, u_{j-1} read, w written.  The
    fixed-point apply reads the fixed-point copy of u_j (16 bytes per row,
    gathered) and u_j itself for <u_j, w'> (16 more)."""
    chunks = (n + 31) // 32
    per_entry = 4 if packed else (8 if real else 16) + 4
    return nnz * per_entry + 8 * (chunks + 1) + (4 if fixed else 3) * 16 * n


def apply_kernel_flops(n, nnz, real=True, fixed=False):
    """FP64 flops of one Lanczos apply launch: 2 (real) or 4 (complex) FMAs per
    non-zero (none in the fixed-point SpMV), 14 per row for the recurrence
    term and the <v_j, w> partial."""
    return (0 if fixed else nnz * (4 if real else 8)) + 14 * n


KERNEL_KINDS = ["lanczos_apply", "lanczos_update", "krylov_step", "combine", "observables"]


def profiled_solve(te, ev, v_dev):
    """One extra solve with CUDA events around every launch (outside the timed
    region: the events serialise launches that otherwise overlap)."""
    ev.profile(True)
    ev.reset(None, device_ptr=v_dev.data_ptr())
    ev.run()
    apply_ms, apply_n = ev.kernel_time(0)
    kernel_ms = {name: ev.kernel_time(k) for k, name in enumerate(KERNEL_KINDS)}
    ev.profile(False)
    return apply_ms, apply_n, kernel_ms


def run_gb300(args):
    ws, rank, local = dist_info()
    dist = init_dist(ws, local)
    import torch
    import timeevolver_gb300 as te
    torch.cuda.set_device(local)
    te.lib().te_set_device(local)
    n, Hc, Oc, v = build_problem()
    nnz = len(Hc[2])

    # ---- device-resident solves
    H = te.Matrix.from_coo(n, Hc)
    O = te.Matrix.from_coo(n, Oc)
    info = H.info()
    ev = te.Evolver(H, v, T_FINAL, SAMPLING, [("sparse", O)], tol=TOL, m=M_KRYLOV)
    options = {te.OPT_FIXED_SPMV: spmv_option(args.spmv)}
    for opt, val in options.items():
        ev.set_option(opt, val)
    v_dev = torch.from_numpy(v.view(np.float64).copy()).cuda()
    for _ in range(args.warmup):
        ev.reset(None, device_ptr=v_dev.data_ptr())
        ev.run()
    torch.cuda.synchronize()
    stream = torch.cuda.ExternalStream(ev.stream())
    start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    launches = 0
    steps_per_solve = 0
    barrier(dist)
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        start.record(stream)
        for _ in range(args.steps):
            ev.reset(None, device_ptr=v_dev.data_ptr())
            r = ev.run()
            launches += te.lib().te_evolver_launch_count(ev.handle)
            steps_per_solve = r.n_steps
        stop.record(stream)
        stop.synchronize()
    torch.cuda.synchronize()
    barrier(dist)
    ms = start.elapsed_time(stop)
    ms = max_over_ranks(dist, ms)
    status = r.status
    apply_ms, apply_n, kernel_ms = profiled_solve(te, ev, v_dev)
    ev.close()
    fixed_layout = H.fixed_layout()

    # ---- end to end through the C ABI with host buffers
    e2e_times = []
    h2d = 32 * nnz + 32 * len(Oc[2]) + 16 * n
    d2h = 8 * (int(T_FINAL / SAMPLING) + 1) + 16 * n
    if args.warmup > 0:  # one untimed call, as for the device-timed solves
        te.evolve(Hc, v, T_FINAL, SAMPLING, [("sparse", Oc)], tol=TOL, m=M_KRYLOV, options=options)
    for _ in range(max(1, args.steps)):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        out = te.evolve(Hc, v, T_FINAL, SAMPLING, [("sparse", Oc)], tol=TOL, m=M_KRYLOV, options=options)
        torch.cuda.synchronize()
        e2e_times.append(time.perf_counter() - t0)
    e2e_s = max_over_ranks(dist, float(np.mean(e2e_times)))

    if rank != 0:
        if dist is not None:
            dist.destroy_process_group()
        return
    value = replica_seconds_per_solve(ms, args.steps, ws)
    peaks = load_peaks(te)
    fixed = fixed_layout["state"] > 0
    b_format = apply_kernel_bytes(n, nnz, info["real"], fixed, fixed_layout["state"] == 2)
    b_apply = spmv_bytes(n, nnz)
    f_apply = apply_kernel_flops(n, nnz, info["real"], fixed)
    avg_apply_s = apply_ms / 1000.0 / max(1, apply_n)
    achieved = b_apply / avg_apply_s / 1e9
    traffic = ncu_traffic(fixed)
    iters = kernel_ms["lanczos_update"][1]  # one update pass per Lanczos iteration
    vw = steps_per_solve + int(T_FINAL / SAMPLING)  # V.w per step and per sample after t=0
    b_whole = whole_solve_bytes(n, nnz, iters, vw, M_KRYLOV)
    line = {
        "metric": METRIC, "value": value, "unit": "s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": False, "scaling": "weak",
        "vs_baseline": None, "dtype": "complex128 (FP64)", "data": "synthetic (Bose-Hubbard model, seeded state)",
        "config": bench_config(n, nnz),
        "run_info": {"krylov_steps_per_solve": steps_per_solve, "status": status, "err": r.err,
                     "spmv": "fixed" if fixed else "fp64", "parallelism": "replicas" if ws > 1 else "single GPU",
                     "e2e_per_call_s": [round(x, 4) for x in e2e_times],
                     "e2e_calls": "every call uploads H, the observable and v from host memory and reads the "
                                  "samples and the state back; device buffers released by the previous call are "
                                  "reused (the library's buffer cache)"},
        "e2e": {"value": e2e_s, "unit": "s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "gpu_launches": int(launches),
        "roofline": {"bound": "hbm",
                     "kernel": ("lanczos_apply_fix_kernel (fixed-point SELL-32 SpMV%s + FP64 recurrence epilogue)"
                                % (", value dictionary of %d values" % fixed_layout["n_values"]
                                   if fixed_layout["state"] == 2 else "")
                                if fixed else "lanczos_apply_kernel (SELL-32 SpMV + recurrence epilogue)"),
                     "achieved": achieved, "peak": peaks["hbm_gbs"], "unit": "GB/s",
                     "frac": achieved / peaks["hbm_gbs"], "peak_source": peaks["source"],
                     "traffic": traffic, "algorithmic_bytes_per_launch": b_apply,
                     "algorithmic_bytes": "complex128 CSR SpMV, 20 nnz + 4 (n + 1) + 32 n",
                     "format_bytes_per_launch": b_format,
                     "format_frac": b_format / avg_apply_s / 1e9 / peaks["hbm_gbs"],
                     "avg_launch_us": avg_apply_s * 1e6, "launches": apply_n,
                     "fp64": {"achieved_tflops": f_apply / avg_apply_s / 1e12, "peak_tflops": peaks["fp64_tflops"],
                              "peak_source": "measured (te_probe_fp64_tflops)",
                              "frac": f_apply / avg_apply_s / 1e12 / peaks["fp64_tflops"],
                              "flops_per_launch": f_apply}},
        "whole_solve": {"algorithmic_bytes": b_whole, "achieved_gbs": b_whole / value / 1e9,
                        "frac": b_whole / value / 1e9 / peaks["hbm_gbs"], "lanczos_iterations": int(iters),
                        "v_w_products": vw,
                        "accounting": "per Lanczos iteration 20 nnz + 4 (n + 1) + 32 n + 64 n; "
                                      "per V.w product 16 n m + 16 n"},
        "kernel_ms_per_solve": {k: round(v_[0], 3) for k, v_ in kernel_ms.items()},
        "clocks": clk.summary(),
    }
    if not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(Hc, Oc, v)
    if ws == 1 and not args.no_other_workloads:
        line["other_workloads"] = other_workloads(args)
    print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


def other_workloads(args):
    """The load-imbalanced, batched and adjoint workloads measured in the same
    run (each its own full line: clocks sampled in its timed region, 1 warm-up
    and 2 timed steps, no CPU leg), so that their numbers come from the same
    box and record as the headline."""
    sub = argparse.Namespace(**vars(args))
    sub.steps, sub.warmup, sub.no_cpu_baseline = 2, 1, True
    out = {}
    for name, fn in (("zipf_1e7", run_zipf), ("batched_256", run_batched), ("adjoint_l10", run_adjoint)):
        t0 = time.perf_counter()
        try:
            out[name] = fn(sub)
        except Exception as exc:  # report, do not hide the headline
            out[name] = {"error": "%s: %s" % (type(exc).__name__, exc)}
        out[name]["wall_s"] = round(time.perf_counter() - t0, 1)
    return out


def oracle_solve(Hc, Oc, v, cores):
    """One whole solve of the workload by the oracle on `cores` threads."""
    import oracle
    return oracle.evolve(Hc, v, T_FINAL, SAMPLING, [("sparse", Oc)], tol=TOL, m=M_KRYLOV, n_threads=cores)


def cpu_baseline(Hc, Oc, v):
    """The oracle (CPU restatement of the reference algorithm) on all host
    cores: one whole solve of the workload (about 10 s on 16 Grace cores)."""
    import oracle
    oracle.build()
    cores = os.cpu_count()
    t0 = time.perf_counter()
    r = oracle_solve(Hc, Oc, v, cores)
    el = time.perf_counter() - t0
    return {"value": el, "unit": "s", "cores": cores, "kind": "port",
            "sample": "one whole solve (t=%g, %d Krylov steps, status %d), not extrapolated"
                      % (T_FINAL, r["n_steps"], r["status"])}


def run_reference(args):
    """The reference algorithm on the host cores: the oracle timed over whole
    solves of the workload (warmup + steps calls), inputs from the oracle's own
    model builders."""
    ws, rank, local = dist_info()
    if rank != 0:
        return
    import oracle
    oracle.build()
    t0 = time.perf_counter()
    n, Hc, Oc, v = build_problem_oracle()
    build_s = time.perf_counter() - t0
    cores = os.cpu_count()
    times = []
    for i in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        r = oracle_solve(Hc, Oc, v, cores)
        el = time.perf_counter() - t0
        if i >= args.warmup:
            times.append(el)
    value = float(np.mean(times))
    sample = "whole solves (t=%g, %d Krylov steps each), %d timed after %d untimed" % (
        T_FINAL, r["n_steps"], len(times), args.warmup)
    line = {"metric": METRIC, "value": value, "unit": "s", "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": value * 1000, "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
            "dtype": "complex128 (FP64)", "data": "synthetic (Bose-Hubbard model, seeded state)", "impl": "reference",
            "config": bench_config(n, len(Hc[2])),
            "run_info": {"krylov_steps_per_solve": int(r["n_steps"]), "status": int(r["status"]), "err": r["err"],
                         "per_call_s": [round(x, 3) for x in times], "model_build_s": round(build_s, 1)},
            "cpu_baseline": {"value": value, "unit": "s", "cores": cores, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": "s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


BATCH_METRIC = "batched solves/s (256 Bose-Hubbard chains L=6..10, N=L, m=32, tol 1e-8)"
BATCH_WORKLOAD = ("256 open Bose-Hubbard chains, L~U{6..10}, N=L (dims 462..92378), J~U(0.5,1.5), U~U(0,4), "
                  "t~U(1,20), v = all bosons on site 0, tol=1e-8, m=32, <n_0> at 0 and t; numpy default_rng(4)")


def batched_instances(count=256, seed=4):
    """The batched workload: seeded random chains (the C++ model builder)."""
    from timeevolver_gb300 import models
    rng = np.random.default_rng(seed)
    out = []
    cache = {}
    for _ in range(count):
        L = int(rng.integers(6, 11))
        J = float(rng.uniform(0.5, 1.5))
        U = float(rng.uniform(0.0, 4.0))
        t = float(rng.uniform(1.0, 20.0))
        B, H = models.bose_hubbard(L, L, J, U)
        if L not in cache:
            cache[L] = (B, models.operator_matrix([models.number_operator(0, 1.0)], B))
        Bb, O = cache[L]
        v = np.zeros(len(B), dtype=np.complex128)
        v[B.index([L] + [0] * (L - 1))] = 1.0
        out.append(dict(L=L, coo=H, n0=O, v=v, t=t, n=len(B)))
    return out


def run_batched(args):
    """Batched launch vs a per-instance loop of the plain GPU evolver."""
    import torch
    import timeevolver_gb300 as te
    te.lib().te_set_device(0)
    specs = batched_instances()
    mats = [(te.Matrix.from_coo(s["n"], s["coo"]), te.Matrix.from_coo(s["n"], s["n0"])) for s in specs]
    inst = [dict(H=H, v=s["v"], t=s["t"], sampling_step=s["t"], tol=1e-8, m=32, observables=[O])
            for s, (H, O) in zip(specs, mats)]
    batch = te.Batch(inst)
    stream = torch.cuda.ExternalStream(batch.stream())
    for _ in range(args.warmup):
        batch.run()
    start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    launches = 0
    with ClockSampler(0) as clk:
        start.record(stream)
        for _ in range(args.steps):
            res = batch.run()
            launches += batch.launch_count()
        stop.record(stream)
        stop.synchronize()
    batch_ms = start.elapsed_time(stop) / args.steps
    graph_samples = [batch.samples(i) for i in range(len(specs))]
    # the same batch in one persistent launch per run
    batch.set_option(te.BATCH_OPT_PERSISTENT, 1)
    for _ in range(args.warmup):
        batch.run()
    torch.cuda.synchronize()
    p_launches = 0
    start.record(stream)
    for _ in range(args.steps):
        res_p = batch.run()
        p_launches += batch.launch_count()
    stop.record(stream)
    stop.synchronize()
    pers_ms = start.elapsed_time(stop) / args.steps
    pers_diff = [i for i in range(len(specs))
                 if res_p[i] != res[i] or not np.array_equal(batch.samples(i), graph_samples[i])]
    batch.set_option(te.BATCH_OPT_PERSISTENT, 0)
    # per-instance loop of the plain evolver (evolvers created once, reset and run)
    evs = [te.Evolver(H, s["v"], s["t"], s["t"], [("sparse", O)], tol=1e-8, m=32) for s, (H, O) in zip(specs, mats)]
    for ev, s in zip(evs, specs):
        ev.run()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    loop_launches = 0
    single = []
    for ev, s in zip(evs, specs):
        ev.reset(s["v"])
        single.append(ev.run())
        loop_launches += te.lib().te_evolver_launch_count(ev.handle)
    torch.cuda.synchronize()
    loop_ms = (time.perf_counter() - t0) * 1e3
    same_steps = sum(int(r["n_steps"] == x.n_steps) for r, x in zip(res, single))
    steps = [r["n_steps"] for r in res]
    line = {"metric": BATCH_METRIC, "value": len(specs) / (batch_ms / 1e3), "unit": "solves/s", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": batch_ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "complex128 (FP64)",
            "data": "synthetic (seeded Bose-Hubbard chains)",
            "config": {"workload": BATCH_WORKLOAD, "total_rows": int(sum(s["n"] for s in specs)),
                       "krylov_steps_min_mean_max": [int(min(steps)), float(np.mean(steps)), int(max(steps))]},
            "clocks": clk.summary(),
            "timing": "batch arms: CUDA events on the batch stream; per-instance loop: host wall clock between "
                      "device synchronisations",
            "per_instance_loop": {"value": len(specs) / (loop_ms / 1e3), "unit": "solves/s", "ms": loop_ms,
                                  "gpu_launches": int(loop_launches),
                                  "instances_with_equal_step_count": same_steps},
            "speedup_vs_loop": loop_ms / batch_ms, "gpu_launches": int(launches),
            "persistent_launch": {"value": len(specs) / (pers_ms / 1e3), "unit": "solves/s", "ms": pers_ms,
                                  "gpu_launches": int(p_launches), "same_results_as_graph_path": not pers_diff, "instances_differing": pers_diff[:8],
                                  "speedup_vs_loop": loop_ms / pers_ms}}
    return line


ADJ_METRIC = "grads/s (adjoint d<n_0(T)>/d(J_1..J_9, U), Bose-Hubbard L=10 N=10, T=5, tol 1e-10, m=40)"
ADJ_WORKLOAD = ("Bose-Hubbard open chain L=10 N=10 (dim 92378), H = sum_b J_b H_hop,b + U H_int, J_b~U(0.8,1.2) "
                "(numpy default_rng(2)), U=2; v = all bosons on site 0; loss <n_0(T)>, T=5, tol=1e-10, m=40; "
                "checkpoint interval 0.5, Gauss-Legendre nodes per interval")


def run_adjoint(args, nodes=16):
    """Adjoint gradient vs one plain forward evolution, and central FD on the GPU."""
    import torch
    import timeevolver_gb300 as te
    from timeevolver_gb300 import models
    te.lib().te_set_device(0)
    L = 10
    B, mats = models.bose_hubbard_term_matrices(L, L)
    n = len(B)
    rng = np.random.default_rng(2)
    theta = np.concatenate([rng.uniform(0.8, 1.2, L - 1), [2.0]])
    v = np.zeros(n, dtype=np.complex128)
    v[B.index([L] + [0] * (L - 1))] = 1.0
    terms = [te.Matrix.from_coo(n, m) for m in mats]
    O = te.Matrix.from_coo(n, models.operator_matrix([models.number_operator(0, 1.0)], B))
    adj = te.Adjoint(terms, O, v, T=5.0, tol=1e-10, m=40, checkpoint_interval=0.5, nodes_per_interval=nodes)
    for _ in range(args.warmup):
        adj.run(theta)
        adj.forward(theta)
    torch.cuda.synchronize()
    with ClockSampler(0) as clk:
        t0 = time.perf_counter()
        for _ in range(args.steps):
            loss, grad = adj.run(theta)
        torch.cuda.synchronize()
        t_grad = (time.perf_counter() - t0) / args.steps
    st = adj.stats()
    phases = adj.phase_times()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        loss_f = adj.forward(theta)
    torch.cuda.synchronize()
    t_fwd = (time.perf_counter() - t0) / args.steps
    fwd_steps = adj.stats()["forward_steps"]
    # central differences of the plain forward loss, Richardson-extrapolated
    # over h and h/2 (the O(h^2) term is ~1e-6 relative at h = 1e-4), each
    # loss evaluated at tol 1e-12 so that the evolution's own error stays
    # far below the 1e-6 target
    h, fd_tol = 1e-4, 1e-12
    fd_adj = te.Adjoint(terms, O, v, T=5.0, tol=fd_tol, m=40, checkpoint_interval=0.5, nodes_per_interval=nodes)

    def central(k, step):
        e = np.zeros_like(theta)
        e[k] = step
        return (fd_adj.forward(theta + e) - fd_adj.forward(theta - e)) / (2 * step)

    fd = np.array([(4.0 * central(k, h / 2) - central(k, h)) / 3.0 for k in range(len(theta))])
    rel = float(np.max(np.abs(grad - fd)) / np.max(np.abs(fd)))
    line = {"metric": ADJ_METRIC, "value": 1.0 / t_grad, "unit": "grads/s", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_grad * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "complex128 (FP64)", "data": "synthetic (seeded couplings)",
            "config": {"workload": ADJ_WORKLOAD, "n": n, "nodes_per_interval": nodes, "sample_nodes": st["nodes"],
                       "loss": loss, "plain_forward_loss": loss_f},
            "cost_vs_forward": t_grad / t_fwd, "forward_s": t_fwd,
            "forward_krylov_steps": {"plain": fwd_steps, "adjoint_forward": st["forward_steps"],
                                     "costate": st["backward_steps"]},
            "phase_ms": {k: round(v, 3) for k, v in phases.items()},
            "fd_check": {"method": "central differences, Richardson over h and h/2", "step": h, "fd_tol": fd_tol,
                         "max_abs_diff_rel": rel, "target_rel": 1e-6, "grad": grad.tolist(), "fd": fd.tolist()},
            "gpu_launches_per_gradient": int(st["launches"]), "clocks": clk.summary(),
            "timing": "host wall clock between device synchronisations (gradient and forward alike)"}
    return line


ZIPF_N, ZIPF_T = 10_000_000, 100.0
ZIPF_METRIC = "exp(-iHt)v s (synthetic Zipf(1.5) Hermitian, dim 1e7, t=100, tol 1e-8, m=40)"
ZIPF_WORKLOAD = ("synthetic complex Hermitian H=(A+A^H)/2, dim 1e7, rows of A with Zipf(1.5) lengths clipped to "
                 "[2,256], distinct uniform columns, re/im ~ N(0,1) (device generator, seed 1), scaled by a "
                 "30-step power-iteration estimate of ||H||_2; v complex Gaussian (numpy default_rng(1)); t=100, "
                 "tol=1e-8, m=40, samples at 0 and t")
ZIPF_CPU_N, ZIPF_CPU_T = 1_000_000, 10.0


def run_zipf(args):
    """The load-imbalanced workload: one solve per step with H and v in HBM,
    the apply kernel's roofline, and a CPU sample on a smaller instance."""
    import torch
    import timeevolver_gb300 as te
    te.lib().te_set_device(0)
    t0 = time.perf_counter()
    H, est = te.Matrix.zipf(ZIPF_N, 1.5, 2, 256, 1, 30)
    gen_s = time.perf_counter() - t0
    info = H.info()
    n, nnz = info["n_rows"], info["nnz"]
    rng = np.random.default_rng(1)
    v = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    v /= np.linalg.norm(v)
    v_dev = torch.from_numpy(v.view(np.float64).copy()).cuda()
    ev = te.Evolver(H, v, ZIPF_T, ZIPF_T, [], tol=TOL, m=M_KRYLOV)
    options = {te.OPT_FIXED_SPMV: spmv_option(args.spmv)}
    for opt, val in options.items():
        ev.set_option(opt, val)
    for _ in range(args.warmup):
        ev.reset(None, device_ptr=v_dev.data_ptr())
        ev.run()
    torch.cuda.synchronize()
    stream = torch.cuda.ExternalStream(ev.stream())
    start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    launches = 0
    with ClockSampler(0) as clk:
        start.record(stream)
        for _ in range(args.steps):
            ev.reset(None, device_ptr=v_dev.data_ptr())
            r = ev.run()
            launches += te.lib().te_evolver_launch_count(ev.handle)
        stop.record(stream)
        stop.synchronize()
    value = start.elapsed_time(stop) / 1e3 / args.steps
    apply_ms, apply_n, kernel_ms = profiled_solve(te, ev, v_dev)
    ev.close()
    # end to end through the public call: start vector from the host, state back
    e2e = []
    if args.warmup > 0:  # one untimed call, as for the device-timed solves
        te.evolve(H, v, ZIPF_T, ZIPF_T, [], tol=TOL, m=M_KRYLOV, options=options)
    for _ in range(max(1, args.steps)):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        out = te.evolve(H, v, ZIPF_T, ZIPF_T, [], tol=TOL, m=M_KRYLOV, options=options)
        torch.cuda.synchronize()
        e2e.append(time.perf_counter() - t0)
    peaks = load_peaks(te)
    fl = H.fixed_layout()
    fixed = fl["state"] > 0
    b_format = apply_kernel_bytes(n, nnz, info["real"], fixed, fixed and fl["state"] == 2)
    if fl["state"] == 3:  # column blocks: the int64 row sums written, re-read per block, read by the epilogue
        b_format += 2 * fl["n_values"] * 16 * n
    b_apply = spmv_bytes(n, nnz)
    f_apply = apply_kernel_flops(n, nnz, info["real"], fixed)
    avg = apply_ms / 1e3 / max(1, apply_n)
    line = {"metric": ZIPF_METRIC, "value": value, "unit": "s", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": value * 1e3, "higher_is_better": False, "scaling": "weak",
            "vs_baseline": None, "dtype": "complex128 (FP64)", "data": "synthetic (device generator, seeded)",
            "config": {"workload": ZIPF_WORKLOAD, "n": n, "nnz": nnz, "norm_estimate": est,
                       "spmv": "fixed" if fixed else "fp64",
                       "generation_s": gen_s, "krylov_steps_per_solve": r.n_steps, "status": r.status,
                       "err": r.err, "l2": "inputs larger than L2 (H %.1f GB)" % (nnz * 20 / 1e9)},
            "e2e": {"value": float(np.mean(e2e)), "unit": "s", "h2d_bytes_per_step": 16 * n,
                    "d2h_bytes_per_step": 16 * n + 16},
            "gpu_launches": int(launches),
            "roofline": {"bound": "hbm",
                         "kernel": ("fix_block_kernel x %d + fix_epilogue_kernel (fixed-point SpMV in column "
                                    "blocks, complex H)" % fl["n_values"] if fl["state"] == 3
                                    else "lanczos_apply_fix_kernel (fixed-point SELL-32 SpMV, complex H)" if fixed
                                    else "lanczos_apply_kernel (SELL-32 SpMV, complex H)"),
                         "achieved": b_apply / avg / 1e9, "peak": peaks["hbm_gbs"], "unit": "GB/s",
                         "frac": b_apply / avg / 1e9 / peaks["hbm_gbs"], "peak_source": peaks["source"],
                         "traffic": None, "algorithmic_bytes_per_launch": b_apply,
                         "algorithmic_bytes": "complex128 CSR SpMV, 20 nnz + 4 (n + 1) + 32 n",
                         "format_bytes_per_launch": b_format,
                         "format_frac": b_format / avg / 1e9 / peaks["hbm_gbs"], "avg_launch_us": avg * 1e6,
                         "launches": apply_n,
                         "fp64": {"achieved_tflops": f_apply / avg / 1e12, "peak_tflops": peaks["fp64_tflops"],
                                  "frac": f_apply / avg / 1e12 / peaks["fp64_tflops"],
                                  "flops_per_launch": f_apply}},
            "kernel_ms_per_solve": {k: round(v_[0], 3) for k, v_ in kernel_ms.items()},
            "clocks": clk.summary()}
    if not args.no_cpu_baseline:
        line["cpu_baseline"] = zipf_cpu_baseline(te, nnz, r.n_steps)
    return line


def zipf_cpu_baseline(te, nnz_full, steps_full):
    """The oracle on all host cores on the same generator at dim 1e6, one
    solve to t=10, scaled by the non-zeros and the Krylov step counts."""
    import oracle
    oracle.build()
    Hs, _ = te.Matrix.zipf(ZIPF_CPU_N, 1.5, 2, 256, 1, 30)
    coo = Hs.to_coo()
    rng = np.random.default_rng(1)
    v = rng.standard_normal(ZIPF_CPU_N) + 1j * rng.standard_normal(ZIPF_CPU_N)
    v /= np.linalg.norm(v)
    cores = os.cpu_count()
    t0 = time.perf_counter()
    r = oracle.evolve(coo, v, ZIPF_CPU_T, ZIPF_CPU_T, [], tol=TOL, m=M_KRYLOV, n_threads=cores)
    el = time.perf_counter() - t0
    per_step = el / max(1, r["n_steps"]) * nnz_full / len(coo[2])
    return {"value": per_step * steps_full, "unit": "s", "cores": cores, "kind": "port",
            "sample": "same generator at dim 1e6 (%d non-zeros), t=%g: %d Krylov steps in %.1f s; scaled by the "
                      "non-zero ratio to %.3f s per Krylov step at dim 1e7 and to the %d steps of the full solve "
                      "(extrapolated)" % (len(coo[2]), ZIPF_CPU_T, r["n_steps"], el, per_step, steps_full)}


def ncu_case(t_final, config="plain", zipf_n=2_000_000, spmv=None, fixed_blocks=None):
    """A short solve of the same workload for ncu captures (t_final instead of
    the full time; the Zipf matrix at a smaller dimension)."""
    import timeevolver_gb300 as te
    te.build()
    te.lib().te_set_device(0)
    if config == "zipf":
        H, est = te.Matrix.zipf(zipf_n, 1.5, 2, 256, 1, 30)
        if fixed_blocks is not None:
            H.set_fixed_blocks(fixed_blocks)
        rng = np.random.default_rng(1)
        v = rng.standard_normal(zipf_n) + 1j * rng.standard_normal(zipf_n)
        v /= np.linalg.norm(v)
        out = te.evolve(H, v, t_final, t_final, [], tol=TOL, m=M_KRYLOV,
                        options={te.OPT_FIXED_SPMV: spmv_option(spmv)})
        print("ncu case: zipf n=%d nnz=%d t=%g, %d Krylov steps, status %d, %d launches"
              % (zipf_n, H.info()["nnz"], t_final, out["n_steps"], out["status"], out["launches"]))
        return
    n, Hc, Oc, v = build_problem()
    out = te.evolve(Hc, v, t_final, t_final, [("sparse", Oc)], tol=TOL * t_final / T_FINAL, m=M_KRYLOV,
                    options={te.OPT_FIXED_SPMV: spmv_option(spmv)})
    print("ncu case: t=%g, spmv %s, %d Krylov steps, status %d, %d launches"
          % (t_final, spmv, out["n_steps"], out["status"], out["launches"]))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-other-workloads", action="store_true",
                    help="plain config: skip the load-imbalanced, batched and adjoint workloads that the default run "
                         "measures after the headline and attaches to its line")
    ap.add_argument("--config", default="plain", choices=["plain", "batched", "adjoint", "zipf"],
                    help="plain: the L=12 single evolution (headline); batched: 256 chains in one batch; "
                         "adjoint: gradients of <n_0(T)> for L=10; zipf: the dim-1e7 load-imbalanced matrix")
    ap.add_argument("--ncu-case", type=float, default=None, metavar="T",
                    help="run one short solve to time T (for ncu captures) and exit")
    ap.add_argument("--spmv", default=None, choices=["fixed", "fp64"],
                    help="SpMV arithmetic of the Lanczos passes: fixed-point integer products (the default) or "
                         "FP64 FMAs")
    ap.add_argument("--fixed-blocks", type=int, default=None,
                    help="column blocks of the fixed-point form in --ncu-case runs of --config zipf "
                         "(te_matrix_set_fixed_blocks: 0 automatic, 1 none, 2..8)")
    ap.add_argument("--zipf-n", type=int, default=2_000_000,
                    help="dimension of the Zipf matrix in --ncu-case runs of --config zipf")
    args = ap.parse_args()
    if args.ncu_case is not None:
        ncu_case(args.ncu_case, args.config, args.zipf_n, args.spmv, args.fixed_blocks)
        return
    if args.impl == "reference":
        run_reference(args)
    elif args.config in ("batched", "adjoint", "zipf"):
        import timeevolver_gb300 as te
        te.build()
        fn = {"batched": run_batched, "adjoint": run_adjoint, "zipf": run_zipf}[args.config]
        print(json.dumps(fn(args)), flush=True)
    else:
        import timeevolver_gb300 as te
        te.build()
        run_gb300(args)


if __name__ == "__main__":
    main()
