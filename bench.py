"""Benchmark of the wave-solver hot path: FP32 batched forward + adjoint + kernel accumulation.

Workload (the batched FP32 configuration): 32 sources at x = -200 + 12.5 (s + 0.5) Mm over a
400 Mm box, nx = 512, nz = 300 polytrope, supergranule stream-function flow (vx peak 240 m/s)
and a 5 % Gaussian sound-speed bump, 3600 steps of 2 s, receivers every 2 Mm.  One bench step
is one full forward solve (with partial states kept in HBM every 15 steps) plus one full
adjoint solve with the kernel integral accumulated at every record, for all 32 sources.
Metric: grid-point steps per second, forward and adjoint steps counted once each.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

--impl reference times the CPU restatement of the reference Fortran (the FP64 oracle; the
Fortran itself cannot be built here) on all host cores, one solve per core, on a bounded
sample of the same workload.  Under torchrun only rank 0 runs it.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOAD = "batch32: 32 sources, nx=512 (400 Mm), nz=300 polytrope, psi flow 240 m/s + 5% c bump, 3600 steps"
METRIC = "fwd+adj grid-pt-steps/s: FP32 batched vs FP64 plain, 1 GB300, <=1e-4 rel err"
UNIT = "grid-pt-steps/s"


def words_per_point_step(nx, nz, npmlbot=20, npmltop=10, npmlhor=9, V=4, B=3):
    """Algorithmic words per grid-point step of the fused schedule: 15 V + 10 + 5 B + 15 Naux/N."""
    naux = 2 * nx * (npmlbot + npmltop) + 2 * (2 * npmlhor) * nz
    return 15 * V + 10 + 5 * B + 15 * naux / (nx * nz)


def column_words_per_point(nz, c2d=True, flows=True, npmlbot=20, npmltop=10, bg_shared_by=1):
    """Algorithmic words per grid point of one column-pass launch (one RK stage), averaged over
    the five stages: reads xi_z, v_z, v_x, dxi_x/dx, and with flows FXX, FXZ; the 2-D background
    c2rho0 and v0z (once per launch when the bg_shared_by solves of the batch share it); the RHS
    ring tiles (rhs v_z of stage s-2 in stages 3-5, rhs v_x and v_z of stage s-1 in stages 2-5);
    writes p, the partial RHS of v_x and rhs v_z; PML rows add psi_vz and psi_p (state read,
    ring read in stages 2-5, ring write) and az, bz, fdz."""
    bg = ((1 if c2d else 0) + (1 if flows else 0)) / bg_shared_by
    reads = 4 + (2 if flows else 0) + bg + 3 / 5 + 2 * 4 / 5
    writes = 3
    pml = (npmlbot + npmltop) / nz * (2 * (1 + 4 / 5 + 1) + 3)
    return reads + writes + pml


def ncu_traffic(kernel):
    """DRAM bytes per launch of `kernel` from the committed ncu summary (None if absent)."""
    try:
        with open(os.path.join(ROOT, "profiles", "ncu_traffic.json")) as f:
            return json.load(f)[kernel]["dram_bytes_per_launch"]
    except (OSError, KeyError, ValueError):
        return None


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms while running."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index=0):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            p = [v.strip() for v in ln.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                smax = float(p[2])
            except ValueError:
                continue
            for n, v in zip(names, p[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peak_hbm():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


# ----------------------------------------------------------------------------------------------
def run_reference(args):
    """CPU arm: the FP64 oracle on all host cores, one solve per core (bounded sample)."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    import numpy as np
    from oracle import oracle as O
    from sparc_flows_gb300 import model as M

    run, model, specs, psi, cmul = M.workload("batch32")
    cores = os.cpu_count() or 1
    nsolve = min(cores, len(specs))
    sample_steps = int(os.environ.get("SPARC_CPU_SAMPLE_STEPS", "40"))
    xlocs = [s.xloc for s in specs[:nsolve]]
    O.build()

    def sample():
        t0 = time.perf_counter()
        O.run_batch(run.replace(nsteps=sample_steps), model, xlocs, psi, sample_steps, nsolve)
        return time.perf_counter() - t0

    for _ in range(args.warmup):
        sample()
    ts = [sample() for _ in range(args.steps)]
    units = nsolve * run.nx * run.nz * sample_steps
    value = units * len(ts) / sum(ts)
    desc = (f"{nsolve} forward solves of the batch32 grid ({sample_steps} steps each, one per host thread); "
            "adjoint steps cost the same per grid-point step")
    out = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "higher_is_better": True,
           "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
           "ms_per_step": 1e3 * sum(ts) / len(ts), "scaling": "weak", "vs_baseline": None, "dtype": "f64",
           "data": "synthetic", "config": {"workload": WORKLOAD, "sample": desc},
           "cpu_baseline": {"value": value, "unit": UNIT, "cores": nsolve, "kind": "port", "sample": desc},
           "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)


def cpu_baseline_quick():
    """Bounded oracle sample for the gb300 line's cpu_baseline (~10-20 s)."""
    from oracle import oracle as O
    from sparc_flows_gb300 import model as M

    run, model, specs, psi, cmul = M.workload("batch32")
    cores = os.cpu_count() or 1
    nsolve = min(cores, len(specs))
    steps = int(os.environ.get("SPARC_CPU_SAMPLE_STEPS", "40"))
    O.build()
    t0 = time.perf_counter()
    O.run_batch(run.replace(nsteps=steps), model, [s.xloc for s in specs[:nsolve]], psi, steps, nsolve)
    dt = time.perf_counter() - t0
    v = nsolve * run.nx * run.nz * steps / dt
    return {"value": v, "unit": UNIT, "cores": nsolve, "kind": "port",
            "sample": f"{nsolve} FP64 forward solves x {steps} steps of the batch32 grid on {nsolve} host threads"}


def plain64_oracle_records(nsteps):
    """Seismograms of the plain FP64 workload from the FP64 oracle (the checker of the fp64_plain
    figure); runs in a spawned process while the GPU is timed."""
    from oracle import oracle as O
    from sparc_flows_gb300 import model as M

    run, model, specs, _, _ = M.workload("plain64")
    run = run.replace(nsteps=nsteps)
    sp = specs[0]
    sim = O.OracleSim(run, model)
    sim.set_forward_source(sp.xloc, sp.spatial, sp.sigma, sp.temporal, sp.nu0, run.nsteps + 8)
    seis = sim.run_steps(run.nsteps)
    sim.close()
    return seis


def gradient_stage(pipe, model, dev, reps=20, cpu=True):
    """The gradient post-processing of grad.py on this batch's own kernels: sparc_gradient (kernel
    sum, hessian preconditioning, x/z filters, antisymmetrisation), a conjugate-gradient direction
    and three line-search models, timed with CUDA events; the oracle's NumPy restatement of
    grad.py timed on the host beside it (grad.py is NumPy, so this is the reference's own
    arithmetic cost, without its FITS reads)."""
    import numpy as np
    import torch

    from sparc_flows_gb300 import gradient as GR

    fk = pipe.final_kernels(summed=False)
    kp, hs = fk["kernel_psi"].contiguous(), fk["hessian"].contiguous()
    nsrc, nz, nx = kp.shape
    rho = torch.as_tensor(np.ascontiguousarray(model[:, 2]), dtype=torch.float64, device=dev)
    ws = GR.Workspace(nx, nz, dev)
    stream = torch.cuda.current_stream()
    g = GR.gradient_psi(kp, hs, rho, ws=ws)
    gp, pp = 0.9 * g, -g
    GR.update_direction("cg", g, gp, pp, ws=ws)
    torch.cuda.synchronize()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
    ev[0].record(stream)
    for _ in range(reps):
        GR.gradient_psi(kp, hs, rho, ws=ws)
    ev[1].record(stream)
    for _ in range(reps):
        u, _ = GR.update_direction("cg", g, gp, pp, ws=ws)
        GR.linesearch_models(g, u, [0.01, 0.02, 0.03], ws=ws)
    ev[2].record(stream)
    torch.cuda.synchronize()
    grad_ms = ev[0].elapsed_time(ev[1]) / reps
    upd_ms = ev[1].elapsed_time(ev[2]) / reps
    n = nz * nx
    grad_bytes = (2 * nsrc * n + n + nz) * 8  # per-source kernels and hessians read once, gradient written
    peak, peak_kind = measured_peak_hbm()
    out = {"workload": f"{nsrc} sources, nz={nz}, nx={nx}, FP64 (grad.py:188-202, 204-250, 351-378)",
           "gradient_ms": grad_ms, "update_and_linesearch_ms": upd_ms,
           "gradient_algorithmic_bytes": grad_bytes,
           "gradient_achieved_gbs": grad_bytes / (grad_ms * 1e-3) / 1e9,
           "gradient_frac_of_hbm": grad_bytes / (grad_ms * 1e-3) / 1e9 / peak, "peak_kind": peak_kind,
           "launches": {"gradient": 4, "cg_direction": 5, "linesearch_models": 5}}
    if cpu:
        from oracle import grad_oracle as go
        kh, hh, gh = kp.cpu().numpy(), hs.cpu().numpy(), g.cpu().numpy()
        t0 = time.perf_counter()
        ref = go.gradient_psi(kh, hh, model[:, 2])
        t1 = time.perf_counter()
        uh, _ = go.cg_update(gh, 0.9 * gh, -gh)
        go.ls_models(gh, uh, [0.01, 0.02, 0.03])
        t2 = time.perf_counter()
        out["cpu_numpy_ms"] = {"gradient": (t1 - t0) * 1e3, "update_and_linesearch": (t2 - t1) * 1e3,
                               "cores": 1, "kind": "port"}
        out["rel_err_vs_numpy"] = float(np.linalg.norm(gh - ref) / np.linalg.norm(ref))
    return out


def tt_stage(seis, run, specs, dev, cpu=True):
    """The travel-time adjoint source (ADJOINT_SOURCE_FILT) of every source of the batch from its
    own seismograms: all nine ridge filters with 5-60 Mm receiver ranges and 10-18 min windows,
    data = 0.95 times the synthetic one record later.  GPU time with CUDA events around
    TTAdjoint.run; the oracle's per-receiver restatement timed on one host core for one source."""
    import numpy as np
    import torch

    from sparc_flows_gb300.ttadjoint import TTAdjoint

    s = seis.double().contiguous()
    nb, nt, nx = s.shape
    d = (0.95 * torch.roll(s, 1, dims=1)).contiguous()
    modes = {p: (5.0, 60.0, 10.0 + p) for p in range(9)}
    freq = {"allmodes": (1.5, 6.0)}
    t_min = np.arange(nt) * (run.outputcad / 60.0)
    x00s = [sp.xloc for sp in specs]
    tt = TTAdjoint(nx, nt, nb, run.xlength_cm, run.outputcad, device=dev)
    tt.run(s, d, x00s, t_min, modes, freq)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    res = tt.run(s, d, x00s, t_min, modes, freq)
    e1.record()
    torch.cuda.synchronize()
    gpu_ms = e0.elapsed_time(e1)
    out = {"workload": f"{nb} sources, {nt} records x {nx} columns, 9 ridge filters, FP64 (driver.f90:1758-2238)",
           "gpu_ms_all_sources": gpu_ms, "measurements": int(res["nmeas"].sum())}
    if cpu:
        # a source in the middle of the box: every receiver in its ranges carries signal (the edge
        # columns x = 0 and nx - 1 are held at zero, and a window there measures rounding noise,
        # differently in any two FFT implementations)
        from oracle import tt_oracle as TO
        bm = nb // 2
        t0 = time.perf_counter()
        ref = TO.adjoint_source(s[bm].cpu().numpy(), d[bm].cpu().numpy(), x00s[bm], run.xlength_cm, t_min,
                                run.outputcad, modes, freq)
        cpu_s = time.perf_counter() - t0
        a = res["adj"][bm].cpu().numpy()
        out["cpu_numpy_ms_one_source"] = cpu_s * 1e3
        out["cpu_kind"] = "port (per-receiver 2-D transforms as the reference, numpy.fft, 1 core)"
        out["gpu_ms_per_source"] = gpu_ms / nb
        out["oracle_source"] = bm
        out["rel_err_vs_oracle"] = float(np.linalg.norm(a - ref["adj"]) / max(np.linalg.norm(ref["adj"]), 1e-300))
    tt.close()
    return out


# ----------------------------------------------------------------------------------------------
def run_gpu(args):
    import numpy as np
    import torch
    import torch.distributed as dist

    from sparc_flows_gb300 import model as M
    from sparc_flows_gb300.pipeline import FwdAdjKernels

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    # the oracle's plain64 records (the fp64_plain figure's checker), computed on one host core in
    # a spawned process while the GPU runs; started before the first CUDA call
    oracle_job = None
    if rank == 0 and not args.no_plain and not args.no_cpu:
        import concurrent.futures as cf
        import multiprocessing as mp
        pool = cf.ProcessPoolExecutor(max_workers=1, mp_context=mp.get_context("spawn"))
        oracle_job = (pool, pool.submit(plain64_oracle_records, min(args.nsteps or 1800, 1800)))
    if world > 1:
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = f"cuda:{local}"

    run, model, specs, psi, cmul = M.workload("batch32")
    if world > 1:
        # weak scaling: 32 sources per GPU, the 32 * world sources of the job spread uniformly
        # over the box and split contiguously between the ranks (distributed.shard)
        from sparc_flows_gb300.distributed import shard, sum_kernels
        nall = len(specs) * world
        allspecs = [M.SourceSpec(-200.0 + (400.0 / nall) * (s + 0.5)) for s in range(nall)]
        specs = shard(allspecs, rank, world)
    if args.nsteps:
        run = run.replace(nsteps=args.nsteps)
    pipe = FwdAdjKernels(run, model, specs, psi=psi, cmul=cmul, precision=32, device=dev)
    stream = torch.cuda.current_stream()

    def barrier():
        if world > 1:
            dist.barrier()

    def job_step():
        """Forward + adjoint + kernels of this rank's sources, then the kernel sum over every source
        of the job (grad.py:188-196), the only exchange between ranks."""
        pipe.run_all()
        if world > 1:
            sum_kernels({"kacc": pipe.kacc.sum(0)})

    for _ in range(args.warmup):
        job_step()
    torch.cuda.synchronize()
    barrier()
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        ev0.record(stream)
        for _ in range(args.steps):
            job_step()
        ev1.record(stream)
        torch.cuda.synchronize()
    barrier()
    torch.cuda.synchronize()
    ms = ev0.elapsed_time(ev1)
    t = torch.tensor([ms], device=dev)
    if world > 1:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    ms = float(t.item())
    units = pipe.point_steps() * args.steps * world
    value = units / (ms * 1e-3)

    # ---- per-pass timing (CUDA events on the launching stream, outside the timed loop)
    passes = pipe.fwd.profile_passes(nsteps=20)

    # ---- the FP64 plain single-source path (plain64: nx=256, no flow, 1800 steps), same pipeline
    plain = None
    if not args.no_plain:
        prun, pmodel, pspecs, ppsi, pcmul = M.workload("plain64")
        if args.nsteps:
            prun = prun.replace(nsteps=min(args.nsteps, prun.nsteps))
        pp = FwdAdjKernels(prun, pmodel, pspecs, psi=ppsi, cmul=pcmul, precision=64, device=dev)
        pp.run_all()
        torch.cuda.synchronize()
        q0, q1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        q0.record(stream)
        for _ in range(2):
            pp.run_all()
        q1.record(stream)
        torch.cuda.synchronize()
        pms = q0.elapsed_time(q1) / 2
        plain = {"workload": "plain64: 1 source, nx=256 (200 Mm), nz=300, no flow, 1800 steps, FP64",
                 "value": pp.point_steps() / (pms * 1e-3), "unit": UNIT, "ms_per_run": pms,
                 "column_kernel": pp.fwd.column_kernel_name()}
        plain_seis = pp.seis[0].double().cpu().numpy()
        pp.close()
        if oracle_job is not None:
            pool, fut = oracle_job
            ref = fut.result()
            pool.shutdown()
            plain["seismograms_rel_l2_vs_oracle"] = float(np.linalg.norm(plain_seis - ref) / np.linalg.norm(ref))
            plain["oracle"] = "FP64 CPU restatement (physics2d.f90:943-1094, step.f90:43-119), same inputs"

    # ---- end-to-end through the public API: pinned host inputs in, host kernels/seismograms out
    nrec = run.nrec
    data_h = torch.zeros((len(specs), nrec, run.nx), dtype=torch.float32).pin_memory()
    psi_h = torch.as_tensor(psi, dtype=torch.float64).pin_memory()
    kern_h = torch.empty((4, run.nz, run.nx), dtype=torch.float64).pin_memory()
    seis_h = torch.empty((len(specs), nrec, run.nx), dtype=torch.float32).pin_memory()
    h2d = data_h.numel() * 4 + psi_h.numel() * 8
    d2h = kern_h.numel() * 8 + seis_h.numel() * 4
    e2e_steps = max(1, min(args.steps, 2))
    torch.cuda.synchronize()
    barrier()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(e2e_steps):
        data_d = data_h.to(dev, non_blocking=True)
        psi_d = psi_h.to(dev, non_blocking=True)
        pipe.fwd.update_flow(psi_d)
        pipe.adj.update_flow(psi_d)
        seis, kacc = pipe.run_all(data_d)
        kern_h.copy_(kacc.sum(0), non_blocking=True)
        seis_h.copy_(seis, non_blocking=True)
    e1.record(stream)
    torch.cuda.synchronize()
    e2e_ms = e0.elapsed_time(e1)
    te = torch.tensor([e2e_ms], device=dev)
    if world > 1:
        dist.all_reduce(te, op=dist.ReduceOp.MAX)
    e2e_ms = float(te.item())
    e2e_value = pipe.point_steps() * e2e_steps * world / (e2e_ms * 1e-3)

    # ---- the same batch with the forward field checkpointed in HBM every 16 records and recomputed
    # per segment during the adjoint run (one run after a warm-up; kernels equal the stored run's)
    checkpointed = None
    if rank == 0 and not args.no_checkpoint:
        ckp = FwdAdjKernels(run, model, specs, psi=psi, cmul=cmul, precision=32, device=dev, checkpoint_every=16)
        ckp.run_all()
        torch.cuda.synchronize()
        c0, c1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        c0.record(stream)
        ckp.run_all()
        c1.record(stream)
        torch.cuda.synchronize()
        cms = c0.elapsed_time(c1)
        checkpointed = {"every_records": 16, "value": ckp.point_steps() / (cms * 1e-3), "unit": UNIT,
                        "ms_per_run": cms, "forward_solves_per_run": 2,
                        "partial_state_bytes": ckp.snaps.numel() * ckp.snaps.element_size() + ckp.ckpt.numel(),
                        "stored_partial_state_bytes": pipe.snaps.numel() * pipe.snaps.element_size()}
        ckp.close()

    # ---- accuracy of the FP32 batched path against FP64 on one source of the same workload
    accuracy = None
    if rank == 0 and not args.no_accuracy:
        from sparc_flows_gb300.accuracy import fp32_vs_fp64
        accuracy = fp32_vs_fp64("batch32", source=15, nsteps=run.nsteps, device=dev)

    if rank == 0:
        words = words_per_point_step(run.nx, run.nz)
        peak, peak_kind = measured_peak_hbm()
        achieved = words * 4 * value / world / 1e9  # GB/s on one GPU, whole step
        dom = max(passes["per_class_ms"], key=passes["per_class_ms"].get)
        # dominant kernel: the column pass, five launches per step, timed with CUDA events
        col_launch_ms = passes["per_class_ms"]["column"] / 5
        col_bytes = column_words_per_point(run.nz, bg_shared_by=len(specs)) * 4 * len(specs) * run.nx * run.nz
        col_achieved = col_bytes / (col_launch_ms * 1e-3) / 1e9
        col_kernel = pipe.fwd.column_kernel_name()
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": WORKLOAD, "sources_per_gpu": len(specs), "nx": run.nx, "nz": run.nz,
                       "nsteps": run.nsteps, "step": "forward + adjoint + kernel integral of all sources",
                       "l2": "inputs larger than L2 (working set ~0.4 GB state + 28 GB partial states per GPU)",
                       "parallelism": (f"dp{world}: {len(specs) * world} sources sharded over {world} GPUs, "
                                       "one FP64 kernel-sum all-reduce per step" if world > 1 else
                                       "1 GPU, 32 sources in one batch")},
            "roofline": {"bound": "hbm", "achieved": col_achieved, "peak": peak, "unit": "GB/s",
                         "frac": col_achieved / peak, "traffic": ncu_traffic(col_kernel),
                         "kernel": col_kernel, "peak_kind": peak_kind,
                         "algorithmic_bytes_per_launch": col_bytes, "launch_ms": col_launch_ms,
                         "step": {"achieved": achieved, "frac": achieved / peak,
                                  "algorithmic_bytes_per_point_step": words * 4,
                                  "dominant_pass": dom, "pass_ms_per_step": passes["per_class_ms"],
                                  "pass_share": passes["share"]}},
            "clocks": clk.summary(),
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                    "steps": e2e_steps},
            "gpu_launches": pipe.launch_count() * args.steps,
        }
        if plain is not None:
            plain["fp32_batched_over_fp64_plain"] = (value / world) / plain["value"]
            line["fp64_plain"] = plain
        if accuracy is not None:
            line["accuracy"] = accuracy
        if checkpointed is not None:
            line["checkpointed"] = checkpointed
        if not args.no_gradient:
            line["gradient"] = gradient_stage(pipe, model, dev, cpu=not args.no_cpu)
            line["tt_adjoint_source"] = tt_stage(seis_h.to(dev), run, specs, dev, cpu=not args.no_cpu)
        if not args.no_cpu:
            line["cpu_baseline"] = cpu_baseline_quick()
        print(json.dumps(line), flush=True)
    pipe.close()
    if world > 1:
        dist.destroy_process_group()


def run_uneven(args):
    """48 independent solves (nx 256/384/512, 1800/2700/3600 steps, flow 0-300 m/s, dc/c 0-5 %,
    seed 0), grouped by (nx, steps) into batched plans that run concurrently on their own
    streams.  value = useful grid-point steps (forward + adjoint) / device time of K full runs."""
    import torch
    from sparc_flows_gb300 import model as M
    from sparc_flows_gb300.uneven import UnevenBatch

    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    solves = M.uneven_solves(48, seed=0)
    if args.nsteps:
        solves = [M.Solve(s.nx, min(s.nsteps, args.nsteps), s.vpeak_ms, s.dcc, s.xloc) for s in solves]
    ub = UnevenBatch(solves, precision=32, device=f"cuda:{local}", autotune=args.autotune)
    for _ in range(args.warmup):
        ub.run()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        e0.record()
        for _ in range(args.steps):
            ub.run()
        torch.cuda.synchronize()
        e1.record()
        torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    value = ub.point_steps() * args.steps / (ms * 1e-3)
    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": 1, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
                "config": {"workload": "uneven48: 48 solves, nx 256/384/512, 1800/2700/3600 steps, "
                                       "flow U(0,300) m/s, dc/c U(0,0.05), seed 0",
                           "groups": {f"{k[0]}x{k[1]}": len(v) for k, v in ub.groups.items()},
                           "column_pass_autotuned": {f"{k[0]}x{k[1]}": list(v["choice"]) for k, v in ub.tuned.items()},
                           "l2": "inputs larger than L2", "parallelism": "9 batched plans on 9 concurrent streams"},
                "clocks": clk.summary(), "gpu_launches": None}
        if args.accuracy:
            errs = ub.errors_against_fp64()
            names = [k for k in errs[0] if k not in ("nx", "nsteps")]
            line["per_solve_error_vs_fp64"] = {
                "solves": [{"nx": e["nx"], "nsteps": e["nsteps"], **{k: e[k] for k in names}} for e in errs],
                "max": {k: max(e[k] for e in errs) for k in names},
                "how": "rel-L2 of each solve's FP32 seismograms and scaled kernels against the same solve "
                       "run through FP64 plans"}
        print(json.dumps(line), flush=True)
    ub.close()


def run_3d(args):
    """The 3-D configuration: 4 sources on a 256 x 256 x 300 grid (200 Mm box), axisymmetric
    outflow, FP32.  One bench step = 100 time steps of the batch (the checkpoint interval);
    value = grid-point steps / device time.  e2e: the same through WaveSolver3D with the source
    table uploaded from the host and the v_z records read back every bench step."""
    import numpy as np
    import torch
    from sparc_flows_gb300 import model as M
    from sparc_flows_gb300.solver3d import WaveSolver3D

    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    nx = ny = 256
    nz, nsrc, chunk = 300, 4, 100
    model, xl, v0, pats = M.workload_3d(nx, ny, nz, nsrc)
    ws = WaveSolver3D(nx, ny, model, xl, nbatch=nsrc, precision=32, flows=True, steps_out=15,
                      device=f"cuda:{local}")
    ws.set_flow(*v0)
    run = M.uneven_run(512, 3600)
    amp = M.source_time_series(run, M.SourceSpec(0.0), 3600 + 8)[1:]
    ws.set_source(pats, amp)
    ws.reset(0)
    for _ in range(args.warmup):
        ws.forward(chunk)
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        e0.record(stream)
        for _ in range(args.steps):
            ws.forward(chunk)
        e1.record(stream)
        torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    units = ws.point_steps(chunk) * args.steps
    value = units / (ms * 1e-3)
    # end to end: the source table from pinned host memory in, the records to pinned host memory out
    amp_h = torch.as_tensor(amp).pin_memory()
    rec_h = torch.empty((chunk // 15 + 1, nsrc, ny, nx), dtype=torch.float32).pin_memory()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(max(1, args.steps)):
        ws.set_source(pats, amp_h.numpy())
        rec = ws.forward(chunk)
        rec_h[:rec.shape[0]].copy_(rec, non_blocking=True)
        torch.cuda.synchronize()
    e2e_s = time.perf_counter() - t0
    e2e = units / args.steps * max(1, args.steps) / e2e_s
    ws.close()
    # forward + adjoint + kernel integral of the same batch with the forward field checkpointed in
    # HBM every 100 steps and recomputed per segment (pipeline3d); a run of `fa_steps` steps
    from sparc_flows_gb300.pipeline3d import FwdAdjKernels3D
    fa_steps = args.nsteps or 200
    fak = FwdAdjKernels3D(nx, ny, model, xl, pats, amp, fa_steps, flow=v0, precision=32, steps_out=15,
                          checkpoint_every=100, device=f"cuda:{local}")
    fak.run_all()
    torch.cuda.synchronize()
    f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    f0.record(stream)
    fak.run_all()
    f1.record(stream)
    torch.cuda.synchronize()
    fa_ms = f0.elapsed_time(f1)
    fwd_adj = {"workload": f"{nsrc} sources, {nx} x {ny} x {nz}, {fa_steps} steps, forward + adjoint + kernel "
                           "integral, checkpoint every 100 steps (recomputed per segment)",
               "value": fak.point_steps() / (fa_ms * 1e-3), "unit": UNIT, "ms_per_run": fa_ms,
               "solves_per_run": 3, "records": fak.nrec, "checkpoint_bytes": int(fak.ckpt.numel()),
               "record_buffer_bytes": int(fak.snaps.numel() * fak.snaps.element_size())}
    fak.close()
    words = 15 * 6 + 10 + 5 * 3 + 15 * (2 * 20 / nz)  # 15 V + 10 + 5 B + 15 Naux/N, 20 PML levels: 117 words
    peak, peak_kind = measured_peak_hbm()
    achieved = words * 4 * value / 1e9
    line = {"metric": "3-D grid-pt-steps/s (FP32 batched, option 16)", "value": value, "unit": UNIT,
            "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": "3d4: 4 sources, 256 x 256 x 300 polytrope, 200 Mm box, outflow 300 m/s, "
                                   "100 time steps per bench step", "l2": "inputs larger than L2 (8 GB of fields)"},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": None, "peak_kind": peak_kind,
                         "algorithmic_bytes_per_point_step": words * 4, "scope": "whole step"},
            "clocks": clk.summary(),
            "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": amp_h.numel() * 8,
                    "d2h_bytes_per_step": int(rec_h.numel() * 4)},
            "gpu_launches": None, "fwd_adj_kernels": fwd_adj}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--nsteps", type=int, default=0, help="override the 3600 time steps (testing only)")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-plain", action="store_true", help="skip the FP64 plain reference path")
    ap.add_argument("--no-accuracy", action="store_true", help="skip the FP32-vs-FP64 accuracy report")
    ap.add_argument("--no-gradient", action="store_true", help="skip the gradient post-processing figures")
    ap.add_argument("--no-checkpoint", action="store_true", help="skip the checkpointed-run figures")
    ap.add_argument("--autotune", action="store_true", help="uneven48: pick each group's column pass first, timed with every group running at once")
    ap.add_argument("--accuracy", action="store_true",
                    help="uneven48: each solve's FP32 error against the same solve in FP64 (one more FP64 run)")
    ap.add_argument("--workload", default="batch32", choices=["batch32", "uneven48", "3d4"],
                    help="uneven48: 48 solves of mixed grids, lengths and backgrounds (seed 0)")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "3d4":
        run_3d(args)
    elif args.workload == "uneven48":
        run_uneven(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
