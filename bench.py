"""Benchmark: batched 2-D Rayleigh-Benard FP64 time steps on one GB300.

Workload (default, the batched configuration the headline metric is quoted
on): 256 independent RBC instances, Nx and Ny drawn iid from {33, 65, 129}
(numpy default_rng(99)), Ra log-uniform in [1e4, 1e7] (same generator),
Pr = 1, aspect 1, dt = 0.005, IMEX Euler, 3/2 dealiasing, case "linear",
T = conductive profile + 1e-3 U(-1,1) noise with seed 100 + i.

A step = one time step of every instance (all 256), replayed from one CUDA
graph of eleven fused line-program launches.  ``value`` = instance-steps/s with
the state resident in HBM; ``e2e`` = the same through the public API with the
state in pinned host memory (one H2D copy of every instance's state before and
one D2H copy after each step, inside the timed region).  ``plain`` = the same
instances run one by one on the per-instance GPU path.  ``persistent`` = the
same batch with several steps of every instance in one persistent launch
(pgx_run_persistent), replayed from a graph.  ``adjoint`` = the
adjoint steady-state search (129 x 129, Ra 1e5, 200-step horizon, checkpoints
every 20 steps): gradients/s, cost against the forward sweep, finite-difference
check on 20 random directions, 50 descent iterations.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
                    [--instances 256] [--workload c4|c1|c3|c2|c5] [--adjoint-iters 50]
Under torchrun every rank runs its own batch (weak scaling, no collective on
the data path); rank 0 prints one JSON line.
"""
import argparse
import json
import os
import statistics
import subprocess
import tempfile
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "2D RBC FP64 steps/s at 1 GB300: plain vs batched-graph; adjoint grads/s at 1e-6 rel"
# DFMA throughput of one GB300 at 2070 MHz measured with the same probe kernel (profiles/gb300_fp64_probe.txt);
# used only when the in-process measurement (fp64_peak below) cannot run
FP64_PEAK_FALLBACK_TFLOPS = 1.256
# committed ncu summary of the dominant pass on the 256-instance workload: DRAM bytes per step of the pass
TRAFFIC_PROFILE = os.path.join(ROOT, "profiles", "line_program_batched_c4_p2_traffic.txt")


def workload_specs(kind, n_instances, rank=0):
    """(shape, ra, dt, seed, amplitude, aspect) for every instance of the workload."""
    if kind == "c4":
        rng = np.random.default_rng(99)
        sizes = rng.choice([33, 65, 129], size=(n_instances * (rank + 1), 2))[n_instances * rank:]
        ras = 10.0 ** rng.uniform(4.0, 7.0, n_instances * (rank + 1))[n_instances * rank:]
        return [((int(a), int(b)), float(ra), 0.005, 100 + n_instances * rank + i, 1e-3, 1.0)
                for i, ((a, b), ra) in enumerate(zip(sizes, ras))]
    if kind == "c1":
        return [((65, 65), 1e5, 0.01, 0, 1e-3, 1.0)]
    if kind == "c3":
        return [((513, 257), 1e8, 1e-3, 2, 1e-3, 2.0)]
    raise ValueError(kind)


WORKLOAD_NAMES = {
    "c4": "batched 2D RBC: {n} instances, Nx,Ny iid {{33,65,129}}, Ra log-uniform [1e4,1e7], Pr 1, dt 0.005",
    "c1": "plain 2D RBC 65x65, Ra 1e5, Pr 1, dt 0.01",
    "c3": "large plain 2D RBC 513x257, aspect 2, Ra 1e8, Pr 1, dt 1e-3",
}


def max_over_ranks(x):
    """Max of a host scalar over the ranks of the default process group (nccl: through the
    rank's GPU; gloo: on the host)."""
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(x)], device=dev, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def aggregate_value(n_inst_per_rank, world, steps, total_ms_max):
    """Whole-job instance-steps/s: every rank steps its own instances; time = the slowest rank."""
    return n_inst_per_rank * world * steps / (total_ms_max / 1e3)


# ------------------------------------------------------------------ CPU side
_WORKER = {}
BLAS_ENV = ("OMP_NUM_THREADS", "OPENBLAS_NUM_THREADS", "MKL_NUM_THREADS")


def _oracle_init(specs):
    sys.path.insert(0, ROOT)
    from oracle import rbc2d as orb
    sols = []
    for shape, ra, dt, seed, amp, aspect in specs:
        ns = orb.NavierStokes(case="linear", shape=shape, ra=ra, pr=1.0, dt=dt, aspect=aspect, dealias=True,
                              integrator="eu", beta=1.0, tsave=None)
        orb.seeded_temperature(ns, seed, amp)
        sols.append(ns)
    _WORKER["sols"] = sols


def _oracle_steps(steps):
    sols = _WORKER["sols"]
    t0 = time.perf_counter()
    for _ in range(steps):
        for ns in sols:
            ns.update()
    return time.perf_counter() - t0, len(sols) * steps


def _oracle_flavour():
    """How the CPU oracle runs here: with its compiled banded sweeps (oracle/kernels.c, the
    counterpart of the reference's Fortran) when built, else NumPy loops throughout."""
    sys.path.insert(0, ROOT)
    from oracle import _ck
    return "NumPy restatement of the reference path" + (", banded sweeps in compiled C" if _ck.lib() else "")


class CpuPort:
    """The CPU oracle (NumPy restatement of the reference path) on ``cores`` spawned
    processes, each owning a slice of the instances; solvers are built once."""

    def __init__(self, specs, cores):
        import multiprocessing as mp
        self.chunks = [c for c in (specs[i::cores] for i in range(cores)) if c]
        ctx = mp.get_context("spawn")
        self.pools = []
        # one BLAS thread per worker process: the processes are the parallelism
        saved = {k: os.environ.get(k) for k in BLAS_ENV}
        os.environ.update({k: "1" for k in BLAS_ENV})
        try:
            for c in self.chunks:
                self.pools.append(ctx.Pool(1, initializer=_oracle_init, initargs=(c,)))
        finally:
            for k, v in saved.items():
                if v is None:
                    os.environ.pop(k, None)
                else:
                    os.environ[k] = v

    def step(self, steps=1):
        """Advance every instance ``steps`` steps; returns (instance-steps done, wall s of stepping)."""
        res = [p.apply_async(_oracle_steps, (steps,)) for p in self.pools]
        out = [r.get() for r in res]
        return sum(o[1] for o in out), max(o[0] for o in out)

    def close(self):
        for p in self.pools:
            p.close()
            p.join()


def cpu_sample(specs, steps, warmup):
    """The one CPU measurement of both CPU legs (the GPU arm's ``cpu_baseline`` and the reference
    arm): every instance of the workload in single-threaded spawned processes on all host cores,
    ``warmup`` untimed steps, then ``steps`` timed steps.  Returns (instance-steps/s, cores,
    description, wall s of the timed steps)."""
    cores = min(host_cores(), len(specs))
    port = CpuPort(specs, cores)
    for _ in range(max(warmup, 1)):
        port.step(1)
    done, wall = 0, 0.0
    for _ in range(steps):
        d, w = port.step(1)
        done, wall = done + d, wall + w
    port.close()
    desc = ("all %d instances x %d timed step(s) after %d warm-up, CPU oracle (%s) in %d single-threaded spawned "
            "processes, %.1f s of stepping (%.0f core-s)"
            % (len(specs), steps, max(warmup, 1), _oracle_flavour(), cores, wall, wall * cores))
    return done / wall, cores, desc, wall


def host_cores():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


# ------------------------------------------------------------------ clocks
class ClockSampler:
    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index, path=None):
        self.proc = None
        self.path = path or os.path.join(tempfile.gettempdir(), "pgx_bench_clocks.csv")
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(gpu_index), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "50"], stdout=self.f,
                                         stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.f.close()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                smax.append(float(parts[1]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[4:8]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "samples": len(sm),
                "reasons": sorted(reasons)}


# ------------------------------------------------------------------ GPU side
def build_batch(specs, split=None):
    from pypde_gb300.navier.fused import FusedBatch
    from pypde_gb300.navier.rbc2d import NavierStokes
    solvers = []
    for shape, ra, dt, seed, amp, aspect in specs:
        ns = NavierStokes(case="linear", shape=shape, ra=ra, pr=1.0, dt=dt, aspect=aspect, dealias=True,
                          integrator="eu", beta=1.0, tsave=None)
        ns.set_temperature_noise(seed, amp)
        solvers.append(ns)
    return solvers, FusedBatch(solvers, split=split)


def time_steps(fn, steps, stream, between=None):
    """Per-step CUDA events on ``stream``; returns the list of step times in ms.  ``between`` runs
    before every step, outside the events (the L2 flush of small working sets)."""
    import torch
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    for a, b in ev:
        if between is not None:
            between()
        a.record(stream)
        fn()
        b.record(stream)
    torch.cuda.synchronize()
    return [a.elapsed_time(b) for a, b in ev]


def fp64_peak(stream, reps=5):
    """DFMA throughput of this GPU now (TFLOP/s): the library's FMA probe kernel on every SM
    (4 CTAs x 256 threads each, 8 independent chains a thread), CUDA events on ``stream``, best
    of ``reps`` launches of about 20 ms."""
    import torch
    from pypde_gb300 import _lib
    L = _lib.lib()
    sms = torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
    ctas, threads = 4 * sms, 256
    out = torch.empty(ctas * threads, dtype=torch.float64, device="cuda")
    iters = 4000
    for _ in range(2):   # size the launch to about 20 ms
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        _lib.check(L.pgx_fp64_fma_probe(out.data_ptr(), ctas, threads, iters, stream.cuda_stream), "fp64 probe")
        b.record(stream)
        torch.cuda.synchronize()
        iters = max(1000, int(iters * 20.0 / max(a.elapsed_time(b), 1e-3)))
    best = 0.0
    for _ in range(reps):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        _lib.check(L.pgx_fp64_fma_probe(out.data_ptr(), ctas, threads, iters, stream.cuda_stream), "fp64 probe")
        b.record(stream)
        torch.cuda.synchronize()
        best = max(best, L.pgx_fp64_fma_probe_flops(ctas, threads, iters) / (a.elapsed_time(b) * 1e-3) / 1e12)
    return best


def committed_traffic(pass_name, workload, n_inst):
    """DRAM bytes (read + write) per step of ``pass_name`` from the committed ncu summary, with the
    commit it was captured at, or (None, why)."""
    if workload != "c4" or n_inst != 256:
        return None, "no committed capture for this workload"
    try:
        fields = {}
        for line in open(TRAFFIC_PROFILE):
            if ":" in line and not line.startswith(" "):
                k, v = line.split(":", 1)
                fields[k.strip()] = v.strip()
        if fields.get("pass") != pass_name:
            return None, "the committed capture is of pass %s" % fields.get("pass")
        return float(fields["dram_bytes_per_step"]), "%s (captured at commit %s)" % (
            os.path.relpath(TRAFFIC_PROFILE, ROOT), fields.get("commit", "?"))
    except (OSError, KeyError, ValueError) as e:
        return None, "no committed capture (%s)" % e


def batch_parity(fb, saved, specs, every=16, steps=5):
    """The benched batch from its initial state, ``steps`` graph replays, against the CPU oracle on
    every ``every``-th instance: max over instances and state arrays of max|gpu - oracle| / max|oracle|."""
    import torch
    from oracle import rbc2d as orb
    fb.state_arena.copy_(saved)
    for _ in range(steps):
        fb.step()
    torch.cuda.synchronize()
    worst, checked = 0.0, 0
    for i in range(0, len(specs), every):
        shape, ra, dt, seed, amp, aspect = specs[i]
        ref = orb.NavierStokes(case="linear", shape=shape, ra=ra, pr=1.0, dt=dt, aspect=aspect, dealias=True,
                               integrator="eu", beta=1.0, tsave=None)
        orb.seeded_temperature(ref, seed, amp)
        for _ in range(steps):
            ref.update()
        st = fb.solvers[i].state()
        for name, arr in (("T", ref.That), ("U", ref.Uhat), ("V", ref.Vhat), ("P", ref.Phat), ("pres", ref.pres)):
            worst = max(worst, float(np.max(np.abs(st[name] - arr)) / max(np.max(np.abs(arr)), 1e-300)))
        checked += 1
    return {"max_rel_err": worst, "tolerance": 1e-8, "ok": worst < 1e-8, "instances_checked": checked,
            "steps": steps, "how": "every %dth instance of the benched batch (its tuned tiles and graph), from the "
                                   "initial state, against the CPU oracle" % every}


def per_pass_times(fb, reps, stream, between=None):
    out = []
    for i in range(len(fb.launches)):
        fb.run_pass(i)  # warm
        ms = time_steps(lambda: fb.run_pass(i), reps, stream, between)  # noqa: B023
        out.append(sum(ms) / reps)
    return out


L2_BYTES = 129e6


def l2_flusher(work_bytes):
    """(callable or None, description): working sets the L2 could hold are flushed between timed steps by
    writing a buffer of twice its size."""
    import torch
    if work_bytes >= 2 * L2_BYTES:
        return None, "no flush: the working set (%.1f MB) exceeds the 129 MB L2" % (work_bytes / 1e6)
    buf = torch.empty(int(2 * L2_BYTES) // 8, dtype=torch.float64, device="cuda")
    return (lambda: buf.fill_(0.0)), ("L2 flushed between timed steps (a 258 MB write): the working set "
                                      "(%.1f MB) fits the 129 MB L2" % (work_bytes / 1e6))


def run_gpu(args, rank, world):
    import torch
    import torch.distributed as dist
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    specs = workload_specs(args.workload, args.instances, rank)

    # CPU baseline first (spawned pool, before heavy GPU work), rank 0 only, N = 1 only
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        v, ncores, desc, _ = cpu_sample(specs, args.steps, args.warmup)
        cpu = {"value": v, "unit": "instance-steps/s", "cores": ncores, "kind": "port", "blas_threads": 1,
               "sample": desc}

    solvers, fb = build_batch(specs, {"auto": None, "on": True, "off": False}[args.split])
    n_inst = len(solvers)
    stream = torch.cuda.current_stream()
    tuned = None
    if args.tiles:  # tiles saved by an earlier run (same workload): no tuning launches
        with open(args.tiles) as f:
            fb._build_launches(json.load(f)["forward"])
        tuned = "loaded from %s" % args.tiles
    elif not args.no_tune:
        tuned = fb.autotune()
    if args.save_tiles:
        with open(args.save_tiles, "w") as f:
            json.dump({"forward": fb.tiles()}, f)
    if args.graph_groups:
        fb.capture(1, groups="shape%d" % -args.graph_groups if args.graph_groups < 0 else args.graph_groups)
        group_times = None
    elif args.no_tune:
        fb.capture(1)
        group_times = None
    else:  # instance groups as parallel branches of the step's graph: tuned like the tiles
        group_times = {str(k): round(v, 4) for k, v in fb.tune_groups().items()}
        if not args.no_graph_tiles:   # the dominant pass's tiles once more, inside the step's graph
            group_times["in_graph"] = {k: [list(v[0]), v[1]] for k, v in fb.tune_in_graph().items()}
        # the fastest of a few recordings of the final graph (the same launches and branches)
        group_times["recordings"] = [round(t, 4) for t in fb.capture_best()]
    state_bytes = fb.state_arena.numel() * 8
    initial_state = fb.state_arena.clone()   # tuning restores the state: this is the seeded initial state
    work_bytes = fb.scratch_bytes()
    flush, l2_note = l2_flusher(work_bytes)

    # warmup + timed region (graph replay), barrier + sync on both sides; the clock sampler starts
    # before the warm-up so that it is producing samples when the timed region begins
    clocks = ClockSampler(local, args.clocks_csv)
    time.sleep(0.5)
    for _ in range(args.warmup):
        fb.step()
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    step_ms = time_steps(fb.step, args.steps, stream, flush)
    wall = time.perf_counter() - t0
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    clk = clocks.stop()
    total_ms = sum(step_ms)
    if world > 1:
        total_ms = max_over_ranks(total_ms)
    value = aggregate_value(n_inst, world, args.steps, total_ms)
    finite = int(sum(bool(torch.isfinite(I.arrays["TG"]).all()) for I in fb.insts))

    # e2e: public API (FusedBatch.step_host), state in pinned host memory, copied in before and out
    # after every step; instance groups on their own streams overlap one group's copies with
    # another's passes
    host = torch.empty(fb.state_arena.numel(), dtype=torch.float64, pin_memory=True)
    host.copy_(fb.state_arena)
    groups = fb.host_pipeline(args.e2e_groups, branches=1)

    def e2e_step():
        fb.step_host(host)

    for _ in range(2):
        e2e_step()
    torch.cuda.synchronize()
    e2e_ms = time_steps(e2e_step, args.steps, stream, flush)
    e2e_total = sum(e2e_ms)
    if world > 1:
        e2e_total = max_over_ranks(e2e_total)
    e2e = {"value": n_inst * world * args.steps / (e2e_total / 1e3), "unit": "instance-steps/s",
           "h2d_bytes_per_step": state_bytes, "d2h_bytes_per_step": state_bytes, "stream_groups": groups}

    if rank != 0:
        return None

    # the benched batch against the oracle: a fixed sample, from the initial state, tuned tiles and graph
    parity = batch_parity(fb, initial_state, specs) if args.workload == "c4" else None

    # roofline of the dominant pass: algorithmic flops / CUDA-event time per launch, against the DFMA
    # throughput measured here, now (same process, same clocks)
    pt = per_pass_times(fb, 5, stream, flush)
    try:
        peak, peak_src = fp64_peak(stream), ("DFMA throughput measured in this run by the library's FMA probe "
                                             "kernel (pgx_fp64_fma_probe, every SM); MEASURED_PEAKS.json "
                                             "carries only HBM and bf16")
    except Exception as e:  # pragma: no cover - probe missing from an old build
        peak, peak_src = FP64_PEAK_FALLBACK_TFLOPS, "committed DFMA measurement at 2070 MHz (%s)" % e
    work = fb.pass_work()
    passes = []
    for (name, fl, by), ms in zip(work, pt):
        passes.append({"pass": name, "ms": round(ms, 4), "gflop": round(fl / 1e9, 4),
                       "frac_fp64": round(fl / (ms * 1e-3) / 1e12 / peak, 4)})
    dom = max(range(len(pt)), key=lambda i: pt[i])
    fl_dom = work[dom][1]
    achieved = fl_dom / (pt[dom] * 1e-3) / 1e12
    traffic, traffic_src = committed_traffic(work[dom][0], args.workload, n_inst)
    roofline = {"bound": "fp64", "kernel": "line_program_batched_fft (%s)" % work[dom][0],
                "achieved": round(achieved, 4), "peak": round(peak, 4), "unit": "TFLOP/s",
                "frac": round(achieved / peak, 4), "traffic": traffic, "traffic_source": traffic_src,
                "peak_source": peak_src, "flops_per_launch": fl_dom, "algorithmic_bytes_per_launch": work[dom][2],
                "launch_ms": round(pt[dom], 4)}
    step_fl = sum(w[1] for w in work)
    step_fp64 = {"tflops": round(step_fl / (total_ms / args.steps * 1e-3) / 1e12, 4),
                 "frac": round(step_fl / (total_ms / args.steps * 1e-3) / 1e12 / peak, 4),
                 "gflop_per_step": round(step_fl / 1e9, 3)}

    # one by one on the per-instance GPU path (same fused kernels, one CUDA graph per instance)
    plain = None
    if n_inst > 1 and not args.no_plain:
        per = []
        for i in range(n_inst):
            one = fb.single(i)
            if not args.no_tune:
                one.autotune(reps=2)
            one.capture(1)
            for _ in range(2):
                one.step()
            per.append(sum(time_steps(one.step, 3, stream)) / 3)
            del one
        plain = {"value": n_inst / (sum(per) / 1e3), "unit": "instance-steps/s",
                 "how": "the same %d instances one at a time, per-instance CUDA graph of the fused step" % n_inst}
    # op-by-op drop-in path (NavierStokes.update: one kernel per pypde operation) on a sample
    eager = None
    if not args.no_plain:
        sample = solvers[: min(8, n_inst)]
        eager = {}
        for label, fused in (("plain", False), ("default", None)):
            for ns in sample:
                ns.update(fused=fused)
            torch.cuda.synchronize()
            t = time.perf_counter()
            for ns in sample:
                for _ in range(2):
                    ns.update(fused=fused)
            torch.cuda.synchronize()
            eager[label] = round(2 * len(sample) / (time.perf_counter() - t), 2)
        eager.update({"unit": "instance-steps/s",
                      "how": "NavierStokes.update() per call, %d instances x 2 steps, host wall clock: plain = "
                             "update(fused=False), op by op; default = update(), the fused passes launched "
                             "eagerly" % len(sample)})

    # the same batch as persistent launches (several steps of every instance in one launch of a resident
    # grid, tiles re-picked for one CTA size), recorded in a CUDA graph
    persistent = None
    if args.workload == "c4" and n_inst > 1 and args.persistent_steps > 0:
        T, per_sm, K = 128, 6, args.persistent_steps
        fb.persistent_tiles(T, per_sm)
        fb.state_arena.copy_(initial_state)
        info = fb.persistent(nsteps=K, threads=T)
        fb.capture_persistent()
        for _ in range(2):
            fb.step_persistent()
        torch.cuda.synchronize()
        reps = max(1, args.steps // K)
        ms = time_steps(fb.step_persistent, reps, stream, flush)
        err, where = fb.persistent_error()
        persistent = {"value": round(n_inst * K * reps / (sum(ms) / 1e3), 2), "unit": "instance-steps/s",
                      "ms_per_step": round(sum(ms) / (reps * K), 4), "steps_per_launch": K, "launches": reps,
                      "threads": info["threads"], "ctas_per_sm": info["ctas_per_sm"], "items_per_launch": info["nitems"],
                      "error": err,
                      "how": "pgx_run_persistent: %d steps of all %d instances per launch (work queue, per-instance "
                             "pass counters), tiles re-picked from the autotuner's timings for %d-thread CTAs, "
                             "%d per SM; one CUDA-graph replay per launch" % (K, n_inst, T, per_sm)}

    line = {
        "metric": METRIC,
        "value": round(value, 2),
        "unit": "instance-steps/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": round(total_ms / args.steps, 4),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": "synthetic: seeded U(-1,1) temperature noise on the conductive profile (seeds 100+i)",
        "config": {"workload": WORKLOAD_NAMES[args.workload].format(n=n_inst), "instances_per_gpu": n_inst,
                   "sizes": sorted({s[0] for s in specs}),
                   "form": "batched, CUDA-graph replay of %d fused passes%s, instances in %d parallel graph "
                           "branches" % (len(fb.progs), " (per-field convection passes)" if fb.split else "",
                                         fb.graph_groups),
                   "l2": l2_note, "parallelism": "instance-parallel"},
        "e2e": e2e,
        "gpu_launches": fb.graph_launches * args.steps,
        "roofline": roofline,
        "parity": parity,
        "clocks": clk,
        "cpu_baseline": cpu,
        "step_fp64": step_fp64,
        "passes": passes,
        "plain": plain,
        "persistent": persistent,
        "eager": eager,
        "graph_groups": {"groups": fb.graph_groups, "tuned_ms_per_step": group_times},
        "finite_instances": finite,
        "host_wall_s": round(wall, 3),
    }
    if world == 1 and args.adjoint_iters >= 0 and args.workload == "c4":
        line["adjoint"] = run_adjoint(args, stream)
    line["autotuned_tiles"] = {k: list(v[:5]) for k, v in tuned.items()} if isinstance(tuned, dict) else tuned
    # the per-pass fractions and the parity check also inside roofline (a key every reader parses), and in
    # full at the end of the line (the part of a long output that is kept when only its tail is)
    roofline["passes_frac_fp64"] = {p["pass"]: p["frac_fp64"] for p in passes}
    if parity is not None:
        roofline["parity_max_rel_err"] = parity["max_rel_err"]
    for k in ("step_fp64", "parity", "passes"):
        line[k] = line.pop(k)
    return line


def run_adjoint(args, stream):
    """Adjoint steady-state search, 129 x 129, Ra 1e5, Pr 1, dt 0.01: J = ||Phi^200(X) - X|| from the
    conductive state + 1e-2 U(-1,1) noise (seed 3), checkpoints every 20 steps; gradient by the fused
    reverse-mode passes; central differences (h = 1e-6) on 20 random unit directions; descent."""
    import torch
    from pypde_gb300.navier.adjoint import descend, random_directions
    from pypde_gb300.navier.fused_adjoint import FusedAdjoint, HorizonGradient, HorizonGradientGroups
    from pypde_gb300.navier.rbc2d import NavierStokes
    H, every, shape = args.adjoint_horizon, 20, (129, 129)
    ns = NavierStokes(case="linear", shape=shape, ra=1e5, pr=1.0, dt=0.01, dealias=True, integrator="eu",
                      tsave=None)
    ns.set_temperature_noise(3, 1e-2)
    fa = FusedAdjoint([ns])
    if args.adjoint_profile:
        # fixed launch order for a launch-list capture: forward steps, then adjoint steps (eager)
        for _ in range(args.adjoint_profile):
            fa.step_eager()
        for _ in range(args.adjoint_profile):
            fa.adjoint_step_eager()
        torch.cuda.synchronize()
        return {"profile_order": [p.name for p in fa.progs] * args.adjoint_profile +
                                 [p.name for p in fa.aprogs] * args.adjoint_profile}
    if not args.no_tune:
        fa.autotune(reps=2)
        fa.autotune_adjoint(reps=2)
    fa.capture(1)
    fa.capture_adjoint()
    hg = HorizonGradient(fa, H, every)
    X = fa.state_arena.clone()
    for _ in range(2):  # warm-up (the first call of each records its CUDA graph)
        hg.value_and_grad(X)
        hg.value(X)
    torch.cuda.synchronize()

    flush = l2_flusher(0)[0]   # the L2 is flushed between timed calls

    def timed(fn, reps):
        res = []
        ms = time_steps(lambda: res.append(fn()), reps, stream, flush)
        return sum(ms) / reps, res[-1]

    reps = max(2, min(args.steps, 5))
    ms_j, _ = timed(lambda: hg.value(X), reps)
    ms_g, (J, g) = timed(lambda: hg.value_and_grad(X), reps)
    # per-step costs: one fused forward step and one adjoint step (graph replays)
    ms_f1, _ = timed(fa.step, 50)
    ms_a1, _ = timed(fa.adjoint_step, 50)
    # central differences on random unit directions of the (T, U, V) coefficient space
    shapes = [v.shape for v in fa.views(X)[0].values()]
    dirs = random_directions(shapes, args.adjoint_fd, seed=17, device="cuda")
    h, errs = 1e-6, []
    for d in dirs:
        D = torch.zeros_like(X)
        for v, e in zip(fa.views(D)[0].values(), d):
            v.copy_(e)
        fd = (float(hg.value(X + h * D)[0]) - float(hg.value(X - h * D)[0])) / (2 * h)
        ad = float((g * D).sum())
        errs.append(abs(fd - ad) / abs(ad))
    # many searches at once: a batch of instances of the same configuration (noise seeds 3, 4, ...)
    batched = None
    if args.adjoint_batch > 1:
        solvers = []
        for i in range(args.adjoint_batch):
            nsi = NavierStokes(case="linear", shape=shape, ra=1e5, pr=1.0, dt=0.01, dealias=True, integrator="eu",
                               tsave=None)
            nsi.set_temperature_noise(3 + i, 1e-2)
            solvers.append(nsi)
        hgs = HorizonGradientGroups(solvers, H, every, groups=args.adjoint_groups, tune=not args.no_tune)
        Xs = hgs.states()
        for _ in range(2):
            hgs.value_and_grad(Xs)
        torch.cuda.synchronize()
        ms_b, outs = timed(lambda: hgs.value_and_grad(Xs), 2)
        batched = {"instances": args.adjoint_batch, "groups": len(hgs.parts), "ms_per_batch_grad": round(ms_b, 3),
                   "grads_per_s": round(args.adjoint_batch * 1e3 / ms_b, 3),
                   "finite": all(bool(torch.isfinite(g).all()) for _, g in outs)}
        del hgs, outs, solvers
        torch.cuda.empty_cache()
    # steady-state search: descent iterations, one gradient evaluation each
    t0 = time.perf_counter()
    _, hist = descend(hg.value_and_grad, X, args.adjoint_iters)
    torch.cuda.synchronize()
    wall_desc = time.perf_counter() - t0
    return {"config": "129x129, aspect 1, Ra 1e5, Pr 1, dt 0.01, horizon %d steps, checkpoint every %d, "
                      "X0 = conductive + 1e-2 U(-1,1) (seed 3); J = ||Phi^H(X) - X||_2 over (T, U, V)" % (H, every),
            "grads_per_s": round(1e3 / ms_g, 3), "ms_per_grad": round(ms_g, 3), "ms_per_objective": round(ms_j, 3),
            "cost_ratio_grad_vs_forward": round(ms_g / min(ms_j, H * ms_f1), 3),
            "cost_ratio_basis": "gradient (forward sweep + checkpointed reverse sweep, one graph) over the "
                                "faster of: the objective's own graph, H single-step forward replays",
            "ms_forward_step": round(ms_f1, 4), "ms_adjoint_step": round(ms_a1, 4),
            "adjoint_launches_per_step": fa.adjoint_launches_per_step,
            "fd_check": {"directions": len(dirs), "h": h, "max_rel_err": max(errs) if errs else None,
                         "median_rel_err": statistics.median(errs) if errs else None},
            "descent": {"iterations": args.adjoint_iters, "accepted": len(hist) - 1, "J_first": hist[0],
                        "J_last": hist[-1], "wall_s": round(wall_desc, 3),
                        "step": "alpha J / |grad J|^2, alpha adapted by acceptance"},
            "batched": batched,
            "J": float(J[0]), "autotuned_adjoint_tiles": getattr(fa, "atuned", None)}


def dense_dct_passes(f, c, g, axis, mma, st):
    """c = Fwd f, g = Bwd c along ``axis`` (N x N, N lines) as LOAD / DENSE / STORE line programs with
    the dense Chebyshev DCT matrices, the contraction on the FP64 tensor cores (``mma``) or as FMA
    chains; 8 lines per CTA."""
    import ctypes
    from pypde_gb300 import _lib
    from pypde_gb300._dev import to_dev
    from pypde_gb300.navier.fused import dense_dct_host
    N = f.shape[0]
    mats = dense_dct_host(N)
    keep = [to_dev(mats["dct_fwd"]), to_dev(mats["dct_bwd"])]
    runs = []
    for src, dst, A in ((f, c, keep[0]), (c, g, keep[1])):
        P = _lib.PgxProgram()
        P.axis, P.lines_len, P.tb, P.lcap, P.nslots, P.fft_n, P.nthreads = axis, 1, 8, (N + 1) | 1, 1, 0, 256
        ops = [_lib.op("LOAD", a=0, arr=0, len=0), _lib.op("DENSE", a=0, mat=0, len=0, k=_lib.DENSE_MMA if mma else 0),
               _lib.op("STORE", a=0, arr=1)]
        P.nops = len(ops)
        for i, o in enumerate(ops):
            P.ops[i] = o
        inst = _lib.PgxInstance()
        for i, t in enumerate((src, dst)):
            inst.arr[i].ptr, inst.arr[i].s0, inst.arr[i].s1 = t.data_ptr(), t.stride(0), t.stride(1)
            inst.arr[i].n0, inst.arr[i].n1 = t.shape
        inst.mat[0] = A.data_ptr()
        inst.len[0], inst.len[1] = N, N
        runs.append((P, inst))
    L = _lib.lib()

    def run():
        for P, inst in runs:
            _lib.check(L.pgx_run(ctypes.byref(P), ctypes.byref(inst), st), "dense dct")
    run.keep = keep
    return run


def run_microbench(args):
    """Kernel microbench (seed 1): DCT-I forward + backward along each axis of N x N fields,
    N = 33 ... 1025, and the ADI Helmholtz solve (I - 0.01 Laplacian) u = f with Dirichlet bases
    at 257^2 and 1025^2, by the ADI plan and exactly by fast diagonalisation; CUDA-event times, round-trip
    error against the input, residual of each solve's operator."""
    import torch
    import pypde_gb300 as pg
    from pypde_gb300 import _lib
    stream = torch.cuda.current_stream()
    st = stream.cuda_stream
    L = _lib.lib()
    rng = np.random.default_rng(1)
    flush = l2_flusher(0)[0]   # the fields fit the L2: flushed between timed calls
    dct = []
    for N in (33, 65, 129, 257, 513, 1025):
        f = torch.as_tensor(rng.uniform(-1, 1, (N, N)), device="cuda")
        c = torch.empty_like(f)
        g = torch.empty_like(f)
        row = {"N": N}
        for axis in (0, 1):
            s0, s1 = (N, 1)

            def fb():
                L.pgx_dct1(f.data_ptr(), s0, s1, N, c.data_ptr(), s0, s1, N, N, N, axis, _lib.DCT_FWD, st)
                L.pgx_dct1(c.data_ptr(), s0, s1, N, g.data_ptr(), s0, s1, N, N, N, axis, _lib.DCT_BWD, st)

            for _ in range(3):
                fb()
            ms = time_steps(fb, max(args.steps, 5), stream, flush)
            err = float((g - f).abs().max() / f.abs().max())
            t = statistics.median(ms)
            flops = 2 * 2.5 * N * np.log2(2 * (N - 1)) * N
            row["axis%d" % axis] = {"ms_fwd_bwd": round(t, 5), "roundtrip_err": err,
                                    "tflops": round(flops / (t * 1e-3) / 1e12, 4)}
            # the same transforms as dense matrices: tensor cores (DMMA) and FMA chains
            for mma in (True, False):
                fb2 = dense_dct_passes(f, c, g, axis, mma, st)
                for _ in range(3):
                    fb2()
                t2 = statistics.median(time_steps(fb2, max(args.steps, 5), stream, flush))
                err2 = float((g - f).abs().max() / f.abs().max())
                row["axis%d" % axis]["dense_mma" if mma else "dense_fma"] = {
                    "ms_fwd_bwd": round(t2, 5), "roundtrip_err": err2,
                    "tflops": round(2 * 2.0 * N * N * N / (t2 * 1e-3) / 1e12, 4)}
        dct.append(row)
    from oracle import spectral as sp
    hh, hfd = [], []
    for N in (257, 1025):
        fld = pg.Field([pg.Base(N, "CD"), pg.Base(N, "CD")])
        fh = rng.uniform(-1, 1, (N, N))
        f = torch.as_tensor(fh, device="cuda")
        S, B, I = sp.stencil("CD", N), sp.B2(N), sp.I2(N)
        C, A = B @ S, I @ S
        Bf = B @ fh @ B.T
        for exact in (False, True):
            sol = (pg.solverplan_hholtz2d_fd if exact else pg.solverplan_hholtz2d_adi)(fld.xs, lam=0.01)
            run = lambda: sol.solve_lhs(sol.solve_rhs(f))  # noqa: E731
            for _ in range(3):
                x = run()
            ms = time_steps(run, max(args.steps, 5), stream, flush)
            x = x.cpu().numpy()
            if exact:   # residual of the unsplit operator (C - lam A) X C^T - lam C X A^T = B F B^T
                r = (C - 0.01 * A) @ x @ C.T - 0.01 * C @ x @ A.T - Bf
                hfd.append({"N": N, "ms": round(statistics.median(ms), 4), "launches": 4,
                            "residual": float(np.max(np.abs(r)) / np.max(np.abs(Bf)))})
            else:       # residual of the ADI-factored system A_x X A_y^T = B F B^T, A = C - lam I S
                Ax = C - 0.01 * A
                r = Ax @ x @ Ax.T - Bf
                hh.append({"N": N, "ms": round(statistics.median(ms), 4), "launches": 4,
                           "residual": float(np.max(np.abs(r)) / np.max(np.abs(Bf)))})
    return {"metric": "kernel microbench: DCT-I fwd+bwd per axis and Helmholtz solves", "dct": dct,
            "helmholtz_adi": hh, "helmholtz_exact_fd": hfd, "dtype": "f64", "data": "synthetic U(-1,1), seed 1",
            "l2": "flushed between timed calls (a 258 MB write)",
            "residual": "max |operator(x) - B F B^T| / max |B F B^T| with the premultiplied operator of each plan "
                        "(ADI: its factored operator; exact: the unsplit one, bounded by the host eigendecomposition)"}


def run_reference(args, rank, world):
    """Reference arm: the CPU oracle (NumPy restatement of pypde's path; the reference
    itself is Python and does not ship to the GPU host) on all host cores."""
    if rank != 0:
        return None
    specs = workload_specs(args.workload, args.instances)
    full = len(specs)
    value, cores, desc, total_wall = cpu_sample(specs, args.steps, args.warmup)
    return {"metric": METRIC, "value": round(value, 3), "unit": "instance-steps/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(total_wall / args.steps * 1e3, 3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic: seeded U(-1,1) temperature noise (seeds 100+i)", "impl": "reference",
            "config": {"workload": WORKLOAD_NAMES[args.workload].format(n=full), "instances_per_gpu": full},
            "cpu_baseline": {"value": round(value, 3), "unit": "instance-steps/s", "cores": cores, "kind": "port",
                             "blas_threads": 1, "sample": desc},
            "e2e": {"value": round(value, 3), "unit": "instance-steps/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="c4", choices=["c4", "c1", "c3", "c2", "c5"])
    ap.add_argument("--instances", type=int, default=256)
    ap.add_argument("--no-plain", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-tune", action="store_true")
    ap.add_argument("--persistent-steps", type=int, default=4,
                    help="c4: steps per launch of the persistent form measured beside the graph form (0: skip)")
    ap.add_argument("--tiles", default=None, help="use the tiles saved by --save-tiles instead of tuning")
    ap.add_argument("--adjoint-groups", type=int, default=1,
                    help="instance groups of the batched gradient, each on its own stream (measured on the "
                         "32-instance batch: 1 group 22.5, 4 groups 20.5, 8 groups 17.0 gradients/s)")
    ap.add_argument("--no-graph-tiles", action="store_true", help="skip the in-graph second look at P2's tiles")
    ap.add_argument("--graph-groups", type=int, default=0,
                    help="instance groups as parallel branches of the step's graph (0: tuned, -K: K "
                         "per instance shape)")
    ap.add_argument("--clocks-csv", default=None, help="where the nvidia-smi samples of the timed region go")
    ap.add_argument("--e2e-groups", type=lambda v: v if v.startswith("shape") else int(v), default="shape",
                    help="instance groups of the end-to-end step, each on its own stream (a number, or "
                         "'shape': one group per instance shape, 'shapeK': K per shape)")
    ap.add_argument("--split", default="auto", choices=["auto", "on", "off"],
                    help="per-field convection passes (auto: for batches of up to 4 instances)")
    ap.add_argument("--save-tiles", default=None)
    ap.add_argument("--adjoint-iters", type=int, default=50, help="descent iterations (-1: skip the adjoint part)")
    ap.add_argument("--adjoint-horizon", type=int, default=200)
    ap.add_argument("--adjoint-fd", type=int, default=20, help="finite-difference directions")
    ap.add_argument("--adjoint-batch", type=int, default=32, help="instances of the batched gradient measurement")
    ap.add_argument("--adjoint-profile", type=int, default=0,
                    help="c5 only: run N eager forward and N adjoint steps (fixed launch order) and exit")
    args = ap.parse_args()
    if args.warmup < 3 and args.impl == "gb300":
        args.warmup = 3
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if args.workload == "c2":
        print(json.dumps(run_microbench(args)))
        return
    if args.workload == "c5":  # the adjoint steady-state search alone
        import torch
        torch.cuda.set_device(0)
        print(json.dumps({"metric": METRIC, "adjoint": run_adjoint(args, torch.cuda.current_stream())}))
        return
    if args.impl == "reference":
        line = run_reference(args, rank, world)
    else:
        if world > 1:
            import torch.distributed as dist
            dist.init_process_group("nccl")
        line = run_gpu(args, rank, world)
        if world > 1:
            import torch.distributed as dist
            dist.destroy_process_group()
    if line is not None:
        print(json.dumps(line))


if __name__ == "__main__":
    main()
