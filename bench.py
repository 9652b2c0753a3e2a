#!/usr/bin/env python3
"""Aggregate bead-steps/s of the batched SOP engine on GB300.

Workload (default): the batched ensemble -- 512 independent trajectories, N
log-uniform in [60, 1500] beads (structure seed = trajectory index), kBT
uniform in [0.5, 0.8] kcal/mol, a Philox stream each, FP32, k = 20, R0 = 2,
eps = 1, sigma = 3.8, neighbour list 32 A every 50 steps, pair list 16 A every
10 steps, h = 0.05, zeta = 0.05, started from the native structures.  The step
loop runs as a CUDA graph of 10 steps per replay; one bench step is one replay
(10 Langevin steps of every trajectory).  Inputs are the project's seeded
synthetic structures.  The ensemble is held as two contexts (engine.Ensemble,
`--parts`), each on its own CUDA stream, cut at equal bead counts: one
context's list rebuilds and kernel tails overlap the other's step kernels.

Timing: W untimed bench steps, then K bench steps, each bracketed by CUDA
events (recorded on the first context's stream, which the other streams wait
on at the start and which waits on them at the end), with a 256 MiB write
(flushes the 129 MB L2) before every step outside the events; a barrier and
synchronize on both sides; the max over ranks.  Under torchrun each rank runs its own 512-trajectory
ensemble (replicas: trajectories are independent, no collective), so the
scaling is weak.

Beside the headline the line carries:
  roofline      the step kernels timed alone, one launch per context on the
                contexts' streams (algorithmic bytes / CUDA-event time);
                traffic is a profile figure from the committed ncu capture
  e2e           a 300-step job through the C ABI from host arrays, coordinates
                copied out every step; set-up time and the steady rate apart
  cpu_baseline  the reference algorithm on all host cores, bounded sample
  plain         the plain single-molecule path on the 128-, 4,000- and
                50,000-bead structures: rate, each stage's roofline, one-core
                CPU baseline
  plain_loop    the plain path looping over every 8th ensemble molecule
  served        the served request stream (Poisson 200 jobs/s for 60 s, 150 GB
                budget, steps scaled by 1/50), p50 / p99 latency

`--impl reference` times the reference's algorithm on the host cores (the
serial FP32 CPU restatement of its host routines and kernels, all threads,
one trajectory per task): K steps of all 512 trajectories, and more until
5 s have passed.
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
from concurrent.futures import ThreadPoolExecutor

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

from sop_gb300 import system  # noqa: E402

METRIC = "aggregate bead-steps/s (batched ensemble)"
UNIT = "bead-steps/s"
N_TRAJ = 512
MD_STEPS = 10
E2E_STEPS = 300      # bench steps of the end-to-end job (3,000 Langevin steps)
CUT = [0.0, 32.0, 0.0, 32.0, 0.0, 16.0, 0.0, 16.0]   # absolute NL / PL cut-offs (A)


def workload_config(total_beads: int) -> dict:
    return {
        "workload": "batched ensemble: 512 trajectories, N log-uniform [60,1500] (seed = index), "
                    "kBT U[0.5,0.8], FP32, NL 32 A / 50 steps, PL 16 A / 10 steps, h = 0.05, "
                    "zeta = 0.05, CUDA graph of 10 steps per replay",
        "trajectories": N_TRAJ,
        "beads_per_replica": int(total_beads),
        "md_steps_per_bench_step": MD_STEPS,
        "l2": "flushed before every timed step (256 MiB write); working set exceeds L2 only for the lists",
    }


def ensemble(rank: int):
    ns, ts = system.ensemble_spec(N_TRAJ, 60, 1500, 0.5, 0.8, seed=4)
    mols = [system.generate(int(n), rank * N_TRAJ + k) for k, n in enumerate(ns)]
    return mols, ts


def measured_peaks() -> tuple[float, str]:
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def profile_traffic(workload: str = "ensemble", parts: int = 0, form: int = 0) -> float | None:
    """DRAM bytes per launch of the step kernel from the committed ncu summary
    of that workload (None when there is none).  For the ensemble, `parts`
    contexts whose step kernels run in `form` (1 one kernel, 2 force + finish):
    the bytes of one launch of every context's step kernels together.  A
    profile figure: ncu's dram__bytes_read.sum + dram__bytes_write.sum of one
    capture of the same kernels on the same workload, not measured during this
    run."""
    p = os.path.join(ROOT, "profiles", f"step_kernel_{workload}.md")
    key = (f"traffic_bytes_per_launch_{parts}_parts_form{form}:" if parts
           else "traffic_bytes_per_launch:")
    try:
        for line in open(p):
            if line.strip().startswith(key):
                return float(line.split(":", 1)[1].split()[0])
    except Exception:
        pass
    return None


class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *a):
        self.out = ""
        if self.proc:
            time.sleep(0.3)
            self.proc.terminate()
            try:
                self.out, _ = self.proc.communicate(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self) -> dict:
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in getattr(self, "out", "").splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for name, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def max_over_ranks(x: float, world: int, device) -> float:
    """The largest x over the ranks (the slowest rank's time); x itself on
    one rank."""
    if world <= 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(beads_per_rank: int, md_steps: int, world: int, t_max: float) -> float:
    """Bead-steps/s of the whole job: every rank runs its own replica of the
    workload (weak scaling), timed by the slowest rank."""
    return world * beads_per_rank * md_steps / t_max


def launches_per_bench_step(p, s0: int, form: int = 1) -> int:
    """Kernels of the engine in one replay starting after step s0 (form 1:
    one step kernel per step; 2: force + finish kernels; 3 and 4: one
    launch per run of steps between list rebuilds)."""
    nl_kernels = 12    # bbox reset, bbox, grid, grid base, assign, 3 scan, scatter, cellsort,
                       # stage_xs, nl
    n = 0
    runs = 0
    in_run = False
    for k in range(MD_STEPS):
        st = s0 + 1 + k
        nl = p.nnlup > 0 and st % p.nnlup == 0
        pl = nl or p.nplup <= 1 or st % p.nplup == 0
        n += (nl_kernels if nl else 0) + (1 if pl else 0)
        n += 1 if nl and k > 0 else 0   # the clock advance ahead of a mid-block rebuild
        if form in (3, 4):
            if pl or not in_run:
                runs += 1
            in_run = True
        else:
            n += 2 if form == 2 else 1
    return n + runs + 1   # the block's closing step advance


def step_kernel_bytes(e, mols) -> tuple[float, dict]:
    """Algorithmic bytes of one launch of the fused step kernel:
    80 N (Langevin: read x, v, f; write x, v as float4) + 32 N (read x, write f)
    + 4 B (bond r0) + 4 P_rep + 8 P_att (+4 P_att for per-contact epsilon)."""
    ls = e.list_sizes()
    N = sum(m.n for m in mols)
    B = sum(len(m.bond_i) for m in mols)
    byts = 112.0 * N + 4.0 * B + 4.0 * ls["nil_rep"] + 12.0 * ls["nil_att"]
    return byts, ls


def cpu_baseline(mols, ts, seconds_target: float = 15.0) -> dict:
    """The reference algorithm on the host cores (one molecule per thread)."""
    from oracle import pyoracle as O
    cores = os.cpu_count() or 1
    runs = [O.RefRun(m, m.xyz, CUT, 0.05, 0.05, float(t), 50, 10, 1234, k)
            for k, (m, t) in enumerate(zip(mols, ts))]
    # initial lists and forces (step 0) outside the timing
    with ThreadPoolExecutor(cores) as ex:
        list(ex.map(lambda r: r.advance(0), runs))
    beads = sum(m.n for m in mols)
    steps = 10
    # one trajectory per task, largest first: the pool balances the load
    big_first = sorted(runs, key=lambda r: -r.n)

    t0 = time.perf_counter()
    with ThreadPoolExecutor(cores) as ex:
        list(ex.map(lambda r: r.advance(steps), big_first))
    dt = time.perf_counter() - t0
    # scale the sample to about `seconds_target` of wall time
    more = max(0, int(steps * (seconds_target / max(dt, 1e-3) - 1.0)))
    more = min(more, 400)
    t0 = time.perf_counter()
    with ThreadPoolExecutor(cores) as ex:
        list(ex.map(lambda r: r.advance(more), big_first))
    dt2 = time.perf_counter() - t0 if more else 0.0
    tot_steps = steps + more
    tot_t = dt + dt2
    for r in runs:
        r.close()
    return {"value": beads * tot_steps / tot_t, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": f"all {len(mols)} trajectories ({beads} beads), {tot_steps} Langevin steps "
                      f"each, serial FP32 restatement of the reference's host list filters, "
                      f"force kernels and integrator, one trajectory per task on {cores} threads"}


SERVED_RATE = 200.0          # jobs/s (Poisson)
SERVED_SECONDS = 60.0        # arrival window
STEP_SCALE = 50              # steps log-uniform [1e4, 1e6] scaled by 1/STEP_SCALE
SERVED_STEPS = (1e4 / STEP_SCALE, 1e6 / STEP_SCALE)
SERVED_BUDGET = 150 * 10**9  # device bytes for coordinates, velocities, topology, lists
SERVED_BOXL = 1.0e6          # holds a fully extended 20,000-bead chain without self-images
PLAIN_EVERY = 20             # every 20th job (5%) also runs alone on the plain path


def served_stream(local: int) -> dict:
    """Continuous batching on the Poisson request stream: jobs are submitted at
    their arrival times (structures generated ahead by a pool of host threads),
    admitted by the HBM budget, retired when done; then every PLAIN_EVERY-th
    job again alone on the plain path."""
    from sop_gb300 import engine
    req = system.request_stream(SERVED_RATE, SERVED_SECONDS, (50, 20000), SERVED_STEPS,
                                (0.5, 0.8), seed=5)
    njob = len(req["n"])

    def make(k):
        m = system.generate(int(req["n"][k]), 100000 + k)
        return m, (m.extended_xyz() if req["extended"][k] else m.xyz)

    p = engine.baseline_params(device=local, boxl=SERVED_BOXL)
    lat, work, statuses = {}, 0, []
    gen = ThreadPoolExecutor(max(2, min(8, (os.cpu_count() or 4) // 2)))
    futs = [gen.submit(make, k) for k in range(njob)]
    with engine.Server(p, SERVED_BUDGET, 20000) as srv:
        ids = {}
        nxt = 0
        late = []
        t0 = time.perf_counter()
        while len(lat) < njob:
            now = time.perf_counter() - t0
            if now > 1200.0:
                raise RuntimeError("served stream did not drain in 1200 s")
            while nxt < njob and req["arrival"][nxt] <= now:
                m, x = futs[nxt].result()
                late.append(time.perf_counter() - t0 - req["arrival"][nxt])
                ids[srv.submit(m, x, int(req["steps"][nxt]), float(req["T"][nxt]),
                               traj=nxt)] = nxt
                futs[nxt] = None
                nxt += 1
            s = srv.stats()
            if s["queued"] == 0 and s["active"] == 0 and nxt < njob:
                time.sleep(max(0.0, min(1e-3, req["arrival"][nxt] - now)))
                continue
            srv.advance(1)
            for j in srv.finished():
                r = srv.result(j)
                k = ids[j]
                lat[k] = r["latency_s"]
                work += int(req["n"][k]) * int(r["steps"])
                statuses.append(r["status"])
        wall = time.perf_counter() - t0
        stats = srv.stats()
    gen.shutdown()
    served_rate = work / wall
    # the plain path on every PLAIN_EVERY-th job, one context at a time
    sample = list(range(0, njob, PLAIN_EVERY))
    pw, pt = 0, 0.0
    for k in sample:
        m, x = make(k)
        ep = engine.plain(m, x, p, T=float(req["T"][k]), traj=k, nsteps=int(req["steps"][k]))
        t1 = time.perf_counter()
        ep.step(int(req["steps"][k]))
        pt += time.perf_counter() - t1
        pw += int(req["n"][k]) * int(req["steps"][k])
        ep.close()
    lv = np.array([lat[k] for k in range(njob)])
    return {"value": served_rate, "unit": UNIT,
            "latency_p50_s": float(np.percentile(lv, 50)),
            "latency_p99_s": float(np.percentile(lv, 99)),
            "jobs": njob, "bead_steps": work, "wall_s": wall,
            "arrival_window_s": SERVED_SECONDS,
            "submit_lag_p99_s": float(np.percentile(np.array(late), 99)),
            "offered_bead_steps_per_s": float((req["n"].astype(np.float64) * req["steps"]).sum()
                                              / SERVED_SECONDS),
            "plain_sequential": pw / pt, "served_over_plain": served_rate / (pw / pt),
            "plain_sample_jobs": len(sample),
            "failed_jobs": int(sum(1 for s in statuses if s & 3)),
            "device_bytes": stats["device_bytes"],
            "config": f"Poisson {SERVED_RATE:.0f} jobs/s for {SERVED_SECONDS:.0f} s ({njob} jobs), "
                      f"N log-uniform [50,20000], steps log-uniform [{SERVED_STEPS[0]:.0f},"
                      f"{SERVED_STEPS[1]:.0f}] (the [1e4,1e6] range scaled by 1/{STEP_SCALE}), "
                      f"kBT U[0.5,0.8], half native / half extended, HBM budget "
                      f"{SERVED_BUDGET / 1e9:.0f} GB, boxl {SERVED_BOXL:.0f} A; latency from "
                      f"submission at the arrival time to retirement; plain_sequential: every "
                      f"{PLAIN_EVERY}th job ({len(sample)} jobs) alone, one context at a time"}


PLAIN = {  # workload: (beads, structure seed, per-contact epsilon range)
    "plain128": (128, 0, None),
    "plain4000": (4000, 1, None),
    "plain50k": (50000, 2, (0.7, 1.3)),
}


def plain_measure(workload: str, local: int, K: int, warmup: int, lanes: int = 0, form: int = 0,
                  cpu_seconds: float = 5.0, window: int = 0) -> dict:
    """The plain single-molecule path on one synthetic structure: whole-step
    rate, each stage's HBM roofline, and the reference algorithm on one host
    core (cpu_seconds of it; 0 skips it)."""
    import torch
    from sop_gb300 import engine
    dev = torch.device("cuda", local)
    torch.cuda.set_device(local)
    nbead, seed, eps = PLAIN[workload]
    mol = system.generate(nbead, seed, eps)
    p = engine.baseline_params(device=local, graph_steps=MD_STEPS, lanes_per_bead=lanes,
                               step_split=form, step_window=window)
    e = engine.plain(mol, mol.xyz, p, T=0.6)
    stream = torch.cuda.ExternalStream(e.stream(), device=dev)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    for _ in range(warmup):
        e.step_async(MD_STEPS)
    e.sync()
    s_start = e.status(0)[1]
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(K)]
    torch.cuda.synchronize(dev)
    with ClockSampler(local) as clk:
        with torch.cuda.stream(stream):
            for k in range(K):
                flush.zero_()
                ev[k][0].record(stream)
                e.step_async(MD_STEPS)
                ev[k][1].record(stream)
        torch.cuda.synchronize(dev)
        e.sync()
    t = sum(a.elapsed_time(b) for a, b in ev) / 1e3
    value = mol.n * MD_STEPS * K / t
    ls = e.list_sizes()
    N, B = mol.n, len(mol.bond_i)
    peak, peak_kind = measured_peaks()
    stage_bytes = {
        # read x, v, f, incr; write x, p, v, incr, f (float4); bond r0; list entries
        0: 112.0 * N + 4.0 * B + 4.0 * ls["nil_rep"] + 12.0 * ls["nil_att"],
        # stream both directions of the NL rows and write the PL rows; counts and x_i
        1: 24.0 * N + 8.0 * (ls["nnl_rep"] + ls["nil_rep"]) + 2.0 * (24.0 * ls["nnl_att"]
                                                                 + 16.0 * ls["nil_att"]),
        # cell binning (bbox, cells, sorted copy) + writing both directions of the NL
        2: 64.0 * N + 8.0 * ls["nnl_rep"] + 8.0 * ls["nnl_att"],
    }
    names = {0: "force + Langevin step (k_step; + k_finish in the two-kernel form)",
             1: "pair-list rebuild (k_pl)",
             2: "neighbour-list rebuild (binning + k_nl)"}
    stages = {}
    for st in (0, 1, 2):
        reps = 20
        kev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
               for _ in range(reps)]
        with torch.cuda.stream(stream):
            for k in range(reps):
                flush.zero_()
                kev[k][0].record(stream)
                e.launch_stage(st, 0)
                kev[k][1].record(stream)
        torch.cuda.synchronize(dev)
        tk = statistics.median(a.elapsed_time(b) for a, b in kev) / 1e3
        ach = stage_bytes[st] / tk / 1e9
        stages[names[st]] = {"us": tk * 1e6, "bytes": stage_bytes[st], "achieved_gbs": ach,
                             "frac": ach / peak}
    e.sync()
    tuning = e.tuning()
    e.close()
    s0 = stages[names[0]]
    n_launch = sum(launches_per_bench_step(p, s_start + k * MD_STEPS, tuning["form"])
                   for k in range(K))
    cpu = None
    if cpu_seconds > 0:
        # the reference algorithm on one host core, in whole neighbour-list
        # periods (50 steps, one O(N^2) list build each) until cpu_seconds passed
        from oracle import pyoracle as O
        r = O.RefRun(mol, mol.xyz, CUT, 0.05, 0.05, 0.6, 50, 10, 1234, 0)
        r.advance(0)
        done, t_cpu = 0, 0.0
        while t_cpu < cpu_seconds:
            t0 = time.perf_counter()
            r.advance(50)
            t_cpu += time.perf_counter() - t0
            done += 50
        r.close()
        cpu = {"value": mol.n * done / t_cpu, "unit": UNIT, "cores": 1, "kind": "port",
               "sample": f"{done} Langevin steps of this molecule (whole 50-step neighbour-list "
                         f"periods), serial FP32 restatement of the reference's host list filters, "
                         f"force kernels and integrator, one thread"}
    traffic = profile_traffic(workload)
    return {"metric": f"bead-steps/s (plain path, {nbead:,} beads)", "value": value, "unit": UNIT,
            "steps": K, "warmup": warmup, "ms_per_step": 1e3 * t / K,
            "us_per_md_step": 1e6 * t / (K * MD_STEPS),
            "config": {"workload": f"plain path, one molecule of {nbead:,} beads (seed {seed})"
                                   + (", per-contact epsilon U[0.7,1.3]" if eps else "")
                                   + ", NL 32 A / 50 steps, PL 16 A / 10 steps, "
                                   "CUDA graph of 10 steps per replay",
                       "md_steps_per_bench_step": MD_STEPS,
                       "l2": "flushed before every timed step (256 MiB write)"},
            "roofline": {"bound": "hbm", "achieved": s0["achieved_gbs"], "peak": peak,
                         "unit": "GB/s", "frac": s0["frac"], "traffic": traffic,
                         "traffic_source": (f"ncu capture, profiles/step_kernel_{workload}.md"
                                            if traffic else None),
                         "kernel": names[0], "peak_source": peak_kind},
            "cpu_baseline": cpu, "tuning": tuning, "stages": stages, "lists": ls,
            "gpu_launches": int(n_launch), "clocks": clk.summary()}


def plain_one(args, local: int) -> None:
    """`--workload plainN`: the plain path's own JSON line."""
    d = plain_measure(args.workload, local, args.steps, args.warmup, args.lanes, args.form,
                      0.0 if args.no_cpu_baseline else 5.0, args.window)
    line = {"metric": d.pop("metric"), "value": d.pop("value"), "unit": d.pop("unit"),
            "n_gpus": 1, "steps": d.pop("steps"), "warmup": d.pop("warmup"),
            "ms_per_step": d.pop("ms_per_step"), "higher_is_better": True, "scaling": "none",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic", **d}
    print(json.dumps(line), flush=True)


REF_MIN_SECONDS = 5.0


def run_reference(args, rank: int) -> None:
    """The reference's algorithm on the host cores: each step is the bench
    step's 10 Langevin steps of all 512 trajectories, one trajectory per task
    on every host thread.  K steps are timed, and more until REF_MIN_SECONDS
    have passed; the rate is over every timed step."""
    from oracle import pyoracle as O
    mols, ts = ensemble(0)
    cores = os.cpu_count() or 1
    runs = [O.RefRun(m, m.xyz, CUT, 0.05, 0.05, float(t), 50, 10, 1234, k)
            for k, (m, t) in enumerate(zip(mols, ts))]
    beads = int(sum(m.n for m in mols))
    # largest first, one trajectory per task: the pool balances the load
    big_first = sorted(runs, key=lambda r: -r.n)
    with ThreadPoolExecutor(cores) as ex:
        list(ex.map(lambda r: r.advance(0), runs))

        def one():
            list(ex.map(lambda r: r.advance(MD_STEPS), big_first))

        for _ in range(args.warmup):
            one()
        t0 = time.perf_counter()
        steps = 0
        while steps < args.steps or time.perf_counter() - t0 < REF_MIN_SECONDS:
            one()
            steps += 1
        dt = time.perf_counter() - t0
    for r in runs:
        r.close()
    val = beads * MD_STEPS * steps / dt
    line = {"impl": "reference", "metric": METRIC, "value": val, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * dt / steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic", "config": workload_config(beads),
            "cpu_baseline": {"value": val, "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": f"{steps} timed steps ({args.steps} asked, more until "
                                       f"{REF_MIN_SECONDS:.0f} s passed; {dt:.1f} s), each "
                                       f"{MD_STEPS} Langevin steps of all 512 trajectories "
                                       f"({beads} beads), serial FP32 restatement of the "
                                       f"reference algorithm, one trajectory per task on "
                                       f"{cores} threads"},
            "e2e": {"value": val, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    if rank == 0:
        print(json.dumps(line), flush=True)


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-plain", action="store_true", help="skip the plain-loop comparison")
    ap.add_argument("--no-served", action="store_true", help="skip the served request stream")
    ap.add_argument("--lanes", type=int, default=0,
                    help="lanes per bead of the step kernel (2, 4, 8, 16); 0: autotuned")
    ap.add_argument("--form", type=int, default=0,
                    help="form of the step: 1 one kernel, 2 force + finish kernels, 3 persistent "
                         "(the steps between rebuilds in one launch); 0: autotuned")
    ap.add_argument("--window", type=int, default=0,
                    help="shared-memory window of the step in beads; 0: autotuned, -1: none")
    ap.add_argument("--parts", type=int, default=2,
                    help="ensemble: contexts (each on its own stream) the trajectories are split "
                         "over, at equal bead counts")
    ap.add_argument("--workload", default="ensemble", choices=["ensemble", *PLAIN],
                    help="ensemble: the batched ensemble (with the served stream beside it); "
                         "plain128 / plain4000 / plain50k: the plain path on one structure")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))

    if args.impl == "reference":
        if rank == 0:
            run_reference(args, rank)
        return

    if args.workload in PLAIN:
        if rank == 0:
            plain_one(args, local)
        return

    import torch
    import torch.distributed as dist
    from sop_gb300 import engine

    if world > 1:
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)

    def barrier():
        if world > 1:
            dist.barrier()

    mols, ts = ensemble(rank)
    total = sum(m.n for m in mols)
    p = engine.baseline_params(device=local, graph_steps=MD_STEPS, lanes_per_bead=args.lanes,
                               step_split=args.form, step_window=args.window)

    def build():
        # the persistent form (--form 3) runs in one context only
        ens = engine.Ensemble(p, parts=1 if args.form == 3 else args.parts)
        for k, (m, t) in enumerate(zip(mols, ts)):
            ens.add(m, m.xyz, T=float(t), traj=rank * N_TRAJ + k)
        ens.commit()
        return ens

    e = build()
    streams = [torch.cuda.ExternalStream(s, device=dev) for s in e.streams()]
    s0 = streams[0]
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)

    def fork_join(enqueue, ev0, ev1):
        """ev0 on the first stream, the others wait on it; enqueue(); the
        first stream waits on the others' ends; ev1 on the first stream."""
        ev0.record(s0)
        for st in streams[1:]:
            st.wait_event(ev0)
        enqueue()
        for st in streams[1:]:
            j = torch.cuda.Event()
            j.record(st)
            s0.wait_event(j)
        ev1.record(s0)

    for _ in range(args.warmup):
        e.step_async(MD_STEPS)
    e.sync()
    s_start = [eng.status(0)[1] for eng in e.engines]
    tuning = e.tuning()

    K = args.steps
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(K)]
    barrier()
    torch.cuda.synchronize(dev)
    with ClockSampler(local) as clk:
        with torch.cuda.stream(s0):
            for k in range(K):
                flush.zero_()
                fork_join(lambda: e.step_async(MD_STEPS), *ev[k])
        torch.cuda.synchronize(dev)
        e.sync()
    barrier()
    ms = [a.elapsed_time(b) for a, b in ev]
    s_end = [eng.status(0)[1] for eng in e.engines]
    if any(b - a != K * MD_STEPS for a, b in zip(s_start, s_end)):
        raise RuntimeError("a neighbour-list overflow re-ran steps outside the timed region")
    statuses = [e.status(m)[0] for m in range(len(mols))]
    t_local = sum(ms) / 1e3
    t_max = max_over_ranks(t_local, world, dev)
    value = whole_job_rate(total, MD_STEPS * K, world, t_max)

    # ---- roofline of the dominant kernel (the fused step kernel), timed alone:
    # one launch per context, the contexts' launches side by side
    byts, ls = step_kernel_bytes(e, mols)
    reps = 50
    kev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
           for _ in range(reps)]
    with torch.cuda.stream(s0):
        for k in range(reps):
            flush.zero_()
            fork_join(lambda: [eng.launch_stage(0, 0) for eng in e.engines], *kev[k])
    torch.cuda.synchronize(dev)
    t_kernel = statistics.median(a.elapsed_time(b) for a, b in kev) / 1e3
    peak, peak_kind = measured_peaks()
    achieved = byts / t_kernel / 1e9
    forms = {tu.get("form") for tu in tuning}
    traffic = profile_traffic(parts=len(e.engines), form=forms.pop()) if len(forms) == 1 else None
    n_parts = len(e.engines)
    e.close()

    # ---- end to end through the C ABI: host arrays in, coordinates out every step
    e2e = None
    if not args.no_e2e:
        K2 = E2E_STEPS
        pinned = [torch.empty((total, 3), dtype=torch.float32, pin_memory=True).numpy()
                  for _ in range(2)]
        h2d = 0
        for m in mols:
            h2d += 12 * m.n * 2 + 12 * len(m.bond_i) + 8 * len(m.ang_i) + 16 * len(m.nat_i) + 4 * m.n
        barrier()
        t0 = time.perf_counter()
        e2 = build()
        t_setup = time.perf_counter() - t0
        # each step's coordinates are copied out while the next step runs:
        # queue step k and its download, then wait for download k-1
        prev = None
        for k in range(K2):
            e2.step_async(MD_STEPS)
            t = e2.download_all_async(pinned[k & 1])
            if prev is not None:
                e2.download_wait(prev)
            prev = t
        e2.download_wait(prev)
        e2.sync()
        dt = time.perf_counter() - t0
        e2.close()
        barrier()
        dt = max_over_ranks(dt, world, dev)
        t_setup = max_over_ranks(t_setup, world, dev)
        e2e = {"value": whole_job_rate(total, MD_STEPS * K2, world, dt), "unit": UNIT,
               "h2d_bytes_per_step": int(h2d / K2), "d2h_bytes_per_step": int(12 * total),
               "steps": K2, "setup_s": t_setup,
               "steady_value": whole_job_rate(total, MD_STEPS * K2, world, dt - t_setup),
               "note": f"wall clock of a {K2}-step job through the C ABI: creation of the "
                       f"{n_parts} contexts, upload of every structure from host arrays and "
                       "set-up (setup_s), then per step 10 Langevin steps and a download of "
                       "every coordinate (sop_download_all_async of each context into its rows "
                       "of page-locked memory, waited for one step later); value includes the "
                       "set-up, steady_value excludes it"}

    cpu = None
    plain = None
    if rank == 0 and not args.no_cpu_baseline:
        cpu = cpu_baseline(mols, ts)
    if rank == 0 and not args.no_plain:
        # the plain path looping over the same trajectories: one context each
        sample = list(range(0, len(mols), 8))
        nst = 200
        beads = 0
        t_plain = 0.0
        for k in sample:
            m = mols[k]
            ep = engine.plain(m, m.xyz, engine.baseline_params(device=local, graph_steps=MD_STEPS),
                              T=float(ts[k]), traj=k)
            ep.step(MD_STEPS)
            t0 = time.perf_counter()
            ep.step(nst)
            t_plain += time.perf_counter() - t0
            beads += m.n
            ep.close()
        plain = {"value": beads * nst / t_plain, "unit": UNIT,
                 "sample": f"{len(sample)} of the trajectories (every 8th), {nst} steps each, "
                           f"one plain context at a time (the reference's single-molecule loop)"}

    plains = None
    if rank == 0 and not args.no_plain:
        plains = {w: plain_measure(w, local, max(K, 20), args.warmup,
                                   cpu_seconds=0.0 if args.no_cpu_baseline else 3.0)
                  for w in PLAIN}

    served = None
    if rank == 0 and not args.no_served:
        served = served_stream(local)

    if rank == 0:
        n_launch = sum(launches_per_bench_step(p, s0_ + k * MD_STEPS, tu.get("form", 1))
                       for s0_, tu in zip(s_start, tuning) for k in range(K))
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": K,
            "warmup": args.warmup, "ms_per_step": 1e3 * t_max / K, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": dict(workload_config(total), contexts=n_parts,
                           streams=f"{n_parts} contexts, one CUDA stream each, cut at equal "
                                   "bead counts; joined at every bench step"),
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic,
                         "traffic_source": ("ncu capture of this kernel on this workload, "
                                            "profiles/step_kernel_ensemble.md" if traffic else None),
                         "kernel": "force + Langevin step (k_step; + k_finish in the two-kernel "
                                   "form), one launch per context side by side",
                         "step_form": [tu.get("form") for tu in tuning],
                         "bytes_per_launch": byts, "launch_us": t_kernel * 1e6,
                         "peak_source": peak_kind},
            "cpu_baseline": cpu,
            "e2e": e2e,
            "gpu_launches": int(n_launch),
            "clocks": clk.summary(),
            "plain_loop": plain,
            "batched_over_plain": (value / world / plain["value"]) if plain else None,
            "served": served,
            "plain": plains,
            "lists": ls,
            "tuning": tuning,
            "contexts": n_parts,
            "molecule_errors": int(sum(1 for s in statuses if s & 3)),
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
