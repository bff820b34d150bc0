#!/usr/bin/env python3
"""Benchmark of the GB300 event-loop engine: executed events/s on sDMD's event loop.

Workload (default, --workload c4): the uneven batch -- 512 independent single
random-sequence chains of 5-60 residues, box edge scaled to constant density,
Andersen NVT at 280-400 K -- built from seeded synthetic inputs through the
host-side C builder, all systems in one launch.  The path is the FP32 screen with
FP64 refine and eager advance (every pop moves every atom, as the reference
does), so every event equals the reference's bit for bit
(tests/test_gpu_bench_path.py).  A "step" is E executed events of the event loop
(src/SGThread.c:75-151) on every system of the batch.

  value     executed events/s with the state resident in HBM, CUDA events on the
            engine's stream, L2 flushed before each step;
  e2e       the same metric through the public C ABI with host buffers (create +
            upload, tree build, run, download inside the timed region), over the
            same trajectory segment as `value` -- its final state is checked equal;
  plain_fp64  the plain single-replica all-FP64 GPU form (one ALA x 10 replica,
            FP64 prediction of every candidate) and the ratio the metric names;
  roofline  the loop kernel's algorithmic bytes per launch over its CUDA-event
            duration, against the measured HBM copy bandwidth.

--impl reference runs the reference's CPU algorithm (the oracle's C restatement,
compiled on this host) on the same batch: the same E events per system per
step, the same warm-up steps before the timed ones, one single-threaded loop
per host core as the reference runs one system per process.

Multi-GPU (torchrun): the event loop of one system is sequential, so ranks run
independent batches (different seeds): "replicas only", weak scaling.
"""
import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

METRIC = "events/s per GB300: batched FP32-screen vs plain FP64, at matched NVE drift"


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class Dist:
    def __init__(self):
        self.rank, self.world, self.local = dist_env()
        self.pg = None
        if self.world > 1:
            import torch.distributed as td
            os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
            td.init_process_group("gloo", rank=self.rank, world_size=self.world)
            self.td = td

    def barrier(self):
        if self.world > 1:
            self.td.barrier()

    def max(self, v):
        if self.world == 1:
            return v
        import torch
        t = torch.tensor([float(v)], dtype=torch.float64)
        self.td.all_reduce(t, op=self.td.ReduceOp.MAX)
        return float(t.item())

    def sum(self, v):
        if self.world == 1:
            return v
        import torch
        t = torch.tensor([float(v)], dtype=torch.float64)
        self.td.all_reduce(t, op=self.td.ReduceOp.SUM)
        return float(t.item())


class ClockSampler:
    """nvidia-smi samples (200 ms) during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.p = None

    def start(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                                       "--format=csv,noheader,nounits", "-lms", "200"],
                                      stdout=self.f, stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None

    def stop(self):
        if self.p is not None:
            self.p.terminate()
            try:
                self.p.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.p.kill()
        self.f.flush()
        rows = []
        with open(self.f.name) as fh:
            for line in fh:
                parts = [x.strip() for x in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        os.unlink(self.f.name)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no nvidia-smi samples"], "samples": 0}
        def num(x):
            try:
                return float(x)
            except ValueError:
                return None
        sm = [num(r[1]) for r in rows if num(r[1]) is not None]
        mx = [num(r[2]) for r in rows if num(r[2]) is not None]
        reasons = set()
        for r in rows:
            for name, val in zip(["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"], r[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(rows)}


WORKLOADS = {
    "c1": "C1: one ALA x 10 chain (59 atoms), 40 A cube, Andersen NVT 300 K",
    "c2": "C2: 256 random-sequence 16-mer peptides at 5 mM, 440 A periodic cube, Andersen NVT 300 K "
          "(full-rebuild-sweep configuration)",
    "c3": "C3: 64 replicas of ALA x 10, temperatures geometric 270-500 K, on-device replica exchange every "
          "1e4 events per replica",
    "c4": "C4: 512 single random-sequence chains of 5-60 residues, box edge 40 A * (N/59)^(1/3) (floor 27 A), "
          "Andersen NVT 280-400 K",
    "c5": "C5: 8 replicas of 400 random-sequence 10-mers (~42k atoms) in a smooth cylindrical wall of radius "
          "60 A with a 120 A periodic axis (compressed rigid-chain packing), Andersen NVT 310 K",
}


def build_workload(name, rank):
    from sdmd_gb300 import workloads as W
    if name not in WORKLOADS:
        raise SystemExit(f"unknown workload {name}")
    make = {"c1": lambda: [W.c1(seed=1 + rank)], "c2": lambda: [W.c2(seed=1 + rank)],
            "c3": lambda: W.c3(seed=1 + rank), "c4": lambda: W.c4(seed=1 + rank),
            "c5": lambda: W.c5(seed=1 + rank)}[name]
    return make()


def run_config(args, systems, world):
    """The workload's description, identical in both arms of the benchmark."""
    return {"workload": WORKLOADS[args.workload], "n_systems": len(systems) * world,
            "n_atoms": sum(s.n for s in systems) * world, "events_per_step": args.events_per_step * len(systems),
            "events_per_system_per_step": args.events_per_step,
            "segment": f"{args.warmup} warm-up steps, then {args.steps} timed steps, from the state after the "
                       "full-rebuild sweep",
            "l2": "flushed between steps (256 MiB write)"}


def neighbourhood_mean(s):
    """Mean 27-cell neighbourhood population (candidates P per predicted atom)."""
    import numpy as np
    cn = s.scal["cellnum"]
    occ = np.zeros((cn[2], cn[1], cn[0]), np.int64)
    np.add.at(occ, (s.a["cz"][1:], s.a["cy"][1:], s.a["cx"][1:]), 1)
    tot = np.zeros_like(occ)
    for dz in (-1, 0, 1):
        for dy in (-1, 0, 1):
            for dx in (-1, 0, 1):
                tot += np.roll(occ, (dz, dy, dx), axis=(0, 1, 2))
    return float(tot[s.a["cz"][1:], s.a["cy"][1:], s.a["cx"][1:]].mean())


def system_bytes(s):
    """Host<->device bytes of one system: static arrays once, dynamic arrays both ways."""
    from sdmd_gb300.system import DYNAMIC_ARRAYS, STATIC_ARRAYS
    st = sum(s.a[k].nbytes for k, _ in STATIC_ARRAYS)
    dy = sum(s.a[k].nbytes for k, _ in DYNAMIC_ARRAYS)
    return st, dy


def peaks():
    try:
        with open(os.path.join(REPO, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def autotune_candidates(systems):
    """CTA sizes the autotuner tries: up to 512 threads for large systems (which run
    with helper blocks), 128-256 for a single small one, 64-256 for batches."""
    if min(s.n for s in systems) >= 2048:
        return (128, 256, 512)
    return (128, 256) if len(systems) == 1 else (64, 128, 256)


def load_traffic():
    p = os.path.join(REPO, "profiles", "traffic.json")
    try:
        with open(p) as f:
            return json.load(f)
    except Exception:
        return {}


def event_bytes(s, advance):
    """Algorithmic bytes per executed event of one system: the candidates' state
    read for the target and the partner (P per atom, 56 B each), both atoms' own
    state and new events, the two tree paths; eager advance adds every atom's
    position and event time, read and written, at every pop."""
    P = neighbourhood_mean(s)
    logn = math.ceil(math.log2(max(s.n, 2)))
    b = 2 * P * 56 + 2 * 104 + 2 * logn * 12
    if advance == "eager":
        pops = 1.0 + s.counters.get("recal", 0) / max(s.counters.get("frame", 1), 1)
        b += pops * s.n * 56
    return b, P


def plain_fp64_rate(device, events=3000):
    """The metric's denominator: the plain single-replica all-FP64 GPU form -- one
    ALA x 10 replica, every candidate predicted in FP64, eager advance -- timed
    with CUDA events on the engine's stream after a warm-up run."""
    from sdmd_gb300 import workloads as W
    from sdmd_gb300.engine import ADVANCE_EAGER, SCREEN_FP64, Engine
    s = W.c1()
    with Engine([s], advance=ADVANCE_EAGER, screen=SCREEN_FP64, device=device) as e:
        e.prepare(full=True)
        e.run(1000)
        e.run(events)
        ms = e.last_ms()[1]
    return {"value": round(events / ms * 1e3, 3), "unit": "events/s",
            "workload": "one ALA x 10 replica (59 atoms), 40 A cube, Andersen NVT 300 K; plain FP64 prediction, "
                        "eager advance", "events": events}


def run_ours(args, D):
    import numpy as np
    if D.rank == 0:
        import __graft_entry__ as G
        G.build()
    D.barrier()
    from sdmd_gb300.engine import (ADVANCE_EAGER, ADVANCE_LAZY, SCREEN_FP32, SCREEN_FP64, Engine,
                                   autotune_threads)
    import torch
    torch.cuda.set_device(D.local)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")   # > 129 MB L2

    systems = build_workload(args.workload, D.rank)
    if args.systems:   # the first K systems of the batch (small profiling cases)
        systems = systems[:args.systems]
    cfg = run_config(args, systems, D.world)
    E = args.events_per_step
    adv = ADVANCE_LAZY if args.advance == "lazy" else ADVANCE_EAGER
    scr = SCREEN_FP32 if args.screen == "fp32" else SCREEN_FP64
    tuned = None
    if args.threads:
        threads = args.threads
    else:   # CTA size from the autotuner (short runs on copies of the workload)
        threads, tuned = autotune_threads(systems, advance=adv, screen=scr, device=D.local,
                                          candidates=autotune_candidates(systems))
    eng = Engine(systems, threads=threads, device=D.local, advance=adv, screen=scr)
    eng.prepare(full=True)
    sweep_ms = eng.last_ms()[0]
    eng.download()
    after_sweep = [s.copy() for s in systems]

    remd = None
    if args.workload == "c3":   # one step = one exchange round: E events per replica, then the exchange
        from sdmd_gb300.system import glibc_rng_state
        remd = {"num": np.arange(1, len(systems) + 1), "T": np.array([s.scal["temperature"] for s in systems]),
                "rng": glibc_rng_state(20201), "attempted": 0, "accepted": 0}

    def step(e, state):
        if state is None:
            e.run(E)
            return None
        out = e.run_remd(1, state["num"], state["T"], state["rng"], every_events=E, attempted=state["attempted"],
                         accepted=state["accepted"])
        return dict(num=out["num"], T=out["T"], rng=out["rng"], attempted=out["attempted"],
                    accepted=out["accepted"])

    for _ in range(args.warmup):
        remd = step(eng, remd)
    eng.download()
    seg0 = [s.copy() for s in systems]            # the timed segment starts here (both measurements)
    remd0 = None if remd is None else dict(remd)
    D.barrier()
    torch.cuda.synchronize()
    clocks = ClockSampler(D.local)
    clocks.start()
    frame0 = sum(s.counters["frame"] for s in systems)
    step_ms = []
    launches = loop_launches = 0
    loop_ms = 0.0
    t_wall0 = time.perf_counter()
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        remd = step(eng, remd)
        step_ms.append(eng.last_ms()[1])
        a, b, c = eng.last_run_stats()
        launches += a
        loop_launches += b
        loop_ms += c
    torch.cuda.synchronize()
    wall = time.perf_counter() - t_wall0
    clk = clocks.stop()
    D.barrier()
    eng.download()
    events = sum(s.counters["frame"] for s in systems) - frame0
    t_dev = sum(step_ms) / 1e3
    t_max = D.max(t_dev)
    ev_all = D.sum(events)
    value = ev_all / t_max
    info = eng.launch_info()

    # e2e through the C ABI with host buffers, over the same segment: each step
    # uploads the state, rebuilds the tree, runs E events and downloads
    st_b, dy_b = 0, 0
    for s in seg0:
        a, b = system_bytes(s)
        st_b += a
        dy_b += b
    work = [s.copy() for s in seg0]
    st_e2e = None if remd0 is None else dict(remd0)
    e2e_t = []
    e2e_events = 0
    for k in range(args.steps):
        f0 = sum(s.counters["frame"] for s in work)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        with Engine(work, threads=threads, device=D.local, advance=adv, screen=scr) as e2:
            e2.prepare(full=False)
            st_e2e = step(e2, st_e2e)
            e2.download()
        e2e_t.append(time.perf_counter() - t0)
        e2e_events += sum(s.counters["frame"] for s in work) - f0
    e2e_value = D.sum(e2e_events) / D.max(sum(e2e_t))
    same = all(all(np.array_equal(a.a[k], b.a[k]) for k in ("x", "vx", "ev_time", "ev_partner")) and
               a.counters == b.counters for a, b in zip(work, systems))

    # roofline of the loop kernel: algorithmic bytes per launch over its CUDA-event time
    per_sys = [event_bytes(s, args.advance) for s in after_sweep]
    per_event = sum(b for b, _ in per_sys) / len(per_sys)   # every system runs E events per step
    P_mean = sum(p for _, p in per_sys) / len(per_sys)
    kname = info["loop_kernel"]
    n_launch = max(loop_launches, 1)
    bytes_per_launch = per_event * events / n_launch
    launch_s = loop_ms / 1e3 / n_launch
    peak, peak_kind = peaks()
    achieved = bytes_per_launch / launch_s / 1e9
    traffic = load_traffic().get(f"{kname}_{args.workload}_{args.advance}_dram_bytes_per_event")
    roof = {"bound": "hbm", "achieved": round(achieved, 3), "peak": peak, "unit": "GB/s",
            "frac": round(achieved / peak, 6), "peak_kind": peak_kind,
            "traffic": None if traffic is None else round(traffic * events / n_launch, 1),
            "kernel": kname, "launches": loop_launches, "bytes_per_event": round(per_event, 1),
            "P_candidates": round(P_mean, 2)}
    # the full-rebuild sweep: its algorithmic bytes (every atom's state read once,
    # its new event written, the cell lists and bond lists read) over its device time
    b_sweep = 0
    for s0 in after_sweep:
        ncell = int(np.prod(s0.scal["cellnum"]))
        b_sweep += 104 * s0.n + 4 * (ncell + s0.n) + 4 * int(s0.a["bond_j"].size)
    sweep = {"ms": round(sweep_ms, 3), "bytes": b_sweep, "GBps": round(b_sweep / (sweep_ms / 1e3) / 1e9, 3),
             "frac_hbm": round(b_sweep / (sweep_ms / 1e3) / 1e9 / peak, 6)}

    plain = cpu = drift = None
    if D.rank == 0:
        plain = plain_fp64_rate(D.local)
        if not args.no_cpu:
            cpu = cpu_baseline(after_sweep, args.cpu_seconds)
        if not args.no_drift and remd is None:   # outside every timed region
            drift = measure_nve_drift(after_sweep[:16], threads, D.local, adv, scr)

    if D.rank == 0:
        eng_cfg = {"advance": args.advance, "screen": args.screen, "threads_per_system": threads,
                   "helper_blocks": info["helper_blocks"], "staged": info["staged"], "loop_kernel": kname,
                   "replicas": "independent per rank" if D.world > 1 else None}
        if tuned is not None:
            eng_cfg["autotune"] = {str(k): round(v, 1) for k, v in tuned.items()}
        if remd is not None:
            eng_cfg["exchange"] = {"every_events": E, "attempted": int(remd["attempted"]),
                                   "accepted": int(remd["accepted"])}
        line = {"metric": METRIC, "value": round(value, 3), "unit": "events/s", "n_gpus": D.world,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(t_max * 1e3 / args.steps, 3),
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": "f32+f64" if args.screen == "fp32" else "f64",
                "data": "synthetic (seeded random-sequence peptides, bundled Library_Ding force field)",
                "config": cfg, "engine": eng_cfg,
                "e2e": {"value": round(e2e_value, 3), "unit": "events/s", "h2d_bytes_per_step": st_b + dy_b,
                        "d2h_bytes_per_step": dy_b, "same_trajectory_as_value": bool(same)},
                "plain_fp64": plain,
                "vs_plain_fp64": None if plain is None else round(value / plain["value"], 2),
                "exact": "every event equals the reference's (eager advance)" if args.advance == "eager" else
                         "lazy advance: rounding differs from the reference",
                "roofline": roof, "sweep": sweep, "cpu_baseline": cpu, "nve_drift": drift, "clocks": clk,
                "gpu_launches": launches, "wall_s_timed": round(wall, 3)}
        print(json.dumps(line))


def measure_nve_drift(systems0, threads, device, adv, scr, events=20000):
    """The metric's "matched NVE drift": from the same post-sweep states with the
    thermostat off, the energy change of the measured path and of plain FP64
    (eager advance), as |dE| / (N kT) per 10^6 executed events, worst system.  E
    is CalKinetE + CalPotenE on the device plus the constraint-step energy the
    reference's CalPotenE leaves out.  Forming or breaking a hydrogen bond changes
    that bookkeeping by the bond's energy (the reference's sum is not conserved
    across HB events), so systems with HB or HB-neighbour events in the window are
    left out of the worst case and counted."""
    from sdmd_gb300.energy import constraint_energy, nve_drift
    from sdmd_gb300.engine import ADVANCE_EAGER, SCREEN_FP64, Engine
    out = {"unit": "|dE|/(N kT) per 1e6 executed events (worst of the systems)", "limit": 1e-4,
           "thermostat": "off", "systems": len(systems0)}
    for name, a, sc in (("measured_path", adv, scr), ("fp64_eager", ADVANCE_EAGER, SCREEN_FP64)):
        ss = [s.copy() for s in systems0]
        for s in ss:
            s.scal["thermostat"] = 0
        with Engine(ss, threads=threads, device=device, advance=a, screen=sc) as e:
            e.prepare(full=True)
            pot, kin = e.energies()
            e.download()
            e0 = [pot[k] + kin[k] + constraint_energy(s) for k, s in enumerate(ss)]
            f0 = [s.counters["frame"] for s in ss]
            h0 = [s.counters["hb"] + s.counters["hbneighbor"] for s in ss]
            e.run(events)
            pot, kin = e.energies()
            e.download()
            e1 = [pot[k] + kin[k] + constraint_energy(s) for k, s in enumerate(ss)]
        worst, ev_tot, with_hb = 0.0, 0, 0
        for k, s in enumerate(ss):
            ev = s.counters["frame"] - f0[k]
            ev_tot += ev
            if s.counters["hb"] + s.counters["hbneighbor"] > h0[k]:
                with_hb += 1
                continue
            worst = max(worst, nve_drift(e0[k], e1[k], s.n, float(s.scal["temperature"]), ev))
        out[name] = {"events": int(ev_tot), "drift": worst if with_hb < len(ss) else None,
                     "systems_with_hb_events_left_out": with_hb}
    return out


def cpu_baseline(systems, seconds):
    """The oracle (C restatement of the reference's loop) on one host core, on a
    bounded sample of the same workload: events of the first systems of the batch
    from their post-sweep states."""
    from oracle import oracle as O
    k = min(len(systems), 4)
    loops = []
    for s0 in systems[:k]:
        s = s0.copy()
        loops.append(O.Loop(s))
    t0 = time.perf_counter()
    for L in loops:
        L.run(200)
    rate = 200 * k / max(time.perf_counter() - t0, 1e-6)
    n = int(max(500, min(rate * seconds / k, 5e6)))
    t0 = time.perf_counter()
    for L in loops:
        L.run(n)
    dt = time.perf_counter() - t0
    return {"value": round(n * k / dt, 3), "unit": "events/s", "cores": 1, "kind": "port",
            "sample": f"{n} events on each of the first {k} systems of the batch from their post-sweep states "
                      "(oracle/sdmd_oracle.c, gcc -O2)"}


def _ref_worker_main(conn, workload, rank, idx):
    """One host process of the reference arm: the oracle loop on its systems of the
    batch, E events each per command, timed around the whole command."""
    sys.path.insert(0, REPO)
    from oracle import oracle as O
    systems = build_workload(workload, rank)
    loops = []
    for k in idx:
        s = systems[k].copy()
        O.predict_all(s)
        loops.append(O.Loop(s))
    conn.send(("ready", 0.0, 0))
    while True:
        n = conn.recv()
        if n is None:
            break
        f0 = sum(L.system.counters["frame"] for L in loops)
        t0 = time.perf_counter()
        for L in loops:
            L.run(n)
        dt = time.perf_counter() - t0
        conn.send(("done", dt, sum(L.system.counters["frame"] for L in loops) - f0))
    conn.close()


def run_reference(args, D):
    """The reference's CPU algorithm (oracle port) on this host's cores: the same
    batch, the same E events per system per step and the same warm-up steps, one
    single-threaded loop per core with the systems spread over the cores."""
    if D.rank != 0:
        return
    from oracle import oracle as O
    O.build()
    from sdmd_gb300 import build as B
    B.build_host()
    import multiprocessing as mp
    systems = build_workload(args.workload, 0)   # built (and cached) once, before the workers load it
    if args.systems:
        systems = systems[:args.systems]
    cfg = run_config(args, systems, 1)
    if args.workload == "c3":
        cfg["reference_note"] = "exchange rounds not replayed: the replicas run E events per step"
    cores = min(len(systems), os.cpu_count() or 1)
    groups = [list(range(k, len(systems), cores)) for k in range(cores)]
    ctx = mp.get_context("spawn")
    pipes, procs = [], []
    for g in groups:
        a, b = ctx.Pipe()
        p = ctx.Process(target=_ref_worker_main, args=(b, args.workload, 0, g))
        p.start()
        pipes.append(a)
        procs.append(p)
    for a in pipes:
        a.recv()

    def one_step():
        for a in pipes:
            a.send(args.events_per_step)
        res = [a.recv() for a in pipes]
        return max(r[1] for r in res), sum(r[2] for r in res)

    for _ in range(args.warmup):
        one_step()
    times, total = [], 0
    for _ in range(args.steps):
        t, n = one_step()
        times.append(t)
        total += n
    for a in pipes:
        a.send(None)
    for p in procs:
        p.join()
    value = total / sum(times)
    line = {"impl": "reference", "metric": METRIC, "value": round(value, 3), "unit": "events/s", "n_gpus": D.world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(sum(times) * 1e3 / args.steps, 3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded random-sequence peptides, bundled Library_Ding force field)", "config": cfg,
            "cpu_baseline": {"value": round(value, 3), "unit": "events/s", "cores": cores, "kind": "port",
                             "per_core": round(value / cores, 3),
                             "sample": f"the whole workload: {args.events_per_step} events per system per step on "
                                       f"all {len(systems)} systems, {cores} single-threaded loops (one per core, "
                                       "the systems spread over them), after the same warm-up steps"},
            "e2e": {"value": round(value, 3), "unit": "events/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", default="c4", choices=sorted(WORKLOADS))
    ap.add_argument("--events-per-step", type=int, default=None, help="executed events per system per step")
    ap.add_argument("--threads", type=int, default=0)
    ap.add_argument("--systems", type=int, default=0, help="run only the first K systems of the batch")
    ap.add_argument("--advance", choices=["eager", "lazy"], default="eager")
    ap.add_argument("--screen", choices=["fp32", "fp64"], default="fp32")
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-drift", action="store_true")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.events_per_step is None:
        args.events_per_step = {"c3": 10000, "c4": 5000}.get(args.workload, 20000)
    D = Dist()
    if args.impl == "reference":
        run_reference(args, D)
    else:
        run_ours(args, D)


if __name__ == "__main__":
    main()
