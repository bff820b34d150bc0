#!/usr/bin/env python3
"""Benchmark of the GB300 event-loop engine: executed events/s on sDMD's event loop.

Workload (default, --workload c2): the full-rebuild-sweep configuration -- 256
random-sequence 16-residue peptides at 5 mM in a periodic 440 A cube
(~42k atoms), Andersen NVT at 300 K, built from seeded synthetic inputs through
the host-side C builder.  A "step" is one chunk of E executed events of the
event loop (src/SGThread.c:75-151) on that system; `value` = executed events/s
with the state resident in HBM, timed with CUDA events on the engine's stream;
`e2e` = the same metric through the public C ABI with host buffers (create +
upload, tree build, run, download inside the timed region).

--impl reference times the reference's CPU algorithm (the oracle's C
restatement, compiled on this host) on the same workload and prints the same
line with "impl": "reference".

Besides the timed value, the line reports the loop kernel's roofline figures, the
oracle on one host core (`cpu_baseline`) and, for single systems, the NVE energy
drift of the measured path and of plain FP64 from the same state (`nve_drift`).

Multi-GPU (torchrun): the event loop of one system is sequential, so ranks run
independent replicas (different seeds): "replicas only", weak scaling.
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


def build_workload(name, rank):
    from sdmd_gb300 import workloads as W
    if name == "c2":
        return [W.c2(seed=1 + rank)], {"workload": "C2: 256 random-sequence 16-mer peptides at 5 mM, 440 A periodic "
                                                   "cube, Andersen NVT 300 K (full-rebuild-sweep configuration)"}
    if name == "c1":
        return [W.c1(seed=1 + rank)], {"workload": "C1: one ALA x 10 chain, 40 A cube, Andersen NVT 300 K"}
    if name == "c3":
        return W.c3(seed=1 + rank), {"workload": "C3: 64 replicas of ALA x 10, temperatures geometric 270-500 K, "
                                                 "on-device replica exchange every 1e4 events per replica"}
    if name == "c4":
        return W.c4(seed=1 + rank), {"workload": "C4: 512 single random-sequence chains of 5-60 residues, box edge "
                                                 "40 A * (N/59)^(1/3) (floor 27 A), Andersen NVT 280-400 K"}
    raise SystemExit(f"unknown workload {name}")


def neighbourhood_mean(s):
    """Mean 27-cell neighbourhood population (candidates P per predicted atom)."""
    import numpy as np
    cn = s.scal["cellnum"]
    n = s.n
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


def load_traffic():
    p = os.path.join(REPO, "profiles", "traffic.json")
    try:
        with open(p) as f:
            return json.load(f)
    except Exception:
        return {}


def run_ours(args, D):
    import numpy as np
    if D.rank == 0:
        import __graft_entry__ as G
        G.build()
    D.barrier()
    from sdmd_gb300.engine import Engine
    from sdmd_gb300.system import System
    import torch
    torch.cuda.set_device(D.local)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")   # > 129 MB L2

    systems, cfg = build_workload(args.workload, D.rank)
    natoms = sum(s.n for s in systems)
    E = args.events_per_step
    host_copy = [s.copy() for s in systems]

    from sdmd_gb300.engine import ADVANCE_EAGER, ADVANCE_LAZY, SCREEN_FP32, SCREEN_FP64
    adv = ADVANCE_LAZY if args.advance == "lazy" else ADVANCE_EAGER
    scr = SCREEN_FP32 if args.screen == "fp32" else SCREEN_FP64
    tuned = None
    if args.threads:
        threads = args.threads
    else:   # CTA size from the autotuner (short runs on copies of the workload)
        from sdmd_gb300.engine import autotune_threads
        threads, tuned = autotune_threads(systems, advance=adv, screen=scr, device=D.local,
                                          candidates=(128, 256) if len(systems) == 1 else (64, 128, 256))
    eng = Engine(systems, threads=threads, device=D.local, advance=adv, screen=scr)
    eng.prepare(full=True)
    sweep_ms = eng.last_ms()[0]
    eng.download()
    after_sweep = [s.copy() for s in systems]

    remd = None
    if args.workload == "c3":   # one step = one exchange round: E events per replica, then the exchange
        import numpy as np
        from sdmd_gb300.system import glibc_rng_state
        remd = {"num": np.arange(1, len(systems) + 1), "T": np.array([s.scal["temperature"] for s in systems]),
                "rng": glibc_rng_state(20201), "attempted": 0, "accepted": 0}

    def step():
        if remd is None:
            eng.run(E)
            return
        out = eng.run_remd(1, remd["num"], remd["T"], remd["rng"], every_events=E, attempted=remd["attempted"],
                           accepted=remd["accepted"])
        remd.update(num=out["num"], T=out["T"], rng=out["rng"], attempted=out["attempted"],
                    accepted=out["accepted"])

    for _ in range(args.warmup):
        step()
    D.barrier()
    torch.cuda.synchronize()
    clocks = ClockSampler(D.local)
    clocks.start()
    frame0 = sum(s.counters["frame"] for s in systems)
    eng.download()
    frame0 = sum(s.counters["frame"] for s in systems)
    step_ms = []
    launches = loop_launches = 0
    loop_ms = 0.0
    t_wall0 = time.perf_counter()
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        step()
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

    # e2e through the C ABI with host buffers: upload, tree build, run, download
    st_b, dy_b = 0, 0
    for s in after_sweep:
        a, b = system_bytes(s)
        st_b += a
        dy_b += b
    e2e_t = []
    e2e_events = 0
    work = [s.copy() for s in after_sweep]
    for k in range(args.steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        with Engine(work, threads=threads, device=D.local, advance=adv, screen=scr) as e2:
            e2.prepare(full=False)
            if remd is None:
                e2.run(E)
            else:
                e2.run_remd(1, remd["num"], remd["T"], remd["rng"], every_events=E)
            e2.download()
        e2e_t.append(time.perf_counter() - t0)
        e2e_events += E * len(work)
    e2e_value = D.sum(e2e_events) / D.max(sum(e2e_t))

    # roofline of the loop kernel: algorithmic bytes per executed event
    P = neighbourhood_mean(after_sweep[0])
    logn = math.ceil(math.log2(max(after_sweep[0].n, 2)))
    pops_per_event = 1.0 + after_sweep[0].counters.get("recal", 0) / max(after_sweep[0].counters.get("frame", 1), 1)
    per_event = 2 * P * 56 + 2 * 104 + 2 * logn * 12
    if args.advance == "eager":
        per_event += pops_per_event * after_sweep[0].n * 56   # every pop moves every atom and event time
    kname = "loop_kernel_screen" if args.screen == "fp32" else "loop_kernel_fp64"
    n_launch = max(loop_launches, 1)
    bytes_per_launch = per_event * events / n_launch
    launch_s = loop_ms / 1e3 / n_launch          # CUDA events around each event-loop launch
    peak, peak_kind = peaks()
    achieved = bytes_per_launch / launch_s / 1e9
    traffic = load_traffic().get(f"{kname}_{args.workload}_{args.advance}_dram_bytes_per_event")
    roof = {"bound": "hbm", "achieved": round(achieved, 3), "peak": peak, "unit": "GB/s",
            "frac": round(achieved / peak, 6), "peak_kind": peak_kind,
            "traffic": None if traffic is None else round(traffic * events / n_launch, 1),
            "kernel": kname, "launches": loop_launches, "bytes_per_event": round(per_event, 1),
            "P_candidates": round(P, 2)}
    # the full-rebuild sweep: its algorithmic bytes (every atom's state read once,
    # its new event written, the cell list and bond lists read) over its device time
    s0 = after_sweep[0]
    ncell = int(np.prod(s0.scal["cellnum"]))
    b_sweep = 104 * s0.n + 4 * (ncell + s0.n) + 4 * int(s0.a["bond_j"].size)
    sweep = {"ms": round(sweep_ms, 3), "bytes": b_sweep, "GBps": round(b_sweep / (sweep_ms / 1e3) / 1e9, 3),
             "frac_hbm": round(b_sweep / (sweep_ms / 1e3) / 1e9 / peak, 6)}

    cpu = None
    if D.rank == 0 and D.world >= 1 and not args.no_cpu:
        cpu = cpu_baseline(after_sweep[0], args.cpu_seconds)
    drift = None
    if D.rank == 0 and len(systems) == 1 and not args.no_drift:   # outside every timed region
        drift = measure_nve_drift(after_sweep[0], threads, D.local, adv, scr)

    if D.rank == 0:
        if tuned is not None:
            cfg["autotune"] = {str(k): round(v, 1) for k, v in tuned.items()}
        if remd is not None:
            cfg["exchange"] = {"every_events": E, "attempted": int(remd["attempted"]),
                               "accepted": int(remd["accepted"])}
        cfg.update({"n_atoms": natoms, "n_systems": len(systems) * D.world, "events_per_step": E * len(systems),
                    "l2": "flushed between steps (256 MiB write)", "advance": args.advance, "screen": args.screen,
                    "threads_per_system": threads, "replicas": "independent per rank" if D.world > 1 else None})
        line = {"metric": METRIC, "value": round(value, 3), "unit": "events/s", "n_gpus": D.world,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(t_max * 1e3 / args.steps, 3),
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": "f32+f64" if args.screen == "fp32" else "f64",
                "data": "synthetic (seeded random-sequence peptides, bundled Library_Ding force field)",
                "config": cfg,
                "e2e": {"value": round(e2e_value, 3), "unit": "events/s", "h2d_bytes_per_step": st_b + dy_b,
                        "d2h_bytes_per_step": dy_b},
                "roofline": roof, "sweep": sweep, "cpu_baseline": cpu, "nve_drift": drift, "clocks": clk,
                "gpu_launches": launches, "wall_s_timed": round(wall, 3)}
        print(json.dumps(line))


def measure_nve_drift(s0, threads, device, adv, scr, events=200000, events_ref=20000):
    """The metric's "matched NVE drift": from the same post-sweep state with the
    thermostat off, the energy change of the measured path (FP32 screen, lazy
    advance) and of the reference's algorithm (plain FP64, eager advance, fewer
    events: it is slower), as |dE| / (N kT) per 10^6 executed events.  E is
    CalKinetE + CalPotenE on the device plus the constraint-step energy the
    reference's CalPotenE leaves out; HB events change that bookkeeping, so their
    count is reported with each run."""
    from sdmd_gb300.energy import constraint_energy, nve_drift
    from sdmd_gb300.engine import ADVANCE_EAGER, SCREEN_FP64, Engine
    out = {"unit": "|dE|/(N kT) per 1e6 executed events", "limit": 1e-4, "thermostat": "off"}
    kT = float(s0.scal["temperature"])
    for name, a, sc, n in (("measured_path", adv, scr, events), ("fp64_eager", ADVANCE_EAGER, SCREEN_FP64, events_ref)):
        s = s0.copy()
        s.scal["thermostat"] = 0
        with Engine([s], threads=threads, device=device, advance=a, screen=sc) as e:
            e.prepare(full=True)
            pot, kin = e.energies()
            e.download()
            e0, f0 = pot[0] + kin[0] + constraint_energy(s), s.counters["frame"]
            e.run(n)
            pot, kin = e.energies()
            e.download()
            e1 = pot[0] + kin[0] + constraint_energy(s)
        ev = s.counters["frame"] - f0
        out[name] = {"events": int(ev), "drift": nve_drift(e0, e1, s.n, kT, ev),
                     "hb_events": int(s.counters["hb"] + s.counters["hbneighbor"])}
    return out


def cpu_baseline(system, seconds):
    """The oracle (C restatement of the reference's loop) on this host, single
    core, on a bounded sample: events from the same post-sweep state."""
    from oracle import oracle as O
    s = system.copy()
    loop = O.Loop(s)
    t0 = time.perf_counter()
    rc, _, _ = loop.run(500)
    dt = time.perf_counter() - t0
    rate = 500 / max(dt, 1e-6)
    n = int(max(1000, min(rate * seconds, 5e6)))
    t0 = time.perf_counter()
    rc, _, _ = loop.run(n)
    dt = time.perf_counter() - t0
    return {"value": round(n / dt, 3), "unit": "events/s", "cores": 1, "kind": "port",
            "sample": f"{n} events of the same system from the post-sweep state (oracle/sdmd_oracle.c, gcc -O2)"}


_WORKER_SYSTEMS = {}


def _ref_worker(job):
    """One host process of the reference arm: the oracle loop on system k of the batch."""
    workload, k, n_events = job
    sys.path.insert(0, REPO)
    from oracle import oracle as O
    if workload not in _WORKER_SYSTEMS:   # built (or loaded) once per worker process
        _WORKER_SYSTEMS[workload] = build_workload(workload, 0)[0]
    s = _WORKER_SYSTEMS[workload][k].copy()
    O.predict_all(s)
    loop = O.Loop(s)
    t0 = time.perf_counter()
    loop.run(n_events)
    return n_events, time.perf_counter() - t0


def run_reference_batch(args, D, systems, cfg):
    """A batch of independent systems: one single-threaded reference loop per host
    core, min(#systems, cores) at once, events summed over the wall time."""
    import multiprocessing as mp
    cores = min(len(systems), os.cpu_count() or 1)
    n_ev = max(200, int(args.events_per_step * args.cpu_seconds / 60))   # bounded sample per core and step
    ctx = mp.get_context("spawn")
    with ctx.Pool(cores) as pool:
        pool.map(_ref_worker, [(args.workload, k, 200) for k in range(cores)])   # warm-up: imports, builds
        times, total = [], 0
        for _ in range(args.steps):
            res = pool.map(_ref_worker, [(args.workload, k, n_ev) for k in range(cores)])
            times.append(max(r[1] for r in res))   # the loops run concurrently; their set-up is not timed
            total += sum(r[0] for r in res)
    value = total / sum(times)
    cfg.update({"n_atoms": sum(s.n for s in systems), "n_systems": len(systems),
                "events_per_step": n_ev * cores})
    line = {"impl": "reference", "metric": METRIC, "value": round(value, 3), "unit": "events/s", "n_gpus": D.world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(sum(times) * 1e3 / args.steps, 3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded random-sequence peptides, bundled Library_Ding force field)", "config": cfg,
            "cpu_baseline": {"value": round(value, 3), "unit": "events/s", "cores": cores, "kind": "port",
                             "sample": f"{n_ev} events on each of {cores} systems of the batch per step, one "
                                       "single-threaded loop per core (the reference runs one replica per process)"},
            "e2e": {"value": round(value, 3), "unit": "events/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def run_reference(args, D):
    """The reference's CPU algorithm (oracle port) on this host's cores."""
    if D.rank != 0:
        return
    from oracle import oracle as O
    O.build()
    import __graft_entry__ as G
    from sdmd_gb300 import build as B
    B.build_host()
    systems, cfg = build_workload(args.workload, 0)
    if len(systems) > 1:
        run_reference_batch(args, D, systems, cfg)
        return
    s = systems[0]
    O.predict_all(s)
    loop = O.Loop(s)
    t0 = time.perf_counter()
    loop.run(500)
    rate = 500 / max(time.perf_counter() - t0, 1e-6)
    n = int(max(1000, min(rate * args.cpu_seconds / max(args.steps, 1), 5e6)))
    for _ in range(args.warmup):
        loop.run(max(n // 10, 100))
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        loop.run(n)
        times.append(time.perf_counter() - t0)
    value = n * args.steps / sum(times)
    cfg.update({"n_atoms": s.n, "events_per_step": n})
    line = {"impl": "reference", "metric": METRIC, "value": round(value, 3), "unit": "events/s", "n_gpus": D.world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(sum(times) * 1e3 / args.steps, 3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded random-sequence peptides, bundled Library_Ding force field)", "config": cfg,
            "cpu_baseline": {"value": round(value, 3), "unit": "events/s", "cores": 1, "kind": "port",
                             "sample": f"{n} events per step of the same system after the full-rebuild sweep; the "
                                       "reference's loop is single-threaded (one system = one core)"},
            "e2e": {"value": round(value, 3), "unit": "events/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", default="c2")
    ap.add_argument("--events-per-step", type=int, default=None)
    ap.add_argument("--threads", type=int, default=0)
    ap.add_argument("--advance", choices=["eager", "lazy"], default="lazy")
    ap.add_argument("--screen", choices=["fp32", "fp64"], default="fp32")
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-drift", action="store_true")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.events_per_step is None:
        args.events_per_step = 10000 if args.workload == "c3" else 20000   # C3: one exchange per 1e4 events
    D = Dist()
    if args.impl == "reference":
        run_reference(args, D)
    else:
        run_ours(args, D)


if __name__ == "__main__":
    main()
