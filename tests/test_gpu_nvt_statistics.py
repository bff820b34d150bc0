"""NVT temperature and potential-energy means of the benchmarked path against the
reference's algorithm (GPU; CPU oracle side on a spawned process pool).

ALA x 10 in a 40 A cube under Andersen NVT at 300 K (T* = 0.5962).  Replicas
differ only in their rand() stream.  The GPU runs its replicas in one batched
launch of the benchmarked path (FP32 screen, eager advance); the oracle -- the
C restatement of the reference's loop -- runs its own replicas on host cores.
Every `chunk` executed events each replica records T = 2 KE / (3 N) (CalSysTem,
src/ToolFunctions.c:755-757) and the potential energy (CalPotenE, :659-752).
After the equilibration chunks, each replica's time average is one sample; the
means over replicas must agree within 4 combined standard errors, and the
replica that shares its seed with an oracle replica must give the oracle's
series exactly.

Run as a script for a long measurement, e.g.
  python tests/test_gpu_nvt_statistics.py --events 10000000 --replicas 8
which prints the two sides' means and errors as JSON.
"""
import argparse
import json
import os
import sys
import time

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if REPO not in sys.path:
    sys.path.insert(0, REPO)


def _replicas(seeds):
    from sdmd_gb300 import workloads as W
    from sdmd_gb300.system import glibc_rng_state
    base = W.c1()
    out = []
    for sd in seeds:
        s = base.copy()
        s.rng = glibc_rng_state(sd)
        out.append(s)
    return out


def gpu_series(seeds, n_chunks, chunk):
    from sdmd_gb300.engine import ADVANCE_EAGER, SCREEN_FP32, Engine
    systems = _replicas(seeds)
    n = systems[0].n
    T, U = np.zeros((len(seeds), n_chunks)), np.zeros((len(seeds), n_chunks))
    with Engine(systems, advance=ADVANCE_EAGER, screen=SCREEN_FP32, threads=64) as e:
        e.prepare(full=True)
        for k in range(n_chunks):
            e.run(chunk)
            pot, kin = e.energies()
            T[:, k] = 2 * kin / (3 * n)
            U[:, k] = pot
    return T, U


def _cpu_one(args):
    seed, n_chunks, chunk = args
    sys.path.insert(0, REPO)
    from oracle import oracle as O
    s = _replicas([seed])[0]
    O.predict_all(s)
    loop = O.Loop(s)
    T, U = np.zeros(n_chunks), np.zeros(n_chunks)
    for k in range(n_chunks):
        rc, _, _ = loop.run(chunk)
        assert rc == 0
        T[k] = 2 * O.kinetic_energy(s) / (3 * s.n)
        U[k] = O.potential_energy(s)
    return T, U


def cpu_series(seeds, n_chunks, chunk, pool):
    res = pool.map(_cpu_one, [(sd, n_chunks, chunk) for sd in seeds])
    return np.stack([r[0] for r in res]), np.stack([r[1] for r in res])


def summary(x, equil):
    m = x[:, equil:].mean(1)                  # one time average per replica
    return float(m.mean()), float(m.std(ddof=1) / np.sqrt(len(m)))


def compare(n_events, replicas, chunk=1000, equil_frac=0.2):
    import multiprocessing as mp
    n_chunks = max(int(n_events // chunk), 10)
    equil = int(n_chunks * equil_frac)
    gpu_seeds = [7000 + k for k in range(replicas)]
    cpu_seeds = [7000] + [9000 + k for k in range(replicas - 1)]   # one shared seed, the rest independent
    with mp.get_context("spawn").Pool(min(replicas, os.cpu_count() or 1)) as pool:
        t0 = time.time()
        Tc, Uc = cpu_series(cpu_seeds, n_chunks, chunk, pool)
        cpu_s = time.time() - t0
    t0 = time.time()
    Tg, Ug = gpu_series(gpu_seeds, n_chunks, chunk)
    gpu_s = time.time() - t0
    out = {"events_per_replica": n_chunks * chunk, "replicas": replicas, "chunk": chunk,
           "equilibration_chunks": equil, "gpu_s": round(gpu_s, 1), "cpu_s": round(cpu_s, 1)}
    for name, g, c in (("T", Tg, Tc), ("PE", Ug, Uc)):
        mg, eg = summary(g, equil)
        mc, ec = summary(c, equil)
        out[name] = {"gpu": [mg, eg], "oracle": [mc, ec], "z": abs(mg - mc) / np.hypot(eg, ec)}
    out["shared_seed_identical"] = bool(np.array_equal(Tg[0], Tc[0]) and np.array_equal(Ug[0], Uc[0]))
    return out


@pytest.mark.gpu
def test_nvt_means_agree_with_the_reference_algorithm():
    import __graft_entry__ as G
    G.build()
    r = compare(n_events=60000, replicas=16)
    assert r["shared_seed_identical"], r
    for q in ("T", "PE"):
        assert r[q]["z"] < 4.0, r
    # the thermostat holds the target temperature (T* = 0.5962) within the errors
    mg, eg = r["T"]["gpu"]
    assert abs(mg - 0.5962) < 4 * eg + 0.01, r


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--events", type=float, default=1e6)
    ap.add_argument("--replicas", type=int, default=8)
    ap.add_argument("--chunk", type=int, default=1000)
    a = ap.parse_args()
    import __graft_entry__ as G
    G.build()
    print(json.dumps(compare(int(a.events), a.replicas, a.chunk)))
