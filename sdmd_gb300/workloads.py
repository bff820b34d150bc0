"""The benchmark configurations, built from seeded synthetic inputs.

Every system goes through the same path a user's input does: .gro text (here
generated: random-sequence peptides, relaxed and placed without overlap) plus
parameter.txt, read by the host-side C builder with the reference's semantics
and the force-field tables of Library_Ding.  No public dataset is involved.

  C1  one ALA x 10 chain (59 atoms), extended start, 40 A cube, Andersen NVT at
      300 K (T* = 300 * 0.0019872041 = 0.5962), Thermo_Freq 6, cutoff 9 A
  C2  256 chains x 16 residues, residues uniform over the 20 amino acids,
      random rigid placement at 5 mM: cube edge (256 / (0.005 N_A))^(1/3) = 440 A
  C3  64 replicas of C1, temperatures geometric 270-500 K
  C4  512 single chains of 5-60 residues, box edge scaled to C1's density,
      temperatures 280-400 K

  C5  8 replicas of 400 random-sequence 10-mers (about 42k atoms) in a smooth
      cylindrical wall of radius 60 A (axis x, 120 A periodic), Andersen NVT
      310 K.  Overlap-free insertion stalls far below this density (0.031 atoms
      per A^3), so the chains are placed in a longer cylinder and compressed to
      the target length as rigid bodies (the host generator's compressive
      packing); the replicas share that start and differ in their thermostat
      random streams.
"""
import json
import os
import tempfile

import numpy as np

from .host import AMINO_ACIDS, build_system, generate_gro, params_text
from .system import glibc_rng_state

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
DATA = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data")   # holds Library_Ding (force-field tables)
BOLTZMANN = 0.0019872041                               # kcal/mol/K (src/REMDExec.c:19)


CACHE = os.environ.get("SDMD_WORKLOAD_CACHE", os.path.join(tempfile.gettempdir(), "sdmd_workloads"))


def cached(key, make):
    """Build a System once per machine session (keyed by the workload parameters
    and the host library's build time) and reload it from an .npz afterwards."""
    from .host import HOST_LIB
    from .system import System
    os.makedirs(CACHE, exist_ok=True)
    stamp = int(os.path.getmtime(HOST_LIB)) if os.path.exists(HOST_LIB) else 0
    path = os.path.join(CACHE, f"{key}_{stamp}.npz")
    if os.path.exists(path):
        d = np.load(path, allow_pickle=False)
        s = System()
        for k in d.files:
            if k.startswith("a/"):
                s.a[k[2:]] = d[k].copy()
        s.scal = json.loads(str(d["scal"]))
        s.counters = json.loads(str(d["counters"]))
        s.rng = d["rng"].copy()
        s.time = float(d["time"])
        return s
    s = make()
    tmp = path + f".{os.getpid()}.tmp.npz"
    np.savez(tmp, scal=json.dumps(s.scal), counters=json.dumps(s.counters), rng=s.rng, time=s.time,
             **{f"a/{k}": v for k, v in s.a.items()})
    os.replace(tmp, path)
    return s


def _datadir(param_kw, wall_atom=None):
    """A run directory: parameter.txt and the force-field library.  With
    `wall_atom`, the library's Wall.txt names that atom type instead: the shipped
    one names PHO, which the reference's atom model table lacks (src/Models.c
    129-206), so ReadWall would stop."""
    d = tempfile.mkdtemp(prefix="sdmd_wl_")
    lib = os.path.join(DATA, "Library_Ding")
    if wall_atom is None:
        os.symlink(lib, os.path.join(d, "Library_Ding"))
    else:
        os.makedirs(os.path.join(d, "Library_Ding"))
        for e in os.listdir(lib):
            if e != "Wall.txt":
                os.symlink(os.path.join(lib, e), os.path.join(d, "Library_Ding", e))
        with open(os.path.join(d, "Library_Ding", "Wall.txt"), "w") as f:
            f.write(f"Wall\n   ATOM {wall_atom:<7s} {wall_atom:<4s} 12.0  N N\n")
    with open(os.path.join(d, "parameter.txt"), "w") as f:
        f.write(params_text(**param_kw))
    return d


def random_sequences(n, length, seed, lo=None, hi=None):
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        L = length if lo is None else int(rng.integers(lo, hi + 1))
        out.append([AMINO_ACIDS[k] for k in rng.integers(0, 20, L)])
    return out


def c1(seed=1, temperature_k=300.0, thermostat="Andersen", box=40.0, rng_seed=1575263273):
    def make():
        d = _datadir(dict(temp=round(temperature_k * BOLTZMANN, 4), thermostat=thermostat, time=1e9))
        gro = generate_gro(d, [["ALA"] * 10], (box, box, box), seed=seed)
        return build_system(d, gro_text=gro, seed=rng_seed)

    return cached(f"c1_{seed}_{temperature_k}_{thermostat}_{box}_{rng_seed}", make)


def c2(n_chains=256, length=16, seed=1, temperature_k=300.0, thermostat="Andersen", conc_mM=5.0,
       rng_seed=1575263273):
    edge = (n_chains / (conc_mM * 1e-3 * 6.02214076e23) * 1e27) ** (1.0 / 3.0)   # A

    def make():
        d = _datadir(dict(temp=round(temperature_k * BOLTZMANN, 4), thermostat=thermostat, time=1e9))
        gro = generate_gro(d, random_sequences(n_chains, length, seed), (edge, edge, edge), seed=seed)
        return build_system(d, gro_text=gro, seed=rng_seed)

    return cached(f"c2_{n_chains}_{length}_{seed}_{temperature_k}_{thermostat}_{conc_mM}_{rng_seed}", make)


def c3(n_replicas=64, t_lo=270.0, t_hi=500.0, seed=1):
    base = c1(seed=seed)
    out = []
    for k in range(n_replicas):
        s = base.copy()
        t = t_lo * (t_hi / t_lo) ** (k / max(n_replicas - 1, 1))
        s.scal["temperature"] = t * BOLTZMANN
        s.rng = glibc_rng_state(1000 + k)
        out.append(s)
    return out


def _c4_specs(n_systems, lo, hi, seed, t_lo, t_hi, rng_seed0):
    rng = np.random.default_rng(seed)
    seqs = random_sequences(n_systems, 0, seed, lo, hi)
    temps = rng.uniform(t_lo, t_hi, n_systems)
    out = []
    for k, seq in enumerate(seqs):
        T = float(temps[k])
        natoms_est = 10.45 * len(seq)
        edge = max(27.0, 40.0 * (natoms_est / 59.0) ** (1.0 / 3.0))
        out.append((k, seq, T, edge, seed * 100003 + k, rng_seed0 + k, f"c4_{k}_{len(seq)}_{seed}_{round(T, 3)}"))
    return out


def _c4_one(spec):
    k, seq, T, edge, gro_seed, rng_seed, key = spec

    def make():
        d = _datadir(dict(temp=round(T * BOLTZMANN, 4), thermostat="Andersen", time=1e9))
        gro = generate_gro(d, [seq], (edge, edge, edge), seed=gro_seed)
        return build_system(d, gro_text=gro, seed=rng_seed)

    return cached(key, make)


def c4(n_systems=512, lo=5, hi=60, seed=1, t_lo=280.0, t_hi=400.0, rng_seed0=5000, workers=None):
    """512 single chains, lengths uniform lo..hi residues with random sequences, box
    edge 40 A * (N / 59)^(1/3) (C1's atom density) floored at 27 A (three 9 A
    cells), temperatures uniform t_lo..t_hi.  Each system is built (and cached)
    separately, the missing ones in parallel on all host cores (spawned worker
    processes); returns the list of Systems."""
    specs = _c4_specs(n_systems, lo, hi, seed, t_lo, t_hi, rng_seed0)
    from .host import HOST_LIB
    stamp = int(os.path.getmtime(HOST_LIB)) if os.path.exists(HOST_LIB) else 0
    missing = [sp for sp in specs if not os.path.exists(os.path.join(CACHE, f"{sp[-1]}_{stamp}.npz"))]
    if len(missing) > 1:
        import multiprocessing as mp
        n = workers or min(len(missing), os.cpu_count() or 1)
        with mp.get_context("spawn").Pool(n) as pool:
            for _ in pool.imap_unordered(_c4_touch, missing):
                pass
    return [_c4_one(sp) for sp in specs]


def c5(n_replicas=8, n_chains=400, length=10, seed=1, temperature_k=310.0, radius=60.0, axis=120.0,
       margin=4.0, rng_seed=1575263273):
    """n_replicas copies of one packing of n_chains random-sequence chains inside a
    smooth cylindrical wall (radius `radius`, periodic axis x of length `axis`),
    atoms at least `margin` from the wall; replica k's thermostat stream is
    glibc srand(2000 + k).  The wall atom is a CA (the cylinder-wall golden case's
    choice)."""
    def make():
        d = _datadir(dict(temp=round(temperature_k * BOLTZMANN, 4), thermostat="Andersen", time=1e9,
                          wall_exist="smooth", wall_type="cylinder"), wall_atom="CA")
        gro = generate_gro(d, random_sequences(n_chains, length, seed), (axis, 2 * radius, 2 * radius), wall=2,
                           margin=margin, seed=seed)
        return build_system(d, gro_text=gro, seed=rng_seed)

    base = cached(f"c5_{n_chains}_{length}_{seed}_{temperature_k}_{radius}_{axis}_{margin}_{rng_seed}", make)
    out = []
    for k in range(n_replicas):
        s = base.copy()
        s.rng = glibc_rng_state(2000 + k)
        out.append(s)
    return out


def _c4_touch(spec):
    _c4_one(spec)
    return spec[0]

