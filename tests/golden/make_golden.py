#!/usr/bin/env python3
"""Generate the golden fixtures under tests/golden/ from the reference itself.

Runs only where the reference's sources are (the checkout named by the
SDMD_REFERENCE environment variable, /root/reference by default): builds the
reference's unmodified C sources with the oracle recipe (oracle/ref/Makefile -> oracle/_ref/sdmd_ref_harness), runs each case, and
packs the dumps into compressed .npz fixtures that travel with the repository:

  pre/*        state after SDEnergyMin/PBC/LinkList, before the full-rebuild sweep
               (src/SGThread.c:42-52), static topology + tables included
  sweep/*      every atom's event after Predict(1..N) (src/SGThread.c:47-52)
  cbt/*        the event tree after CreateCBT (src/CBT.c:16-30)
  trace/*      per popped event: ints (target, partner, type, sub, executed, ...),
               doubles (dt, time, v_target, v_partner, new event times)
  ckpt<K>/*    state after K executed events
  final/*      state at the end of the traced run
  meta/*       event count, checkpoints, the harness summary, and the run's inputs
               (.gro text, parameter.txt, the test-local Wall.txt when there is one)

Usage: python tests/golden/make_golden.py [case ... | remd]

remd_rearrange.npz holds the exchange server's rearrange() on seeded replica
ladders, run by the reference's own Server.c.
"""
import os
import shutil
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
REF = os.environ.get("SDMD_REFERENCE", "/root/reference")   # the reference checkout
HARNESS = os.path.join(REPO, "oracle", "_ref", "sdmd_ref_harness")

PARAM_TEMPLATE = """Continue?          new
Time               {time}
T(reduced)         {temp}
Dump_Rate          {dump}
CutOff_R(A)        {cutoff}
Force_Field        Ding
Thermostat         {thermostat}
Thermo_Freq        {thermo_freq}
CGModel            no
WallExist?         {wall_exist}
WallType           {wall_type}
WallDyn            {wall_dyn}
Flow               no
Obstruct?          {obstruct}
Tunnel?            no
SphObst?           {sphobst}
"""

_DT = {"d": np.float64, "q": np.int64, "i": np.int32, "b": np.uint8}


def read_sections(path):
    """Parse the harness's section files ("SDMD" name[32] type pad[3] int64 count data)."""
    out = {}
    with open(path, "rb") as f:
        buf = f.read()
    off = 0
    while off < len(buf):
        assert buf[off:off + 4] == b"SDMD", (path, off)
        name = buf[off + 4:off + 36].split(b"\0", 1)[0].decode()
        typ = chr(buf[off + 36])
        count = int(np.frombuffer(buf, np.int64, 1, off + 40)[0])
        off += 48
        dt = np.dtype(_DT[typ])
        out[name] = np.frombuffer(buf, dt, count, off).copy()
        off += count * dt.itemsize
    return out


def build_harness():
    subprocess.check_call(["make", "-s", "-C", os.path.join(REPO, "oracle", "ref")])


def run_case(name, gro_text, params, n_events, ckpts, wall_lib=None, keep_trace_full=4000, sparse=False, args=()):
    work = tempfile.mkdtemp(prefix="sdmd_golden_")
    try:
        ind, outd, dumpd = (os.path.join(work, d) for d in ("in", "out", "dump"))
        for d in (ind, outd, dumpd):
            os.makedirs(d)
        lib = os.path.join(ind, "Library_Ding")
        if wall_lib is None:
            os.symlink(os.path.join(REF, "input", "Library_Ding"), lib)
        else:
            shutil.copytree(os.path.join(REF, "input", "Library_Ding"), lib)
            os.chmod(lib, 0o755)
            wp = os.path.join(lib, "Wall.txt")
            if os.path.exists(wp):
                os.chmod(wp, 0o644)
            with open(wp, "w") as f:
                f.write(wall_lib)
        with open(os.path.join(ind, "parameter.txt"), "w") as f:
            f.write(PARAM_TEMPLATE.format(**params))
        with open(os.path.join(ind, "sys.gro"), "w") as f:
            f.write(gro_text)
        ck = ",".join(str(c) for c in ckpts) if ckpts else "-"
        r = subprocess.run([HARNESS, dumpd, str(n_events), ck, "--", "-i", ind, "-o", outd, "-f", "sys.gro", *args],
                           capture_output=True, text=True, cwd=work)
        if r.returncode != 0:
            raise RuntimeError(f"harness failed for {name}: {r.stdout[-2000:]} {r.stderr[-2000:]}")
        summary = [l for l in r.stdout.splitlines() if l.startswith("harness:")]
        arrays = {}
        for stage, fn in [("pre", "pre.bin"), ("sweep", "sweep.bin"), ("cbt", "cbt.bin"),
                          ("final", "final.bin"), ("trace", "trace.bin")]:
            for k, v in read_sections(os.path.join(dumpd, fn)).items():
                arrays[f"{stage}/{k}"] = v
        for c in ckpts:
            p = os.path.join(dumpd, f"ckpt_{c}.bin")
            if os.path.exists(p):
                for k, v in read_sections(p).items():
                    arrays[f"ckpt{c}/{k}"] = v
        ti = arrays.pop("trace/trace_i").reshape(-1, 12)
        td = arrays.pop("trace/trace_d").reshape(-1, 10)
        if not sparse:
            # compact per-pop record for every pop, full detail for the first pops
            arrays["trace/ids"] = ti[:, :5].copy()          # target partner type sub executed
            arrays["trace/dt"] = td[:, 0].copy()
            arrays["trace/full_i"] = ti[:keep_trace_full].copy()
            arrays["trace/full_d"] = td[:keep_trace_full].copy()
        else:
            # long runs: only the executed HB / HB-neighbour pops (with their pop index)
            sel = np.nonzero((ti[:, 4] == 1) & ((ti[:, 2] == 2) | (ti[:, 2] == 3)))[0]
            arrays["trace/sparse_pop"] = sel.astype(np.int64)
            arrays["trace/sparse_i"] = ti[sel].copy()
            arrays["trace/sparse_d"] = td[sel].copy()
        arrays["trace/n_pops"] = np.array([len(ti)], np.int64)
        arrays["meta/n_events"] = np.array([n_events], np.int64)
        arrays["meta/ckpts"] = np.array(ckpts, np.int64)
        arrays["meta/summary"] = np.frombuffer(("\n".join(summary)).encode(), np.uint8)
        arrays["meta/rng_pre"] = rng_state_after(int(arrays["pre/seed"][0]), int(arrays["pre/rand_calls"][0]))
        # the run's own inputs, so that the host-side builder can be checked against pre/*
        arrays["meta/gro"] = np.frombuffer(gro_text.encode(), np.uint8)
        arrays["meta/parameter"] = np.frombuffer(PARAM_TEMPLATE.format(**params).encode(), np.uint8)
        if wall_lib is not None:
            arrays["meta/wall_lib"] = np.frombuffer(wall_lib.encode(), np.uint8)
        if args:
            arrays["meta/args"] = np.frombuffer(" ".join(args).encode(), np.uint8)
        out = os.path.join(HERE, f"{name}.npz")
        np.savez_compressed(out, **arrays)
        print(f"{name}: {summary[0] if summary else ''} -> {os.path.getsize(out) / 1024:.0f} KiB")
    finally:
        shutil.rmtree(work, ignore_errors=True)


def rng_state_after(seed, calls):
    """glibc TYPE_3 rand() state after srand(seed) and `calls` draws:
    [tab[0..30], front, rear] as int32 (layout of sdmd_rng)."""
    r = [0] * 31
    r[0] = seed if seed != 0 else 1
    for i in range(1, 31):
        hi, lo = divmod(r[i - 1], 127773)
        w = 16807 * lo - 2836 * hi
        if w < 0:
            w += 2147483647
        r[i] = w
    f, b = 3, 0
    for _ in range(310 + calls):
        r[f] = (r[f] + r[b]) & 0xFFFFFFFF
        f += 1
        b += 1
        if f >= 31:
            f = 0
        elif b >= 31:
            b = 0
    tab = np.array(r, np.uint32).view(np.int32)
    return np.concatenate([tab, np.array([f, b], np.int32)])


def base_params(**kw):
    p = dict(time=5000, temp=0.6, dump=1e9, cutoff=9.0, thermostat="Andersen", thermo_freq=6.0,
             wall_exist="no", wall_type="no", sphobst="no", obstruct="no", wall_dyn="no")
    p.update(kw)
    return p


def cases():
    with open(os.path.join(REF, "input", "ala10.gro")) as f:
        ala10 = f.read()
    out = {
        # the reference's shipped ala10 input (150 A box), Andersen NVT at T*=0.6
        "ala10_nvt": dict(gro_text=ala10, params=base_params(), n_events=10000, ckpts=[1000, 5000]),
        # same, NVE: the strict bit-exact case (no RNG in the loop)
        "ala10_nve": dict(gro_text=ala10, params=base_params(thermostat="no"), n_events=10000, ckpts=[1000, 5000]),
        # long NVT run: HB formation/breaking and HB-neighbour events start near 1e5 events
        "ala10_nvt_long": dict(gro_text=ala10, params=base_params(), n_events=150000,
                               ckpts=[50000, 104000, 110000, 125000], sparse=True),
    }
    extra = os.path.join(HERE, "inputs")
    if os.path.isdir(extra):
        for fn in sorted(os.listdir(extra)):
            if fn.endswith(".case.py"):
                spec = {}
                with open(os.path.join(extra, fn)) as f:
                    exec(f.read(), {"base_params": base_params, "extra": extra, "REF": REF}, spec)
                out[fn[:-len(".case.py")]] = spec["CASE"]
    return out


def bundle_force_field():
    """Copy the reference's force-field input tables (Library_Ding, MIT licence,
    input/Library_Ding/ of alexzheng42/sDMD) into the package's data directory:
    the workload generator, the tests and the benchmark build systems from them on
    machines without the reference."""
    src = os.path.join(REF, "input", "Library_Ding")
    dst = os.path.join(REPO, "sdmd_gb300", "data", "Library_Ding")
    if os.path.isdir(dst):
        shutil.rmtree(dst)
    shutil.copytree(src, dst)
    for root, dirs, files in os.walk(dst):
        for f in files:
            os.chmod(os.path.join(root, f), 0o644)
    with open(os.path.join(dst, "PROVENANCE.txt"), "w") as f:
        f.write("Force-field input tables of sDMD (alexzheng42/sDMD, input/Library_Ding), MIT licence,\n"
                "Copyright (c) 2018 Size Zheng.  Copied unchanged by tests/golden/make_golden.py as input data.\n")


SERVER = os.path.join(REPO, "oracle", "_ref", "sdmd_ref_server_rearrange")


def remd_golden():
    """The exchange server's rearrange() (src/Server.c:145-192) run by the reference
    itself (oracle/ref/server_driver.c) on seeded replica ladders: per case, the
    srand seed, the starting (num, T) records, every round's energies, and every
    round's resulting (num, T).  Energies are drawn around a common mean with a
    spread comparable to the temperature gaps, so swaps are both accepted and
    rejected."""
    rng = np.random.default_rng(20201)
    arrays = {}
    for case, (n, rounds, seed) in enumerate([(8, 60, 1), (16, 60, 7), (64, 40, 20201), (3, 80, 99)]):
        T0 = 270.0 * (500.0 / 270.0) ** (np.arange(n) / max(n - 1, 1)) * 0.0019872041
        num0 = np.arange(1, n + 1, dtype=np.int32)
        E = -150.0 + rng.normal(0.0, 2.0, (rounds, n))
        lines = [f"{seed} {n} {rounds}"]
        for r in range(rounds):
            for i in range(n):
                lines.append(f"{num0[i]} {float(T0[i])!r} {float(E[r, i])!r}")
        res = subprocess.run([SERVER], input="\n".join(lines) + "\n", capture_output=True, text=True, check=True)
        out = [l.split() for l in res.stdout.splitlines()]
        assert len(out) == rounds * n
        arrays[f"c{case}/seed"] = np.array([seed], np.int64)
        arrays[f"c{case}/T0"] = T0
        arrays[f"c{case}/num0"] = num0
        arrays[f"c{case}/E"] = E
        arrays[f"c{case}/num"] = np.array([int(o[0]) for o in out], np.int32).reshape(rounds, n)
        arrays[f"c{case}/T"] = np.array([float.fromhex(o[1]) for o in out]).reshape(rounds, n)
    arrays["meta/cases"] = np.array([4], np.int64)
    out = os.path.join(HERE, "remd_rearrange.npz")
    np.savez_compressed(out, **arrays)
    print(f"remd_rearrange: 4 cases -> {os.path.getsize(out) / 1024:.0f} KiB")


def main(argv):
    if not os.path.isdir(REF):
        sys.exit("the reference sources are not present; golden fixtures can only be regenerated where they are")
    bundle_force_field()
    if argv == ["--force-field-only"]:
        return
    build_harness()
    if argv == ["remd"]:
        remd_golden()
        return
    all_cases = cases()
    names = argv or list(all_cases)
    for n in names:
        run_case(n, **all_cases[n])
    if not argv:
        remd_golden()


if __name__ == "__main__":
    main(sys.argv[1:])
