"""The reference's checkpoint file, savedData.dat, through the host library
(no GPU).  Runs where the reference's sources are: the reference itself writes
and reads the files (its SaveDAT / ReadBreakPoint, through
oracle/_ref/libsdmd_ref_bridge.so in child processes).

  read      a checkpoint the reference wrote after K events, applied onto a
            system built from the same inputs, holds the reference's state at K
            (rand() restarted from the saved seed, as ReadBreakPoint does);
  bytes     writing that state back with the file as template reproduces the
            file byte for byte;
  continue  the oracle continues M events from it, the host library writes the
            checkpoint, the reference reads it in a continue run: its state is
            the oracle's, and N more events of the reference's own loop equal N
            more oracle events.
"""
import ctypes as C
import os

import numpy as np
import pytest

from tests.test_ref_bridge import DYN, LIB, _fill, case_dir, in_child

pytestmark = pytest.mark.skipif(not os.path.exists(LIB),
                                reason="the reference's sources are not here (oracle/_ref not built)")
COUNTERS = ["frame", "collision", "bond", "hb", "hbneighbor", "thermostat", "pcc", "wall", "hb_formed",
            "alpha_hb_formed"]


def _driver(ind, outd):
    from sdmd_gb300.system import sdmd_system
    L = C.CDLL(LIB)
    L.sdmd_bridge_fill.argtypes = [C.POINTER(sdmd_system), C.POINTER(C.c_void_p)]
    L.bd_init.argtypes = [C.c_int, C.POINTER(C.c_char_p)]
    L.bd_run.argtypes = [C.c_long]
    L.bd_run.restype = C.c_long
    argv = [b"sDMD", b"-i", ind.encode(), b"-o", outd.encode(), b"-f", b"sys.gro"]
    assert L.bd_init(len(argv), (C.c_char_p * len(argv))(*argv)) == 0
    return L


def _child_new_run_and_save(ind, outd, k_events, q):
    try:
        L = _driver(ind, outd)
        L.bd_sweep()
        L.bd_run(k_events)
        L.bd_save()
        s = _fill(L)
        q.put(("ok", s.a, s.counters, s.time))
    except Exception as e:
        q.put(("error", repr(e)))


def _child_continue(ind, outd, n_events, q):
    try:
        L = _driver(ind, outd)          # parameter.txt says "continue": ReadBreakPoint
        L.bd_tree()
        s0 = _fill(L)
        L.bd_run(n_events)
        s1 = _fill(L)
        q.put(("ok", s0.a, s0.rng, s0.counters, s0.time, s1.a, s1.counters, s1.time))
    except Exception as e:
        q.put(("error", repr(e)))


def host_lib():
    from sdmd_gb300 import host as H
    from sdmd_gb300.system import sdmd_system
    L = H.lib()
    L.sdmd_saved_read.argtypes = [C.c_char_p, C.POINTER(C.c_void_p), C.c_char_p, C.c_int]
    L.sdmd_saved_apply.argtypes = [C.c_void_p, C.POINTER(sdmd_system), C.c_char_p, C.c_char_p, C.c_int]
    L.sdmd_saved_write.argtypes = [C.c_char_p, C.c_void_p, C.POINTER(sdmd_system), C.c_char_p, C.c_int]
    L.sdmd_saved_free.argtypes = [C.c_void_p]
    return L


def read_saved(path):
    L = host_lib()
    h = C.c_void_p()
    err = C.create_string_buffer(512)
    assert L.sdmd_saved_read(str(path).encode(), C.byref(h), err, 512) == 0, err.value
    return h


def apply_saved(h, system):
    L = host_lib()
    st = system.struct()
    err = C.create_string_buffer(512)
    assert L.sdmd_saved_apply(h, C.byref(st), system.names, err, 512) == 0, err.value
    system.pull_scalars(st)


def write_saved(path, tpl, system):
    L = host_lib()
    err = C.create_string_buffer(512)
    assert L.sdmd_saved_write(str(path).encode(), tpl, C.byref(system.struct()), err, 512) == 0, err.value


@pytest.mark.parametrize("case,k,m,n", [("ala10_nvt", 2000, 1500, 1500), ("sheet2", 20000, 15000, 15000)])
def test_checkpoint_read_write_continue(case, k, m, n):
    from oracle import oracle as O
    from sdmd_gb300.host import build_system
    from sdmd_gb300.system import glibc_rng_state
    work, ind, outd = case_dir(case)
    d = np.load(os.path.join(os.path.dirname(__file__), "golden", f"{case}.npz"))
    # a continue run needs Time > currenttime + Dump_Rate (src/Initialization.c:494-505)
    par = os.path.join(ind, "parameter.txt")
    lines = open(par).read().splitlines()
    lines = [("Dump_Rate          1.0" if l.startswith("Dump_Rate") else l) for l in lines]
    lines = [("Time               100000" if l.startswith("Time") else l) for l in lines]
    open(par, "w").write("\n".join(lines) + "\n")
    a_ref, c_ref, t_ref = in_child(_child_new_run_and_save, ind, outd, k)
    f1 = os.path.join(outd, "savedData.dat")
    seed = int(d["pre/seed"][0])

    # read: the continue state of a system built from the same inputs
    h = read_saved(f1)
    s = build_system(ind, gro_text=bytes(d["meta/gro"]).decode(), seed=seed)
    apply_saved(h, s)
    for key in DYN:
        assert np.array_equal(s.a[key], a_ref[key]), key
    assert s.time == t_ref and all(s.counters[c] == c_ref[c] for c in COUNTERS)
    assert np.array_equal(s.rng, glibc_rng_state(seed))

    # bytes: the same state written with the file as template is the file
    f1b = os.path.join(work, "rewritten.dat")
    write_saved(f1b, h, s)
    assert open(f1b, "rb").read() == open(f1, "rb").read()

    # continue: the oracle runs M events from the checkpoint (continue mode keeps the
    # stored events), the host library writes it, the reference reads it back
    loop = O.Loop(s)
    assert loop.run(m)[0] == 0
    write_saved(f1, h, s)
    with open(par, "rb") as f:
        txt = f.read()
    with open(par, "wb") as f:
        f.write(txt.replace(b"new", b"continue", 1))
    a0, rng0, c0, t0, a1, c1, t1 = in_child(_child_continue, ind, outd, n)
    for key in DYN:
        assert np.array_equal(a0[key], s.a[key]), key
    assert t0 == s.time and all(c0[c] == s.counters[c] for c in COUNTERS)
    assert np.array_equal(rng0, glibc_rng_state(seed))   # ReadBreakPoint's srand(seed)
    # ... and the reference's own loop from there equals the oracle's from the same read
    # (the static model is built from the inputs of the new run)
    with open(par, "wb") as f:
        f.write(txt)
    h2 = read_saved(f1)
    s2 = build_system(ind, gro_text=bytes(d["meta/gro"]).decode(), seed=seed)
    apply_saved(h2, s2)
    assert O.Loop(s2).run(n)[0] == 0
    for key in DYN:
        assert np.array_equal(a1[key], s2.a[key]), key
    assert t1 == s2.time and all(c1[c] == s2.counters[c] for c in COUNTERS)
    for hh in (h, h2):
        host_lib().sdmd_saved_free(hh)


def differing_defined_bytes(mine, ref):
    """Offsets where two savedData.dat images differ, leaving out the bytes the
    reference's SaveDAT writes without defining them: the atom records' pointer
    fields (PropertyStr.bond / .constr: its heap addresses), residue and peptide
    record 0 (malloc'd), the residue records' bytes past the name, and velocity[0]
    of atoms that had a thermostat event (ThermostatEvent copies an uninitialised
    speed[0], src/Events.c:397-418)."""
    if len(mine) != len(ref):
        return np.array([min(len(mine), len(ref))])
    n_atoms, n_prot, n_aa = np.frombuffer(ref[:12], np.int32)
    aa0 = 12 + 4 * (n_atoms + 1) ** 2 + 48 + 20 + 32
    at = aa0 + 32 * (n_aa + 1) + 24 * (n_prot + 1)
    mask = np.ones(len(ref), bool)
    mask[aa0: aa0 + 32] = False
    mask[aa0 + 32 * (n_aa + 1): aa0 + 32 * (n_aa + 1) + 24] = False
    for k in range(n_aa + 1):
        mask[aa0 + 32 * k + 4: aa0 + 32 * k + 8] = False
    for i in range(n_atoms + 1):
        mask[at + 312 * i + 120: at + 312 * i + 136] = False
        mask[at + 312 * i + 136 + 48: at + 312 * i + 136 + 56] = False
    a, b = np.frombuffer(mine, np.uint8), np.frombuffer(ref, np.uint8)
    return np.nonzero((a != b) & mask)[0]


@pytest.mark.parametrize("case,k", [("ala10_nvt", 2000), ("sheet2", 20000), ("ala10_cyl", 3000)])
def test_new_run_template_writes_the_reference_file(case, k):
    """A new run's checkpoint without a file to start from: sdmd_saved_new builds
    the template from the system the host library built (same inputs and seed),
    and writing the reference's state after K events with it gives the file the
    reference's own SaveDAT wrote, byte for byte but for what the reference leaves
    undefined: the atom records' two pointer fields (its heap addresses), residue
    and peptide record 0, the residue records' bytes past the name and the unused
    velocity[0] after a thermostat event."""
    from sdmd_gb300.host import build_system
    from sdmd_gb300.system import System, sdmd_system
    work, ind, outd = case_dir(case)
    d = np.load(os.path.join(os.path.dirname(__file__), "golden", f"{case}.npz"))
    a_ref, c_ref, t_ref = in_child(_child_new_run_and_save, ind, outd, k)
    ref = open(os.path.join(outd, "savedData.dat"), "rb").read()
    seed = int(d["pre/seed"][0])
    built = build_system(ind, gro_text=bytes(d["meta/gro"]).decode(), seed=seed)
    # the template comes from the host library's own handle of the same build
    from sdmd_gb300 import host as H
    L = host_lib()
    L.sdmd_saved_new.argtypes = [C.c_void_p, C.c_void_p, C.c_uint32, C.POINTER(C.c_void_p), C.c_char_p, C.c_int]
    params = H.read_parameters(os.path.join(ind, "parameter.txt"))
    hs = C.c_void_p()
    err = C.create_string_buffer(512)
    assert H.lib().sdmd_build_system_gro_text(ind.encode(), bytes(d["meta/gro"]), C.byref(params), seed, 20000,
                                               C.byref(hs), err, 512) == 0, err.value
    tpl = C.c_void_p()
    assert L.sdmd_saved_new(hs, C.byref(params), seed, C.byref(tpl), err, 512) == 0, err.value
    s = System()
    s.a, s.scal, s.counters, s.time = dict(built.a), dict(built.scal), dict(c_ref), t_ref
    for key in DYN:
        s.a[key] = a_ref[key]
    s.rng = built.rng.copy()
    path = os.path.join(work, "new_template.dat")
    write_saved(path, tpl, s)
    mine = open(path, "rb").read()
    bad = differing_defined_bytes(mine, ref)
    assert len(bad) == 0, f"{len(bad)} bytes differ, first at offset {bad[0]}"
    L.sdmd_saved_free(tpl)
    H.lib().sdmd_host_free(hs)
