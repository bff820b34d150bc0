"""The bridge compiled into the reference (sdmd_gb300/bridge/sdmd_ref_bridge.c)
against the reference's own code (no GPU).

oracle/ref/Makefile links the bridge with the reference's unmodified sources
and a driver (oracle/ref/bridge_driver.c) into oracle/_ref/libsdmd_ref_bridge.so,
where the reference's sources are.  Each scenario runs in a child process: the
reference keeps its state in globals.

  fill      after the reference's own InputData + Prepare() set-up, the filled
            sdmd_system equals the host builder's, field for field;
  hand-off  the filled state runs K events in the oracle (the GPU's checker),
            is written back, and the reference's own loop continues for M events
            from it (continue mode: the tree is rebuilt): the result equals K + M
            events of one uninterrupted oracle run -- positions, velocities,
            events, cells, HB state (the reference itself checks its HB map bits
            at every HB event), counters and rand() state.
"""
import ctypes as C
import multiprocessing as mp
import os
import shutil
import tempfile

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB = os.path.join(REPO, "oracle", "_ref", "libsdmd_ref_bridge.so")
pytestmark = pytest.mark.skipif(not os.path.exists(LIB),
                                reason="the reference's sources are not here (oracle/_ref not built)")
POOLED = {"con_step_off", "pair_step_off", "con_step_d", "con_step_e", "con_step_acc", "pair_step_d", "pair_step_e",
          "pair_step_acc"}
DYN = ["x", "y", "z", "vx", "vy", "vz", "cx", "cy", "cz", "type", "hb_bond", "hb_itype", "nb_partner", "nb_status",
       "nb_pnum", "ev_time", "ev_partner", "ev_counter", "ev_pcounter", "ev_potential", "ev_type", "ev_sub",
       "cell_list"]


def case_dir(case):
    d = np.load(os.path.join(REPO, "tests", "golden", f"{case}.npz"))
    work = tempfile.mkdtemp(prefix="sdmd_bridge_")
    ind, outd = os.path.join(work, "in"), os.path.join(work, "out")
    os.makedirs(outd)
    os.makedirs(ind)
    lib = os.path.join(ind, "Library_Ding")
    shutil.copytree(os.path.join(REPO, "sdmd_gb300", "data", "Library_Ding"), lib)
    if "meta/wall_lib" in d.files:
        with open(os.path.join(lib, "Wall.txt"), "wb") as f:
            f.write(bytes(d["meta/wall_lib"]))
    with open(os.path.join(ind, "parameter.txt"), "wb") as f:
        f.write(bytes(d["meta/parameter"]))
    with open(os.path.join(ind, "sys.gro"), "wb") as f:
        f.write(bytes(d["meta/gro"]))
    return work, ind, outd


def _bridge(ind, outd):
    from sdmd_gb300.system import sdmd_system
    L = C.CDLL(LIB)
    L.sdmd_bridge_fill.argtypes = [C.POINTER(sdmd_system), C.POINTER(C.c_void_p)]
    L.sdmd_bridge_readback.argtypes = [C.POINTER(sdmd_system)]
    L.bd_init.argtypes = [C.c_int, C.POINTER(C.c_char_p)]
    L.bd_run.argtypes = [C.c_long]
    L.bd_run.restype = C.c_long
    argv = [b"sDMD", b"-i", ind.encode(), b"-o", outd.encode(), b"-f", b"sys.gro"]
    assert L.bd_init(len(argv), (C.c_char_p * len(argv))(*argv)) == 0
    return L


def _fill(L):
    from sdmd_gb300.host import system_from_struct
    from sdmd_gb300.system import sdmd_system
    st = sdmd_system()
    owner = C.c_void_p()
    assert L.sdmd_bridge_fill(C.byref(st), C.byref(owner)) == 0
    return system_from_struct(C.pointer(st))


def _child_fill(case, q):
    try:
        work, ind, outd = case_dir(case)
        s = _fill(_bridge(ind, outd))
        q.put(("ok", s.a, s.scal, s.rng, s.counters, s.time))
    except Exception as e:   # reported to the parent
        q.put(("error", repr(e)))


def _child_handoff(case, k_events, m_events, q):
    try:
        from oracle import oracle as O
        work, ind, outd = case_dir(case)
        L = _bridge(ind, outd)
        s0 = _fill(L)
        straight = s0.copy()
        O.predict_all(straight)
        assert O.Loop(straight).run(k_events + m_events)[0] == 0
        mid = s0.copy()
        O.predict_all(mid)
        assert O.Loop(mid).run(k_events)[0] == 0
        assert L.sdmd_bridge_readback(C.byref(mid.struct())) == 0
        L.bd_tree()                                   # continue mode: the reference rebuilds its tree
        L.bd_run(m_events)                            # ... and runs its own loop
        s1 = _fill(L)
        q.put(("ok", s1.a, straight.a, s1.rng, straight.rng, s1.counters, straight.counters, s1.time, straight.time))
    except Exception as e:
        q.put(("error", repr(e)))


def _run_child(target, args):
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    p = ctx.Process(target=target, args=(*args, q))
    p.start()
    import queue
    out = None
    for _ in range(600):   # the reference exits the process on its own errors: notice that
        try:
            out = q.get(timeout=1)
            break
        except queue.Empty:
            if not p.is_alive():
                break
    if out is None:
        try:
            out = q.get(timeout=2)
        except queue.Empty:
            out = ("error", f"child ended with exit code {p.exitcode} and no result")
    p.join(timeout=60)
    return out


def in_child(target, *args):
    """Run target(*args, queue) in a fresh process and return its result.  A child
    that ends without any result is started once more: the reference's runs are
    deterministic, so a real failure fails both times, while a transient failure
    of the process start-up on a loaded machine does not fail the test."""
    out = _run_child(target, args)
    if out[0] == "error" and out[1].startswith("child ended"):
        out = _run_child(target, args)
    assert out[0] == "ok", out
    return out[1:]


def steps(a, kind, k):
    off, n = int(a[f"{kind}_step_off"][k]), int(a[f"{kind}_step_n"][k])
    return [(a[f"{kind}_step_d"][q], a[f"{kind}_step_e"][q], a[f"{kind}_step_acc"][q]) for q in range(off, off + n)]


@pytest.mark.parametrize("case", ["ala10_nvt", "ala10_cyl", "mixed6", "sheet2", "ala10_sph", "ala10_obst"])
def test_fill_equals_the_host_builder(case):
    from sdmd_gb300.host import build_system
    a, scal, rng, counters, time = in_child(_child_fill, case)
    work, ind, outd = case_dir(case)
    d = np.load(os.path.join(REPO, "tests", "golden", f"{case}.npz"))
    ref = build_system(ind, gro_text=bytes(d["meta/gro"]).decode(), seed=int(d["pre/seed"][0]))
    for k, v in ref.a.items():
        if k in POOLED:
            continue
        assert a[k].shape == v.shape and np.array_equal(a[k], v), k
    for kind, n in (("con", len(ref.a["con_step_n"])), ("pair", len(ref.a["pair_step_n"]))):
        for k in range(n):
            assert steps(a, kind, k) == steps(ref.a, kind, k), (kind, k)
    for k, v in ref.scal.items():
        if k not in ("n_con_steps", "n_pair_steps"):
            assert scal[k] == v, k
    assert np.array_equal(rng, ref.rng)               # glibc's rand() state, read through initstate()
    assert counters == ref.counters and time == ref.time


@pytest.mark.parametrize("case,k,m", [("ala10_nvt", 3000, 3000), ("sheet2", 30000, 30000)])
def test_handoff_to_the_reference_loop_and_back(case, k, m):
    a, b, ra, rb, ca, cb, ta, tb = in_child(_child_handoff, case, k, m)
    for key in DYN:
        assert np.array_equal(a[key], b[key]), key
    assert np.array_equal(ra, rb) and ca == cb and ta == tb
    assert ca["frame"] == k + m
    if case == "sheet2":
        assert ca["hb"] > 0


def _child_obstacles(ind, outd, q):
    try:
        s = _fill(_bridge(ind, outd))
        q.put(("ok", s.a["sphobst"], s.a["obst"], s.scal.get("wall_type")))
    except Exception as e:
        q.put(("error", repr(e)))


@pytest.mark.parametrize("obstruct,sphobst", [
    ("1 y 60.0", "1 70 70 70 8"),
    ("3 z 90.25 ; x 58 ; y 91.5", "2   60.5 61.5 62.5 9.0 and 95 96 97 10.5"),
    ("no", "3 55 55 55 6 , 99 99 99 6 , 55 99 55 7.25"),
])
def test_obstacle_lines_read_as_the_reference_reads_them(obstruct, sphobst):
    """The Obstruct? and SphObst? lines, with other spacings and separator tokens:
    the host library's parse (through its builder) equals the reference's
    ReadParameter (src/Initialization.c:634-724) as the bridge fills it."""
    from sdmd_gb300.host import build_system
    work, ind, outd = case_dir("ala10_obst")
    text = open(os.path.join(ind, "parameter.txt")).read().splitlines()
    text = [(f"Obstruct?          {obstruct}" if l.startswith("Obstruct?") else
             f"SphObst?           {sphobst}" if l.startswith("SphObst?") else l) for l in text]
    with open(os.path.join(ind, "parameter.txt"), "w") as f:
        f.write("\n".join(text) + "\n")
    sph, obst, wall_type = in_child(_child_obstacles, ind, outd)
    d = np.load(os.path.join(REPO, "tests", "golden", "ala10_obst.npz"))
    mine = build_system(ind, gro_text=bytes(d["meta/gro"]).decode(), seed=int(d["pre/seed"][0]))
    assert np.array_equal(mine.a["sphobst"], sph) and len(sph) == 4 * int(sphobst.split()[0])
    assert np.array_equal(mine.a["obst"], obst)
    if obstruct != "no":
        assert len(obst) == 3 * int(obstruct.split()[0]) and mine.scal["wall_type"] == wall_type
