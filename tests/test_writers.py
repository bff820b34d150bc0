"""The host library's output writers against the reference's own (no GPU).

sdmd_write_* (sdmd_gb300/host/writers.c) write the reference's text outputs from
an engine state.  Here the reference's unmodified sources (oracle/_ref, with the
bridge) set up a golden case, run their own loop, and write their outputs with
SaveData (src/DataSave.c); the bridge then fills an sdmd_system from that same
state, and the host library's writers must produce the same bytes: the
trajectory (.gro, .pdb, .xyz), the connection map (with the hydrogen bonds the
run formed), the HB counts and the energy / temperature series (two frames each,
appended).
"""
import ctypes as C
import os

import numpy as np
import pytest

from tests.test_ref_bridge import LIB, REPO, _bridge, _fill, case_dir, in_child

pytestmark = pytest.mark.skipif(not os.path.exists(LIB),
                                reason="the reference's sources are not here (oracle/_ref not built)")

TRJ, POT, KIN, TEM, CNT, HBN, XYZ, PDB, LGF = 0, 1, 2, 3, 4, 5, 6, 7, 8   # enum FileType (src/DMD.h:212-228)
NAMES = {TRJ: "out_trj.gro", POT: "out_pot.txt", KIN: "out_kin.txt", TEM: "out_tem.txt", CNT: "out_cnt.txt",
         HBN: "out_HBn.txt", XYZ: "out_xyz.xyz", PDB: "out_pdb.pdb"}


def _child_frames(case, runs, q):
    """The reference writes one frame after each run; the state of each frame is
    filled through the bridge and returned with the reference's energies."""
    try:
        work, ind, outd = case_dir(case)
        L = _bridge(ind, outd)
        L.bd_potential.restype = C.c_double
        L.bd_kinetic.restype = C.c_double
        L.bd_temperature.restype = C.c_double
        L.bd_save_type.argtypes = [C.c_int]
        L.bd_sweep()
        frames = []
        for n in runs:
            L.bd_run(n)
            for t in (TRJ, POT, KIN, TEM, CNT, HBN, XYZ, PDB):
                L.bd_save_type(t)
            s = _fill(L)
            frames.append((s.a, s.scal, s.counters, s.time, L.bd_potential(), L.bd_kinetic(), L.bd_temperature()))
        files = {t: open(os.path.join(outd, name), "rb").read() for t, name in NAMES.items()}
        q.put(("ok", frames, files, ind))
    except Exception as e:
        q.put(("error", repr(e)))


def _host_writers():
    from sdmd_gb300.host import lib
    from sdmd_gb300.system import sdmd_system
    L = lib()
    P = C.POINTER(sdmd_system)
    for f in ("sdmd_write_gro", "sdmd_write_pdb", "sdmd_write_xyz"):
        getattr(L, f).argtypes = [C.c_char_p, C.c_int, P, C.c_char_p, C.c_char_p]
    for f in ("sdmd_write_cnt", "sdmd_write_hbn"):
        getattr(L, f).argtypes = [C.c_char_p, C.c_int, P]
    L.sdmd_write_series.argtypes = [C.c_char_p, C.c_int, C.c_double, C.c_double]
    return L


@pytest.mark.parametrize("case,runs", [("ala10_nvt", (2000, 2000)), ("sheet2", (30000, 20000))])
def test_writers_match_the_reference(case, runs, tmp_path):
    from sdmd_gb300.host import build_system
    from sdmd_gb300.system import System
    frames, ref_files, ind = in_child(_child_frames, case, runs)
    d = np.load(os.path.join(REPO, "tests", "golden", f"{case}.npz"))
    named = build_system(ind, gro_text=bytes(d["meta/gro"]).decode(), seed=int(d["pre/seed"][0]))
    L = _host_writers()
    out = {t: str(tmp_path / name).encode() for t, name in NAMES.items()}
    for k, (a, scal, counters, time, pot, kin, tem) in enumerate(frames):
        s = System()
        s.a, s.scal, s.counters, s.time = a, scal, counters, time
        s.rng = np.zeros(33, np.int32)
        st = C.byref(s.struct())
        app = 1 if k else 0
        assert L.sdmd_write_gro(out[TRJ], app, st, named.names, named.resnames) == 0
        assert L.sdmd_write_pdb(out[PDB], app, st, named.names, named.resnames) == 0
        assert L.sdmd_write_xyz(out[XYZ], app, st, named.names, b"") == 0   # no log written: the timer is empty
        assert L.sdmd_write_cnt(out[CNT], app, st) == 0
        assert L.sdmd_write_hbn(out[HBN], app, st) == 0
        for t, v in ((POT, pot), (KIN, kin), (TEM, tem)):
            assert L.sdmd_write_series(out[t], app, time, v) == 0
    for t, name in NAMES.items():
        mine = open(out[t], "rb").read()
        assert mine == ref_files[t], f"{name} differs"
    if case == "sheet2":
        assert frames[-1][2]["hb_formed"] > 0          # the map carries formed hydrogen bonds
        assert b" 4 " in ref_files[CNT] or b" 5 " in ref_files[CNT] or b" 12 " in ref_files[CNT]


def _child_log(case, q):
    try:
        work, ind, outd = case_dir(case)
        L = _bridge(ind, outd)
        L.bd_save_type.argtypes = [C.c_int]
        L.bd_save_type(LGF)                           # SaveLog, as Prepare() calls it
        q.put(("ok", open(os.path.join(outd, "out_log.txt"), "rb").read(), ind))
    except Exception as e:
        q.put(("error", repr(e)))


@pytest.mark.parametrize("case", ["ala10_nvt", "sheet2", "ala10_cyl", "mixed6", "ala10_sph", "ala10_obst"])
def test_log_matches_the_reference(case, tmp_path):
    """out_log.txt from the host library equals the reference's SaveLog output
    line for line after the first, which carries the wall-clock time."""
    from sdmd_gb300 import host as H
    ref, ind = in_child(_child_log, case)
    d = np.load(os.path.join(REPO, "tests", "golden", f"{case}.npz"))
    L = H.lib()
    L.sdmd_write_log.argtypes = [C.c_char_p, C.c_void_p, C.c_void_p, C.c_char_p, C.c_double, C.c_uint32, C.c_double,
                                 C.c_double]
    params = H.read_parameters(os.path.join(ind, "parameter.txt"))
    seed = int(d["pre/seed"][0])
    hs = C.c_void_p()
    err = C.create_string_buffer(512)
    assert L.sdmd_build_system_gro_text(ind.encode(), bytes(d["meta/gro"]), C.byref(params), seed, 20000, C.byref(hs),
                                        err, 512) == 0, err.value
    path = tmp_path / "out_log.txt"
    assert L.sdmd_write_log(str(path).encode(), hs, C.byref(params), b"2000_01_01_00_00_00", 0.0, seed, 0.0, 0.0) == 0
    L.sdmd_host_free(hs)
    mine = path.read_bytes().split(b"\n")
    theirs = ref.split(b"\n")
    assert mine[0] == b"#Log file at 2000_01_01_00_00_00"
    assert mine[1:] == theirs[1:]


SYSINFO = 9   # enum FileType: sysInfo


def _child_sysinfo(case, q):
    try:
        work, ind, outd = case_dir(case)
        L = _bridge(ind, outd)
        L.bd_save_type.argtypes = [C.c_int]
        L.bd_save_type(SYSINFO)                       # SaveSysInfo, as Prepare() calls it for a new run
        q.put(("ok", open(os.path.join(outd, "SysInfo.dat"), "rb").read(), ind))
    except Exception as e:
        q.put(("error", repr(e)))


def walk_sysinfo(mine, ref):
    """Walk two SysInfo.dat images record by record (src/DataSave.c:280-331), the
    lists following the reference's non-NULL pointers, and return the first
    difference: every defined field equal, every pointer equally NULL or not.
    Left out: residue / peptide record 0 and a residue record's bytes past its
    name (malloc'd), and padding."""
    pos = [0]

    def take(n):
        a, b = mine[pos[0]:pos[0] + n], ref[pos[0]:pos[0] + n]
        pos[0] += n
        return a, b

    def same(a, b, keep, what):
        for lo, hi in keep:
            if a[lo:hi] != b[lo:hi]:
                raise AssertionError(f"{what}: bytes {lo}-{hi} differ at file offset {pos[0] - len(a) + lo}")

    def ptr(a, b, off, what):
        pa, pb = int.from_bytes(a[off:off + 8], "little"), int.from_bytes(b[off:off + 8], "little")
        if (pa == 0) != (pb == 0):
            raise AssertionError(f"{what}: link at byte {off} is {'set' if pa else 'NULL'} here, "
                                 f"{'set' if pb else 'NULL'} in the reference")
        return pb != 0

    def steps(first, what):
        more = first
        while more:
            a, b = take(32)
            same(a, b, [(0, 24)], what + " step")
            more = ptr(a, b, 24, what + " step")

    def constr(what):
        a, b = take(40)
        same(a, b, [(0, 4), (8, 16), (24, 32)], what)
        st = ptr(a, b, 16, what)
        nxt = ptr(a, b, 32, what)
        steps(st, what)
        return nxt

    a, b = take(12)
    same(a, b, [(0, 12)], "header")
    n_atoms, n_prot, n_aa = np.frombuffer(b, np.int32)
    for k in range(n_aa + 1):
        a, b = take(32)
        if k:
            same(a, b, [(0, 4), (8, 32)], f"aa[{k}]")
    for k in range(n_prot + 1):
        a, b = take(24)
        if k:
            same(a, b, [(0, 24)], f"pep[{k}]")
    for i in range(n_atoms + 1):
        a, b = take(136)
        same(a, b, [(0, 120)], f"property[{i}]")
        ptr(a, b, 120, f"property[{i}].bond")
        more = ptr(a, b, 128, f"property[{i}].constr")
        while more:
            more = constr(f"atom {i} constraint")
        a, b = take(16)
        same(a, b, [(0, 9), (12, 16)], f"HB[{i}]")
    a, b = take(48)
    same(a, b, [(0, 48)], "HBPotential")
    for t in range(12):
        for k in range(32 * 32):
            if constr(f"table {t} entry {k}"):
                raise AssertionError("a pair-table entry with a next link")
    assert pos[0] == len(ref) == len(mine), (pos[0], len(ref), len(mine))


@pytest.mark.parametrize("case", ["ala10_nvt", "sheet2", "ala10_cyl", "mixed6"])
def test_sysinfo_matches_the_reference(case, tmp_path):
    from sdmd_gb300 import host as H
    ref, ind = in_child(_child_sysinfo, case)
    d = np.load(os.path.join(REPO, "tests", "golden", f"{case}.npz"))
    L = H.lib()
    L.sdmd_write_sysinfo.argtypes = [C.c_char_p, C.c_void_p]
    params = H.read_parameters(os.path.join(ind, "parameter.txt"))
    hs = C.c_void_p()
    err = C.create_string_buffer(512)
    assert L.sdmd_build_system_gro_text(ind.encode(), bytes(d["meta/gro"]), C.byref(params), int(d["pre/seed"][0]),
                                        20000, C.byref(hs), err, 512) == 0, err.value
    path = tmp_path / "SysInfo.dat"
    assert L.sdmd_write_sysinfo(str(path).encode(), hs) == 0
    L.sdmd_host_free(hs)
    walk_sysinfo(path.read_bytes(), ref)


WALLINFO = 10   # enum FileType: wallInfo


def _child_wallinfo(case, q):
    try:
        work, ind, outd = case_dir(case)
        L = _bridge(ind, outd)
        L.bd_save_type.argtypes = [C.c_int]
        L.bd_save_type(WALLINFO)                      # SaveWallInfo, as Prepare() calls it for a smooth wall
        q.put(("ok", open(os.path.join(outd, "WallInfo.dat"), "rb").read(), ind))
    except Exception as e:
        q.put(("error", repr(e)))


def test_wallinfo_matches_the_reference(tmp_path):
    """WallInfo.dat of the cylinder-wall case equals the reference's SaveWallInfo
    output byte for byte (the wall's atom record as ReadWall builds it)."""
    from sdmd_gb300 import host as H
    ref, ind = in_child(_child_wallinfo, "ala10_cyl")
    d = np.load(os.path.join(REPO, "tests", "golden", "ala10_cyl.npz"))
    L = H.lib()
    L.sdmd_write_wallinfo.argtypes = [C.c_char_p, C.c_void_p]
    params = H.read_parameters(os.path.join(ind, "parameter.txt"))
    hs = C.c_void_p()
    err = C.create_string_buffer(512)
    assert L.sdmd_build_system_gro_text(ind.encode(), bytes(d["meta/gro"]), C.byref(params), int(d["pre/seed"][0]),
                                        20000, C.byref(hs), err, 512) == 0, err.value
    path = tmp_path / "WallInfo.dat"
    assert L.sdmd_write_wallinfo(str(path).encode(), hs) == 0
    L.sdmd_host_free(hs)
    assert len(ref) == 136 + 176
    assert path.read_bytes() == ref


OBSTINFO = 11   # enum FileType: obstInfo


def _child_obstinfo(case, q):
    try:
        work, ind, outd = case_dir(case)
        L = _bridge(ind, outd)
        L.bd_save_type.argtypes = [C.c_int]
        L.bd_save_type(OBSTINFO)                      # SaveObstInfo, as Prepare() calls it for obstruction walls
        q.put(("ok", open(os.path.join(outd, "ObstInfo.dat"), "rb").read(), ind))
    except Exception as e:
        q.put(("error", repr(e)))


def test_obstinfo_matches_the_reference(tmp_path):
    """ObstInfo.dat of the two-plane case equals the reference's SaveObstInfo output
    byte for byte (each obstruction wall's atom record)."""
    from sdmd_gb300 import host as H
    ref, ind = in_child(_child_obstinfo, "ala10_obst")
    d = np.load(os.path.join(REPO, "tests", "golden", "ala10_obst.npz"))
    L = H.lib()
    L.sdmd_write_obstinfo.argtypes = [C.c_char_p, C.c_void_p]
    params = H.read_parameters(os.path.join(ind, "parameter.txt"))
    hs = C.c_void_p()
    err = C.create_string_buffer(512)
    assert L.sdmd_build_system_gro_text(ind.encode(), bytes(d["meta/gro"]), C.byref(params), int(d["pre/seed"][0]),
                                        20000, C.byref(hs), err, 512) == 0, err.value
    path = tmp_path / "ObstInfo.dat"
    assert L.sdmd_write_obstinfo(str(path).encode(), hs) == 0
    L.sdmd_host_free(hs)
    assert len(ref) == 2 * (136 + 176)
    assert path.read_bytes() == ref
