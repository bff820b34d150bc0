"""The reference's analysis tool reads the engine's output files (no GPU).

sAnalysis (the reference's analysis/ sources, built by oracle/ref/Makefile) reads
a run's trajectory, connection map, SysInfo.dat and log.  It runs twice on the
ALA x 10 run of tests/golden/cli_ala10: once on the reference executable's own
files, once with SysInfo.dat and out_log.txt written by the host library from the
same inputs (sdmd_write_sysinfo / sdmd_write_log; the engine's executable writes
them the same way, and its text outputs equal the reference's byte for byte,
tests/test_gpu_cli.py).  Every file the analyses write -- the unwrapped
trajectory, HB statistics, radius of gyration, Ramachandran and contact maps --
must be the same.
"""
import ctypes as C
import os
import shutil
import subprocess

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ANALYSIS = os.path.join(REPO, "oracle", "_ref", "sAnalysis")
CASE = os.path.join(REPO, "tests", "golden", "cli_ala10")
DEBUG_SEED = 1575263273
FLAGS = ["-trj", "out_trj.gro", "-cnt", "out_cnt.txt", "-sys", "SysInfo.dat", "-log", "out_log.txt", "-rPBC", "-HB",
         "-RG", "-Ramach", "-ConMap"]

pytestmark = pytest.mark.skipif(not os.path.exists(ANALYSIS),
                                reason="the reference's analysis sources are not here (oracle/_ref not built)")


def _analyse(d):
    before = set(os.listdir(d))
    r = subprocess.run([ANALYSIS, "-path", str(d) + "/", *FLAGS], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout[-2000:]
    return {name: (d / name).read_bytes() for name in sorted(set(os.listdir(d)) - before)}


def test_analysis_reads_the_engine_files(tmp_path):
    from sdmd_gb300 import host as H
    ref_dir, mine_dir, ind = tmp_path / "ref", tmp_path / "mine", tmp_path / "in"
    shutil.copytree(os.path.join(CASE, "expected"), ref_dir)
    shutil.copytree(os.path.join(CASE, "expected"), mine_dir)
    shutil.copytree(os.path.join(CASE, "in"), ind)
    shutil.copytree(os.path.join(REPO, "sdmd_gb300", "data", "Library_Ding"), ind / "Library_Ding")
    L = H.lib()
    params = H.read_parameters(str(ind / "parameter.txt"))
    hs = C.c_void_p()
    err = C.create_string_buffer(512)
    assert L.sdmd_build_system(str(ind).encode(), b"sys.gro", C.byref(params), None, DEBUG_SEED, 20000, C.byref(hs),
                               err, 512) == 0, err.value
    L.sdmd_write_sysinfo.argtypes = [C.c_char_p, C.c_void_p]
    L.sdmd_write_log.argtypes = [C.c_char_p, C.c_void_p, C.c_void_p, C.c_char_p, C.c_double, C.c_uint32, C.c_double,
                                 C.c_double]
    assert L.sdmd_write_sysinfo(str(mine_dir / "SysInfo.dat").encode(), hs) == 0
    assert L.sdmd_write_log(str(mine_dir / "out_log.txt").encode(), hs, C.byref(params), b"2000_01_01_00_00_00", 0.0,
                            DEBUG_SEED, 0.0, 0.0) == 0
    L.sdmd_host_free(hs)
    assert (mine_dir / "SysInfo.dat").read_bytes() != (ref_dir / "SysInfo.dat").read_bytes()   # pointer fields differ
    ref, mine = _analyse(ref_dir), _analyse(mine_dir)
    assert "rPBCGRO.gro" in ref and "HBInfo.txt" in ref and "RG.txt" in ref
    assert sorted(mine) == sorted(ref)
    for name in ref:
        assert mine[name] == ref[name], f"{name} differs"


REMD_CASE = os.path.join(REPO, "tests", "golden", "remd_ala10")
REMD_FLAGS = FLAGS[:8] + ["-rPBC", "-HB", "-En", "-REMD", "-reNo", "3", "-rate", "10", "-temp", "300"]


def test_remd_analysis_reads_the_engine_files(tmp_path):
    """The REMD analysis (energies per replica, then WHAM over the temperature
    ladder of out_REMD<id>.txt, reading input/REMDConfig.txt) on the reference
    clients' files and on the same run with each replica's SysInfo and log
    written by the host library (sdmd_write_sysinfo / sdmd_write_log_replica):
    every output the same."""
    from sdmd_gb300 import host as H
    ref_dir, mine_dir, ind = tmp_path / "ref", tmp_path / "mine", tmp_path / "in"
    for d in (ref_dir, mine_dir):
        shutil.copytree(os.path.join(REMD_CASE, "expected"), d)
        (d / "input").mkdir()
        shutil.copy(os.path.join(REMD_CASE, "in", "REMDConfig.txt"), d / "input" / "REMDConfig.txt")
    for k in (1, 2):   # the three SysInfo files differ only in heap addresses: one is kept
        shutil.copy(ref_dir / "SysInfo0.dat", ref_dir / f"SysInfo{k}.dat")
    shutil.copytree(os.path.join(REMD_CASE, "in"), ind)
    shutil.copytree(os.path.join(REPO, "sdmd_gb300", "data", "Library_Ding"), ind / "Library_Ding")
    cfg = H.read_remd_config(ind / "REMDConfig.txt")
    L = H.lib()
    L.sdmd_write_sysinfo.argtypes = [C.c_char_p, C.c_void_p]
    L.sdmd_write_log_replica.argtypes = [C.c_char_p, C.c_void_p, C.c_void_p, C.c_char_p, C.c_double, C.c_uint32,
                                         C.c_double, C.c_double, C.POINTER(H.sdmd_replica)]
    for k in range(cfg["n"]):
        params = H.read_parameters(str(ind / "parameter.txt"))
        params.temperature = cfg["T"][k]            # T(reduced) "no": the replica's -REMD temperature
        hs = C.c_void_p()
        err = C.create_string_buffer(512)
        assert L.sdmd_build_system(str(ind).encode(), b"sys.gro", C.byref(params), None, DEBUG_SEED, 20000,
                                   C.byref(hs), err, 512) == 0, err.value
        r = H.sdmd_replica(port=cfg["port"], output_rate=int(cfg["exchange_time"]), num=int(cfg["num"][k]),
                           T=cfg["T"][k], server=b"localhost", extra=str(k).encode())
        assert L.sdmd_write_sysinfo(str(mine_dir / f"SysInfo{k}.dat").encode(), hs) == 0
        assert L.sdmd_write_log_replica(str(mine_dir / f"out_log{k}.txt").encode(), hs, C.byref(params),
                                        b"2000_01_01_00_00_00", 0.0, DEBUG_SEED, 0.0, 0.0, C.byref(r)) == 0
        L.sdmd_host_free(hs)

    def analyse(d):
        before = set(os.listdir(d))
        out = subprocess.run([ANALYSIS, "-path", str(d) + "/", *REMD_FLAGS], capture_output=True, text=True,
                             timeout=300)
        assert out.returncode == 0, out.stdout[-2000:]
        return {name: (d / name).read_bytes() for name in sorted(set(os.listdir(d)) - before)}

    ref, mine = analyse(ref_dir), analyse(mine_dir)
    assert {"FreeEnergy.txt", "CvPotT.txt", "REMD_T0.txt", "Energy2.txt"} <= set(ref)
    assert sorted(mine) == sorted(ref)
    for name in ref:
        assert mine[name] == ref[name], f"{name} differs"
