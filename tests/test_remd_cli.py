"""The REMD launcher's host side against a whole REMD run of the reference (no GPU).

tests/golden/remd_ala10 holds the outputs of the reference's own sServer and
three sDMD clients, started as its launcher sREMD starts them
(tests/golden/make_remd_golden.py).  Here, without a device: each replica's
command line as the launcher builds it, its log (SaveLog with the REMD lines),
its SysInfo file, the out_REMD lines (SaveRE) and the checkpoint's REMDInfo
record, written by the host library, against the reference's files; and the
launcher's usage and failures.  The run itself is tests/test_gpu_remd_cli.py.
"""
import ctypes as C
import os
import shutil
import subprocess

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CASE = os.path.join(REPO, "tests", "golden", "remd_ala10")
DEBUG_SEED = 1575263273


def _inputs(tmp_path):
    ind = tmp_path / "in"
    shutil.copytree(os.path.join(CASE, "in"), ind)
    shutil.copytree(os.path.join(REPO, "sdmd_gb300", "data", "Library_Ding"), ind / "Library_Ding")
    return ind


def _config(ind):
    from sdmd_gb300 import host as H
    return H.read_remd_config(ind / "REMDConfig.txt")


def _build(ind, T):
    from sdmd_gb300 import host as H
    L = H.lib()
    params = H.read_parameters(str(ind / "parameter.txt"))
    params.temperature = T                  # T(reduced) "no": the replica's -REMD temperature
    hs = C.c_void_p()
    err = C.create_string_buffer(512)
    assert L.sdmd_build_system(str(ind).encode(), b"sys.gro", C.byref(params), None, DEBUG_SEED, 20000, C.byref(hs),
                               err, 512) == 0, err.value
    return L, params, hs


def test_each_replica_writes_the_reference_log_and_sysinfo(tmp_path):
    """out_log<id>.txt (but for its first line, the start time) and SysInfo<id>.dat
    of each replica equal the reference client's."""
    from sdmd_gb300 import host as H
    from tests.test_writers import walk_sysinfo
    ind = _inputs(tmp_path)
    cfg = _config(ind)
    assert cfg["n"] == 3 and cfg["exchange_time"] == 5
    for k in range(cfg["n"]):
        L, params, hs = _build(ind, cfg["T"][k])
        r = H.sdmd_replica(port=cfg["port"], output_rate=int(cfg["exchange_time"]), num=int(cfg["num"][k]),
                           T=cfg["T"][k], server=b"localhost", extra=str(k).encode())
        L.sdmd_write_log_replica.argtypes = [C.c_char_p, C.c_void_p, C.c_void_p, C.c_char_p, C.c_double, C.c_uint32,
                                             C.c_double, C.c_double, C.POINTER(H.sdmd_replica)]
        path = tmp_path / f"out_log{k}.txt"
        assert L.sdmd_write_log_replica(str(path).encode(), hs, C.byref(params), b"2000_01_01_00_00_00", 0.0,
                                        DEBUG_SEED, 0.0, 0.0, C.byref(r)) == 0
        mine = path.read_text().splitlines()
        ref = open(os.path.join(CASE, "expected", f"out_log{k}.txt")).read().splitlines()
        assert mine[1:] == ref[1:], f"replica {k}"
        L.sdmd_write_sysinfo.argtypes = [C.c_char_p, C.c_void_p]
        sysinfo = tmp_path / f"SysInfo{k}.dat"
        assert L.sdmd_write_sysinfo(str(sysinfo).encode(), hs) == 0
        walk_sysinfo(sysinfo.read_bytes(), open(os.path.join(CASE, "expected", "SysInfo0.dat"), "rb").read())
        L.sdmd_host_free(hs)


def test_remd_lines_and_the_checkpoint_record(tmp_path):
    """SaveRE's line format, and the REMDInfo record (the checkpoint's last 128
    bytes) that sdmd_saved_set_replica gives the template, against the reference
    client's last checkpoint."""
    from sdmd_gb300 import host as H
    ind = _inputs(tmp_path)
    cfg = _config(ind)
    L = H.lib()
    L.sdmd_write_remd.argtypes = [C.c_char_p, C.c_int, C.c_double, C.c_double, C.c_int32]
    for k in range(cfg["n"]):
        ref = open(os.path.join(CASE, "expected", f"out_REMD{k}.txt")).read()
        path = tmp_path / f"out_REMD{k}.txt"
        for q, line in enumerate(ref.splitlines()):
            t, T, num = line.split()
            assert L.sdmd_write_remd(str(path).encode(), q > 0, float(t), float(T), int(num)) == 0
        assert path.read_text() == ref
        # the checkpoint's REMDInfo: the replica's record at its last dump
        saved = open(os.path.join(CASE, "expected", f"savedData{k}.dat"), "rb").read()
        rec = saved[-128:]
        num_k, T_k = np.frombuffer(rec[112:116], np.int32)[0], np.frombuffer(rec[120:128], np.float64)[0]
        _, params, hs = _build(ind, cfg["T"][k])
        tpl = C.c_void_p()
        err = C.create_string_buffer(512)
        L.sdmd_saved_new.argtypes = [C.c_void_p, C.c_void_p, C.c_uint32, C.POINTER(C.c_void_p), C.c_char_p, C.c_int]
        assert L.sdmd_saved_new(hs, C.byref(params), DEBUG_SEED, C.byref(tpl), err, 512) == 0
        r = H.sdmd_replica(port=cfg["port"], output_rate=int(cfg["exchange_time"]), num=int(num_k), T=float(T_k),
                           server=b"localhost", extra=str(k).encode())
        L.sdmd_saved_set_replica.argtypes = [C.c_void_p, C.POINTER(H.sdmd_replica)]
        assert L.sdmd_saved_set_replica(tpl, C.byref(r)) == 0
        from sdmd_gb300.system import sdmd_system
        L.sdmd_host_view.restype = C.POINTER(sdmd_system)
        L.sdmd_saved_write.argtypes = [C.c_char_p, C.c_void_p, C.POINTER(sdmd_system), C.c_char_p, C.c_int]
        out = tmp_path / f"savedData{k}.dat"
        assert L.sdmd_saved_write(str(out).encode(), tpl, L.sdmd_host_view(hs), err, 512) == 0, err.value
        mine = out.read_bytes()
        assert len(mine) == len(saved) and mine[-128:] == rec, f"replica {k}"
        back = H.sdmd_replica()
        L.sdmd_saved_read.argtypes = [C.c_char_p, C.POINTER(C.c_void_p), C.c_char_p, C.c_int]
        sv = C.c_void_p()
        ref_path = os.path.join(CASE, "expected", f"savedData{k}.dat").encode()
        assert L.sdmd_saved_read(ref_path, C.byref(sv), err, 512) == 0
        L.sdmd_saved_replica.argtypes = [C.c_void_p, C.POINTER(H.sdmd_replica)]
        assert L.sdmd_saved_replica(sv, C.byref(back)) == 1
        assert (back.num, back.T, back.extra, back.server) == (num_k, T_k, str(k).encode(), b"localhost")
        L.sdmd_saved_free(sv)
        L.sdmd_saved_free(tpl)
        L.sdmd_host_free(hs)


def run(args, **kw):
    from sdmd_gb300 import build
    build.build_all()
    return subprocess.run([build.REMD_APP, *args], capture_output=True, text=True, timeout=300, **kw)


def test_launcher_usage_and_failures(tmp_path):
    r = run(["-h"])
    assert r.returncode == 0 and "-args" in r.stdout
    r = run(["-f", str(tmp_path / "missing.txt"), "-args", "sDMD", "-i", str(tmp_path), "-o", str(tmp_path)])
    assert r.returncode == 1 and "!!ERROR!!" in r.stderr
    r = run(["-f", str(tmp_path / "missing.txt")])          # no -args
    assert r.returncode == 1


def test_launcher_builds_every_replica_then_needs_a_device(tmp_path):
    from sdmd_gb300 import engine
    if engine.device_count() > 0:
        pytest.skip("on a GPU machine the run itself is tests/test_gpu_remd_cli.py")
    ind = _inputs(tmp_path)
    out = tmp_path / "out"
    out.mkdir()
    r = run(["-f", str(ind / "REMDConfig.txt"), "-args", "sDMD", "-i", str(ind), "-o", str(out), "-f", "sys.gro",
             "-pot", "-tem", "-end"], env=dict(os.environ, SDMD_DEBUG_RANDOM="1"))
    assert r.returncode == 1
    assert "3 replicas, exchange every 5 time units" in r.stdout
    assert "!!ERROR!!: sdmd_gpu_create" in r.stderr
