"""The engine's REMD launcher against a whole REMD run of the reference (GPU).

tests/golden/remd_ala10 holds the outputs of the reference's own sServer and
three sDMD clients, started as its launcher sREMD starts them, with the server's
seed fixed (tests/golden/make_remd_golden.py): ALA x 10 at 275, 350 and 450 K,
exchanges every 5 time units, dumps every 10, Time 30, -pot -tem.  sremd-gb300
runs the same launcher command line on the same inputs with the same seeds
(SDMD_DEBUG_RANDOM for the clients', SDMD_SERVER_SEED for the server's), all three
replicas in one engine batch, and every replica's files must equal the
reference client's: trajectory, connection map, energies and temperatures at
every dump, the out_REMD lines of every exchange (time, new temperature, ladder
index), the log (but for its first line, the start time), SysInfo (field by
field, as tests/test_writers.py walks it) and the last checkpoint (but for the
bytes the reference leaves undefined, as tests/test_saved_data.py compares them).
tests/golden/remd_ala10_continue is the reference's continue run from those
checkpoints (each replica's read from the output folder, its temperature record
with it) to Time 50.
"""
import os
import shutil
import subprocess

import pytest

pytestmark = pytest.mark.gpu

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.parametrize("case", ["remd_ala10", "remd_ala10_continue"])
def test_launcher_writes_the_reference_replicas_outputs(tmp_path, case):
    import __graft_entry__ as G
    G.build()
    from sdmd_gb300 import build
    from tests.test_saved_data import differing_defined_bytes
    from tests.test_writers import walk_sysinfo
    CASE = os.path.join(REPO, "tests", "golden", case)
    ind, outd = tmp_path / "in", tmp_path / "out"
    shutil.copytree(os.path.join(CASE, "in"), ind)
    shutil.copytree(os.path.join(REPO, "sdmd_gb300", "data", "Library_Ding"), ind / "Library_Ding")
    outd.mkdir()
    for k in range(3):   # a continue run reads each replica's checkpoint from the output folder
        if (ind / f"savedData{k}.dat").exists():
            shutil.copy(ind / f"savedData{k}.dat", outd / f"savedData{k}.dat")
    launch = dict(line.split(" ", 1) for line in open(os.path.join(CASE, "expected", "launch.txt")).read().splitlines())
    env = dict(os.environ, SDMD_DEBUG_RANDOM="1", SDMD_SERVER_SEED=launch["server_seed"].strip())
    cmd = [build.REMD_APP, "-f", str(ind / "REMDConfig.txt"), "-args", "sDMD", "-i", str(ind), "-o", str(outd), "-f",
           "sys.gro", *launch["flags"].split(), "-end"]
    r = subprocess.run(cmd, env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    assert "Finished!" in r.stdout
    for k in range(3):
        for name in (f"out_trj{k}.gro", f"out_cnt{k}.txt", f"out_pot{k}.txt", f"out_tem{k}.txt", f"out_REMD{k}.txt"):
            mine = (outd / name).read_bytes()
            ref = open(os.path.join(CASE, "expected", name), "rb").read()
            assert mine == ref, f"{name} differs from the reference's"
        mine = (outd / f"out_log{k}.txt").read_text().splitlines()
        ref = open(os.path.join(CASE, "expected", f"out_log{k}.txt")).read().splitlines()
        assert mine[0].startswith("#Log file at ") and mine[1:] == ref[1:]
        expected_sys = os.path.join(CASE, "expected", "SysInfo0.dat")   # a new run's only
        assert (outd / f"SysInfo{k}.dat").exists() == os.path.exists(expected_sys)
        if os.path.exists(expected_sys):
            walk_sysinfo((outd / f"SysInfo{k}.dat").read_bytes(), open(expected_sys, "rb").read())
        bad = differing_defined_bytes((outd / f"savedData{k}.dat").read_bytes(),
                                      open(os.path.join(CASE, "expected", f"savedData{k}.dat"), "rb").read())
        assert len(bad) == 0, f"savedData{k}.dat differs at {bad[:5]}"
