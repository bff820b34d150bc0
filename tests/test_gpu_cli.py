"""The engine's sDMD executable against the reference's own executable (GPU).

tests/golden/cli_ala10 holds a whole run of the reference's unmodified sDMD
(tests/golden/make_cli_golden.py: its own main and command line, the fixed
-DDEBUG_RANDOM seed): ALA x 10 under Andersen NVT to Time 40 with Dump_Rate 10
and -pot -kin -tem -HBn.  sdmd-gb300 runs the same command line on the same
inputs with the same seed (SDMD_DEBUG_RANDOM), its event loop on the GPU, and
every output file must equal the reference's byte for byte: the trajectory, the
connection map, the energies, the temperature and the HB counts at every dump,
and the last checkpoint (savedData.dat, but for the bytes the reference leaves
undefined, as tests/test_saved_data.py compares them), the log (but for its
first line, the start time) and a new run's SysInfo.dat (field by field, as
tests/test_writers.py walks it); an output file already in
the folder is kept under the run's start time, as the reference's BackupFile
does.  cli_ala10_continue is the
reference's continue run from that checkpoint (read from the output folder, as
ReadBreakPoint does) to Time 70.
"""
import os
import shutil
import subprocess

import pytest

pytestmark = pytest.mark.gpu

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
OUTPUTS = ["out_trj.gro", "out_cnt.txt", "out_pot.txt", "out_kin.txt", "out_tem.txt", "out_HBn.txt"]


@pytest.mark.parametrize("case", ["cli_ala10", "cli_ala10_continue"])
def test_executable_writes_the_reference_outputs(tmp_path, case):
    import __graft_entry__ as G
    G.build()
    from sdmd_gb300 import build
    CASE = os.path.join(REPO, "tests", "golden", case)
    ind, outd = tmp_path / "in", tmp_path / "out"
    shutil.copytree(os.path.join(CASE, "in"), ind)
    shutil.copytree(os.path.join(REPO, "sdmd_gb300", "data", "Library_Ding"), ind / "Library_Ding")
    outd.mkdir()
    if (ind / "savedData.dat").exists():      # a continue run's checkpoint
        shutil.copy(ind / "savedData.dat", outd / "savedData.dat")
    (outd / "out_trj.gro").write_text("an earlier run\n")   # kept under the run's start time
    flags = open(os.path.join(CASE, "expected", "flags.txt")).read().split()
    env = dict(os.environ, SDMD_DEBUG_RANDOM="1")
    r = subprocess.run([build.APP, "-i", str(ind), "-o", str(outd), "-f", "sys.gro", *flags], env=env,
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    assert "Finished!" in r.stdout
    kept = [p for p in outd.iterdir() if p.name.startswith("out_trj@") and p.name.endswith(".gro")]
    assert len(kept) == 1 and kept[0].read_text() == "an earlier run\n"     # BackupFile
    for name in OUTPUTS:
        mine = (outd / name).read_bytes()
        ref = open(os.path.join(CASE, "expected", name), "rb").read()
        assert mine == ref, f"{name} differs from the reference's"
    mine, ref = (outd / "out_log.txt").read_text().splitlines(), open(os.path.join(CASE, "expected", "out_log.txt")).read().splitlines()
    assert mine[0].startswith("#Log file at ") and mine[1:] == ref[1:]   # the first line is the start time
    expected_sys = os.path.join(CASE, "expected", "SysInfo.dat")      # written by a new run only
    assert (outd / "SysInfo.dat").exists() == os.path.exists(expected_sys)
    if os.path.exists(expected_sys):
        from tests.test_writers import walk_sysinfo
        walk_sysinfo((outd / "SysInfo.dat").read_bytes(), open(expected_sys, "rb").read())
    from tests.test_saved_data import differing_defined_bytes
    bad = differing_defined_bytes((outd / "savedData.dat").read_bytes(),
                                  open(os.path.join(CASE, "expected", "savedData.dat"), "rb").read())
    assert len(bad) == 0, f"savedData.dat differs at {bad[:5]}"
