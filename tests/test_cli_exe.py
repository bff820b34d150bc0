"""The engine's sDMD executable without a GPU: it builds with the libraries, reads
the reference's command line, and fails loudly (the reference's "!!ERROR!!"
message, exit code 1) where the reference would, or where no device exists."""
import os
import shutil
import subprocess

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def run(args, **kw):
    from sdmd_gb300 import build
    build.build_all()
    return subprocess.run([build.APP, *args], capture_output=True, text=True, timeout=300, **kw)


def test_usage_and_bad_directories(tmp_path):
    r = run(["-h"])
    assert r.returncode == 0 and "usage" in r.stdout
    r = run(["-i", str(tmp_path / "missing"), "-o", str(tmp_path)])
    assert r.returncode == 1 and "!!ERROR!!" in r.stderr


def test_run_builds_the_system_then_needs_a_device(tmp_path):
    from sdmd_gb300 import engine
    if engine.device_count() > 0:
        return   # on a GPU machine the run itself is tests/test_gpu_cli.py
    ind = tmp_path / "in"
    shutil.copytree(os.path.join(REPO, "tests", "golden", "cli_ala10", "in"), ind)
    shutil.copytree(os.path.join(REPO, "sdmd_gb300", "data", "Library_Ding"), ind / "Library_Ding")
    r = run(["-i", str(ind), "-o", str(tmp_path), "-f", "sys.gro"], env=dict(os.environ, SDMD_DEBUG_RANDOM="1"))
    assert r.returncode == 1
    assert "| timestep                       40.00 |" in r.stdout   # parameters read, system built
    assert "!!ERROR!!: sdmd_gpu_create" in r.stderr
