#!/usr/bin/env python3
"""Generate tests/golden/cli_ala10/: a whole run of the reference's own sDMD
executable, for the end-to-end comparison with the engine's executable.

Needs the reference's executable built by the oracle recipe
(oracle/ref/Makefile -> oracle/_ref/sDMD: the reference's unmodified sources,
its own main, -DDEBUG_RANDOM for the fixed seed).  The run: the ALA x 10 chain of
the ala10_nvt fixture, Andersen NVT, Time 40 with Dump_Rate 10, and the optional
outputs -pot -kin -tem -HBn.  Kept: the inputs (in/parameter.txt, in/sys.gro; the
force-field library is the package's) and the outputs (expected/): the text files
and the last checkpoint.  cli_ala10_continue/ is the continue run from that
checkpoint to Time 70 (its in/ also holds the checkpoint it reads).

Usage: python tests/golden/make_cli_golden.py
"""
import os
import shutil
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
EXE = os.path.join(REPO, "oracle", "_ref", "sDMD")
CASE = os.path.join(HERE, "cli_ala10")
CONT = os.path.join(HERE, "cli_ala10_continue")
FLAGS = ["-pot", "-kin", "-tem", "-HBn"]
OUTPUTS = ["out_trj.gro", "out_cnt.txt", "out_pot.txt", "out_kin.txt", "out_tem.txt", "out_HBn.txt", "savedData.dat",
           "out_log.txt", "SysInfo.dat"]


def parameters(text, time, dump):
    lines = text.splitlines()
    for k, line in enumerate(lines):
        if line.startswith("Time "):
            lines[k] = f"Time               {time}"
        elif line.startswith("Dump_Rate"):
            lines[k] = f"Dump_Rate          {dump}"
    return "\n".join(lines) + "\n"


def run_case(ind, case_dir, extra_inputs=()):
    outd = tempfile.mkdtemp(prefix="sdmd_cli_out_")
    for name in extra_inputs:   # a continue run reads its checkpoint from the output folder
        shutil.copy(os.path.join(ind, name), os.path.join(outd, name))
    subprocess.run([EXE, "-i", ind, "-o", outd, "-f", "sys.gro", *FLAGS], check=True, stdout=subprocess.DEVNULL,
                   timeout=600)
    os.makedirs(os.path.join(case_dir, "in"), exist_ok=True)
    os.makedirs(os.path.join(case_dir, "expected"), exist_ok=True)
    for name in ("parameter.txt", "sys.gro", *extra_inputs):
        shutil.copy(os.path.join(ind, name), os.path.join(case_dir, "in", name))
    for name in OUTPUTS:
        if os.path.exists(os.path.join(outd, name)):   # SysInfo.dat: new runs only
            shutil.copy(os.path.join(outd, name), os.path.join(case_dir, "expected", name))
    with open(os.path.join(case_dir, "expected", "flags.txt"), "w") as f:
        f.write(" ".join(FLAGS) + "\n")
    shutil.rmtree(outd)


def main():
    if not os.path.exists(EXE):
        raise SystemExit(f"{EXE} is missing: build it with make -C oracle/ref")
    d = np.load(os.path.join(HERE, "ala10_nvt.npz"))
    work = tempfile.mkdtemp(prefix="sdmd_cli_golden_")
    ind, outd = os.path.join(work, "in"), os.path.join(work, "out")
    os.makedirs(ind)
    os.makedirs(outd)
    shutil.copytree(os.path.join(REPO, "sdmd_gb300", "data", "Library_Ding"), os.path.join(ind, "Library_Ding"))
    param = parameters(bytes(d["meta/parameter"]).decode(), 40, 10.0)
    with open(os.path.join(ind, "parameter.txt"), "w") as f:
        f.write(param)
    with open(os.path.join(ind, "sys.gro"), "wb") as f:
        f.write(bytes(d["meta/gro"]))
    run_case(ind, CASE)
    # the continue run: the new run's checkpoint, Time 70 (> currenttime + Dump_Rate)
    shutil.copy(os.path.join(CASE, "expected", "savedData.dat"), os.path.join(ind, "savedData.dat"))
    with open(os.path.join(ind, "parameter.txt"), "w") as f:
        f.write(parameters(param, 70, 10.0).replace("new", "continue", 1))
    run_case(ind, CONT, ("savedData.dat",))
    shutil.rmtree(work)
    print("wrote", CASE, CONT)


if __name__ == "__main__":
    main()
