#!/usr/bin/env python3
"""Generate tests/golden/remd_ala10/: a whole REMD run of the reference's own
executables, for the end-to-end comparison with the engine's REMD launcher.

Needs the reference's sDMD and sServer built by the oracle recipe
(oracle/ref/Makefile -> oracle/_ref/: the reference's unmodified sources, its own
mains, -DDEBUG_RANDOM for the clients' fixed seed).  The run is what the
reference's launcher sREMD (src/REMDExec.c) starts, with the server's seed fixed
instead of time(NULL): sServer <port> 3 <seed>, then one sDMD client per replica,
a second apart as the launcher starts them, each with the -args flags and
"-REMD localhost <port> <T> <num> <rate> <id>".  The system is the ALA x 10 chain
of the ala10_nvt fixture, Andersen NVT at T(reduced) "no", Time 30 with Dump_Rate
10; REMDConfig.txt: 275 350 450 K, ExchangeRate 5.  Kept: the inputs (in/) and
every replica's outputs (expected/; SysInfo0.dat stands for the three SysInfo
files, which differ only in the reference's heap addresses).
tests/golden/remd_ala10_continue is the continue run from those checkpoints to
Time 50 (its in/ also holds the checkpoints it reads from the output folder).

Usage: python tests/golden/make_remd_golden.py
"""
import os
import shutil
import socket
import subprocess
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
REF = os.path.join(REPO, "oracle", "_ref")
CASE = os.path.join(HERE, "remd_ala10")
CONT = os.path.join(HERE, "remd_ala10_continue")
TEMPS_K = [275, 350, 450]
EXCHANGE = 5
SERVER_SEED = 12345
FLAGS = ["-pot", "-tem"]
PER_REPLICA = ["out_trj{}.gro", "out_cnt{}.txt", "out_pot{}.txt", "out_tem{}.txt", "savedData{}.dat", "out_log{}.txt",
               "SysInfo{}.dat", "out_REMD{}.txt"]
BOLTZMANN = 0.0019872041


def parameters(text):
    lines = text.splitlines()
    for k, line in enumerate(lines):
        if line.startswith("Time "):
            lines[k] = "Time               30"
        elif line.startswith("Dump_Rate"):
            lines[k] = "Dump_Rate          10.0"
        elif line.startswith("T(reduced)"):
            lines[k] = "T(reduced)         no"
    return "\n".join(lines) + "\n"


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def run_case(ind, outd, port, case, extra_inputs=()):
    """sServer and one sDMD client per replica, as the launcher starts them; the
    inputs and every replica's outputs are kept in `case`."""
    server = subprocess.Popen([os.path.join(REF, "sServer"), str(port), str(len(TEMPS_K)), str(SERVER_SEED)],
                              stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
    clients = []
    for k, t in enumerate(TEMPS_K):
        time.sleep(1.0)   # the launcher starts client k a second after client k - 1
        cmd = [os.path.join(REF, "sDMD"), "-i", ind, "-o", outd, "-f", "sys.gro", *FLAGS, "-REMD", "localhost",
               str(port), "%lf" % (t * BOLTZMANN), str(k + 1), str(EXCHANGE), str(k)]
        clients.append(subprocess.Popen(cmd, stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL))
    for c in clients:
        if c.wait(timeout=600):
            raise SystemExit("a client failed")
    if server.wait(timeout=60):
        raise SystemExit("the server failed")
    if os.path.exists(case):
        shutil.rmtree(case)
    os.makedirs(os.path.join(case, "in"))
    os.makedirs(os.path.join(case, "expected"))
    for name in ("parameter.txt", "sys.gro", "REMDConfig.txt", *extra_inputs):
        shutil.copy(os.path.join(ind, name), os.path.join(case, "in", name))
    for k in range(len(TEMPS_K)):
        for pattern in PER_REPLICA:
            name = pattern.format(k)
            if pattern.startswith("SysInfo") and (k or not os.path.exists(os.path.join(outd, name))):
                continue   # the replicas' SysInfo files differ only in heap addresses: one is kept
            shutil.copy(os.path.join(outd, name), os.path.join(case, "expected", name))
    with open(os.path.join(case, "expected", "launch.txt"), "w") as f:
        f.write(f"server_seed {SERVER_SEED}\nflags {' '.join(FLAGS)}\n")


def main():
    for exe in ("sDMD", "sServer"):
        if not os.path.exists(os.path.join(REF, exe)):
            raise SystemExit(f"{REF}/{exe} is missing: build it with make -C oracle/ref")
    d = np.load(os.path.join(HERE, "ala10_nvt.npz"))
    work = tempfile.mkdtemp(prefix="sdmd_remd_golden_")
    ind, outd = os.path.join(work, "in"), os.path.join(work, "out")
    os.makedirs(ind)
    os.makedirs(outd)
    shutil.copytree(os.path.join(REPO, "sdmd_gb300", "data", "Library_Ding"), os.path.join(ind, "Library_Ding"))
    param = parameters(bytes(d["meta/parameter"]).decode())
    with open(os.path.join(ind, "parameter.txt"), "w") as f:
        f.write(param)
    with open(os.path.join(ind, "sys.gro"), "wb") as f:
        f.write(bytes(d["meta/gro"]))
    port = free_port()
    with open(os.path.join(ind, "REMDConfig.txt"), "w") as f:
        f.write("#REPLICA EXCHANGE MD CONFIGURATION FILE\n")
        f.write(f"ReplicaNum              = {len(TEMPS_K)}\n")
        f.write("Temperatures            = " + " ".join(str(t) for t in TEMPS_K) + "\n")
        f.write(f"SocketPort              = {port}\n")
        f.write(f"ExchangeRate            = {EXCHANGE}\n")
    run_case(ind, outd, port, CASE)
    # the continue run: every replica from its checkpoint (read from the output
    # folder, and its REMDInfo -- port included -- from the file) to Time 50
    saved = [f"savedData{k}.dat" for k in range(len(TEMPS_K))]
    outd2 = os.path.join(work, "out2")
    os.makedirs(outd2)
    for name in saved:
        shutil.copy(os.path.join(outd, name), os.path.join(ind, name))
        shutil.copy(os.path.join(outd, name), os.path.join(outd2, name))
    with open(os.path.join(ind, "parameter.txt"), "w") as f:
        f.write(param.replace("Time               30", "Time               50").replace("new", "continue", 1))
    run_case(ind, outd2, port, CONT, saved)
    shutil.rmtree(work)
    print("wrote", CASE, CONT)


if __name__ == "__main__":
    main()
