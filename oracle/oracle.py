"""ctypes front end of the CPU oracle (oracle/sdmd_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
bench.py's cpu_baseline / reference leg, never by the product package.
"""
import ctypes as C
import os
import subprocess

import numpy as np

from sdmd_gb300.system import TRACE_DTYPE, sdmd_rng, sdmd_system, sdmd_trace_rec

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
LIB = os.path.join(HERE, "liboracle_sdmd.so")
SRC = os.path.join(HERE, "sdmd_oracle.c")


def build(force=False):
    """Compile the oracle restatement (plain C, no FP contraction)."""
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= max(
            os.path.getmtime(SRC), os.path.getmtime(os.path.join(HERE, "sdmd_oracle.h")),
            os.path.getmtime(os.path.join(REPO, "include", "sdmd_gpu.h"))):
        return LIB
    tmp = LIB + ".tmp"
    subprocess.check_call(["gcc", "-O2", "-std=c99", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared",
                           "-I" + os.path.join(REPO, "include"), "-o", tmp, SRC, "-lm"])
    os.replace(tmp, LIB)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        _lib = C.CDLL(build())
        P = C.POINTER
        _lib.oracle_predict_all.argtypes = [P(sdmd_system)]
        _lib.oracle_loop_create.argtypes = [P(sdmd_system)]
        _lib.oracle_loop_create.restype = C.c_void_p
        _lib.oracle_loop_destroy.argtypes = [C.c_void_p]
        _lib.oracle_run.argtypes = [C.c_void_p, C.c_int64, C.c_double, P(sdmd_trace_rec), C.c_int64, P(C.c_int64)]
        _lib.oracle_cbt.argtypes = [C.c_void_p, P(C.c_int32), P(C.c_int32)]
        _lib.oracle_potential_energy.argtypes = [P(sdmd_system)]
        _lib.oracle_potential_energy.restype = C.c_double
        _lib.oracle_kinetic_energy.argtypes = [P(sdmd_system)]
        _lib.oracle_kinetic_energy.restype = C.c_double
        _lib.oracle_rand.argtypes = [P(sdmd_rng)]
        _lib.oracle_rand.restype = C.c_int32
        _lib.oracle_mb.argtypes = [P(sdmd_rng), C.c_double, C.c_double]
        _lib.oracle_mb.restype = C.c_double
        _lib.oracle_log.argtypes = [C.c_double]
        _lib.oracle_log.restype = C.c_double
        _lib.oracle_remd_rearrange.argtypes = [C.c_int32, P(C.c_int32), P(C.c_double), P(C.c_double), P(sdmd_rng)]
        _lib.oracle_run_until.argtypes = [C.c_void_p, C.c_double, C.c_double, P(C.c_int64)]
        _lib.oracle_potential_energy_counted.argtypes = [P(sdmd_system)]
        _lib.oracle_potential_energy_counted.restype = C.c_double
    return _lib


def predict_all(system):
    """Full-rebuild sweep on a sdmd_gb300.system.System (in place)."""
    st = system.struct()
    rc = lib().oracle_predict_all(C.byref(st))
    system.pull_scalars(st)
    return rc


class Loop:
    """Event loop over one System; the System's arrays are updated in place."""

    def __init__(self, system):
        self.system = system
        self.st = system.struct()
        self.h = lib().oracle_loop_create(C.byref(self.st))

    def run(self, max_events, t_end=None, trace_cap=0):
        if t_end is None:
            t_end = self.st.t_end
        tr = np.zeros(max(trace_cap, 1), TRACE_DTYPE)
        n = C.c_int64(0)
        rc = lib().oracle_run(self.h, int(max_events), float(t_end),
                              tr.ctypes.data_as(C.POINTER(sdmd_trace_rec)), int(trace_cap), C.byref(n))
        self.system.pull_scalars(self.st)
        return rc, tr[:min(n.value, trace_cap)], n.value

    def run_until(self, stop_time, t_end=None):
        """Run until the first executed event at time >= stop_time (REMDRun's exchange point)."""
        if t_end is None:
            t_end = self.st.t_end
        n = C.c_int64(0)
        rc = lib().oracle_run_until(self.h, float(t_end), float(stop_time), C.byref(n))
        self.system.pull_scalars(self.st)
        return rc

    def potential_energy_counted(self):
        """CalPotenE on the loop's own state, its FindPair warnings counted (REMDRun)."""
        e = lib().oracle_potential_energy_counted(C.byref(self.st))
        self.system.pull_scalars(self.st)
        return e

    def cbt(self):
        n = self.system.n
        node = np.zeros(2 * n, np.int32)
        leaf = np.zeros(n + 1, np.int32)
        lib().oracle_cbt(self.h, node.ctypes.data_as(C.POINTER(C.c_int32)), leaf.ctypes.data_as(C.POINTER(C.c_int32)))
        return node, leaf

    def close(self):
        if self.h:
            lib().oracle_loop_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()


def potential_energy(system):
    return lib().oracle_potential_energy(C.byref(system.struct()))


def kinetic_energy(system):
    return lib().oracle_kinetic_energy(C.byref(system.struct()))
