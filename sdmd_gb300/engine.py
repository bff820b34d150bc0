"""Python front end of the GB300 event-loop engine (ctypes over libsdmd_gpu.so).

The C ABI (include/sdmd_gpu.h) is the product boundary; this module is the
thin host-side mirror used by the tests and the benchmark.  There is no CPU
fallback: if the CUDA library is missing or no device is present, every call
raises.
"""
import ctypes as C
import os

import numpy as np

from .system import TRACE_DTYPE, sdmd_error_info, sdmd_opts, sdmd_rng, sdmd_system, sdmd_trace_rec

HERE = os.path.dirname(os.path.abspath(__file__))
GPU_LIB = os.path.join(HERE, "libsdmd_gpu.so")

ADVANCE_EAGER, ADVANCE_LAZY = 0, 1
SCREEN_FP64, SCREEN_FP32 = 0, 1

ABI_FUNCS = ["sdmd_gpu_abi_version", "sdmd_gpu_device_count", "sdmd_gpu_strerror", "sdmd_gpu_create",
             "sdmd_gpu_destroy", "sdmd_gpu_prepare", "sdmd_gpu_run", "sdmd_gpu_download", "sdmd_gpu_trace",
             "sdmd_gpu_last_ms", "sdmd_gpu_last_error", "sdmd_rng_seed", "sdmd_rng_next", "sdmd_rng_skip",
             "sdmd_gpu_prepare_noalloc", "sdmd_gpu_last_run_stats", "sdmd_gpu_energies", "sdmd_gpu_run_remd",
             "sdmd_gpu_launch_info", "sdmd_gpu_run_to_dump", "sdmd_gpu_run_to_stops", "sdmd_gpu_exchange"]
LOOP_KERNELS = {0: "loop_kernel_fp64", 1: "loop_kernel_screen", 2: "loop_kernel_screen_r128",
                3: "loop_kernel_screen_coop", 4: "loop_kernel_screen_coop512"}

_lib = None


class sdmd_remd(C.Structure):
    _fields_ = [("num", C.POINTER(C.c_int32)), ("T", C.POINTER(C.c_double)), ("E", C.POINTER(C.c_double)),
                ("every_events", C.c_int64), ("every_time", C.c_double), ("rng", sdmd_rng),
                ("attempted", C.c_int64), ("accepted", C.c_int64), ("exchanges_done", C.c_int64)]


SDMD_EUNSUPPORTED = -17   # include/sdmd_gpu.h


class EngineError(RuntimeError):
    def __init__(self, code, where, info=None):
        self.code = code
        msg = f"{where}: {strerror(code)} ({code})"
        if info is not None and info.code:
            msg += f" [system {info.system}, atom {info.atom}, event {info.event}]"
        super().__init__(msg)


def lib():
    """Load libsdmd_gpu.so (built by __graft_entry__.build()).  Raises if absent."""
    global _lib
    if _lib is None:
        if not os.path.exists(GPU_LIB):
            raise RuntimeError(f"{GPU_LIB} is missing: run __graft_entry__.build() (no CPU fallback exists)")
        L = C.CDLL(GPU_LIB)
        P = C.POINTER
        L.sdmd_gpu_abi_version.restype = C.c_int
        L.sdmd_gpu_device_count.argtypes = [P(C.c_int32)]
        L.sdmd_gpu_strerror.argtypes = [C.c_int]
        L.sdmd_gpu_strerror.restype = C.c_char_p
        L.sdmd_gpu_create.argtypes = [P(sdmd_system), C.c_int32, P(sdmd_opts), P(C.c_void_p)]
        L.sdmd_gpu_destroy.argtypes = [C.c_void_p]
        L.sdmd_gpu_destroy.restype = None
        L.sdmd_gpu_prepare.argtypes = [C.c_void_p, C.c_int32]
        L.sdmd_gpu_prepare_noalloc.argtypes = [C.c_void_p, C.c_int32]
        L.sdmd_gpu_run.argtypes = [C.c_void_p, C.c_int64, C.c_double]
        L.sdmd_gpu_download.argtypes = [C.c_void_p, P(sdmd_system), C.c_int32]
        L.sdmd_gpu_trace.argtypes = [C.c_void_p, C.c_int32, P(sdmd_trace_rec), C.c_int32, P(C.c_int32)]
        L.sdmd_gpu_last_ms.argtypes = [C.c_void_p, P(C.c_double), P(C.c_double)]
        L.sdmd_gpu_last_error.argtypes = [C.c_void_p, P(sdmd_error_info)]
        L.sdmd_gpu_last_run_stats.argtypes = [C.c_void_p, P(C.c_int64), P(C.c_int64), P(C.c_double)]
        L.sdmd_gpu_energies.argtypes = [C.c_void_p, P(C.c_double), P(C.c_double)]
        L.sdmd_gpu_run_remd.argtypes = [C.c_void_p, C.c_int64, C.c_double, P(sdmd_remd)]
        L.sdmd_gpu_run_to_stops.argtypes = [C.c_void_p, P(C.c_double), P(C.c_int64), C.c_double, P(C.c_int32)]
        L.sdmd_gpu_exchange.argtypes = [C.c_void_p, P(sdmd_remd)]
        L.sdmd_gpu_launch_info.argtypes = [C.c_void_p, P(C.c_int32), P(C.c_int32), P(C.c_int32), P(C.c_int32)]
        L.sdmd_rng_seed.argtypes = [P(sdmd_rng), C.c_uint32]
        L.sdmd_rng_seed.restype = None
        L.sdmd_rng_next.argtypes = [P(sdmd_rng)]
        L.sdmd_rng_next.restype = C.c_int32
        L.sdmd_rng_skip.argtypes = [P(sdmd_rng), C.c_int64]
        L.sdmd_rng_skip.restype = None
        _lib = L
    return _lib


def strerror(code):
    try:
        return lib().sdmd_gpu_strerror(int(code)).decode()
    except Exception:
        return "error"


def device_count():
    n = C.c_int32(0)
    lib().sdmd_gpu_device_count(C.byref(n))
    return n.value


class Engine:
    """A handle over a batch of systems (sdmd_gb300.system.System objects)."""

    def __init__(self, systems, advance=ADVANCE_EAGER, screen=SCREEN_FP64, threads=0, trace=0, device=0, helpers=0):
        """helpers: blocks of the eager advance on the screened path (sdmd_opts.helper_blocks:
        0 automatic, -1 off, k > 0 exactly k)."""
        self.systems = list(systems)
        self.structs = (sdmd_system * len(self.systems))(*[s.struct() for s in self.systems])
        o = sdmd_opts()
        o.advance, o.screen, o.threads_per_system, o.device, o.trace_capacity = advance, screen, threads, device, trace
        o.helper_blocks = helpers
        self.opts = o
        h = C.c_void_p()
        rc = lib().sdmd_gpu_create(self.structs, len(self.systems), C.byref(o), C.byref(h))
        if rc:
            raise EngineError(rc, "sdmd_gpu_create")
        self.h = h

    def _check(self, rc, where):
        if rc:
            info = sdmd_error_info()
            lib().sdmd_gpu_last_error(self.h, C.byref(info))
            raise EngineError(rc, where, info)

    def prepare(self, full=True):
        self._check(lib().sdmd_gpu_prepare(self.h, 1 if full else 0), "sdmd_gpu_prepare")

    def prepare_noalloc(self, full=True):
        """sdmd_gpu_prepare_noalloc: the same sweep with its scratch in the library's static array."""
        self._check(lib().sdmd_gpu_prepare_noalloc(self.h, 1 if full else 0), "sdmd_gpu_prepare_noalloc")

    def run(self, max_events, t_end=0.0):
        self._check(lib().sdmd_gpu_run(self.h, int(max_events), float(t_end)), "sdmd_gpu_run")

    def download(self):
        """Copy device state back into the System objects' arrays and scalars."""
        self._check(lib().sdmd_gpu_download(self.h, self.structs, len(self.systems)), "sdmd_gpu_download")
        for s, st in zip(self.systems, self.structs):
            s.pull_scalars(st)

    def trace(self, s=0, cap=None):
        cap = cap if cap is not None else max(self.opts.trace_capacity, 1)
        out = np.zeros(cap, TRACE_DTYPE)
        n = C.c_int32(0)
        self._check(lib().sdmd_gpu_trace(self.h, s, out.ctypes.data_as(C.POINTER(sdmd_trace_rec)), cap,
                                         C.byref(n)), "sdmd_gpu_trace")
        return out[:n.value]

    def last_ms(self):
        a, b = C.c_double(0), C.c_double(0)
        lib().sdmd_gpu_last_ms(self.h, C.byref(a), C.byref(b))
        return a.value, b.value

    def energies(self):
        """(potential, kinetic) energy of every system: CalPotenE / CalKinetE on the device."""
        n = len(self.systems)
        pot, kin = np.zeros(n), np.zeros(n)
        self._check(lib().sdmd_gpu_energies(self.h, pot.ctypes.data_as(C.POINTER(C.c_double)),
                                            kin.ctypes.data_as(C.POINTER(C.c_double))), "sdmd_gpu_energies")
        return pot, kin

    def run_remd(self, n_exchanges, num, T, rng, every_events=0, every_time=0.0, t_end=0.0, attempted=0,
                 accepted=0):
        """Replica exchange on the device (every system is a replica).  num / T are the
        replicas' (ladder index, temperature) records, rng the exchange server's rand()
        state (33 ints).  Returns dict(num, T, E, rng, attempted, accepted, done)."""
        n = len(self.systems)
        num = np.ascontiguousarray(num, np.int32).copy()
        T = np.ascontiguousarray(T, np.float64).copy()
        E = np.zeros(n)
        x = sdmd_remd()
        x.num = num.ctypes.data_as(C.POINTER(C.c_int32))
        x.T = T.ctypes.data_as(C.POINTER(C.c_double))
        x.E = E.ctypes.data_as(C.POINTER(C.c_double))
        x.every_events = int(every_events)
        x.every_time = float(every_time)
        for i in range(31):
            x.rng.tab[i] = int(rng[i])
        x.rng.front, x.rng.rear = int(rng[31]), int(rng[32])
        x.attempted, x.accepted = int(attempted), int(accepted)
        self._check(lib().sdmd_gpu_run_remd(self.h, int(n_exchanges), float(t_end), C.byref(x)), "sdmd_gpu_run_remd")
        out_rng = np.array([x.rng.tab[i] for i in range(31)] + [x.rng.front, x.rng.rear], np.int32)
        return {"num": num, "T": T, "E": E, "rng": out_rng, "attempted": x.attempted, "accepted": x.accepted,
                "done": x.exchanges_done}

    def run_to_stops(self, stop_time, max_events, t_end=0.0):
        """Each system k runs to its first executed event at time >= stop_time[k]
        (<= 0: none) or max_events[k] executed events (0: it does not run).
        Returns at_stop (1 where a system stopped at such an event)."""
        n = len(self.systems)
        stop = np.ascontiguousarray(stop_time, np.float64)
        lim = np.ascontiguousarray(max_events, np.int64)
        at = np.zeros(n, np.int32)
        self._check(lib().sdmd_gpu_run_to_stops(self.h, stop.ctypes.data_as(C.POINTER(C.c_double)),
                                                lim.ctypes.data_as(C.POINTER(C.c_int64)), float(t_end),
                                                at.ctypes.data_as(C.POINTER(C.c_int32))), "sdmd_gpu_run_to_stops")
        return at

    def exchange(self, num, T, rng, attempted=0, accepted=0):
        """One exchange now (CalPotenE, one rearrange() pass over replicas with T != 0,
        new thermostat targets).  Returns dict(num, T, E, rng, attempted, accepted)."""
        n = len(self.systems)
        num = np.ascontiguousarray(num, np.int32).copy()
        T = np.ascontiguousarray(T, np.float64).copy()
        E = np.zeros(n)
        x = sdmd_remd()
        x.num = num.ctypes.data_as(C.POINTER(C.c_int32))
        x.T = T.ctypes.data_as(C.POINTER(C.c_double))
        x.E = E.ctypes.data_as(C.POINTER(C.c_double))
        for i in range(31):
            x.rng.tab[i] = int(rng[i])
        x.rng.front, x.rng.rear = int(rng[31]), int(rng[32])
        x.attempted, x.accepted = int(attempted), int(accepted)
        self._check(lib().sdmd_gpu_exchange(self.h, C.byref(x)), "sdmd_gpu_exchange")
        out_rng = np.array([x.rng.tab[i] for i in range(31)] + [x.rng.front, x.rng.rear], np.int32)
        return {"num": num, "T": T, "E": E, "rng": out_rng, "attempted": x.attempted, "accepted": x.accepted}

    def launch_info(self):
        """dict(threads, helper_blocks, staged, loop_kernel) of the handle's event-loop launch."""
        v = [C.c_int32(0) for _ in range(4)]
        self._check(lib().sdmd_gpu_launch_info(self.h, *[C.byref(x) for x in v]), "sdmd_gpu_launch_info")
        return {"threads": v[0].value, "helper_blocks": v[1].value, "staged": bool(v[2].value),
                "loop_kernel": LOOP_KERNELS.get(v[3].value, str(v[3].value))}

    def last_run_stats(self):
        """(kernels launched, event-loop kernels launched, event-loop kernel ms) of the last run."""
        a, b, c = C.c_int64(0), C.c_int64(0), C.c_double(0)
        lib().sdmd_gpu_last_run_stats(self.h, C.byref(a), C.byref(b), C.byref(c))
        return a.value, b.value, c.value

    def close(self):
        if getattr(self, "h", None):
            lib().sdmd_gpu_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


def autotune_threads(systems, advance=ADVANCE_EAGER, screen=SCREEN_FP64, candidates=(64, 128, 256), events=400,
                     device=0):
    """Pick the threads per system (CTA size) that runs `events` executed events per
    system fastest on copies of `systems` (full-rebuild sweep first, one warm-up
    run, then a timed run).  A size the handle does not support for this batch
    (more than 256 threads without helper blocks) is skipped.  Returns
    (best, {threads: events/s})."""
    rates = {}
    for t in candidates:
        work = [s.copy() for s in systems]
        try:
            e = Engine(work, advance=advance, screen=screen, threads=t, device=device)
        except EngineError as err:
            if err.code == SDMD_EUNSUPPORTED and t > 256:
                continue
            raise
        with e:
            e.prepare(full=True)
            e.run(max(events // 4, 16))
            e.run(events)
            ms = e.last_ms()[1]
        rates[t] = events * len(systems) / max(ms, 1e-6) * 1e3
    best = max(rates, key=rates.get)
    return best, rates

