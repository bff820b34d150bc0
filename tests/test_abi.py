"""The C-ABI library builds, loads and exports every symbol the header declares
(no GPU needed: no compute call is made)."""
import ctypes as C
import os
import re

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    src = open(os.path.join(REPO, "include", "sdmd_gpu.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(sdmd_\w+)\s*\(", src)))


@pytest.fixture(scope="module")
def gpu_lib():
    from sdmd_gb300 import build
    return C.CDLL(build.build_gpu())


def test_header_declares_the_engine_api():
    names = declared_functions()
    for n in ["sdmd_gpu_create", "sdmd_gpu_prepare", "sdmd_gpu_run", "sdmd_gpu_download", "sdmd_gpu_destroy"]:
        assert n in names


def test_library_exports_every_declared_symbol(gpu_lib):
    missing = [n for n in declared_functions() if not hasattr(gpu_lib, n)]
    assert not missing, missing


def test_struct_layout_matches_header(gpu_lib):
    """ctypes mirror sizes equal the C sizes (checked by compiling a probe)."""
    import subprocess
    import tempfile
    from sdmd_gb300 import system as S
    probe = r'''
#include <stdio.h>
#include <stddef.h>
#include "sdmd_gpu.h"
int main(void){printf("%zu %zu %zu %zu %zu %zu\n", sizeof(sdmd_system), sizeof(sdmd_trace_rec), sizeof(sdmd_opts),
 sizeof(sdmd_rng), sizeof(sdmd_counters), offsetof(sdmd_system, time)); return 0;}
'''
    with tempfile.TemporaryDirectory() as t:
        with open(os.path.join(t, "p.c"), "w") as f:
            f.write(probe)
        exe = os.path.join(t, "p")
        subprocess.check_call(["gcc", "-I" + os.path.join(REPO, "include"), "-o", exe, os.path.join(t, "p.c")])
        got = [int(v) for v in subprocess.check_output([exe]).split()]
    want = [C.sizeof(S.sdmd_system), C.sizeof(S.sdmd_trace_rec), C.sizeof(S.sdmd_opts), C.sizeof(S.sdmd_rng),
            C.sizeof(S.sdmd_counters), S.sdmd_system.time.offset]
    assert got == want


def test_host_rng_helpers_match_glibc(gpu_lib):
    """sdmd_rng_seed/next reproduce glibc srand()/rand() (host-only calls)."""
    import ctypes.util
    from sdmd_gb300 import engine, system
    libc = C.CDLL(ctypes.util.find_library("c"))
    r = system.sdmd_rng()
    engine.lib().sdmd_rng_seed(C.byref(r), 1575263273)
    libc.srand(1575263273)
    assert [engine.lib().sdmd_rng_next(C.byref(r)) for _ in range(5000)] == [libc.rand() for _ in range(5000)]


def test_struct_views_the_current_arrays():
    """System.struct() writes every array's address into the sdmd_system it hands
    to the C ABI, reuses them while the arrays are the same objects, and takes
    the new ones when an array is replaced; scalars and the RNG ring are copied."""
    from sdmd_gb300.system import STATIC_ARRAYS, DYNAMIC_ARRAYS, from_fixture
    from tests.conftest import load_golden
    s = from_fixture(load_golden("ala10_nvt"), "pre")
    addr = lambda p: C.cast(p, C.c_void_p).value
    st = s.struct()
    for name, _ in STATIC_ARRAYS + DYNAMIC_ARRAYS:
        assert addr(getattr(st, name)) == s.a[name].ctypes.data, name
    assert [st.rng.tab[i] for i in range(31)] + [st.rng.front, st.rng.rear] == [int(v) for v in s.rng]
    assert st.n_atoms == s.n and st.time == s.time
    s.a["vx"] = s.a["vx"].copy()                      # a replaced array is seen at once
    s.rng[3] += 1
    st = s.struct()
    assert addr(st.vx) == s.a["vx"].ctypes.data
    assert st.rng.tab[3] == int(s.rng[3])
    with pytest.raises(ValueError):
        s.a["x"] = s.a["x"][::2]                      # a strided view is refused
        s.struct()
