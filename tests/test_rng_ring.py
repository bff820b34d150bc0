"""The sample commit's skip of consumed rand() draws (no GPU).

glibc's TYPE_3 state keeps front == rear + 3 (mod 31).  The commit kernel
rotates the table so that rear sits at index 0, draws whole blocks of 31 with
static indices (R[(3 + s) % 31] += R[s]), then the remainder, and writes the
table back with rear advanced by the number of draws.  Replayed here, it must
leave the same state as that many calls of the library's sdmd_rng_next, which
is itself checked against glibc's rand().
"""
import ctypes as C

import numpy as np
import pytest

from sdmd_gb300.system import glibc_rng_state, sdmd_rng


@pytest.fixture(scope="module")
def gpu_lib():
    """The engine library (built for sm_103a; its host-side RNG helpers run on CPU)."""
    from sdmd_gb300 import build
    return C.CDLL(build.build_gpu())


def ring_skip(st, m):
    tab, front, rear = [int(v) & 0xFFFFFFFF for v in st[:31]], int(st[31]), int(st[32])
    assert front == (rear + 3) % 31
    R = [tab[(rear + k) % 31] for k in range(31)]
    for _ in range(m // 31):
        for s in range(31):
            R[(3 + s) % 31] = (R[(3 + s) % 31] + R[s]) & 0xFFFFFFFF
    for s in range(m % 31):
        R[(3 + s) % 31] = (R[(3 + s) % 31] + R[s]) & 0xFFFFFFFF
    out = [0] * 31
    for k in range(31):
        out[(rear + k) % 31] = R[k]
    rear2 = (rear + m) % 31
    return np.array(out, np.uint32).view(np.int32), (rear2 + 3) % 31, rear2


@pytest.mark.parametrize("seed,skip", [(1, 0), (1575263273, 5), (20201, 17), (7, 1000)])
def test_ring_skip_equals_sequential_draws(gpu_lib, seed, skip):
    from sdmd_gb300 import engine
    for m in (0, 1, 2, 30, 31, 32, 61, 62, 100, 1000, 4097):
        st = glibc_rng_state(seed, skip)
        tab, front, rear = ring_skip(st, m)
        r = sdmd_rng()
        for i in range(31):
            r.tab[i] = int(st[i])
        r.front, r.rear = int(st[31]), int(st[32])
        for _ in range(m):
            engine.lib().sdmd_rng_next(C.byref(r))
        assert np.array_equal(tab, np.array([r.tab[i] for i in range(31)], np.int32)), (seed, skip, m)
        assert (front, rear) == (r.front, r.rear), (seed, skip, m)
