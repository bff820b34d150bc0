"""The exchange server's rearrange() (src/Server.c:145-192): the oracle's
restatement against the reference's own Server.c (no GPU).

tests/golden/remd_rearrange.npz holds seeded replica ladders run through the
reference (oracle/ref/server_driver.c): the srand seed, the starting (num, T)
records, each round's energies and each round's resulting (num, T).  The oracle,
fed the same energies and the same rand() stream, must give the same records
round after round.  The device exchange is checked against the oracle in
tests/test_gpu_remd.py.
"""
import ctypes as C

import numpy as np

from oracle import oracle as O
from sdmd_gb300.system import glibc_rng_state, sdmd_rng


def test_rearrange_matches_the_reference_server(golden):
    d = golden("remd_rearrange")
    for c in range(int(d["meta/cases"][0])):
        seed = int(d[f"c{c}/seed"][0])
        T = np.ascontiguousarray(d[f"c{c}/T0"], dtype=np.float64).copy()
        num = np.ascontiguousarray(d[f"c{c}/num0"], dtype=np.int32).copy()
        n = len(num)
        st = glibc_rng_state(seed)   # srand(seed) as the server's main does
        rng = sdmd_rng()
        for i in range(31):
            rng.tab[i] = int(st[i])
        rng.front, rng.rear = int(st[31]), int(st[32])
        energies = d[f"c{c}/E"]
        for r in range(energies.shape[0]):
            E = np.ascontiguousarray(energies[r], dtype=np.float64)
            O.lib().oracle_remd_rearrange(n, num.ctypes.data_as(C.POINTER(C.c_int32)),
                                          T.ctypes.data_as(C.POINTER(C.c_double)),
                                          E.ctypes.data_as(C.POINTER(C.c_double)), C.byref(rng))
            assert np.array_equal(num, d[f"c{c}/num"][r]), (c, r)
            assert np.array_equal(T, d[f"c{c}/T"][r]), (c, r)
