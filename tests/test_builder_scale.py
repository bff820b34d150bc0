"""The host-side builder against the reference's own set-up at multi-chain scale (no GPU).

The golden fixtures hold one to six chains.  Here 32 random 16-residue chains at
the 5 mM concentration of the 256-chain full-rebuild workload (about 5.3k atoms)
go through both set-ups from the same inputs: the reference's InputData and
Prepare (its O(N^2) neighbour search for SDEnergyMin, the random steepest descent
with one rand() draw per violation, GenerateVelocity, PBC and LinkList; run
through the bridge in a child process) and the host library's (the same pairs
found through a grid, in the same order).  Every array of the initial state --
coordinates after the minimisation, velocities, cells, topology, tables, HB
roles -- and the rand() state must agree bit for bit.
"""
import os
import shutil

import numpy as np
import pytest

from tests.test_ref_bridge import LIB, REPO, _bridge, _fill, in_child
from tests.test_builder import POOLED, steps

pytestmark = pytest.mark.skipif(not os.path.exists(LIB),
                                reason="the reference's sources are not here (oracle/_ref not built)")

DEBUG_SEED = 1575263273
N_CHAINS, LENGTH = 32, 16


def _child_setup(ind, outd, q):
    try:
        s = _fill(_bridge(ind, outd))
        q.put(("ok", s.a, s.scal, s.rng))
    except Exception as e:
        q.put(("error", repr(e)))


def test_builder_reproduces_the_reference_at_32_chains(tmp_path):
    from sdmd_gb300 import workloads as W
    from sdmd_gb300.host import build_system
    ind, outd = tmp_path / "in", tmp_path / "out"
    ind.mkdir()
    outd.mkdir()
    shutil.copytree(os.path.join(REPO, "sdmd_gb300", "data", "Library_Ding"), ind / "Library_Ding")
    d = np.load(os.path.join(REPO, "tests", "golden", "ala10_nvt.npz"))
    (ind / "parameter.txt").write_bytes(bytes(d["meta/parameter"]))
    edge = (N_CHAINS / (5.0e-3 * 6.02214076e23) * 1e27) ** (1.0 / 3.0)   # A, 5 mM
    gro = W.generate_gro(str(ind), W.random_sequences(N_CHAINS, LENGTH, 3), (edge, edge, edge), seed=3)
    (ind / "sys.gro").write_text(gro)
    a, scal, rng = in_child(_child_setup, str(ind), str(outd))
    s = build_system(str(ind), gro_text=gro, seed=DEBUG_SEED)
    assert s.n > 5000
    for k, v in a.items():
        if k in POOLED:
            continue
        assert k in s.a and s.a[k].shape == v.shape and np.array_equal(s.a[k], v), k
    for k, v in scal.items():
        if k not in ("n_con_steps", "n_pair_steps"):
            assert s.scal[k] == v, k
    assert np.array_equal(s.rng, rng)

    class R:
        pass
    r = R()
    r.a = a
    for kind in ("con", "pair"):
        for k in range(len(a[f"{kind}_step_n"])):
            assert steps(s, kind, k) == steps(r, kind, k), (kind, k)
