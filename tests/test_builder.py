"""The host-side builder against the reference's own initial state (no GPU).

Each golden fixture stores the inputs of its run (the .gro text, parameter.txt,
and the test-local Wall.txt when the case has a wall).  Building a system from
them must reproduce the reference's state after InputData / SDEnergyMin / PBC /
LinkList (src/DMD.c:195-237, src/SGThread.c:42-46) -- coordinates, velocities,
cells, topology, potential tables, HB roles, wall and the rand() state -- bit
for bit.  Step lists are compared entry by entry: the builder pools shared step
lists once, so the pool offsets differ while every list is the same.
"""
import os
import shutil

import numpy as np
import pytest

from sdmd_gb300.host import build_system
from sdmd_gb300.system import from_fixture

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
POOLED = {"con_step_off", "pair_step_off", "con_step_d", "con_step_e", "con_step_acc", "pair_step_d", "pair_step_e",
          "pair_step_acc"}


def steps(s, kind, k):
    off, n = int(s.a[f"{kind}_step_off"][k]), int(s.a[f"{kind}_step_n"][k])
    return [(s.a[f"{kind}_step_d"][q], s.a[f"{kind}_step_e"][q], s.a[f"{kind}_step_acc"][q]) for q in range(off, off + n)]


@pytest.mark.parametrize("case", ["ala10_nvt", "ala10_nve", "ala10_cyl", "mixed6", "sheet2", "ala10_sph", "ala10_obst"])
def test_builder_reproduces_the_reference_initial_state(golden, case, tmp_path):
    d = golden(case)
    lib = tmp_path / "Library_Ding"
    shutil.copytree(os.path.join(REPO, "sdmd_gb300", "data", "Library_Ding"), lib)
    if "meta/wall_lib" in d.files:
        (lib / "Wall.txt").write_bytes(bytes(d["meta/wall_lib"]))
    (tmp_path / "parameter.txt").write_bytes(bytes(d["meta/parameter"]))
    s = build_system(str(tmp_path), gro_text=bytes(d["meta/gro"]).decode(), seed=int(d["pre/seed"][0]))
    r = from_fixture(d, "pre")
    for k, v in r.a.items():
        if k in POOLED:
            continue
        assert k in s.a and s.a[k].shape == v.shape and np.array_equal(s.a[k], v), k
    for k, v in r.scal.items():
        if k not in ("n_con_steps", "n_pair_steps"):
            assert s.scal[k] == v, k
    for kind, n in (("con", len(r.a["con_step_n"])), ("pair", len(r.a["pair_step_n"]))):
        for k in range(n):
            assert steps(s, kind, k) == steps(r, kind, k), (kind, k)
    assert np.array_equal(s.rng, r.rng) and s.counters == r.counters and s.time == r.time
    if case == "ala10_cyl":
        assert s.scal["wall"] == 2 and s.scal["wall_type"] == 9
