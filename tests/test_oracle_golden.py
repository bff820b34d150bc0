"""The CPU oracle against the reference's own golden fixtures (no GPU).

The fixtures were produced by the reference's unmodified sources
(tests/golden/make_golden.py).  The oracle must reproduce them bit for bit:
the full-rebuild sweep (src/SGThread.c:47-52), the event tree built by CreateCBT
(src/CBT.c:16-30), every popped event of the loop (src/SGThread.c:75-151) and the
state at every checkpoint.
"""
import ctypes as C

import numpy as np
import pytest

from oracle import oracle as O
from sdmd_gb300.system import fixture_dynamic, from_fixture, sdmd_rng

DYN = ["x", "y", "z", "vx", "vy", "vz", "cx", "cy", "cz", "type", "hb_bond", "hb_itype", "nb_partner", "nb_status",
       "nb_pnum", "ev_time", "ev_partner", "ev_counter", "ev_pcounter", "ev_potential", "ev_type", "ev_sub",
       "cell_list"]
SWEEP = ["ev_time", "ev_partner", "ev_type", "ev_sub", "ev_potential", "ev_pcounter", "nb_pnum", "hb_itype"]


def assert_state_equal(sys_, ref, keys=DYN):
    for k in keys:
        a, b = sys_.a[k], ref[k]
        if not np.array_equal(a, b):
            idx = np.nonzero(a != b)[0][:5]
            raise AssertionError(f"{k} differs at {idx}: {a[idx]} vs {b[idx]}")


@pytest.mark.parametrize("case", ["ala10_nve", "ala10_nvt", "ala10_nvt_long", "ala10_cyl", "mixed6", "sheet2",
                                  "ala10_sph", "ala10_obst"])
def test_sweep_and_tree(golden, case):
    d = golden(case)
    s = from_fixture(d, "pre")
    assert O.predict_all(s) == 0
    assert_state_equal(s, fixture_dynamic(d, "sweep"), SWEEP)
    loop = O.Loop(s)
    node, leaf = loop.cbt()
    assert np.array_equal(node, d["cbt/cbt_node"]) and np.array_equal(leaf, d["cbt/cbt_leaf"])


@pytest.mark.parametrize("case", ["ala10_nve", "ala10_nvt", "ala10_cyl", "mixed6", "ala10_sph", "ala10_obst"])
def test_trace_event_for_event(golden, case):
    d = golden(case)
    s = from_fixture(d, "pre")
    O.predict_all(s)
    loop = O.Loop(s)
    rc, tr, n = loop.run(int(d["meta/n_events"][0]), trace_cap=len(d["trace/ids"]) + 10)
    assert rc == 0
    ids, dts = d["trace/ids"], d["trace/dt"]
    assert n == len(ids)
    mine = np.stack([tr["target"], tr["partner"], tr["type"], tr["sub"], tr["executed"]], 1)
    assert np.array_equal(mine, ids)
    assert np.array_equal(tr["dt"], dts)
    full = d["trace/full_d"]
    k = len(full)
    assert np.array_equal(tr["time_now"][:k], full[:, 1])
    assert np.array_equal(tr["vt"][:k], full[:, 2:5])
    ref = fixture_dynamic(d, "final")
    assert_state_equal(s, ref)
    assert s.counters == ref["_counters"] and s.time == ref["_time"]
    if case == "ala10_cyl":   # the smooth cylinder wall (WallTime / WallEvent) is exercised
        assert s.counters["wall"] > 0
    if case == "ala10_sph":   # spherical obstacles (SphObstTime / SphObstEvent) are exercised
        assert ((ids[:, 2] == 9) & (ids[:, 4] == 1)).sum() > 0 and s.counters["wall"] > 0
    if case == "ala10_obst":  # obstruction walls (ObstTime / ObstEvent), capture and escape
        ob = ids[(ids[:, 2] == 6) & (ids[:, 4] == 1)]
        assert set(ob[:, 3]) >= {4, 5} and set(ob[:, 1]) == {-1, -13}


@pytest.mark.parametrize("case", ["ala10_nvt_long", "sheet2"])
def test_long_run_checkpoints(golden, case):
    """Long runs with HB formation and breaking; sheet2's bonds form between its two
    chains (a two-strand sheet), so the inter-protein branches are exercised."""
    d = golden(case)
    s = from_fixture(d, "pre")
    O.predict_all(s)
    loop = O.Loop(s)
    done = 0
    for c in [int(v) for v in d["meta/ckpts"]] + [int(d["meta/n_events"][0])]:
        rc, _, _ = loop.run(c - done)
        done = c
        assert rc == 0
        ref = fixture_dynamic(d, f"ckpt{c}" if f"ckpt{c}/x" in d.files else "final")
        assert_state_equal(s, ref)
        assert s.counters == ref["_counters"]
    assert s.counters["hb"] > 0 and s.counters["hbneighbor"] > 0
    if case == "sheet2":   # some of its HB events pair atoms of different chains
        half = s.n // 2
        assert any(r[2] == 2 and (r[0] <= half) != (r[1] <= half) for r in d["trace/sparse_i"])


def test_rng_matches_glibc_rand():
    """The oracle's rand() restatement reproduces glibc's stream (checked against
    libc here; the reference draws every random number through rand())."""
    import ctypes.util
    libc = C.CDLL(ctypes.util.find_library("c"))
    from tests.golden.make_golden import rng_state_after
    for seed in (1575263273, 1, 987654321):
        st = rng_state_after(seed, 0)
        r = sdmd_rng()
        for i in range(31):
            r.tab[i] = int(st[i])
        r.front, r.rear = int(st[31]), int(st[32])
        libc.srand(seed)
        got = [O.lib().oracle_rand(C.byref(r)) for _ in range(20000)]
        want = [libc.rand() for _ in range(20000)]
        assert got == want


def test_log_is_correctly_rounded():
    """oracle_log is correctly rounded on the Box-Muller domain (0, 1), checked
    against 200-bit mpmath.  (glibc's log misrounds ~0.08% of these inputs by one
    ulp; a correctly rounded log is the platform-independent choice.)"""
    mpmath = pytest.importorskip("mpmath")
    mpmath.mp.prec = 200
    rng = np.random.default_rng(5)
    a = rng.random(6000) * 2 - 1
    b = rng.random(6000) * 2 - 1
    s = a * a + b * b
    s = s[(s < 1) & (s > 0)]
    f = O.lib().oracle_log
    for v in s:
        assert f(float(v)) == float(mpmath.log(mpmath.mpf(float(v)))), float(v).hex()


def test_log_close_to_libm():
    import math
    rng = np.random.default_rng(7)
    s = rng.random(100000)
    f = O.lib().oracle_log
    mine = np.array([f(float(v)) for v in s])
    ref = np.array([math.log(float(v)) for v in s])
    ulp = np.abs(mine - ref) / np.spacing(np.abs(ref))
    assert ulp.max() <= 1.0 and np.mean(mine != ref) < 0.005


def test_oracle_nve_energy_conserved_between_hb_events(golden):
    """The exact restatement conserves KE + PE at every non-HB event (the same
    check the GPU modes pass in test_gpu_lazy.py)."""
    from tests.test_gpu_lazy import assert_conserved_between_hb_events, energy_trace
    d = golden("ala10_nve")
    s = from_fixture(d, "pre")
    O.predict_all(s)
    loop = O.Loop(s)
    from tests.energy import total_energy
    e0 = total_energy(s, O.kinetic_energy, O.potential_energy)
    hb0 = s.counters["hb"] + s.counters["hbneighbor"]
    tr = energy_trace(lambda: loop.run(250), s, 120, O.kinetic_energy, O.potential_energy)
    assert_conserved_between_hb_events(tr, e0, hb0)


@pytest.mark.parametrize("case", ["ala10_nve", "ala10_nvt_long"])
def test_energy_functions_match_reference(golden, case):
    """oracle_kinetic_energy / oracle_potential_energy equal the reference's own
    CalKinetE / CalPotenE (dumped by the harness) at every checkpoint."""
    d = golden(case)
    for st in ["pre"] + [f"ckpt{c}" for c in d["meta/ckpts"]] + ["final"]:
        s = from_fixture(d, "pre", dynamic_stage=None if st == "pre" else st)
        assert O.kinetic_energy(s) == d[f"{st}/kinE"][0]
        assert O.potential_energy(s) == d[f"{st}/potE"][0]


def test_dynamic_wall_follows_the_reference(golden):
    """A compressing cylinder wall (WallDyn compress, -Wsz 2 -Wrt 10): DoWallDyn
    moves the wall once per time unit and invalidates the events of atoms heading
    for it, until the compression is complete.  Every pop of the reference's run,
    and at each checkpoint the state, the box and the wall's own state, equal."""
    d = golden("ala10_cyldyn")
    s = from_fixture(d, "pre")
    assert s.scal["wall_dyn"] == 1
    O.predict_all(s)
    loop = O.Loop(s)
    ids, dts = d["trace/ids"], d["trace/dt"]
    done, pops = 0, []
    for c in [int(v) for v in d["meta/ckpts"]] + [int(d["meta/n_events"][0])]:
        rc, tr, n = loop.run(c - done, trace_cap=len(ids) + 10)
        assert rc == 0
        pops.append(tr[:n])
        done = c
        stage = f"ckpt{c}" if f"ckpt{c}/x" in d.files else "final"
        ref = fixture_dynamic(d, stage)
        assert_state_equal(s, ref)
        assert s.scal["box"] == ref["_box"], (c, s.scal["box"], ref["_box"])
        assert [s.scal["wall_dyn"], s.scal["wall_dyn_sign"], s.scal["wall_dyn_touch"]] == ref["_wall_dyn_i"]
        assert s.scal["wall_dyn_cur_time"] == ref["_wall_dyn_d"][3]
    tr = np.concatenate(pops)
    mine = np.stack([tr["target"], tr["partner"], tr["type"], tr["sub"], tr["executed"]], 1)
    assert np.array_equal(mine, ids) and np.array_equal(tr["dt"], dts)
    assert s.scal["box"][1] < d["pre/box"][1] and s.scal["wall_dyn"] == 0   # compressed, then stopped
