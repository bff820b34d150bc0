"""CUDA engine vs the reference's golden fixtures and the CPU oracle (GPU).

The exact FP64 path must reproduce the reference bit for bit: the full-rebuild
sweep (src/SGThread.c:47-52), the event tree (src/CBT.c), every popped event of
the loop (src/SGThread.c:75-151) and the state at every checkpoint.  All calls go
through the C ABI (libsdmd_gpu.so).
"""
import numpy as np
import pytest

from sdmd_gb300.system import fixture_dynamic, from_fixture

pytestmark = pytest.mark.gpu

DYN = ["x", "y", "z", "vx", "vy", "vz", "cx", "cy", "cz", "type", "hb_bond", "hb_itype", "nb_partner", "nb_status",
       "nb_pnum", "ev_time", "ev_partner", "ev_counter", "ev_pcounter", "ev_potential", "ev_type", "ev_sub",
       "cell_list"]
# every exactness test runs on both prediction paths: plain FP64, and the FP32
# screen with FP64 refine (which must give identical results)
SCREENS = pytest.mark.parametrize("screen", [0, 1], ids=["fp64", "screen32"])

SWEEP = ["ev_time", "ev_partner", "ev_type", "ev_sub", "ev_potential", "ev_pcounter", "nb_pnum", "hb_itype"]


@pytest.fixture(scope="module")
def engine_mod():
    import __graft_entry__ as G
    G.build()
    from sdmd_gb300 import engine
    if engine.device_count() < 1:
        pytest.fail("no CUDA device visible: the GPU tests need one")
    return engine


def assert_state_equal(a, ref, keys=DYN):
    for k in keys:
        x, y = a[k], ref[k]
        if not np.array_equal(x, y):
            idx = np.nonzero(x != y)[0][:5]
            raise AssertionError(f"{k} differs at {idx}: {x[idx]} vs {y[idx]}")


@SCREENS
@pytest.mark.parametrize("case", ["ala10_nve", "ala10_nvt", "ala10_nvt_long", "ala10_cyl", "ala10_sph",
                                  "ala10_obst"])
def test_sweep_matches_reference(golden, engine_mod, case, screen):
    d = golden(case)
    s = from_fixture(d, "pre")
    with engine_mod.Engine([s], screen=screen) as eng:
        eng.prepare(full=True)
        eng.download()
    assert_state_equal(s.a, fixture_dynamic(d, "sweep"), SWEEP)
    assert s.counters["warnings"] == int(d["sweep/warningsum"][0])


@SCREENS
@pytest.mark.parametrize("case", ["ala10_nve", "ala10_nvt", "ala10_cyl", "ala10_sph", "ala10_obst"])
def test_loop_matches_reference_event_for_event(golden, engine_mod, case, screen):
    d = golden(case)
    ids, dts = d["trace/ids"], d["trace/dt"]
    s = from_fixture(d, "pre")
    with engine_mod.Engine([s], trace=len(ids) + 16, screen=screen) as eng:
        eng.prepare(full=True)
        eng.run(int(d["meta/n_events"][0]))
        eng.download()
        tr = eng.trace(0)
    assert len(tr) == len(ids)
    mine = np.stack([tr["target"], tr["partner"], tr["type"], tr["sub"], tr["executed"]], 1)
    bad = np.nonzero((mine != ids).any(1) | (tr["dt"] != dts))[0]
    assert len(bad) == 0, f"first divergence at pop {bad[0]}: {mine[bad[0]]} {tr['dt'][bad[0]]} vs {ids[bad[0]]} {dts[bad[0]]}"
    full = d["trace/full_d"]
    k = len(full)
    assert np.array_equal(tr["time_now"][:k], full[:, 1])
    assert np.array_equal(tr["vt"][:k], full[:, 2:5])
    ref = fixture_dynamic(d, "final")
    assert_state_equal(s.a, ref)
    assert s.counters == ref["_counters"]
    assert s.time == ref["_time"]
    if case == "ala10_cyl":   # WallTime / WallEvent in the cylinder (axis x)
        assert s.counters["wall"] > 0
    if case == "ala10_sph":   # SphObstTime / SphObstEvent
        assert ((ids[:, 2] == 9) & (ids[:, 4] == 1)).sum() > 0


@SCREENS
def test_long_run_with_hb_events(golden, engine_mod, screen):
    """1.5e5 events covering HB formation/breaking and HB-neighbour events, in
    chunks (the device state persists between run calls)."""
    d = golden("ala10_nvt_long")
    s = from_fixture(d, "pre")
    with engine_mod.Engine([s], screen=screen) as eng:
        eng.prepare(full=True)
        done = 0
        for c in [int(v) for v in d["meta/ckpts"]] + [int(d["meta/n_events"][0])]:
            eng.run(c - done)
            done = c
            eng.download()
            ref = fixture_dynamic(d, f"ckpt{c}" if f"ckpt{c}/x" in d.files else "final")
            assert_state_equal(s.a, ref)
            assert s.counters == ref["_counters"], c
    assert s.counters["hb"] > 0 and s.counters["hbneighbor"] > 0


@SCREENS
def test_batch_of_systems_matches_oracle(golden, engine_mod, screen):
    """Several independent systems in one launch (one CTA each): NVE, NVT and NVT
    with other RNG streams; each must equal its own oracle run."""
    from oracle import oracle as O
    d_nvt, d_nve = golden("ala10_nvt"), golden("ala10_nve")
    systems = [from_fixture(d_nve, "pre"), from_fixture(d_nvt, "pre")]
    for seed in (11, 12, 13):
        s = from_fixture(d_nvt, "pre")
        from tests.golden.make_golden import rng_state_after
        s.rng = rng_state_after(seed, 0)
        systems.append(s)
    refs = [s.copy() for s in systems]
    with engine_mod.Engine(systems, threads=64, screen=screen) as eng:
        eng.prepare(full=True)
        eng.run(3000)
        eng.download()
    for s, r in zip(systems, refs):
        O.predict_all(r)
        loop = O.Loop(r)
        rc, _, _ = loop.run(3000)
        assert rc == 0
        assert_state_equal(s.a, r.a)
        assert s.counters == r.counters and s.time == r.time


@SCREENS
def test_batch_of_wall_replicas_matches_oracle(golden, engine_mod, screen):
    """Eight replicas in the smooth cylinder (the shape of the wall benchmark),
    each with its own rand() stream and temperature: each equals its oracle run."""
    from oracle import oracle as O
    from tests.golden.make_golden import rng_state_after
    d = golden("ala10_cyl")
    systems = []
    for k in range(8):
        s = from_fixture(d, "pre")
        s.rng = rng_state_after(100 + k, 0)
        s.scal["temperature"] = 0.55 + 0.02 * k
        systems.append(s)
    refs = [s.copy() for s in systems]
    with engine_mod.Engine(systems, threads=64, screen=screen) as eng:
        eng.prepare(full=True)
        eng.run(6000)
        eng.download()
    walls = 0
    for s, r in zip(systems, refs):
        O.predict_all(r)
        rc, _, _ = O.Loop(r).run(6000)
        assert rc == 0
        assert_state_equal(s.a, r.a)
        assert s.counters == r.counters and s.time == r.time
        walls += s.counters["wall"]
    assert walls > 0


def test_batch_beyond_one_wave_matches_oracle(golden, engine_mod):
    """160 systems at 256 threads: the full build of the screened loop keeps one
    CTA per SM (152 on this part), so the engine runs the 128-register build with
    two.  A system of mixed chains too large to stage in shared memory keeps the
    batch unstaged, so registers are what limits residency.  Every system must equal
    its own oracle run."""
    from oracle import oracle as O
    from sdmd_gb300 import workloads as W
    from tests.golden.make_golden import rng_state_after
    d = golden("ala10_nvt")
    systems = [W.c2(n_chains=6, length=12, seed=5, conc_mM=20.0)]
    for k in range(159):
        s = from_fixture(d, "pre")
        s.rng = rng_state_after(300 + k, 0)
        systems.append(s)
    refs = [s.copy() for s in systems]
    with engine_mod.Engine(systems, threads=256, screen=1) as eng:
        eng.prepare(full=True)
        eng.run(400)
        eng.download()
    for s, r in zip(systems, refs):
        O.predict_all(r)
        rc, _, _ = O.Loop(r).run(400)
        assert rc == 0
        assert_state_equal(s.a, r.a)
        assert s.counters == r.counters and s.time == r.time


@SCREENS
@pytest.mark.parametrize("threads", [32, 96, 256])
def test_block_size_does_not_change_results(golden, engine_mod, threads, screen):
    d = golden("ala10_nvt")
    s = from_fixture(d, "pre")
    with engine_mod.Engine([s], threads=threads, screen=screen) as eng:
        eng.prepare(full=True)
        eng.run(2000)
        eng.download()
    ref = fixture_dynamic(d, "ckpt1000")
    s2 = from_fixture(d, "pre")
    with engine_mod.Engine([s2], threads=threads, screen=screen) as eng:
        eng.prepare(full=True)
        eng.run(1000)
        eng.download()
    assert_state_equal(s2.a, ref)


def test_degenerate_rng_state_is_rejected_on_the_host(golden, engine_mod):
    """An all-zero RNG state would make the rejection sampler loop; the ABI
    refuses it before anything reaches the device."""
    d = golden("ala10_nvt")
    s = from_fixture(d, "pre")
    s.rng[:] = 0
    with pytest.raises(engine_mod.EngineError) as e:
        engine_mod.Engine([s])
    assert e.value.code == -1
