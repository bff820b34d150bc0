"""The benchmarked path against the reference, event for event (GPU).

bench.py times the FP32-screened prediction with eager advance: every pop moves
every atom and every event time (UpdateData / TimeForward, src/ToolFunctions.c
23-36), as the reference does, so the results are the reference's bit for bit.
For large systems the advance of the atoms a pop does not involve runs on helper
blocks on the other SMs (sdmd_opts.helper_blocks), in the same launch.

These tests hold that path to the reference's own golden traces (targets,
partners, types and sub-types of every pop, event times, velocities and the
state at every checkpoint -- zero difference, which meets any relative
tolerance), with and without helper blocks, and to the oracle on the full-size
systems of the benchmark: the 42k-atom full-rebuild-sweep system, a subset of
the uneven batch, and the dense confined batch's shape at a smaller size.
"""
import numpy as np
import pytest

from sdmd_gb300.system import fixture_dynamic, from_fixture

pytestmark = pytest.mark.gpu

DYN = ["x", "y", "z", "vx", "vy", "vz", "cx", "cy", "cz", "type", "hb_bond", "hb_itype", "nb_partner", "nb_status",
       "nb_pnum", "ev_time", "ev_partner", "ev_counter", "ev_pcounter", "ev_potential", "ev_type", "ev_sub",
       "cell_list"]
HELPERS = pytest.mark.parametrize("helpers", [-1, 6], ids=["in-block", "helpers6"])


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


def bench_engine(engine_mod, systems, helpers=0, **kw):
    return engine_mod.Engine(systems, advance=engine_mod.ADVANCE_EAGER, screen=engine_mod.SCREEN_FP32,
                             helpers=helpers, **kw)


@HELPERS
@pytest.mark.parametrize("case", ["ala10_nve", "ala10_nvt", "ala10_cyl", "mixed6", "ala10_sph",
                                  "ala10_obst"])
def test_bench_path_follows_the_reference_trace(golden, engine_mod, case, helpers):
    """Every pop of the golden run: (target, partner, type, sub-type, executed) and
    dt equal; the first pops' clock and target velocities equal; every checkpoint
    state equal."""
    d = golden(case)
    ids, dts = d["trace/ids"], d["trace/dt"]
    s = from_fixture(d, "pre")
    ckpts = [int(v) for v in d["meta/ckpts"]] + [int(d["meta/n_events"][0])]
    with bench_engine(engine_mod, [s], helpers=helpers, trace=len(ids) + 16) as eng:
        eng.prepare(full=True)
        done = 0
        for c in ckpts:
            eng.run(c - done)
            done = c
            eng.download()
            ref = fixture_dynamic(d, f"ckpt{c}" if f"ckpt{c}/x" in d.files else "final")
            assert_state_equal(s.a, ref)
            assert s.counters == ref["_counters"], c
            assert s.time == ref["_time"]
        tr = eng.trace(0)
    assert len(tr) == len(ids)
    mine = np.stack([tr["target"], tr["partner"], tr["type"], tr["sub"], tr["executed"]], 1)
    bad = np.nonzero((mine != ids).any(1) | (tr["dt"] != dts))[0]
    assert len(bad) == 0, f"first divergence at pop {bad[0]}: {mine[bad[0]]} vs {ids[bad[0]]}"
    full = d["trace/full_d"]
    k = len(full)
    assert np.array_equal(tr["time_now"][:k], full[:, 1])
    assert np.array_equal(tr["vt"][:k], full[:, 2:5])
    assert np.array_equal(tr["vp"][:k], full[:, 5:8])


@HELPERS
def test_bench_path_forms_hydrogen_bonds_between_chains(golden, engine_mod, helpers):
    """The two-strand sheet: 1e5 events with 93 inter-chain hydrogen bonds formed
    (HBTime's scan, src/TimePrediction.c:298-483; HBEvent, src/Events.c:275-393).
    Every checkpoint equals the reference's state, and so does every traced HB /
    HB-neighbour pop."""
    d = golden("sheet2")
    s = from_fixture(d, "pre")
    n_pops = int(d["trace/n_pops"][0])
    ckpts = [int(v) for v in d["meta/ckpts"]] + [int(d["meta/n_events"][0])]
    with bench_engine(engine_mod, [s], helpers=helpers, trace=n_pops + 16) as eng:
        eng.prepare(full=True)
        done = 0
        for c in ckpts:
            eng.run(c - done)
            done = c
            eng.download()
            ref = fixture_dynamic(d, f"ckpt{c}" if f"ckpt{c}/x" in d.files else "final")
            assert_state_equal(s.a, ref)
            assert s.counters == ref["_counters"], c
        tr = eng.trace(0)
    assert len(tr) == n_pops
    pops = d["trace/sparse_pop"]
    si, sd = d["trace/sparse_i"], d["trace/sparse_d"]
    mine = np.stack([tr["target"], tr["partner"], tr["type"], tr["sub"], tr["executed"]], 1)[pops]
    assert np.array_equal(mine, si[:, :5])
    assert np.array_equal(tr["vt"][pops], sd[:, 2:5])
    assert s.counters["hb"] > 0


def oracle_run(system, n_events):
    from oracle import oracle as O
    r = system.copy()
    O.predict_all(r)
    rc, _, _ = O.Loop(r).run(n_events)
    assert rc == 0
    return r


def test_full_size_sweep_system_matches_oracle(engine_mod):
    """The 42k-atom system of the full-rebuild-sweep benchmark (256 random-sequence
    16-mers at 5 mM): the parallel screened sweep equals the plain FP64 sequential
    sweep and the oracle's Predict over 1..N bit for bit, including the atoms whose
    pairs straddle the periodic boundary; then 1e4 events of the benchmarked path
    (helper blocks on every free SM) equal the oracle's."""
    from sdmd_gb300 import workloads as W
    base = W.c2()
    s_par, s_seq = base.copy(), base.copy()
    with engine_mod.Engine([s_seq], screen=engine_mod.SCREEN_FP64) as e:
        e.prepare(full=True)
        e.download()
    ref = oracle_run(base, 0)
    sweep_keys = ["ev_time", "ev_partner", "ev_type", "ev_sub", "ev_potential", "ev_pcounter", "nb_pnum"]
    assert_state_equal(s_seq.a, ref.a, sweep_keys)
    with bench_engine(engine_mod, [s_par]) as e:
        e.prepare(full=True)
        e.download()
        assert_state_equal(s_par.a, ref.a, sweep_keys)
        e.run(10000)
        e.download()
    ref = oracle_run(base, 10000)
    assert_state_equal(s_par.a, ref.a)
    assert s_par.counters == ref.counters and s_par.time == ref.time


def test_uneven_batch_subset_matches_oracle(engine_mod):
    """32 systems of the uneven-batch shape (single random-sequence chains of 5-60
    residues, mixed temperatures) in one launch of the benchmarked path: each
    system equals its own oracle run."""
    from sdmd_gb300 import workloads as W
    systems = W.c4(n_systems=32, seed=7)
    lengths = [s.n for s in systems]
    assert min(lengths) < 100 and max(lengths) > 450
    refs = [s.copy() for s in systems]
    with bench_engine(engine_mod, systems, threads=128) as e:
        e.prepare(full=True)
        e.run(3000)
        e.download()
    for s, r in zip(refs, systems):
        o = oracle_run(s, 3000)
        assert_state_equal(r.a, o.a)
        assert r.counters == o.counters and r.time == o.time


@pytest.mark.parametrize("threads", [256, 512])
def test_dense_cylinder_batch_matches_oracle(engine_mod, threads):
    """The dense confined workload's shape at a size the oracle runs in seconds: two
    replicas of 18 random-sequence 10-mers packed near its density (compressed
    rigid-chain packing) inside a smooth cylindrical wall of radius 30 A with a
    27 A periodic axis, differing in their thermostat streams; atoms start 3.4 A
    from the wall (above every wall hard core, 3.27 A), so that wall collisions come
    early.  With helper blocks advancing the atoms a pop does not involve, each
    replica equals its own oracle run after 8000 events, wall collisions included,
    with 256-thread blocks and with the 512-thread build."""
    from sdmd_gb300 import workloads as W
    systems = W.c5(n_replicas=2, n_chains=18, radius=30.0, axis=27.0, margin=3.4)
    refs = [s.copy() for s in systems]
    with bench_engine(engine_mod, systems, helpers=6, threads=threads) as e:
        assert e.launch_info()["loop_kernel"] == ("loop_kernel_screen_coop512" if threads > 256
                                                   else "loop_kernel_screen_coop")
        e.prepare(full=True)
        e.run(8000)
        e.download()
    for s, r in zip(refs, systems):
        o = oracle_run(s, 8000)
        assert_state_equal(r.a, o.a)
        assert r.counters == o.counters and r.time == o.time
    assert all(s.counters["wall"] > 0 for s in systems)
    assert not np.array_equal(systems[0].a["x"], systems[1].a["x"])
