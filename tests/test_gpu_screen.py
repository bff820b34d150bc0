"""The FP32-screened prediction against the plain FP64 path and the oracle (GPU).

The screen only decides which candidates need an exact FP64 recomputation, so
its results must be bit-identical to the plain path's in both advance modes:
the same pops, times, velocities, counters and RNG state.  The multi-chain
system (random residues over the whole library, several peptides per cell
neighbourhood, periodic wrapping) covers candidate kinds the ala10 fixtures
do not: constraint pairs of every residue type, cross-chain HB scans and
many pair-table entries.
"""
import numpy as np
import pytest

from sdmd_gb300.system import from_fixture

pytestmark = pytest.mark.gpu

DYN = ["x", "y", "z", "vx", "vy", "vz", "cx", "cy", "cz", "type", "hb_bond", "hb_itype", "nb_partner", "nb_status",
       "nb_pnum", "ev_time", "ev_partner", "ev_counter", "ev_pcounter", "ev_potential", "ev_type", "ev_sub",
       "cell_list"]


@pytest.fixture(scope="module")
def engine_mod():
    import __graft_entry__ as G
    G.build()
    from sdmd_gb300 import engine
    if engine.device_count() < 1:
        pytest.fail("no CUDA device visible: the GPU tests need one")
    return engine


@pytest.fixture(scope="module")
def mixed_system():
    """24 random-sequence 10-mers at 20 mM (a 125 A periodic cube), 300 K Andersen."""
    from sdmd_gb300 import workloads as W
    return W.c2(n_chains=24, length=10, seed=7, conc_mM=20.0)


def run(engine_mod, s, screen, advance, n, trace=0):
    with engine_mod.Engine([s], screen=screen, advance=advance, trace=trace) as e:
        e.prepare(full=True)
        e.run(n)
        e.download()
        return e.trace(0) if trace else None


def assert_same(a, b):
    for k in DYN:
        if not np.array_equal(a.a[k], b.a[k]):
            idx = np.nonzero(a.a[k] != b.a[k])[0][:5]
            raise AssertionError(f"{k} differs at {idx}: {a.a[k][idx]} vs {b.a[k][idx]}")
    assert a.counters == b.counters
    assert a.time == b.time
    assert np.array_equal(a.rng, b.rng)


@pytest.mark.parametrize("advance", [0, 1], ids=["eager", "lazy"])
def test_screen_equals_fp64_on_ala10(golden, engine_mod, advance):
    d = golden("ala10_nvt_long")
    a, b = from_fixture(d, "pre"), from_fixture(d, "pre")
    ta = run(engine_mod, a, 0, advance, 30000, trace=30016)
    tb = run(engine_mod, b, 1, advance, 30000, trace=30016)
    for k in ("target", "partner", "type", "sub", "executed", "dt", "t_new_time", "p_new_time"):
        assert np.array_equal(ta[k], tb[k]), k
    assert_same(b, a)


@pytest.mark.parametrize("advance", [0, 1], ids=["eager", "lazy"])
def test_screen_equals_fp64_with_a_cylinder_wall(golden, engine_mod, advance):
    d = golden("ala10_cyl")
    a, b = from_fixture(d, "pre"), from_fixture(d, "pre")
    run(engine_mod, a, 0, advance, 40000)
    run(engine_mod, b, 1, advance, 40000)
    assert_same(b, a)
    assert b.counters["wall"] > 0


@pytest.mark.parametrize("advance", [0, 1], ids=["eager", "lazy"])
def test_screen_equals_fp64_on_mixed_chains(engine_mod, mixed_system, advance):
    a, b = mixed_system.copy(), mixed_system.copy()
    run(engine_mod, a, 0, advance, 20000)
    run(engine_mod, b, 1, advance, 20000)
    assert_same(b, a)
    assert b.counters["pcc"] > 0 and b.counters["collision"] > 0


def test_screen_matches_oracle_on_mixed_chains(engine_mod, mixed_system):
    """Eager mode is bit-exact with the reference: the screened path equals the oracle."""
    from oracle import oracle as O
    s, r = mixed_system.copy(), mixed_system.copy()
    run(engine_mod, s, 1, 0, 4000)
    O.predict_all(r)
    rc, _, _ = O.Loop(r).run(4000)
    assert rc == 0
    assert_same(s, r)
