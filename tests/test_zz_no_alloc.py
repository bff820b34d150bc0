"""sdmd_gpu_prepare_noalloc against sdmd_gpu_prepare, through the C ABI (GPU).

The allocation-free entry point keeps its scratch (descriptor table, thermostat
sample buffers, error record) in a static device array that persists between
calls.  Two calls in a row must each give exactly what the allocating entry
point gives from the same state, so stale contents of the first call cannot
leak into the second.  The file sorts last so the test also runs after every
other GPU test has used the library.
"""
import numpy as np
import pytest

from sdmd_gb300.system import from_fixture, glibc_rng_state

pytestmark = pytest.mark.gpu

SDMD_ECAPACITY = -15


@pytest.fixture(scope="module")
def engine_mod():
    import __graft_entry__ as G
    G.build()
    from sdmd_gb300 import engine
    if engine.device_count() < 1:
        pytest.fail("no CUDA device visible: the GPU tests need one")
    return engine


def batch(golden, n):
    base = from_fixture(golden("ala10_nvt"), "pre")
    out = []
    for k in range(n):
        s = base.copy()
        s.rng[:] = glibc_rng_state(1000 + k)   # a different sample stream per system
        out.append(s)
    return out


def snapshot(systems):
    return [(s.state_digest(), np.array(s.rng, copy=True), dict(s.counters), float(s.time)) for s in systems]


def assert_same(a, b):
    for (da, ra, ca, ta), (db, rb, cb, tb) in zip(a, b):
        for k in da:
            assert np.array_equal(da[k], db[k]), k
        assert np.array_equal(ra, rb)
        assert ca == cb
        assert ta == tb


@pytest.mark.parametrize("screen", ["fp64", "fp32"])
@pytest.mark.parametrize("advance", ["eager", "lazy"])
def test_noalloc_sweep_equals_prepare_on_two_calls_in_a_row(golden, engine_mod, screen, advance):
    # on the FP32 screened path sdmd_gpu_prepare runs the parallel sweep and the
    # allocation-free call the sequential one: both must give the same state
    opts = dict(screen=engine_mod.SCREEN_FP32 if screen == "fp32" else engine_mod.SCREEN_FP64,
                advance=engine_mod.ADVANCE_LAZY if advance == "lazy" else engine_mod.ADVANCE_EAGER)
    ref, got = batch(golden, 3), batch(golden, 3)
    with engine_mod.Engine(ref, **opts) as e_ref, engine_mod.Engine(got, **opts) as e_got:
        for call in range(2):
            e_ref.prepare(full=True)
            e_got.prepare_noalloc(full=True)
            e_ref.download()
            e_got.download()
            assert_same(snapshot(got), snapshot(ref))
        # the loop continues identically from either sweep, and continue mode agrees too
        e_ref.run(500)
        e_got.run(500)
        e_ref.prepare(full=False)
        e_got.prepare_noalloc(full=False)
        e_ref.run(500)
        e_got.run(500)
        e_ref.download()
        e_got.download()
        assert_same(snapshot(got), snapshot(ref))
        assert got[0].counters["frame"] == 1000


def test_noalloc_rejects_a_batch_beyond_its_scratch(golden, engine_mod):
    systems = batch(golden, 2000)   # ~3.3 KB of scratch per system: past the 4 MiB array
    with engine_mod.Engine(systems) as e:
        with pytest.raises(engine_mod.EngineError) as info:
            e.prepare_noalloc(full=True)
        assert info.value.code == SDMD_ECAPACITY
        e.prepare(full=True)        # the handle is untouched and still usable
        e.run(10)
