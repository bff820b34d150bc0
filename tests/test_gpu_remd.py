"""Device energies (CalKinetE / CalPotenE) and the on-device replica exchange (GPU).

Energies must equal the reference's own values stored in the golden fixtures, bit
for bit, including checkpoints with formed hydrogen bonds.  The replica exchange
(REMDRun + the server's rearrange) must equal an oracle run of the same replicas:
every replica's loop, CalPotenE at each exchange point, one rearrange() pass with
the server's rand() stream, the new thermostat targets -- for both triggers (a
fixed number of executed events per replica, and the reference's time trigger).
"""
import numpy as np
import pytest

from sdmd_gb300.system import from_fixture, glibc_rng_state

pytestmark = pytest.mark.gpu

BOLTZMANN = 0.0019872041
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


@pytest.mark.parametrize("stage", ["pre", "ckpt50000", "ckpt104000", "ckpt125000", "final"])
def test_energies_equal_the_reference(golden, engine_mod, stage):
    d = golden("ala10_nvt_long")
    s = from_fixture(d, "pre", dynamic_stage=stage)
    s.rng[:] = glibc_rng_state(1)   # checkpoints keep a draw count, not the state; energies do not use it
    with engine_mod.Engine([s]) as e:
        pot, kin = e.energies()
    assert kin[0] == d[f"{stage}/kinE"][0]
    assert pot[0] == d[f"{stage}/potE"][0]


def replicas(golden, n):
    base = from_fixture(golden("ala10_nvt"), "pre")
    T = 270.0 * (500.0 / 270.0) ** (np.arange(n) / (n - 1)) * BOLTZMANN
    out = []
    for k in range(n):
        s = base.copy()
        s.scal["temperature"] = float(T[k])
        s.rng[:] = glibc_rng_state(1000 + k)
        out.append(s)
    return out, T


def oracle_remd(systems, T, server_rng, n_exchanges, every_events=0, every_time=0.0):
    from oracle import oracle as O
    from sdmd_gb300.system import sdmd_rng
    import ctypes as C
    n = len(systems)
    num = np.arange(1, n + 1, dtype=np.int32)
    T = np.array(T, np.float64)
    rng = sdmd_rng()
    for i in range(31):
        rng.tab[i] = int(server_rng[i])
    rng.front, rng.rear = int(server_rng[31]), int(server_rng[32])
    loops = []
    for s in systems:
        O.predict_all(s)
        loops.append(O.Loop(s))
    rate = [(int(s.time / every_time) + 1) * every_time if every_time else 0 for s in systems]
    for _ in range(n_exchanges):
        for k, L in enumerate(loops):
            rc = L.run(every_events)[0] if every_events else L.run_until(rate[k])
            assert rc == 0
        E = np.array([L.potential_energy_counted() for L in loops])
        O.lib().oracle_remd_rearrange(n, num.ctypes.data_as(C.POINTER(C.c_int32)),
                                      T.ctypes.data_as(C.POINTER(C.c_double)),
                                      E.ctypes.data_as(C.POINTER(C.c_double)), C.byref(rng))
        for k, L in enumerate(loops):
            L.st.temperature = float(T[k])
            rate[k] += every_time
    out_rng = np.array([rng.tab[i] for i in range(31)] + [rng.front, rng.rear], np.int32)
    return num, T, E, out_rng


@pytest.mark.parametrize("screen", [0, 1], ids=["fp64", "screen32"])
@pytest.mark.parametrize("trigger", ["events", "time"])
def test_replica_exchange_matches_oracle(golden, engine_mod, screen, trigger):
    n, n_exch = 6, 5
    kw = {"every_events": 1500} if trigger == "events" else {"every_time": 1.0}
    gpu, T = replicas(golden, n)
    ref = [s.copy() for s in gpu]
    server = glibc_rng_state(20201)
    with engine_mod.Engine(gpu, screen=screen) as e:
        e.prepare(full=True)
        out = e.run_remd(n_exch, np.arange(1, n + 1), T, server, **kw)
        e.download()
    num, Tn, E, rng = oracle_remd(ref, T, server, n_exch, **kw)
    assert out["done"] == n_exch
    assert np.array_equal(out["num"], num) and np.array_equal(out["T"], Tn)
    assert np.array_equal(out["E"], E)
    assert np.array_equal(out["rng"], rng)
    assert out["accepted"] > 0 and out["attempted"] >= out["accepted"]
    for s, r in zip(gpu, ref):
        for k in DYN:
            assert np.array_equal(s.a[k], r.a[k]), k
        assert s.counters == r.counters and s.time == r.time
        assert np.array_equal(s.rng, r.rng)


def test_stops_and_exchange_make_the_same_replica_exchange(golden, engine_mod):
    """sdmd_gpu_run_to_stops (each replica to its own exchange point) followed by
    sdmd_gpu_exchange, repeated, is the oracle's replica exchange with the time
    trigger; a system given no events does not move."""
    n, n_exch = 6, 4
    gpu, T = replicas(golden, n)
    ref = [s.copy() for s in gpu]
    server = glibc_rng_state(20201)
    num, Tx, rng = np.arange(1, n + 1), T.copy(), server
    att = acc = 0
    with engine_mod.Engine(gpu, screen=1) as e:
        e.prepare(full=True)
        e.download()
        rate = np.array([(int(s.time / 1.0) + 1) * 1.0 for s in gpu])
        for _ in range(n_exch):
            e.download()
            before = [s.counters["frame"] for s in gpu]
            held = e.run_to_stops(rate, np.zeros(n, np.int64))          # nothing runs
            e.download()
            assert not held.any() and [s.counters["frame"] for s in gpu] == before
            at = e.run_to_stops(rate, np.full(n, 1 << 40, np.int64))
            assert at.all()
            out = e.exchange(num, Tx, rng, att, acc)
            num, Tx, rng, att, acc = out["num"], out["T"], out["rng"], out["attempted"], out["accepted"]
            rate += 1.0
        e.download()
    num_o, T_o, E_o, rng_o = oracle_remd(ref, T, server, n_exch, every_time=1.0)
    assert np.array_equal(num, num_o) and np.array_equal(Tx, T_o)
    assert np.array_equal(out["E"], E_o)
    assert np.array_equal(rng, rng_o)
    for s, r in zip(gpu, ref):
        for k in DYN:
            assert np.array_equal(s.a[k], r.a[k]), k
        assert s.counters == r.counters and s.time == r.time
