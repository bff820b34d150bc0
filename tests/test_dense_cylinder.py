"""The dense confined workload's start (host generator, CPU).

C5 puts about 42k peptide atoms (0.031 per A^3 of the cylinder) inside a smooth
cylindrical wall.  Overlap-free insertion of rigid chains stalls far below that
density, so the generator places the chains in a longer cylinder and compresses
the axis as the chains, kept rigid, push each other apart.  These tests build a
small cylinder near the same density (radius 30 A, 27 A periodic axis; its wall
takes a larger share of the volume, so it holds 8% fewer atoms per A^3) and check
what the event loop needs from its start: no two chains inside each other's hard
cores, every atom inside the wall margin, every chain with the geometry it was
built with, and a system that the reference's input path builds.
"""
import numpy as np
import pytest

from sdmd_gb300 import workloads as W

RADIUS, AXIS, MARGIN, CHAINS = 30.0, 27.0, 4.0, 18


@pytest.fixture(scope="module")
def packed():
    return W.c5(n_replicas=2, n_chains=CHAINS, radius=RADIUS, axis=AXIS, margin=MARGIN)


def positions(s):
    return np.stack([s.a["x"][1:], s.a["y"][1:], s.a["z"][1:]], 1)


def test_density_matches_the_large_cylinder(packed):
    s = packed[0]
    big = 42000 / (np.pi * 56.0 ** 2 * 120.0)              # C5: atoms per A^3 inside the wall margin
    small = s.n / (np.pi * (RADIUS - MARGIN) ** 2 * AXIS)
    assert s.scal["box"][0] == pytest.approx(AXIS)
    assert 0.85 * big < small < 1.15 * big


def test_atoms_inside_the_wall_margin(packed):
    p = positions(packed[0])
    r = np.hypot(p[:, 1] - RADIUS, p[:, 2] - RADIUS)
    assert r.max() <= RADIUS - MARGIN + 1e-3
    assert (p[:, 0] >= 0).all() and (p[:, 0] < AXIS).all()


def test_no_two_chains_overlap(packed):
    s = packed[0]
    p = positions(s)
    prot, typ = s.a["protein"][1:], s.a["type"][1:]
    dmin = np.sqrt(s.a["pair_dmin"].reshape(12, 33, 33)[0])
    worst = np.inf
    for i in range(len(p)):
        d = p[i + 1:] - p[i]
        d[:, 0] -= AXIS * np.round(d[:, 0] / AXIS)          # periodic axis
        r = np.sqrt((d * d).sum(1))
        other = prot[i + 1:] != prot[i]
        lim = dmin[typ[i], typ[i + 1:]]
        gap = (r - lim)[other & (lim > 0)]
        if gap.size:
            worst = min(worst, gap.min())
    assert worst > 0, f"inter-chain hard-core overlap of {-worst:.4f} A"


def test_chains_keep_their_bond_windows(packed):
    """Every bond of the built system is within its window (the energy minimisation
    of the build leaves none violated)."""
    s = packed[0]
    p = positions(s)
    off, bj = s.a["bond_off"], s.a["bond_j"]
    lo, hi = np.sqrt(s.a["bond_dmin"]), np.sqrt(s.a["bond_dmax"])
    for i in range(1, s.n + 1):
        for q in range(off[i], off[i + 1]):
            j = bj[q]
            d = p[j - 1] - p[i - 1]
            d[0] -= AXIS * np.round(d[0] / AXIS)
            r = np.sqrt((d * d).sum())
            assert lo[q] - 1e-3 <= r <= hi[q] + 1e-3, (i, j, r, lo[q], hi[q])


def test_replicas_share_the_start_and_differ_in_their_streams(packed):
    a, b = packed
    assert np.array_equal(a.a["x"], b.a["x"]) and np.array_equal(a.a["vx"], b.a["vx"])
    assert not np.array_equal(a.rng, b.rng)
    assert a.scal["wall"] == b.scal["wall"] != 0
