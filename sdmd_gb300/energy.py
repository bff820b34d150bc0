"""Total energy for NVE drift checks.

The reference applies the CONSTRn step energies in its dynamics (FindPair
"constraint", src/ToolFunctions.c:72-80 and the step walk) but never accumulates
them (CalAccumulatedPoten is only called for the pair tables,
src/Initialization.c:1515, 1636), so its CalPotenE counts 0 for constrained
pairs.  Adding them back to CalKinetE + CalPotenE gives the energy the dynamics
conserves between HB events.
"""
import numpy as np


def constraint_energy(s):
    """Step energy of every constrained pair (i < j with the CONSTR connection bit),
    vectorised over the pairs.  A pair on a step boundary belongs to the shell it
    moves into (FindPair's tolerance: +1e-8 approaching, -1e-8 leaving)."""
    a = s.a
    n = s.n
    off = a["con_off"][: n + 2].astype(np.int64)
    cnt = np.diff(off[: n + 2])[: n + 1]
    i_of = np.repeat(np.arange(n + 1), cnt[: n + 1])
    q_of = np.arange(off[0], off[n + 1])
    j_of = a["con_j"][q_of].astype(np.int64)
    keep = j_of > i_of
    i_of, j_of, q_of = i_of[keep], j_of[keep], q_of[keep]
    if len(q_of) == 0:
        return 0.0
    # the pair carries the constraint bit (2) in i's connection row
    coff = a["conn_off"].astype(np.int64)
    crow = np.repeat(np.arange(n + 1), np.diff(coff[: n + 2])[: n + 1])
    cj = a["conn_j"][coff[0]: coff[n + 1]].astype(np.int64)
    cb = a["conn_bits"][coff[0]: coff[n + 1]]
    ck = crow[(cb & 2) != 0] * (n + 1) + cj[(cb & 2) != 0]
    ok = np.isin(i_of * (n + 1) + j_of, ck)
    i_of, j_of, q_of = i_of[ok], j_of[ok], q_of[ok]
    box = np.array(s.scal["box"], dtype=np.float64)
    cn = np.array(s.scal["cellnum"], dtype=np.int64)
    ci = np.stack([a["cx"][i_of], a["cy"][i_of], a["cz"][i_of]], 1)
    cjj = np.stack([a["cx"][j_of], a["cy"][j_of], a["cz"][j_of]], 1)
    sh = np.where((ci != cjj) & (ci == 0) & (cjj == cn - 1), -box,
                  np.where((ci != cjj) & (ci == cn - 1) & (cjj == 0), box, 0.0))
    pi = np.stack([a["x"][i_of], a["y"][i_of], a["z"][i_of]], 1)
    pj = np.stack([a["x"][j_of], a["y"][j_of], a["z"][j_of]], 1) + sh
    r = pi - pj
    v = np.stack([a["vx"][i_of] - a["vx"][j_of], a["vy"][i_of] - a["vy"][j_of], a["vz"][i_of] - a["vz"][j_of]], 1)
    r2 = np.einsum("ij,ij->i", r, r)
    tol = np.where(np.einsum("ij,ij->i", r, v) < 0, 1e-8, -1e-8)
    so = a["con_step_off"][q_of].astype(np.int64)
    sn = a["con_step_n"][q_of].astype(np.int64)
    e_pool = a["con_step_e"].astype(np.float64)
    d_pool = a["con_step_d"].astype(np.float64)
    cs = np.concatenate([[0.0], np.cumsum(e_pool)])
    tot = 0.0
    done = np.zeros(len(q_of), bool)
    for k in range(int(sn.max()) if len(sn) else 0):
        live = ~done & (k < sn)
        idx = np.nonzero(live)[0]
        hit = idx[r2[idx] < d_pool[so[idx] + k] + tol[idx]]
        tot += float(np.sum(cs[so[hit] + sn[hit]] - cs[so[hit] + k]))
        done[hit] = True
    return tot


def nve_drift(e_start, e_end, n_atoms, kT, events):
    """|E_end - E_start| / (N kT), per 10^6 executed events."""
    return abs(e_end - e_start) / (n_atoms * kT) * (1e6 / max(events, 1))
