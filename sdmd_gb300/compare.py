"""Semantic comparison of two systems' static model (pair tables, constraint
step lists, connection rows), independent of how step lists are pooled."""
import numpy as np


def pair_entries(s):
    a = s.a
    out = {}
    off, n = a["pair_step_off"], a["pair_step_n"]
    for idx in np.nonzero((a["pair_dmin"] != 0) | (n != 0))[0]:
        o, k = int(off[idx]), int(n[idx])
        out[int(idx)] = (float(a["pair_dmin"][idx]), float(a["pair_dmax"][idx]),
                         tuple(a["pair_step_d"][o:o + k]), tuple(a["pair_step_e"][o:o + k]),
                         tuple(a["pair_step_acc"][o:o + k]))
    return out


def constraint_lists(s):
    a = s.a
    out = []
    for i in range(1, s.n + 1):
        row = []
        for q in range(a["con_off"][i], a["con_off"][i + 1]):
            o, k = int(a["con_step_off"][q]), int(a["con_step_n"][q])
            row.append((int(a["con_j"][q]), float(a["con_dmin"][q]), float(a["con_dmax"][q]),
                        tuple(a["con_step_d"][o:o + k]), tuple(a["con_step_e"][o:o + k])))
        out.append(row)
    return out


def conn_rows(s):
    a = s.a
    return [sorted(zip(a["conn_j"][a["conn_off"][i]:a["conn_off"][i + 1]].tolist(),
                       a["conn_bits"][a["conn_off"][i]:a["conn_off"][i + 1]].tolist())) for i in range(0, s.n + 1)]


PLAIN = ["mass", "protein", "aanum", "aatype", "hb_neighbor", "hb_role", "name_code", "bond_off", "bond_j",
         "bond_dmin", "bond_dmax", "con_off", "x", "y", "z", "vx", "vy", "vz", "cx", "cy", "cz", "type", "hb_bond",
         "hb_itype", "nb_partner", "nb_status", "nb_pnum", "ev_time", "ev_partner", "ev_counter", "ev_pcounter",
         "ev_potential", "ev_type", "ev_sub", "cell_list"]


def diff_systems(s, ref):
    """List of human-readable differences (empty when the systems are equivalent)."""
    bad = []
    for k in PLAIN:
        x, y = s.a[k], ref.a[k]
        if x.shape != y.shape:
            bad.append(f"{k}: shape {x.shape} vs {y.shape}")
        elif not np.array_equal(x, y):
            idx = np.nonzero(x != y)[0][:4]
            bad.append(f"{k}: differs at {idx.tolist()}: {x[idx].tolist()} vs {y[idx].tolist()}")
    if pair_entries(s) != pair_entries(ref):
        bad.append("pair tables differ")
    if constraint_lists(s) != constraint_lists(ref):
        bad.append("constraint lists differ")
    if conn_rows(s) != conn_rows(ref):
        bad.append("connection rows differ")
    for k in ["n_atoms", "cellnum", "box", "cellsize", "cutoff", "temperature", "thermo_freq", "thermostat", "wall",
              "wall_type", "hb_barrier"]:
        if np.any(np.asarray(s.scal[k]) != np.asarray(ref.scal[k])):
            bad.append(f"{k}: {s.scal[k]} vs {ref.scal[k]}")
    if not np.array_equal(s.rng, ref.rng):
        bad.append("rng state differs")
    return bad
