"""Test helper: energy of the step-potential constraints.

The reference applies the CONSTRn step energies in its dynamics (FindPair
"constraint", src/ToolFunctions.c:72-80 and the step walk) but never
accumulates them (CalAccumulatedPoten is only called for the pair tables,
src/Initialization.c:1515, 1636), so its CalPotenE counts 0 for constrained
pairs.  Adding them back gives the energy the dynamics actually conserves.
"""
import numpy as np


def constraint_energy(s):
    a = s.a
    box = np.array(s.scal["box"])
    cn = np.array(s.scal["cellnum"])
    tot = 0.0
    for i in range(1, s.n + 1):
        for q in range(a["con_off"][i], a["con_off"][i + 1]):
            j = int(a["con_j"][q])
            if j < i:
                continue
            row = slice(a["conn_off"][i], a["conn_off"][i + 1])
            hit = np.nonzero(a["conn_j"][row] == j)[0]
            if len(hit) == 0 or not (a["conn_bits"][row][hit[0]] & 2):
                continue
            ci = np.array([a["cx"][i], a["cy"][i], a["cz"][i]])
            cj = np.array([a["cx"][j], a["cy"][j], a["cz"][j]])
            sh = np.where((ci != cj) & (ci == 0) & (cj == cn - 1), -box,
                          np.where((ci != cj) & (ci == cn - 1) & (cj == 0), box, 0.0))
            r = np.array([a["x"][i], a["y"][i], a["z"][i]]) - (np.array([a["x"][j], a["y"][j], a["z"][j]]) + sh)
            v = np.array([a["vx"][i] - a["vx"][j], a["vy"][i] - a["vy"][j], a["vz"][i] - a["vz"][j]])
            r2 = float(r @ r)
            # a pair on a step boundary belongs to the shell it moves into: the
            # reference's FindPair tolerance is +ZERO approaching, -ZERO leaving
            tol = 1e-8 if float(r @ v) < 0 else -1e-8
            o, n = int(a["con_step_off"][q]), int(a["con_step_n"][q])
            d, e = a["con_step_d"][o:o + n], a["con_step_e"][o:o + n]
            for k in range(n):
                if r2 < d[k] + tol:
                    tot += float(np.sum(e[k:]))
                    break
    return tot


def total_energy(s, kinetic, potential):
    return kinetic(s) + potential(s) + constraint_energy(s)
