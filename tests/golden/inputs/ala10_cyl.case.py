# ALA x 10 inside a smooth cylinder wall (axis x, radius L_y / 2 = 13.5 A).
# The reference's shipped ala10 peptide, moved to the centre of a 27 A box
# (3 cells of 9 A per axis) and 2 A off the axis along y, so that its farthest
# atom starts 3.54 A from the wall (the largest wall dmin here is 3.27 A) and
# wall events come early; the wall library is a test-local copy naming an
# existing atom type (CA): the shipped Wall.txt names PHO, which AtomModel lacks
# (src/Models.c:129-206), so ReadWall would exit.
import os as _os

import numpy as _np

# REF: the reference checkout, given by make_golden.py
with open(_os.path.join(REF, "input", "ala10.gro")) as _f:
    _lines = _f.read().splitlines()
_n = int(_lines[1])
_body = _lines[2:2 + _n]
_xyz = _np.array([[float(l[20:28]), float(l[28:36]), float(l[36:44])] for l in _body])
_shift = _np.array([1.35, 1.55, 1.35]) - (_xyz.min(0) + _xyz.max(0)) / 2   # nm, in the 2.7 nm box
_out = [_lines[0], _lines[1]]
for _l, _p in zip(_body, _xyz + _shift):
    _out.append(_l[:20] + "".join(f"{v:8.3f}" for v in _p) + _l[44:])
_out.append("   2.70000   2.70000   2.70000")

CASE = dict(gro_text="\n".join(_out) + "\n",
            params=base_params(temp=0.6160, wall_exist="smooth", wall_type="cylinder"),
            n_events=40000, ckpts=[10000, 20000, 30000],
            wall_lib="Wall\n   ATOM CA      CA   12.0  N N\n")
