# Two extended ALA x 10 chains stacked antiparallel 4.8 A apart along the ribbon
# normal (a two-strand sheet), 40 A box, Andersen NVT at T* = 0.6: hydrogen bonds
# form between the chains.  The first chain comes from the package's generator
# (seed 3); the second is that chain turned by 180 degrees about the normal and
# shifted along it.  The .gro text is stored in the fixture.
import os as _os
import sys as _sys

import numpy as _np

_sys.path.insert(0, _os.path.dirname(_os.path.dirname(_os.path.dirname(_os.path.abspath(extra)))))
from sdmd_gb300 import workloads as _W
from sdmd_gb300.host import generate_gro as _gen

_d = _W._datadir(dict(temp=0.6, thermostat="Andersen", time=1e9))
_L = _gen(_d, [["ALA"] * 10], (60.0, 60.0, 60.0), seed=3).splitlines()
_n = int(_L[1])
_body = _L[2:2 + _n]
_X = _np.array([[float(v) for v in l.split()[-3:]] for l in _body])
_X = _X - _X.mean(0)
_normal = _np.linalg.svd(_X, full_matrices=False)[2][2]
# 180-degree turn about the normal: v -> 2 (v.k) k - v
_Y = 2 * _np.outer(_X @ _normal, _normal) - _X + 0.48 * _normal
_box = 4.0
_out = ["two-strand sheet", str(2 * _n)]
for _P in (_X - 0.24 * _normal, _Y - 0.24 * _normal):
    for _l, _p in zip(_body, _P + _box / 2):
        _out.append(_l[:15] + f"{(len(_out) - 1) % 100000:5d}" + "".join(f"{v:8.3f}" for v in _p))
_out.append(f"{_box:10.5f}{_box:10.5f}{_box:10.5f}")

CASE = dict(gro_text="\n".join(_out) + "\n", params=base_params(), n_events=100000, ckpts=[25000, 50000, 75000],
            sparse=True)
