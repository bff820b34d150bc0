# The reference's ala10 input with four spherical obstacles (SphObst?, 12 A
# diameter) placed 0.3-0.7 A from the chain's atoms, so that the first 14k events
# include obstacle collisions: SphObstTime / SphObstEvent
# (src/TimePrediction.c:1020-1071, src/Events.c:752-795), Andersen NVT at T* 0.6.
import os as _os

import numpy as _np

with open(_os.path.join(REF, "input", "ala10.gro")) as _f:
    _gro = _f.read()
_lines = _gro.splitlines()
_n = int(_lines[1])
_xyz = _np.array([[float(l[20:28]), float(l[28:36]), float(l[36:44])] for l in _lines[2:2 + _n]]) * 10
_R = 6.0
_picked = []
for _gx in _np.arange(60.0, 90.0, 0.5):
    for _gy in _np.arange(60.0, 90.0, 0.5):
        for _gz in _np.arange(60.0, 90.0, 0.5):
            _p = _np.array([_gx, _gy, _gz])
            _d = _np.sqrt(((_xyz - _p) ** 2).sum(1)).min()
            _apart = True   # (no generator expressions: this file runs under exec with its own locals)
            for _q in _picked:
                if _np.sqrt(((_p - _q) ** 2).sum()) <= 2 * _R + 2:
                    _apart = False
            if _R + 0.3 <= _d <= _R + 0.7 and _apart:
                _picked.append(_p)
            if len(_picked) == 4:
                break
        if len(_picked) == 4:
            break
    if len(_picked) == 4:
        break
_parts = []
for _p in _picked:
    _parts.append(f"{_p[0]:.2f} {_p[1]:.2f} {_p[2]:.2f} {2 * _R:.1f}")
_sph = " , ".join(_parts)

CASE = dict(gro_text=_gro, params=base_params(sphobst=f"{len(_picked)} {_sph}"), n_events=14000, ckpts=[5000, 10000])
# (14k events: the run's thermostat draw near 14.8k events is one of those where
# glibc's log() is not correctly rounded, so the reference's trajectory leaves the
# correctly rounded one there.)
