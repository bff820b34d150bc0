# The reference's ala10 input with two obstruction walls (Obstruct?): planes at
# x = 65.5 A and z = 84.5 A, each about 4 A from the chain's nearest atom, so that
# the first events include obstacle collisions: ObstTime / ObstEvent
# (src/TimePrediction.c:740-829, src/Events.c:543-617), Andersen NVT at T* 0.6.
# The obstacle atoms read Wall.txt; the library is a test-local copy naming an
# existing atom type (CA): the shipped one names PHO, which AtomModel lacks
# (src/Models.c:129-206).
import os as _os

with open(_os.path.join(REF, "input", "ala10.gro")) as _f:
    _gro = _f.read()

CASE = dict(gro_text=_gro, params=base_params(obstruct="2 x 65.5 , z 84.5"), n_events=14000, ckpts=[5000, 10000],
            wall_lib="Wall\n   ATOM CA      CA   12.0  N N\n")
