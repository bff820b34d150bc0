# The cylinder-wall case (ala10_cyl.case.py) with a compressing wall: WallDyn
# compress, -Wsz 2 -Wrt 10 (the diameter shrinks by 2 A over 10 time units, 0.2 A
# a time unit), so that DoWallDyn (src/Events.c:502-541) moves the wall during the
# run and WallTime widens the box again while an atom is outside it
# (src/TimePrediction.c:674-697).
import os as _os

_spec = {}
with open(_os.path.join(extra, "ala10_cyl.case.py")) as _f:
    exec(_f.read(), {"base_params": base_params, "extra": extra, "REF": REF}, _spec)
CASE = dict(_spec["CASE"])
CASE["params"] = dict(CASE["params"], wall_dyn="compress")
CASE["n_events"] = 20000
CASE["ckpts"] = [5000, 10000, 15000]
CASE["args"] = ("-Wsz", "2", "-Wrt", "10")
