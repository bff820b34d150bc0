"""Host-side mirror of the C ABI structs in include/sdmd_gpu.h.

`System` owns the numpy arrays of one simulated system (atom ids 1..N, entry 0
unused, as in the reference's atom[1..atomnum]) and exposes a ctypes
`sdmd_system` pointing into them.  The arrays are the reference's state
restated as SoA: `x` is atom[i].dynamic->coordinate[1], `ev_time` is
atom[i].dynamic->event.time, `cell_list` is the reference's celllist, and so on
(src/DMD.h:231-466).
"""
import ctypes as C

import numpy as np

NTYPES = 33
NTABLES = 12

i32p = C.POINTER(C.c_int32)
i64p = C.POINTER(C.c_int64)
f64p = C.POINTER(C.c_double)


class sdmd_rng(C.Structure):
    _fields_ = [("tab", C.c_int32 * 31), ("front", C.c_int32), ("rear", C.c_int32)]


class sdmd_counters(C.Structure):
    _fields_ = [("frame", C.c_int64), ("recal", C.c_int64), ("collision", C.c_int64), ("bond", C.c_int64),
                ("hb", C.c_int64), ("hbneighbor", C.c_int64), ("thermostat", C.c_int64), ("pcc", C.c_int64),
                ("wall", C.c_int64), ("warnings", C.c_int64), ("hb_formed", C.c_int32),
                ("alpha_hb_formed", C.c_int32)]


# (field name, ctypes type); array fields are listed with their numpy dtype below
_SCALARS_HEAD = [("n_atoms", C.c_int32), ("cellnum", C.c_int32 * 3), ("n_bonds", C.c_int32),
                 ("n_cons", C.c_int32), ("n_con_steps", C.c_int32), ("n_conn", C.c_int32),
                 ("n_pair_steps", C.c_int32),
                 ("box", C.c_double * 3), ("cellsize", C.c_double * 3), ("cutoff", C.c_double),
                 ("temperature", C.c_double), ("thermo_freq", C.c_double), ("t_end", C.c_double),
                 ("thermostat", C.c_int32), ("wall", C.c_int32), ("wall_pos", C.c_double * 3),
                 ("wall_vel", C.c_double * 3), ("wall_mass", C.c_double), ("wall_type", C.c_int32),
                 ("hb_barrier", C.c_double * 3)]

STATIC_ARRAYS = [("mass", np.float64), ("protein", np.int32), ("aanum", np.int32), ("aatype", np.int32),
                 ("hb_neighbor", np.int32), ("hb_role", np.int32), ("name_code", np.int32),
                 ("bond_off", np.int32), ("bond_j", np.int32), ("bond_dmin", np.float64), ("bond_dmax", np.float64),
                 ("con_off", np.int32), ("con_j", np.int32), ("con_step_off", np.int32), ("con_step_n", np.int32),
                 ("con_dmin", np.float64), ("con_dmax", np.float64), ("con_step_d", np.float64),
                 ("con_step_e", np.float64), ("con_step_acc", np.float64),
                 ("conn_off", np.int32), ("conn_j", np.int32), ("conn_bits", np.int32),
                 ("pair_dmin", np.float64), ("pair_dmax", np.float64), ("pair_step_off", np.int32),
                 ("pair_step_n", np.int32), ("pair_step_d", np.float64), ("pair_step_e", np.float64),
                 ("pair_step_acc", np.float64)]

DYNAMIC_ARRAYS = [("x", np.float64), ("y", np.float64), ("z", np.float64), ("vx", np.float64),
                  ("vy", np.float64), ("vz", np.float64), ("cx", np.int32), ("cy", np.int32), ("cz", np.int32),
                  ("type", np.int32), ("hb_bond", np.int32), ("hb_itype", np.int32), ("nb_partner", np.int32),
                  ("nb_status", np.int32), ("nb_pnum", np.int32), ("ev_time", np.float64),
                  ("ev_partner", np.int32), ("ev_counter", np.int64), ("ev_pcounter", np.int64),
                  ("ev_potential", np.float64), ("ev_type", np.int32), ("ev_sub", np.int32),
                  ("cell_list", np.int32)]

_PTR = {np.float64: f64p, np.int32: i32p, np.int64: i64p}


class sdmd_system(C.Structure):
    _fields_ = (_SCALARS_HEAD
                + [(n, _PTR[t]) for n, t in STATIC_ARRAYS]
                + [(n, _PTR[t]) for n, t in DYNAMIC_ARRAYS]
                + [("time", C.c_double), ("rng", sdmd_rng), ("counters", sdmd_counters)]
                + [("n_sphobst", C.c_int32), ("sphobst", f64p), ("n_obst", C.c_int32), ("obst", f64p)]
                + [("wall_dyn", C.c_int32), ("wall_dyn_sign", C.c_int32), ("wall_dyn_touch", C.c_int32),
                   ("wall_dyn_size", C.c_double), ("wall_dyn_rate", C.c_double), ("wall_dyn_step", C.c_double),
                   ("wall_dyn_cur_time", C.c_double), ("wall_dyn_orig_box", C.c_double * 3)])

MAX_SPHOBST = 64   # SDMD_MAX_SPHOBST


class sdmd_trace_rec(C.Structure):
    _fields_ = [("target", C.c_int32), ("partner", C.c_int32), ("type", C.c_int32), ("sub", C.c_int32),
                ("executed", C.c_int32), ("hb_itype_after", C.c_int32), ("t_new_partner", C.c_int32),
                ("t_new_type", C.c_int32), ("p_new_partner", C.c_int32), ("p_new_type", C.c_int32),
                ("system", C.c_int32), ("pad", C.c_int32), ("dt", C.c_double), ("time_now", C.c_double),
                ("vt", C.c_double * 3), ("vp", C.c_double * 3), ("t_new_time", C.c_double),
                ("p_new_time", C.c_double)]


TRACE_DTYPE = np.dtype([("target", np.int32), ("partner", np.int32), ("type", np.int32), ("sub", np.int32),
                        ("executed", np.int32), ("hb_itype_after", np.int32), ("t_new_partner", np.int32),
                        ("t_new_type", np.int32), ("p_new_partner", np.int32), ("p_new_type", np.int32),
                        ("system", np.int32), ("pad", np.int32), ("dt", np.float64), ("time_now", np.float64),
                        ("vt", np.float64, 3), ("vp", np.float64, 3), ("t_new_time", np.float64),
                        ("p_new_time", np.float64)])
assert TRACE_DTYPE.itemsize == C.sizeof(sdmd_trace_rec)


class sdmd_opts(C.Structure):
    _fields_ = [("advance", C.c_int32), ("screen", C.c_int32), ("threads_per_system", C.c_int32),
                ("device", C.c_int32), ("trace_capacity", C.c_int32), ("helper_blocks", C.c_int32),
                ("reserved", C.c_int32 * 6)]


class sdmd_error_info(C.Structure):
    _fields_ = [("code", C.c_int32), ("system", C.c_int32), ("atom", C.c_int32), ("event", C.c_int64)]


WALL = {"no": 0, "parallel": 1, "cylinder": 2, "sphere": 3}


def glibc_rng_state(seed, skip=0):
    """The rand() stream state after srand(seed) and `skip` draws, as the
    33-entry sdmd_rng layout [tab[0..30], front, rear].  Lehmer-seeded additive
    feedback generator of degree 31 and separation 3 (the first 310 outputs are
    discarded at seeding)."""
    r = [0] * 31
    r[0] = seed if seed != 0 else 1
    for i in range(1, 31):
        hi, lo = divmod(r[i - 1], 127773)
        w = 16807 * lo - 2836 * hi
        if w < 0:
            w += 2147483647
        r[i] = w
    f, b = 3, 0
    for _ in range(310 + skip):
        r[f] = (r[f] + r[b]) & 0xFFFFFFFF
        f += 1
        b += 1
        if f >= 31:
            f = 0
        elif b >= 31:
            b = 0
    tab = np.array(r, np.uint32).view(np.int32)
    return np.concatenate([tab, np.array([f, b], np.int32)])


# (name, dtype, pointer slot) of every array field of sdmd_system
_ARRAY_SLOTS = [(name, dt, getattr(sdmd_system, name).offset // C.sizeof(C.c_void_p))
                for name, dt in STATIC_ARRAYS + DYNAMIC_ARRAYS]
assert all(getattr(sdmd_system, n).offset % C.sizeof(C.c_void_p) == 0 for n, _, _ in _ARRAY_SLOTS)
assert C.sizeof(C.c_void_p) == 8 and C.sizeof(sdmd_system) % 8 == 0
_SLOT_INDEX = np.array([slot for _, _, slot in _ARRAY_SLOTS], np.intp)
assert C.sizeof(sdmd_rng) == 33 * 4


class System:
    """Arrays of one system plus its ctypes view.  Construct with `from_arrays`."""

    def __init__(self):
        self.a = {}
        self.scal = {}
        self.rng = np.zeros(33, np.int32)
        self.counters = {}
        self.time = 0.0
        self._struct = None
        self._ptr_arrays = None   # the arrays whose addresses _ptrs holds
        self._ptrs = None

    @property
    def n(self):
        return int(self.scal["n_atoms"])

    def copy(self):
        o = System()
        o.a = {k: v.copy() for k, v in self.a.items()}
        o.scal = dict(self.scal)
        o.rng = self.rng.copy()
        o.counters = dict(self.counters)
        o.time = self.time
        return o

    def struct(self):
        """ctypes sdmd_system viewing this object's arrays (rebuilt each call; the
        scalars are copied in, the arrays are shared).  The array pointers are
        written as integers into the struct's pointer slots, and the RNG state is
        one 33-word copy: a batch of hundreds of systems is marshalled in a few ms."""
        s = sdmd_system()
        for k, v in self.scal.items():
            if isinstance(v, (list, tuple, np.ndarray)):
                arr = getattr(s, k)
                for i, x in enumerate(v):
                    arr[i] = x
            else:
                setattr(s, k, v)
        arrs = [self.a[name] for name, _, _ in _ARRAY_SLOTS]
        held = self._ptr_arrays
        if held is None or any(a is not b for a, b in zip(arrs, held)):
            # arrays replaced since the last call: check them and take their addresses
            # (the list keeps those very arrays alive, so the addresses stay theirs)
            for (name, dt, _), arr in zip(_ARRAY_SLOTS, arrs):
                if arr.dtype != dt or not arr.flags.c_contiguous:
                    raise ValueError(f"array {name}: need C-contiguous {np.dtype(dt).name}")
            self._ptrs = np.array([arr.__array_interface__["data"][0] for arr in arrs], np.uint64)
            self._ptr_arrays = arrs
        np.frombuffer(s, np.uint64, C.sizeof(sdmd_system) // 8)[_SLOT_INDEX] = self._ptrs
        sph = self.a.get("sphobst")
        if sph is not None and len(sph):   # spherical obstacles: x, y, z, radius each
            if sph.dtype != np.float64 or not sph.flags.c_contiguous or len(sph) % 4:
                raise ValueError("array sphobst: need C-contiguous float64, 4 per obstacle")
            s.n_sphobst = len(sph) // 4
            s.sphobst = sph.ctypes.data_as(f64p)
        ob = self.a.get("obst")
        if ob is not None and len(ob):     # obstruction walls: position[1..3] each
            if ob.dtype != np.float64 or not ob.flags.c_contiguous or len(ob) % 3:
                raise ValueError("array obst: need C-contiguous float64, 3 per obstacle")
            s.n_obst = len(ob) // 3
            s.obst = ob.ctypes.data_as(f64p)
        s.time = self.time
        rng = np.ascontiguousarray(self.rng, np.int32)
        C.memmove(C.addressof(s.rng), rng.ctypes.data, 33 * 4)
        for k, v in self.counters.items():
            setattr(s.counters, k, int(v))
        self._struct = s
        return s

    def pull_scalars(self, s):
        """Copy dynamic scalars (time, RNG, counters) back from a ctypes struct."""
        self.time = s.time
        self.rng[:31] = np.array(s.rng.tab[:], np.int32)
        self.rng[31] = s.rng.front
        self.rng[32] = s.rng.rear
        for k, _ in sdmd_counters._fields_:
            self.counters[k] = getattr(s.counters, k)
        if "wall_dyn" in self.scal:   # a dynamic wall moves the box as the run goes
            self.scal["box"] = list(s.box)
            for k in ("wall_dyn", "wall_dyn_sign", "wall_dyn_touch", "wall_dyn_size", "wall_dyn_rate", "wall_dyn_step",
                      "wall_dyn_cur_time"):
                self.scal[k] = getattr(s, k)

    def state_digest(self):
        """Everything the loop mutates, for exact comparisons."""
        keys = ["x", "y", "z", "vx", "vy", "vz", "cx", "cy", "cz", "type", "hb_bond", "hb_itype", "nb_partner",
                "nb_status", "nb_pnum", "ev_time", "ev_partner", "ev_counter", "ev_pcounter", "ev_potential",
                "ev_type", "ev_sub", "cell_list"]
        return {k: self.a[k].copy() for k in keys}


def _conn_rows(n, triples):
    """Sparse (i, j, bits) triples -> CSR (off[N+2], j[], bits[]) rows for i = 0..N."""
    t = np.asarray(triples, np.int32).reshape(-1, 3)
    order = np.lexsort((t[:, 1], t[:, 0]))
    t = t[order]
    counts = np.bincount(t[:, 0], minlength=n + 1)[: n + 1]
    off = np.zeros(n + 2, np.int32)
    off[1:] = np.cumsum(counts)
    return off, t[:, 1].copy(), t[:, 2].copy()


def from_fixture(npz, stage="pre", dynamic_stage=None):
    """Build a System from a golden fixture (tests/golden/*.npz).  Static data
    comes from `stage` ("pre"); dynamic state from `dynamic_stage` (default the
    same stage)."""
    d = npz
    g = lambda k: d[f"pre/{k}"]
    ds = dynamic_stage or stage
    h = lambda k: d[f"{ds}/{k}"]
    n = int(g("atomnum")[0])
    s = System()
    cellnum = [int(v) for v in g("cellnum")]
    wall_exist = bytes(g("wallExist")).decode()
    wall_type = bytes(g("wallType")).decode()
    wall = 0
    if wall_exist.startswith("sm"):
        wall = {"p": 1, "c": 2, "s": 3}.get(wall_type[:1], 0)
    hbp = g("HBPotential")   # BB_r BB_v SS_r SS_v BS_r BS_v
    s.scal = dict(n_atoms=n, cellnum=cellnum, box=[float(v) for v in g("box")],
                  cellsize=[float(v) for v in g("cellsize")], cutoff=float(g("cutoffr")[0]),
                  temperature=float(g("targetTemperature")[0]), thermo_freq=float(g("thermoF")[0]),
                  t_end=float(g("timestep")[0]),
                  thermostat=0 if bytes(g("thermostatType")).decode() == "no" else 1,
                  wall=wall, wall_pos=[0.0, 0.0, 0.0], wall_vel=[0.0, 0.0, 0.0], wall_mass=0.0, wall_type=0,
                  hb_barrier=[float(hbp[1]), float(hbp[5]), float(hbp[3])])
    if wall and "pre/wall_pos" in d.files:
        s.scal.update(wall_pos=[float(v) for v in g("wall_pos")], wall_vel=[float(v) for v in g("wall_vel")],
                      wall_mass=float(g("wall_mass")[0]), wall_type=int(g("wall_type")[0]))
    a = s.a
    a["mass"] = g("mass").astype(np.float64)
    a["protein"] = g("protein").astype(np.int32)
    a["aanum"] = g("aanum").astype(np.int32)
    a["aatype"] = g("typeofAA").astype(np.int32)
    a["hb_neighbor"] = g("hb_neighbor").astype(np.int32)
    a["hb_role"] = g("hb_role").astype(np.int32)
    names = g("name").reshape(-1, 8)
    code = np.zeros(n + 1, np.int32)
    for i in range(1, n + 1):
        nm = bytes(names[i]).split(b"\0", 1)[0]
        code[i] = 1 if nm == b"H" else (2 if nm == b"O" else 0)
    a["name_code"] = code
    for k in ["bond_off", "bond_j", "con_off", "con_j", "con_step_off", "con_step_n", "pair_step_off", "pair_step_n"]:
        a[k] = g(k).astype(np.int32)
    for k in ["bond_dmin", "bond_dmax", "con_dmin", "con_dmax", "con_step_d", "con_step_e", "con_step_acc",
              "pair_dmin", "pair_dmax", "pair_step_d", "pair_step_e", "pair_step_acc"]:
        a[k] = g(k).astype(np.float64)
    a["bond_off"][0] = 0
    a["con_off"][0] = 0
    a["conn_off"], a["conn_j"], a["conn_bits"] = _conn_rows(n, g("connmap"))
    a["sphobst"] = sphobst_from_parameters(bytes(d["meta/parameter"]).decode()) if "meta/parameter" in d.files \
        else np.zeros(0)
    a["obst"] = g("obst_pos").astype(np.float64) if "pre/obst_pos" in d.files else np.zeros(0)
    if "pre/obst_type" in d.files and not wall:
        s.scal["wall_type"] = int(g("obst_type")[0])   # obstacles are Wall.txt atoms
    if f"{ds}/wall_dyn_i" in d.files:   # a dynamic wall: its state and the box it has moved to
        wi, wd = h("wall_dyn_i"), h("wall_dyn_d")
        s.scal.update(wall_dyn=int(wi[0]), wall_dyn_sign=int(wi[1]), wall_dyn_touch=int(wi[2]),
                      wall_dyn_size=float(wd[0]), wall_dyn_rate=float(wd[1]), wall_dyn_step=float(wd[2]),
                      wall_dyn_cur_time=float(wd[3]), wall_dyn_orig_box=[float(v) for v in wd[4:7]],
                      box=[float(v) for v in h("box_now")])
    _load_dynamic(s, d, ds)
    s.rng = d["meta/rng_pre"].astype(np.int32).copy() if ds == "pre" else np.zeros(33, np.int32)
    for k, v in [("n_bonds", len(a["bond_j"])), ("n_cons", len(a["con_j"])), ("n_con_steps", len(a["con_step_d"])),
                 ("n_conn", len(a["conn_j"])), ("n_pair_steps", len(a["pair_step_d"]))]:
        s.scal[k] = int(v)
    return s


def sphobst_from_parameters(text):
    """The SphObst? line of parameter.txt (its 16th line) as the reference reads it
    (src/Initialization.c:703-724): the count, then x y z diameter per obstacle with
    a separator token between them; returned as x, y, z, radius per obstacle."""
    lines = text.splitlines()
    words = lines[15].split() if len(lines) > 15 else []
    if len(words) < 2 or words[1] == "no":
        return np.zeros(0)
    n, out, q = int(words[1]), [], 2
    for i in range(n):
        x, y, z, dia = (float(v) for v in words[q:q + 4])
        out += [x, y, z, dia / 2]
        q += 4 + (1 if i != n - 1 else 0)
    return np.array(out, np.float64)


def _load_dynamic(s, d, ds):
    a = s.a
    h = lambda k: d[f"{ds}/{k}"]
    for k in ["x", "y", "z", "vx", "vy", "vz", "ev_time", "ev_potential"]:
        a[k] = h(k).astype(np.float64).copy()
    for k in ["cx", "cy", "cz", "type", "hb_bond", "hb_itype", "nb_status", "nb_pnum", "ev_partner", "ev_type",
              "ev_sub", "celllist"]:
        a["cell_list" if k == "celllist" else k] = h(k).astype(np.int32).copy()
    a["ev_counter"] = h("ev_counter").astype(np.int64).copy()
    a["ev_pcounter"] = h("ev_pcounter").astype(np.int64).copy()
    nb = np.stack([h(f"nb_p{k}") for k in range(1, 5)], axis=1).astype(np.int32)
    a["nb_partner"] = np.ascontiguousarray(nb.reshape(-1))
    s.time = float(h("currenttime")[0])
    ec = h("event_counts")
    s.counters = dict(frame=int(h("frame")[0]), recal=int(h("countReCal")[0]), collision=int(ec[0]),
                      bond=int(ec[1]), hb=int(ec[2]), hbneighbor=int(ec[3]), thermostat=int(ec[4]), pcc=int(ec[5]),
                      wall=int(ec[6]), warnings=int(h("warningsum")[0]), hb_formed=int(h("HBnumformed")[0]),
                      alpha_hb_formed=int(h("alphaHBformed")[0]))


def fixture_dynamic(npz, stage):
    """Reference dynamic state of a fixture stage as a {name: array} dict in the
    System naming (for comparisons)."""
    s = System()
    _load_dynamic(s, npz, stage)
    out = dict(s.a)
    out["_time"] = s.time
    out["_counters"] = s.counters
    if f"{stage}/box_now" in npz.files:   # a dynamic wall's box and state
        out["_box"] = [float(v) for v in npz[f"{stage}/box_now"]]
        out["_wall_dyn_i"] = [int(v) for v in npz[f"{stage}/wall_dyn_i"]]
        out["_wall_dyn_d"] = [float(v) for v in npz[f"{stage}/wall_dyn_d"]]
    return out
