"""Python front end of the host-side C builder (libsdmd_host.so, include/sdmd_host.h).

`build_system` reads the reference's own inputs (parameter.txt, a .gro file and
the Library_<ff> force field) and returns a `System` ready for the engine, in
the state the reference reaches right before its full-rebuild sweep.
"""
import ctypes as C
import os

import numpy as np

from .system import DYNAMIC_ARRAYS, STATIC_ARRAYS, System, sdmd_counters, sdmd_system

HERE = os.path.dirname(os.path.abspath(__file__))
HOST_LIB = os.path.join(HERE, "libsdmd_host.so")
DEBUG_RANDOM_SEED = 1575263273   # the reference's fixed seed under -DDEBUG_RANDOM (src/DMD.h:37)


class sdmd_params(C.Structure):
    _fields_ = [("continue_mode", C.c_char * 20), ("time", C.c_double), ("temperature_str", C.c_char * 20),
                ("temperature", C.c_double), ("dump_rate", C.c_double), ("cutoff", C.c_double),
                ("force_field", C.c_char * 20), ("thermostat", C.c_char * 20), ("thermo_freq", C.c_double),
                ("cg", C.c_char * 16), ("wall_exist", C.c_char * 20), ("wall_type", C.c_char * 20),
                ("wall_dyn", C.c_char * 16), ("flow", C.c_char * 32), ("obstruct", C.c_char * 32),
                ("tunnel", C.c_char * 32), ("sphobst", C.c_char * 32),
                ("n_sphobst", C.c_int32), ("sphobst_xyzr", C.c_double * (4 * 64)),
                ("n_obst", C.c_int32), ("obst_pos", C.c_double * (3 * 16))]


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(HOST_LIB):
            raise RuntimeError(f"{HOST_LIB} is missing: run __graft_entry__.build()")
        L = C.CDLL(HOST_LIB)
        P = C.POINTER
        L.sdmd_read_parameters.argtypes = [C.c_char_p, P(sdmd_params)]
        L.sdmd_build_system.argtypes = [C.c_char_p, C.c_char_p, P(sdmd_params), P(C.c_double), C.c_uint32, C.c_int,
                                        P(C.c_void_p), C.c_char_p, C.c_int]
        L.sdmd_build_system_gro_text.argtypes = [C.c_char_p, C.c_char_p, P(sdmd_params), C.c_uint32, C.c_int,
                                                 P(C.c_void_p), C.c_char_p, C.c_int]
        L.sdmd_host_view.argtypes = [C.c_void_p]
        L.sdmd_host_view.restype = P(sdmd_system)
        L.sdmd_host_free.argtypes = [C.c_void_p]
        L.sdmd_host_free.restype = None
        L.sdmd_host_atom_names.argtypes = [C.c_void_p]
        L.sdmd_host_atom_names.restype = C.c_void_p
        L.sdmd_host_residue_names.argtypes = [C.c_void_p]
        L.sdmd_host_residue_names.restype = C.c_void_p
        _lib = L
    return _lib


def read_parameters(path):
    p = sdmd_params()
    rc = lib().sdmd_read_parameters(path.encode(), C.byref(p))
    if rc:
        raise ValueError(f"cannot parse {path}")
    return p


def params_text(time=5000, temp=0.6, dump=1e9, cutoff=9.0, thermostat="Andersen", thermo_freq=6.0,
                wall_exist="no", wall_type="no"):
    """parameter.txt in the reference's positional layout (src/Initialization.c:527-726)."""
    return (f"Continue?          new\nTime               {time}\nT(reduced)         {temp}\n"
            f"Dump_Rate          {dump}\nCutOff_R(A)        {cutoff}\nForce_Field        Ding\n"
            f"Thermostat         {thermostat}\nThermo_Freq        {thermo_freq}\nCGModel            no\n"
            f"WallExist?         {wall_exist}\nWallType           {wall_type}\nWallDyn            no\n"
            f"Flow               no\nObstruct?          no\nTunnel?            no\nSphObst?           no\n")


def _copy_out(view, names_ptr, res_ptr):
    s = view.contents
    n = s.n_atoms
    sizes = {
        "N1": n + 1, "bond_off": n + 2, "con_off": n + 2, "conn_off": n + 2,
        "bond_j": s.n_bonds, "bond_dmin": s.n_bonds, "bond_dmax": s.n_bonds,
        "con_j": s.n_cons, "con_step_off": s.n_cons, "con_step_n": s.n_cons, "con_dmin": s.n_cons,
        "con_dmax": s.n_cons, "con_step_d": s.n_con_steps, "con_step_e": s.n_con_steps,
        "con_step_acc": s.n_con_steps, "conn_j": s.n_conn, "conn_bits": s.n_conn,
        "pair_dmin": 12 * 33 * 33, "pair_dmax": 12 * 33 * 33, "pair_step_off": 12 * 33 * 33,
        "pair_step_n": 12 * 33 * 33, "pair_step_d": s.n_pair_steps, "pair_step_e": s.n_pair_steps,
        "pair_step_acc": s.n_pair_steps, "nb_partner": 4 * (n + 1),
        "cell_list": n + 1 + s.cellnum[0] * s.cellnum[1] * s.cellnum[2],
    }
    out = System()
    for name, dt in STATIC_ARRAYS + DYNAMIC_ARRAYS:
        cnt = sizes.get(name, n + 1)
        ptr = getattr(s, name)
        arr = np.ctypeslib.as_array(ptr, shape=(max(cnt, 1),))[:cnt] if cnt > 0 else np.zeros(0, dt)
        out.a[name] = np.array(arr, dtype=dt, copy=True)
    out.scal = dict(n_atoms=n, cellnum=list(s.cellnum), box=list(s.box), cellsize=list(s.cellsize),
                    cutoff=s.cutoff, temperature=s.temperature, thermo_freq=s.thermo_freq, t_end=s.t_end,
                    thermostat=s.thermostat, wall=s.wall, wall_pos=list(s.wall_pos), wall_vel=list(s.wall_vel),
                    wall_mass=s.wall_mass, wall_type=s.wall_type, hb_barrier=list(s.hb_barrier),
                    n_bonds=s.n_bonds, n_cons=s.n_cons, n_con_steps=s.n_con_steps, n_conn=s.n_conn,
                    n_pair_steps=s.n_pair_steps)
    nsph = s.n_sphobst if s.sphobst else 0
    out.a["sphobst"] = np.array(np.ctypeslib.as_array(s.sphobst, shape=(4 * nsph,)), np.float64) if nsph \
        else np.zeros(0)
    nob = s.n_obst if s.obst else 0
    out.a["obst"] = np.array(np.ctypeslib.as_array(s.obst, shape=(3 * nob,)), np.float64) if nob else np.zeros(0)
    out.pull_scalars(s)
    out.names = C.string_at(names_ptr, 8 * (n + 1)) if names_ptr else None
    out.resnames = C.string_at(res_ptr, 8 * (n + 1)) if res_ptr else None
    return out


def system_from_struct(ptr):
    """A System holding copies of the arrays an sdmd_system (POINTER) points to."""
    return _copy_out(ptr, None, None)


def build_system(datadir, coord_file=None, gro_text=None, params=None, param_path=None, seed=DEBUG_RANDOM_SEED,
                 energy_min_steps=20000):
    """Build a System from the reference's inputs.  Give either a coordinate
    file name inside `datadir` or the .gro text; parameters from `param_path`
    (default <datadir>/parameter.txt) or a filled sdmd_params."""
    if params is None:
        params = read_parameters(param_path or os.path.join(datadir, "parameter.txt"))
    h = C.c_void_p()
    err = C.create_string_buffer(1024)
    if gro_text is not None:
        rc = lib().sdmd_build_system_gro_text(datadir.encode(), gro_text.encode(), C.byref(params), seed,
                                              energy_min_steps, C.byref(h), err, 1024)
    else:
        rc = lib().sdmd_build_system(datadir.encode(), coord_file.encode(), C.byref(params), None, seed,
                                     energy_min_steps, C.byref(h), err, 1024)
    if rc:
        raise ValueError(f"system build failed: {err.value.decode()}")
    try:
        return _copy_out(lib().sdmd_host_view(h), lib().sdmd_host_atom_names(h), lib().sdmd_host_residue_names(h))
    finally:
        lib().sdmd_host_free(h)


AMINO_ACIDS = ["ALA", "ARG", "ASN", "ASP", "CYS", "GLN", "GLU", "GLY", "HIS", "ILE", "LEU", "LYS", "MET", "PHE",
               "PRO", "SER", "THR", "TRP", "TYR", "VAL"]


def generate_gro(datadir, sequences, box, wall=0, margin=5.0, seed=1, ff="Ding"):
    """.gro text for peptides with the given sequences (lists of 3-letter codes)."""
    L = lib()
    L.sdmd_generate_gro.argtypes = [C.c_char_p, C.c_char_p, C.c_int, C.POINTER(C.c_char_p), C.POINTER(C.c_double),
                                    C.c_int, C.c_double, C.c_uint64, C.POINTER(C.c_void_p), C.c_char_p, C.c_int]
    L.sdmd_free_text.argtypes = [C.c_void_p]
    L.sdmd_free_text.restype = None
    seqs = (C.c_char_p * len(sequences))(*[" ".join(s).encode() for s in sequences])
    b = (C.c_double * 3)(*box)
    out = C.c_void_p()
    err = C.create_string_buffer(1024)
    rc = L.sdmd_generate_gro(datadir.encode(), ff.encode(), len(sequences), seqs, b, wall, margin, seed,
                             C.byref(out), err, 1024)
    if rc:
        raise ValueError(f"generation failed: {err.value.decode()}")
    try:
        return C.string_at(out).decode()
    finally:
        L.sdmd_free_text(out)


# ---- the reference's command line and REMD configuration (host/cli.c) ----------
NOUT, NCHARGE, REMD_MAX = 11, 9, 1024
OUT_NAMES = ["saved", "trj", "pot", "kin", "tem", "cnt", "HBn", "xyz", "pdb", "log", "sys"]


class sdmd_cli(C.Structure):
    _fields_ = [("datadir", C.c_char * 1024), ("savedir", C.c_char * 1024), ("coordinate_file", C.c_char * 256),
                ("saved_in", C.c_char * 256), ("out_name", (C.c_char * 256) * NOUT), ("out_on", C.c_int32 * NOUT),
                ("box", C.c_double * 3), ("box_given", C.c_int32), ("wall_dyn_size", C.c_double),
                ("wall_dyn_rate", C.c_double), ("pre_bonds", C.c_int32), ("charge", C.c_int32 * NCHARGE),
                ("charge_no_pbc", C.c_int32), ("remd", C.c_int32), ("remd_server", C.c_char * 256),
                ("remd_port", C.c_int32), ("remd_num", C.c_int32), ("remd_rate", C.c_int32), ("remd_T", C.c_double),
                ("remd_suffix", C.c_char * 64), ("visual", C.c_int32), ("help", C.c_int32)]


class sdmd_remd_config(C.Structure):
    _fields_ = [("n_replicas", C.c_int32), ("port", C.c_int32), ("exchange_time", C.c_double),
                ("T_kelvin", C.c_double * REMD_MAX), ("T", C.c_double * REMD_MAX), ("num", C.c_int32 * REMD_MAX)]


class sdmd_replica(C.Structure):
    """A REMD replica's REMDInfo record (include/sdmd_host.h)."""
    _fields_ = [("port", C.c_int32), ("output_rate", C.c_int32), ("num", C.c_int32), ("T", C.c_double),
                ("server", C.c_char * 50), ("extra", C.c_char * 50)]


def parse_args(argv):
    """sdmd_parse_args over a list of strings (argv[0] is the program name)."""
    L = lib()
    L.sdmd_parse_args.argtypes = [C.c_int, C.POINTER(C.c_char_p), C.POINTER(sdmd_cli), C.c_char_p, C.c_int]
    arr = (C.c_char_p * len(argv))(*[a.encode() for a in argv])
    out = sdmd_cli()
    err = C.create_string_buffer(512)
    rc = L.sdmd_parse_args(len(argv), arr, C.byref(out), err, 512)
    if rc:
        raise ValueError(err.value.decode())
    return out


def read_remd_config(path):
    """sdmd_read_remd_config: dict(n, port, exchange_time, T_kelvin, T, num)."""
    L = lib()
    L.sdmd_read_remd_config.argtypes = [C.c_char_p, C.POINTER(sdmd_remd_config), C.c_char_p, C.c_int]
    cfg = sdmd_remd_config()
    err = C.create_string_buffer(512)
    rc = L.sdmd_read_remd_config(str(path).encode(), C.byref(cfg), err, 512)
    if rc:
        raise ValueError(err.value.decode())
    n = cfg.n_replicas
    return {"n": n, "port": cfg.port, "exchange_time": cfg.exchange_time, "T_kelvin": list(cfg.T_kelvin[:n]),
            "T": np.array(cfg.T[:n]), "num": np.array(cfg.num[:n], np.int32)}
