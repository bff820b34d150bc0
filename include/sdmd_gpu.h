/*
 * sdmd_gpu.h -- C ABI of the GB300 event-loop engine for sDMD.
 *
 * The engine replaces the reference's event loop below ThreadProcess()
 * (src/ToolFunctions.c:12-20): Prepare() (src/SGThread.c:21-64), SingleThreadRun()
 * (src/SGThread.c:67-155), Predict() (src/SGThread.c:158-211), the CBT event queue
 * (src/CBT.c) and event execution (src/Events.c).  Parsing, model building and the
 * output writers stay on the host.
 *
 * Conventions
 *   - Atom ids are 1..N exactly as in the reference (atom[1..atomnum]); every
 *     per-atom array below has N+1 entries and entry 0 is unused.
 *   - Vectors are SoA (x[], y[], z[]), FP64, in the reference's units (A, u,
 *     kcal/mol, 48.88 fs time unit).
 *   - Every function returns SDMD_OK (0) or a negative SDMD_E* code; device-side
 *     physics errors carry (system, atom, event#) retrievable with
 *     sdmd_gpu_last_error().  No function exits the process.
 *   - Handles are not thread-safe; one host thread per handle, one CUDA stream
 *     per handle.  No pointer into caller memory is retained past a call.
 */
#ifndef SDMD_GPU_H
#define SDMD_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SDMD_ABI_VERSION 2

/* ---- status codes ---------------------------------------------------------- */
#define SDMD_OK              0
#define SDMD_EINVAL         -1   /* bad argument / inconsistent sizes            */
#define SDMD_ENOMEM         -2   /* device or host allocation failed             */
#define SDMD_ECUDA          -3   /* CUDA runtime error                           */
#define SDMD_ENODEV         -4   /* no CUDA device                               */
#define SDMD_ENEGTIME       -10  /* predicted event time < 0 (src/TimePrediction.c:168-173) */
#define SDMD_ENAN           -11  /* NaN phi in a velocity update (src/Events.c:1008-1011)   */
#define SDMD_EWALL          -12  /* atom outside the wall (src/TimePrediction.c:700-701)    */
#define SDMD_ELINK          -13  /* cell-list corruption (src/Events.c:182-192)             */
#define SDMD_EHBMAP         -14  /* HB bookkeeping inconsistent (src/Events.c:313-321)      */
#define SDMD_ECAPACITY      -15  /* a fixed device capacity was exceeded                  */
#define SDMD_ETIMEOUT       -16  /* a bounded device-side wait ran out                     */
#define SDMD_EUNSUPPORTED   -17  /* configuration outside the engine's scope              */
#define SDMD_EEVENTTYPE     -18  /* invalid event type popped (src/Events.c:104-108)       */

/* ---- event / sub-event enums (values of src/DMD.h:162-190) ----------------- */
enum {
    SDMD_EV_COLLISION = 0, SDMD_EV_BOND = 1, SDMD_EV_HB = 2, SDMD_EV_HBNEIGHBOR = 3,
    SDMD_EV_THERMOSTAT = 4, SDMD_EV_WALL = 5, SDMD_EV_OBST = 6, SDMD_EV_SPHOBST = 9, SDMD_EV_PCC = 10,
    SDMD_EV_INVALID = 15
};
enum {
    SDMD_SUB_CORE = 0, SDMD_SUB_WELL_BOUNCE = 1, SDMD_SUB_WELL_CAPTURE = 2,
    SDMD_SUB_WELL_ESCAPE = 3, SDMD_SUB_TBD_CAPTURE = 4, SDMD_SUB_TBD_ESCAPE = 5,
    SDMD_SUB_TBD_HBFORM = 6, SDMD_SUB_TBD_HBBREAK = 7, SDMD_SUB_INVALID = 8
};
enum { SDMD_HB_NOEVENT = 0, SDMD_HB_FORM = 1, SDMD_HB_BREAK = 2, SDMD_HB_SKIP = 3 };
enum { SDMD_WALL_NONE = 0, SDMD_WALL_PARALLEL = 1, SDMD_WALL_CYLINDER = 2, SDMD_WALL_SPHERE = 3 };

#define SDMD_NTYPES   33     /* NATOMTYPE + 1 (src/DMD.h:29) */
#define SDMD_NTABLES  12     /* table 0: collision pairs; 1..11: HB classes (src/DMD.c:98-99) */
#define SDMD_INVALID  (-111) /* src/DMD.h:28 */
#define SDMD_MAX_SPHOBST 64  /* spherical obstacles per system */
#define SDMD_MAX_OBST    16  /* obstruction walls per system */
#define SDMD_INFINIT  1e8    /* src/DMD.h:26 */
#define SDMD_ZERO     1e-8   /* src/DMD.h:27 */

/* glibc-compatible additive-feedback RNG state (TYPE_3, degree 31, separation 3):
 * the stream rand() produces after srand(seed).  The reference draws every
 * random number through rand() (src/ToolFunctions.c:517-522). */
typedef struct sdmd_rng {
    int32_t tab[31];
    int32_t front, rear;          /* indices into tab */
} sdmd_rng;

/* Event-type counters, order of src/DMD.c:50-58 */
typedef struct sdmd_counters {
    int64_t frame;                /* executed events  (src/SGThread.c:100) */
    int64_t recal;                /* denied pops      (src/SGThread.c:150) */
    int64_t collision, bond, hb, hbneighbor, thermostat, pcc, wall;
    int64_t warnings;             /* warningsum */
    int32_t hb_formed, alpha_hb_formed;
} sdmd_counters;

/*
 * One simulated system (a replica or an independent system of a batch).
 * Static arrays are read at sdmd_gpu_create/upload; dynamic arrays are read at
 * upload and written by sdmd_gpu_download.
 */
typedef struct sdmd_system {
    /* ---- sizes ---- */
    int32_t n_atoms;
    int32_t cellnum[3];            /* cellnum[1..3] of the reference */
    int32_t n_bonds, n_cons, n_con_steps, n_conn, n_pair_steps;

    /* ---- parameters (src/Initialization.c:512-730) ---- */
    double  box[3];                /* boxDimension[1..3] */
    double  cellsize[3];
    double  cutoff;                /* cutoffr */
    double  temperature;           /* targetTemperature (reduced) */
    double  thermo_freq;           /* thermoF */
    double  t_end;                 /* timestep: the loop runs while time <= t_end */
    int32_t thermostat;            /* 0 none, 1 Andersen */
    int32_t wall;                  /* SDMD_WALL_* ("smooth" walls only) */
    double  wall_pos[3], wall_vel[3], wall_mass;
    int32_t wall_type;             /* atom type of the wall pseudo-atom */
    double  hb_barrier[3];         /* HBPotential BB_v, BS_v, SS_v (src/DMD.h:231-236) */

    /* ---- per-atom static (N+1 entries) ---- */
    const double  *mass;
    const int32_t *protein;        /* sequence.proteinNum */
    const int32_t *aanum;          /* sequence.aminoacidNum (within its protein) */
    const int32_t *aatype;         /* typeofAA (src/Models.c:65) */
    const int32_t *hb_neighbor;    /* HB.neighbor */
    const int32_t *hb_role;        /* HB.role: 'A', 'D', 'S' or 0 */
    const int32_t *name_code;      /* 1: name "H", 2: name "O", 0: other (alpha-HB count only) */

    /* ---- topology ---- */
    const int32_t *bond_off;       /* N+2; bonds of atom i: [bond_off[i], bond_off[i+1]) in list order */
    const int32_t *bond_j;
    const double  *bond_dmin, *bond_dmax;            /* squared lengths */
    const int32_t *con_off;        /* N+2; step-potential constraints of atom i */
    const int32_t *con_j, *con_step_off, *con_step_n;
    const double  *con_dmin, *con_dmax;              /* squared */
    const double  *con_step_d, *con_step_e, *con_step_acc;
    const int32_t *conn_off;       /* N+2; static connection-map bits of atom i (sparse row) */
    const int32_t *conn_j, *conn_bits;               /* bits: 1 BOND_CONNECT, 2 CONSTRAINT_CONNECT */

    /* ---- pair tables [SDMD_NTABLES][SDMD_NTYPES][SDMD_NTYPES] ---- */
    const double  *pair_dmin, *pair_dmax;            /* squared */
    const int32_t *pair_step_off, *pair_step_n;
    const double  *pair_step_d, *pair_step_e, *pair_step_acc;

    /* ---- dynamic per-atom state (N+1 entries) ---- */
    double  *x, *y, *z, *vx, *vy, *vz;
    int32_t *cx, *cy, *cz;         /* cellIndex[1..3] */
    int32_t *type;                 /* typeofAtom (changes on HB form/break) */
    int32_t *hb_bond;              /* HB.bondConnection */
    int32_t *hb_itype;             /* HB.interactionType */
    int32_t *nb_partner;           /* 4*(N+1): neighborPartner[1..4] of atom i at [4*i .. 4*i+3] */
    int32_t *nb_status;            /* HBNeighbor.neighborStatus */
    int32_t *nb_pnum;              /* HBNeighbor.partnerNum */
    double  *ev_time;              /* event.time (relative to the current time) */
    int32_t *ev_partner;
    int64_t *ev_counter, *ev_pcounter;
    double  *ev_potential;
    int32_t *ev_type, *ev_sub;
    int32_t *cell_list;            /* N + ncell + 1: reference celllist (heads at N + cell) */

    /* ---- dynamic scalars ---- */
    double        time;            /* currenttime */
    sdmd_rng      rng;
    sdmd_counters counters;

    /* ---- spherical obstacles (SphObst?, src/Initialization.c:703-724), ABI 2 ----
     * Fixed hard spheres: SphObstTime / SphObstEvent (src/TimePrediction.c:1020-1071,
     * src/Events.c:752-795); an atom's event with obstacle n has partner -1000 n
     * and counts as a wall event.  sphobst: x, y, z, radius per obstacle. */
    int32_t        n_sphobst;      /* 0 .. SDMD_MAX_SPHOBST */
    const double  *sphobst;

    /* ---- obstruction walls (Obstruct?, src/Initialization.c:634-672), ABI 2 ----
     * Planes across one axis: ObstTime / ObstEvent (src/TimePrediction.c:740-829,
     * src/Events.c:543-617) with the potential steps of the pair (atom type,
     * wall_type); obst holds position[1..3] of each obstacle, -1 on the axes it
     * does not cross.  An atom's event with obstacle n across axis d (1..3) has
     * partner -d - 10 n and counts as a wall event.  Obstacles with holes (tunnels)
     * are outside the engine. */
    int32_t        n_obst;         /* 0 .. SDMD_MAX_OBST */
    const double  *obst;

    /* ---- a dynamic smooth wall (WallDyn, -Wsz, -Wrt), ABI 2 ----
     * DoWallDyn (src/Events.c:502-541) after each executed event, and WallTime's
     * widening of the box while an atom is outside a compressed wall
     * (src/TimePrediction.c:674-697); both change box[] as the run goes.  The
     * fields hold DynamicWallStr (src/DMD.h:393-402).  The oracle runs it; the
     * engine returns SDMD_EUNSUPPORTED for wall_dyn != 0. */
    int32_t        wall_dyn;       /* 0 none, 1 compress, 2 expand, 3 pulse */
    int32_t        wall_dyn_sign, wall_dyn_touch;
    double         wall_dyn_size, wall_dyn_rate, wall_dyn_step, wall_dyn_cur_time;
    double         wall_dyn_orig_box[3];
} sdmd_system;

/* one record per popped event; same fields as the reference trace */
typedef struct sdmd_trace_rec {
    int32_t target, partner, type, sub, executed, hb_itype_after;
    int32_t t_new_partner, t_new_type, p_new_partner, p_new_type, system, pad;
    double  dt, time_now;
    double  vt[3], vp[3];
    double  t_new_time, p_new_time;
} sdmd_trace_rec;

/* ---- engine options ---- */
enum { SDMD_ADVANCE_EAGER = 0,   /* x += v*dt for every atom at every pop (bit-exact with the reference) */
       SDMD_ADVANCE_LAZY  = 1 }; /* per-atom local time, FP64 global clock */
enum { SDMD_SCREEN_FP64 = 0,     /* every candidate root in FP64 */
       SDMD_SCREEN_FP32 = 1 };   /* FP32 screen with a proven margin, FP64 refine */

typedef struct sdmd_opts {
    int32_t advance;               /* SDMD_ADVANCE_* */
    int32_t screen;                /* SDMD_SCREEN_* */
    int32_t threads_per_system;    /* 32 (one warp) .. 256, or up to 512 for systems that run with
                                      helper blocks (eager advance, FP32 screen); 0 = 128 */
    int32_t device;                /* CUDA device ordinal */
    int32_t trace_capacity;        /* records kept by sdmd_gpu_run when tracing (0 = off) */
    /* eager advance on the FP32 screened path: blocks on other SMs that advance
     * every atom the pop does not involve, in one cooperative launch with the
     * systems' own blocks (0 = automatic: for up to SMs/2 systems of at least 2,048
     * atoms, every SM the systems leave free; -1 = off; k > 0 = k blocks) */
    int32_t helper_blocks;
    int32_t reserved[6];
} sdmd_opts;

typedef struct sdmd_gpu sdmd_gpu;   /* opaque handle */

typedef struct sdmd_error_info {
    int32_t code, system, atom;
    int64_t event;
} sdmd_error_info;

/* Library / device query.  Returns SDMD_OK if a usable device exists. */
int         sdmd_gpu_abi_version(void);
int         sdmd_gpu_device_count(int32_t *count);
const char *sdmd_gpu_strerror(int code);

/* Create a handle holding n_systems systems on the device and upload their state.
 * Replaces Prepare()'s allocations (src/SGThread.c:21-64). */
int  sdmd_gpu_create(const sdmd_system *systems, int32_t n_systems,
                     const sdmd_opts *opts, sdmd_gpu **out);
void sdmd_gpu_destroy(sdmd_gpu *h);

/* Full-rebuild sweep: Predict() over atoms 1..N of every system
 * (src/SGThread.c:47-52), then build each system's event tree (CreateCBT,
 * src/CBT.c:16-30).  With full_predict == 0 the stored events are kept
 * (continue mode, src/SGThread.c:54-55) and only the trees are built. */
int  sdmd_gpu_prepare(sdmd_gpu *h, int32_t full_predict);

/* Run every system's event loop (src/SGThread.c:75-151) until it has executed
 * max_events more events or its time exceeds t_end (<= 0: the system's own
 * t_end), whichever comes first.  Returns after all systems stopped. */
int  sdmd_gpu_run(sdmd_gpu *h, int64_t max_events, double t_end);

/* SingleThreadRun's dump cadence (src/SGThread.c:128-139): run every system until
 * it executes an event at a time >= dump_time (> 0), after which the reference
 * writes its outputs, or until one of sdmd_gpu_run's limits.  at_dump (may be
 * NULL; n_systems entries) receives 1 for each system that stopped at such an
 * event and 0 for the others; the host then downloads and writes. */
int  sdmd_gpu_run_to_dump(sdmd_gpu *h, double dump_time, int64_t max_events, double t_end, int32_t *at_dump);

/* Copy every system's dynamic state back into the caller's arrays. */
int  sdmd_gpu_download(sdmd_gpu *h, sdmd_system *systems, int32_t n_systems);

/* Copy the last n records of the pop trace of system s (when tracing is on). */
int  sdmd_gpu_trace(sdmd_gpu *h, int32_t s, sdmd_trace_rec *out, int32_t cap, int32_t *n_out);

/* Device time (ms) of the last prepare / run call, measured with CUDA events on
 * the handle's stream. */
int  sdmd_gpu_last_ms(sdmd_gpu *h, double *prepare_ms, double *run_ms);

int  sdmd_gpu_last_error(sdmd_gpu *h, sdmd_error_info *info);

/* Potential (CalPotenE, src/ToolFunctions.c:659-752) and kinetic (CalKinetE,
 * :626-657) energy of every system, in the reference's summation order. */
int  sdmd_gpu_energies(sdmd_gpu *h, double *pot, double *kin);

/* ---- replica exchange (REMDRun, src/REMD.c:29-126; rearrange, src/Server.c:145-192).
 * Every system of the handle is a replica.  After each replica reaches the exchange
 * point -- every_events executed events (every_events > 0), or else the first
 * executed event at time >= the next multiple of every_time (the reference's
 * trigger) -- its CalPotenE is computed and one rearrange() pass over replicas with
 * neighbouring ladder indices swaps (num, T) records with the Metropolis test
 * exp(-(1/T_i - 1/T_j)(E_j - E_i)) against the server's rand() stream.  Each replica's
 * thermostat target becomes its new T.  Runs until n_exchanges exchanges are done or
 * a replica reaches t_end (<= 0: its own t_end). */
typedef struct sdmd_remd {
    int32_t *num;                  /* REMDTempStr.num of each replica (ladder index), in/out */
    double  *T;                    /* REMDTempStr.T of each replica (reduced), in/out */
    double  *E;                    /* out (may be NULL): CalPotenE at the last exchange */
    int64_t  every_events;         /* > 0: exchange every this many executed events per replica */
    double   every_time;           /* else: the reference's time trigger (ExchangeRate) */
    sdmd_rng rng;                  /* the exchange server's rand() state, in/out */
    int64_t  attempted, accepted;  /* cumulative pair attempts / swaps, in/out */
    int64_t  exchanges_done;       /* out */
} sdmd_remd;
int  sdmd_gpu_run_remd(sdmd_gpu *h, int64_t n_exchanges, double t_end, sdmd_remd *remd);

/* The two halves of sdmd_gpu_run_remd, for a host that also dumps between
 * exchanges, as each replica process of the reference does (REMDRun,
 * src/REMD.c:29-126: after an executed event, the dump check, then the exchange
 * check).
 *
 * sdmd_gpu_run_to_stops runs each system k until it executes an event at a time
 * >= stop_time[k] (<= 0: no time stop), or has executed max_events[k] events
 * (0: system k does not run), or one of sdmd_gpu_run's limits.  at_stop (may be
 * NULL; n_systems entries) receives 1 for each system that stopped at such an
 * event (either kind) and 0 for the others.
 *
 * sdmd_gpu_exchange makes one exchange now, with every system at its exchange
 * point: CalPotenE of each, one rearrange() pass (src/Server.c:145-192) over the
 * replicas with T != 0 (a replica whose run has ended takes no part: the
 * reference's server skips a closed connection), and the new thermostat targets
 * of those replicas.  num, T, rng, attempted and accepted are read and updated
 * as by sdmd_gpu_run_remd; E (may be NULL) receives the energies. */
int  sdmd_gpu_run_to_stops(sdmd_gpu *h, const double *stop_time, const int64_t *max_events, double t_end,
                           int32_t *at_stop);
int  sdmd_gpu_exchange(sdmd_gpu *h, sdmd_remd *remd);

/* Kernels launched by the last sdmd_gpu_run (all of them, and event-loop kernels
 * alone) and the device time (ms) of the event-loop kernels alone, measured with
 * CUDA events around each of those launches. */
int  sdmd_gpu_last_run_stats(sdmd_gpu *h, int64_t *launches, int64_t *loop_launches, double *loop_ms);

/* How the handle launches its event loop: threads per system block, helper blocks
 * of the eager advance (0: none), whether whole systems are staged in shared
 * memory, and which loop kernel runs (SDMD_LOOP_*).  Any pointer may be NULL. */
enum { SDMD_LOOP_FP64 = 0, SDMD_LOOP_SCREEN = 1, SDMD_LOOP_SCREEN_R128 = 2, SDMD_LOOP_SCREEN_HELPERS = 3,
       SDMD_LOOP_SCREEN_HELPERS_512 = 4 };
int  sdmd_gpu_launch_info(sdmd_gpu *h, int32_t *threads, int32_t *helper_blocks, int32_t *staged,
                          int32_t *loop_kernel);

/* ---- allocation-free re-sweep ------------------------------------------------
 * No counterpart in the reference (its Prepare() allocates nothing on a GPU).
 *
 * Same contract and bit-identical results as sdmd_gpu_prepare, but the call
 * allocates nothing: no cudaMalloc/cudaFree, no host heap.  The scratch it needs
 * (the descriptor table its launches read, the thermostat sample buffers and an
 * error record) lives in one static device array of SDMD_NOALLOC_SCRATCH_BYTES
 * compiled into the library.  It is meant for callers that must not allocate
 * between create and destroy -- a replica-exchange or annealing driver that
 * re-sweeps after every temperature change while another framework's caching
 * allocator holds the rest of device memory, or a host loop that must not take
 * the allocator's locks or its implicit device synchronisation.
 *
 * Results equal sdmd_gpu_prepare's bit for bit on both prediction paths, but
 * the sweep runs sequentially over each system's atoms (one block per system):
 * on the FP32 screened path sdmd_gpu_prepare runs a parallel sweep instead, so
 * this call takes longer on large systems (about 0.7 s against 18 ms at 42k atoms).
 *
 * Limits and rules:
 *   - the batch must fit: 256-aligned n_systems descriptors plus, with
 *     full_predict and per system with a thermostat, about 28 bytes per atom.
 *     Larger batches return SDMD_ECAPACITY with a message on stderr and change
 *     nothing; use sdmd_gpu_prepare for them.
 *   - the first call on a device looks up the array's address
 *     (cudaGetSymbolAddress) with the handle's device current and keeps it for
 *     the life of the process; make that first call before any stream capture
 *     that could contain it, and make no call after a cudaDeviceReset.
 *   - the array is shared by every handle on a device and keeps its contents
 *     between calls.  Nothing in it must start at zero (each call writes what it
 *     reads), but calls that overlap in time race: serialise them per device.
 */
#define SDMD_NOALLOC_SCRATCH_BYTES (4u << 20)
int  sdmd_gpu_prepare_noalloc(sdmd_gpu *h, int32_t full_predict);

/* glibc-compatible rand() stream helpers (host side). */
void sdmd_rng_seed(sdmd_rng *r, uint32_t seed);
int32_t sdmd_rng_next(sdmd_rng *r);
void sdmd_rng_skip(sdmd_rng *r, int64_t n);

#ifdef __cplusplus
}
#endif
#endif /* SDMD_GPU_H */
