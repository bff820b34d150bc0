/*
 * sdmd_host.h -- host-side C library: builds an engine system (sdmd_system,
 * include/sdmd_gpu.h) from the reference sDMD's own inputs.
 *
 * It reads the same files with the same semantics as the reference's "new run"
 * path: parameter.txt by position (ReadParameter, src/Initialization.c:512-730),
 * a .gro/.pdb coordinate file filtered through the force-field library
 * (ModifyCoordinateFile/ReadGROFile/ReadPDBFile, src/Initialization.c:733-989),
 * the Library_<Force_Field> model files (ReadModel/ScanAA, :1076-1339;
 * CreatePotentialMatrix, :1468-1544; ReadHB/HBNeighborAssign, :1572-1847;
 * ReadWall, :1894-2053), Maxwell-Boltzmann velocities from the seeded rand()
 * stream (GenerateVelocity, :1850-1881), and Prepare()'s set-up up to the
 * full-rebuild sweep: SDEnergyMin, PBC and LinkList (src/SGThread.c:21-46).
 */
#ifndef SDMD_HOST_H
#define SDMD_HOST_H

#include "sdmd_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct sdmd_params {
    char   continue_mode[20];      /* "new" or "continue" */
    double time;                   /* Time: the loop runs while currenttime <= Time */
    char   temperature_str[20];    /* "no" keeps the previous temperature */
    double temperature;            /* reduced (kcal/mol) */
    double dump_rate;
    double cutoff;                 /* A */
    char   force_field[20];        /* "Ding" */
    char   thermostat[20];         /* "Andersen" or "no" */
    double thermo_freq;
    char   cg[16];                 /* "no" */
    char   wall_exist[20];         /* "no" or "smooth" */
    char   wall_type[20];          /* "no", "parallel", "cylinder", "sphere" */
    char   wall_dyn[16];           /* "no" */
    char   flow[32], obstruct[32], tunnel[32], sphobst[32];   /* "no", or the count of spherical obstacles */
    int32_t n_sphobst;                              /* SphObst?: x y z diameter per obstacle, stored */
    double  sphobst_xyzr[4 * SDMD_MAX_SPHOBST];     /* as x, y, z, radius (src/Initialization.c:703-724) */
    int32_t n_obst;                                 /* Obstruct?: an axis letter and a position per */
    double  obst_pos[3 * SDMD_MAX_OBST];            /* obstacle, stored as position[1..3], -1 elsewhere */
} sdmd_params;

typedef struct sdmd_host_system sdmd_host_system;   /* owns every array of an sdmd_system */

/* Parse parameter.txt (positional, 16 lines).  Returns SDMD_OK or SDMD_EINVAL. */
int sdmd_read_parameters(const char *path, sdmd_params *out);

/* Build a system from <datadir>/<coord_file> and <datadir>/Library_<ff>/.
 * box: used only for .pdb files (the reference's -box flag), else NULL.
 * seed: srand() seed; the reference uses time(NULL), or 1575263273 when built
 * with -DDEBUG_RANDOM.  energy_min_steps: SDEnergyMin's step limit (20000 in
 * Prepare()); 0 skips it.  errbuf (may be NULL) receives a message on failure. */
int sdmd_build_system(const char *datadir, const char *coord_file, const sdmd_params *p, const double *box,
                      uint32_t seed, int energy_min_steps, sdmd_host_system **out, char *errbuf, int errlen);

/* Same, from in-memory .gro text (no file I/O for the coordinates). */
int sdmd_build_system_gro_text(const char *datadir, const char *gro_text, const sdmd_params *p, uint32_t seed,
                               int energy_min_steps, sdmd_host_system **out, char *errbuf, int errlen);

/* Synthetic workloads: n_chains peptides (each a string of 3-letter residue
 * codes separated by spaces), relaxed against the model's distance bounds,
 * rotated uniformly at random and placed without overlap in the box (inside a
 * cylinder of radius box[1]/2 about the x axis, `margin` A from its surface,
 * when wall == SDMD_WALL_CYLINDER).  Writes malloc'd .gro text to *gro_out
 * (free with sdmd_free_text). */
int sdmd_generate_gro(const char *datadir, const char *ff, int n_chains, const char *const *sequences,
                      const double box[3], int wall, double margin, uint64_t seed, char **gro_out, char *errbuf,
                      int errlen);
void sdmd_free_text(char *p);

/* ---- the reference's command line (InputData, src/Initialization.c:63-256) ----
 * Flags are read exactly as the reference reads them; arguments that are not
 * flags are skipped.  -i / -o must name existing directories.  Returns SDMD_OK,
 * or SDMD_EINVAL with a message in errbuf.  `help` is set for -h / -help. */
enum { SDMD_OUT_SAVED = 0, SDMD_OUT_TRJ, SDMD_OUT_POT, SDMD_OUT_KIN, SDMD_OUT_TEM, SDMD_OUT_CNT, SDMD_OUT_HBN,
       SDMD_OUT_XYZ, SDMD_OUT_PDB, SDMD_OUT_LOG, SDMD_OUT_SYS, SDMD_CLI_NOUT };
#define SDMD_CLI_NCHARGE 9   /* -arg -asp -glu -his -lys -ter -AlC -AlP -COM */
typedef struct sdmd_cli {
    char    datadir[1024];             /* -i */
    char    savedir[1024];             /* -o */
    char    coordinate_file[256];      /* -f (default coordinate.gro) */
    char    saved_in[256];             /* -si (default savedData.dat; savedData<suffix>.dat with -REMD) */
    char    out_name[SDMD_CLI_NOUT][256];  /* -so -trj -pot -kin -tem -cnt -HBn -xyz -pdb -lgf -sys names */
    int32_t out_on[SDMD_CLI_NOUT];     /* optional outputs switched on (-pot -kin -tem -HBn -xyz / -pdb) */
    double  box[3];                    /* -box x y z */
    int32_t box_given;
    double  wall_dyn_size, wall_dyn_rate;   /* -Wsz, -Wrt */
    int32_t pre_bonds;                 /* -pre */
    int32_t charge[SDMD_CLI_NCHARGE];  /* charge-model selections */
    int32_t charge_no_pbc;             /* -npC */
    int32_t remd;                      /* -REMD server port T num [rate] [suffix] */
    char    remd_server[256];
    int32_t remd_port, remd_num, remd_rate;
    double  remd_T;
    char    remd_suffix[64];
    int32_t visual;                    /* -visual (the OpenGL viewer is not part of this engine) */
    int32_t help;
} sdmd_cli;
int sdmd_parse_args(int argc, const char *const *argv, sdmd_cli *out, char *errbuf, int errlen);

/* ---- REMDConfig.txt as the sREMD launcher reads it (src/REMDExec.c:79-110) ----
 * A comment line, "ReplicaNum = n", "Temperatures = T1 .. Tn" (K, exactly n),
 * "SocketPort = p", "ExchangeRate = r".  T[k] is the reduced temperature replica k
 * runs at: T_kelvin[k] * 0.0019872041 printed with "%lf" and read back, as the
 * launcher hands it over; num[k] = k + 1 is its ladder index and exchange_time
 * the replica's exchange period (atoi of r), the sdmd_remd fields
 * (include/sdmd_gpu.h) of an on-device replica exchange. */
#define SDMD_REMD_MAX_REPLICAS 1024
typedef struct sdmd_remd_config {
    int32_t n_replicas;
    int32_t port;                      /* SocketPort (no socket is used here) */
    double  exchange_time;
    double  T_kelvin[SDMD_REMD_MAX_REPLICAS];
    double  T[SDMD_REMD_MAX_REPLICAS];
    int32_t num[SDMD_REMD_MAX_REPLICAS];
} sdmd_remd_config;
int sdmd_read_remd_config(const char *path, sdmd_remd_config *out, char *errbuf, int errlen);

/* ---- the reference's checkpoint, savedData.dat (SaveDAT, src/DataSave.c:512-585;
 * ReadBreakPoint, src/Initialization.c:360-509) -------------------------------
 * sdmd_saved_read     reads a file into memory, every record kept;
 * sdmd_saved_apply    writes the state a continue run starts from into a system
 *                     built from the same inputs (sdmd_build_system): positions,
 *                     velocities, cells, types, HB state, stored events (the
 *                     engine's continue mode keeps them), cell list, clock and
 *                     event counters; rand() restarts from the saved seed and the
 *                     unsaved counters from zero, as ReadBreakPoint does.  names8
 *                     (may be NULL) are the system's atom names, checked against
 *                     the file's;
 * sdmd_saved_write    writes a system's state in the file's layout, with the
 *                     static records (atom properties, residue and peptide
 *                     tables, the connection map's bond bits, parameters, seed)
 *                     of a file read before -- the reference reads it back with
 *                     ReadBreakPoint. */
typedef struct sdmd_saved sdmd_saved;
typedef struct sdmd_saved_header {
    int32_t  atomnum, cellnum[3];
    int64_t  frame;
    double   timestep, currenttime, temperature, outputrate, box[3];
    uint32_t seed;
    int32_t  remd_flag;
    double   remd_T;
    char     method[20];
} sdmd_saved_header;
int  sdmd_saved_read(const char *path, sdmd_saved **out, char *errbuf, int errlen);
int  sdmd_saved_info(const sdmd_saved *s, sdmd_saved_header *out);
int  sdmd_saved_apply(const sdmd_saved *s, sdmd_system *sys, const char *names8, char *errbuf, int errlen);
int  sdmd_saved_write(const char *path, const sdmd_saved *tpl, const sdmd_system *sys, char *errbuf, int errlen);
/* The template of a new run: a system sdmd_build_system built from p and seed.  Its
   sdmd_saved_write output is the reference's savedData.dat of that run, byte for
   byte except the atom records' two pointer fields (the reference writes its own
   heap addresses there; ReadBreakPoint ignores them). */
int  sdmd_saved_new(const sdmd_host_system *h, const sdmd_params *p, uint32_t seed, sdmd_saved **out, char *errbuf,
                    int errlen);
void sdmd_saved_free(sdmd_saved *s);

/* A replica of the reference's REMD run: REMDInfo (src/DMD.h:383-390) as a
 * client's -REMD flag sets it (src/Initialization.c:170-211) -- the server's
 * port, the exchange period (ExchangeRate), the temperature record (reduced T
 * and ladder index num), the server's name and the extra name that replica's
 * file names carry (its id). */
typedef struct sdmd_replica {
    int32_t port, output_rate, num;
    double  T;
    char    server[50], extra[50];
} sdmd_replica;
/* Sets the REMDInfo record that sdmd_saved_write writes (flag 1 and r's
 * fields); r NULL restores the record of a run without -REMD. */
int  sdmd_saved_set_replica(sdmd_saved *s, const sdmd_replica *r);
/* The file's REMDInfo record: returns its flag (1: a REMD replica's checkpoint,
 * which a continue run takes its temperature record from, src/Initialization.c:475-476),
 * 0 without one, or SDMD_EINVAL. */
int  sdmd_saved_replica(const sdmd_saved *s, sdmd_replica *out);

sdmd_system *sdmd_host_view(sdmd_host_system *h);
void sdmd_host_free(sdmd_host_system *h);

/* Atom names (8 bytes each, entry i*8) and residue names, for output writers. */
const char *sdmd_host_atom_names(const sdmd_host_system *h);
const char *sdmd_host_residue_names(const sdmd_host_system *h);

/*
 * The reference's text outputs, written from an engine state (SaveData,
 * src/DataSave.c).  Each call writes one frame to `path`, appending when `append`
 * is non-zero (the reference appends one frame per dump), in the reference's
 * format byte for byte.  names8 / resnames8: 8-byte name records as above.
 *   sdmd_write_gro     out_trj.gro      SaveGRO           (src/DataSave.c:616-640)
 *   sdmd_write_pdb     out_pdb.pdb      SavePDB           (:588-613)
 *   sdmd_write_xyz     out_xyz.xyz      SaveXYZ           (:488-505); timer is the
 *                      run's start time as DisplayTime prints it (%Y_%m_%d_%H_%M_%S)
 *   sdmd_write_cnt     out_cnt.txt      SaveConnectionMap (:218-233): static bond /
 *                      constraint bits plus the formed hydrogen bonds' HB and
 *                      neighbour bits
 *   sdmd_write_hbn     out_HBn.txt      SaveHB            (:205-216)
 *   sdmd_write_series  out_pot.txt, out_kin.txt, out_tem.txt: one "time value" line
 *                      (SavePot / SaveKin / SaveTemp, :235-278); the value is the
 *                      caller's (sdmd_gpu_energies gives CalPotenE / CalKinetE)
 */
int sdmd_write_gro(const char *path, int append, const sdmd_system *s, const char *names8, const char *resnames8);
int sdmd_write_pdb(const char *path, int append, const sdmd_system *s, const char *names8, const char *resnames8);
int sdmd_write_xyz(const char *path, int append, const sdmd_system *s, const char *names8, const char *timer);
int sdmd_write_cnt(const char *path, int append, const sdmd_system *s);
int sdmd_write_hbn(const char *path, int append, const sdmd_system *s);
int sdmd_write_series(const char *path, int append, double time, double value);
/*   sdmd_write_log     out_log.txt      SaveLog (src/DataSave.c:333-462): the run's
 *                      configuration; timer as for sdmd_write_xyz, old_time the
 *                      run's start time, wall_dyn_size / rate the -Wsz / -Wrt values */
int sdmd_write_log(const char *path, const sdmd_host_system *h, const sdmd_params *p, const char *timer,
                   double old_time, uint32_t seed, double wall_dyn_size, double wall_dyn_rate);
/*   sdmd_write_log_replica  the same for a REMD replica: the REMD lines from r
 *                      (NULL: as sdmd_write_log) */
int sdmd_write_log_replica(const char *path, const sdmd_host_system *h, const sdmd_params *p, const char *timer,
                           double old_time, uint32_t seed, double wall_dyn_size, double wall_dyn_rate,
                           const sdmd_replica *r);
/*   sdmd_write_remd    out_REMD.txt     SaveRE (src/DataSave.c:687-700): after an
 *                      exchange, the replica's time, new temperature and ladder
 *                      index; nothing is written for a temperature <= 0 */
int sdmd_write_remd(const char *path, int append, double time, double T, int32_t num);
/*   sdmd_write_sysinfo SysInfo.dat      SaveSysInfo (src/DataSave.c:280-331): the
 *                      system's static records for the analysis tools, from the built
 *                      system; the reference's heap addresses in its pointer fields
 *                      are written as 1 where it has a link (readers test them for NULL) */
int sdmd_write_sysinfo(const char *path, const sdmd_host_system *h);
/*   sdmd_write_wallinfo WallInfo.dat    SaveWallInfo (src/DataSave.c:280-292): a
 *                      smooth wall's atom record (property and dynamic records) as
 *                      ReadWall builds it; SDMD_EINVAL for a system without a wall */
int sdmd_write_wallinfo(const char *path, const sdmd_host_system *h);
/*   sdmd_write_obstinfo ObstInfo.dat    SaveObstInfo (src/DataSave.c:294-308): each
 *                      obstruction wall's atom record; SDMD_EINVAL without one */
int sdmd_write_obstinfo(const char *path, const sdmd_host_system *h);

#ifdef __cplusplus
}
#endif
#endif
