/*
 * app_common.h -- what the sDMD executable (sdmd_run.c) and the REMD launcher
 * (sremd_run.c) share: one run of the reference's set-up for one system (a
 * single run, or one REMD replica), its output files and its dumps.
 */
#ifndef SDMD_APP_COMMON_H
#define SDMD_APP_COMMON_H

#include <stdint.h>
#include <stddef.h>

#include "sdmd_gpu.h"
#include "sdmd_host.h"

#define APP_DEBUG_SEED 1575263273u   /* the reference's -DDEBUG_RANDOM seed (src/DMD.h:36-38) */

typedef struct app_run {
    sdmd_cli cli;                    /* this run's command line */
    char extra[50];                  /* the extra name its files carry (a replica's id), "" otherwise */
    sdmd_params p;                   /* parameter.txt */
    int is_new;
    uint32_t seed, file_seed;        /* the run's seed; the one its checkpoint records */
    sdmd_host_system *hs;
    sdmd_system *sys;                /* the built system (the host view) */
    const char *names, *resnames;
    sdmd_saved *saved;               /* the checkpoint a continue run started from */
    sdmd_saved *tpl;                 /* the checkpoint's static records */
    int remd;                        /* a REMD replica: rep is its REMDInfo */
    sdmd_replica rep;
    int frames;                      /* dumps written */
    int re_open;                     /* out_REMD<id>.txt created */
    double outputrecord;             /* time of the next dump */
} app_run;

/* The reference's set-up for one run (InputData's parameter and checkpoint reads,
 * Prepare up to the first prediction): the system built from the inputs, a
 * continue run's saved state applied, the checkpoint template, and for a REMD
 * replica (cli->remd) its temperature record.  Prints the error and returns 1 on
 * failure. */
int app_setup(app_run *r, const sdmd_cli *cli, uint32_t seed);
void app_free(app_run *r);

/* "<dir>/<name>" of output `which`, the run's extra name inserted before the
   name's last four characters (AssignName, src/DataSave.c:64-76) */
void app_out_path(char *buf, size_t len, const app_run *r, int which);

/* DisplayTime's start time, %Y_%m_%d_%H_%M_%S (src/ToolFunctions.c:314-322) */
void app_timer(char *buf, size_t len);

/* The configuration block main() prints before the run (src/DMD.c:196-214). */
void app_print_config(const app_run *r);

/* Prepare's SaveLog and, for a new run, SaveSysInfo and a smooth wall's
   SaveWallInfo (src/SGThread.c:27-37). */
int app_start_files(app_run *r, const char *timer);

/* SaveData for every marked file at a dump (src/SGThread.c:132-139): sys is the
   run's downloaded state, pot / kin its CalPotenE / CalKinetE. */
int app_dump(app_run *r, const sdmd_system *sys, double pot, double kin, const char *timer);

/* SaveRE after an exchange (src/DataSave.c:687-700): out_REMD<extra>.txt, backed
   up and created at the replica's first exchange. */
int app_save_re(app_run *r, double time, const char *timer);

/* The end-of-run statistics block (src/DMD.c:244-265). */
void app_print_stats(const sdmd_counters *c);

/* timeEvaluation.dat (src/DMD.c:220-231, 267-277): a continue run prints the
   estimate from the seconds per 100 time units that the last run recorded and
   returns that record (0 when unavailable); at the end, the run's time and event
   count are printed and the record updated. */
double app_time_estimate(const app_run *r);
void app_time_record(const app_run *r, double old_record, double old_time, double seconds, long events);
int64_t app_event_total(const sdmd_counters *c);

int app_engine_fail(sdmd_gpu *h, int rc, const char *where);

#endif
