/*
 * sdmd_run.c -- the sDMD executable with its event loop on the GPU.
 *
 *   sdmd-gb300 -i <input dir> -o <output dir> [-f <coordinates>] [output flags]
 *
 * The reference's command line (InputData, src/Initialization.c:63-256), inputs
 * and outputs: parameter.txt, the coordinate file and Library_<ff>/ from the input
 * directory (a "continue" run also reads savedData.dat from the output directory,
 * as ReadBreakPoint does), the system built
 * as the reference's set-up builds it (src/SGThread.c:21-46), the event loop of
 * SingleThreadRun (src/SGThread.c:67-155) on the engine (FP32 screen, FP64 refine,
 * eager advance: the reference's events exactly), and at every dump -- after the
 * first executed event of each Dump_Rate interval, the first event of a new run
 * included -- the reference's outputs in its formats: out_trj.gro and
 * out_cnt.txt, out_pot/kin/tem.txt, out_HBn.txt and out_xyz.xyz when their flags
 * ask for them (-pdb switches the xyz file on, as the reference's parser does),
 * and savedData.dat (its static records from the inputs, or from the file a
 * continue run started from).  A file already in the output folder is first
 * renamed with the run's start time, as BackupFile does (src/DataSave.c:79-96).
 * out_log.txt (and for a new run SysInfo.dat) is written at the start, as
 * Prepare's SaveLog and SaveSysInfo do.  The end-of-run statistics block is the
 * reference's (src/DMD.c:244-265), and so is timeEvaluation.dat, the seconds per
 * 100 time units that a continue run's estimate is printed from
 * (src/DMD.c:220-231, 267-277).
 *
 * The random seed is time(NULL), as the reference's release build uses, or
 * 1575263273 (the reference's -DDEBUG_RANDOM seed) when SDMD_DEBUG_RANDOM is set.
 */
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include "app_common.h"

int main(int argc, const char *argv[]) {
    sdmd_cli cli;
    char err[1024];
    if (sdmd_parse_args(argc, (const char *const *)argv, &cli, err, sizeof err) != SDMD_OK) {
        fprintf(stderr, "!!ERROR!!: %s\n", err);
        return 1;
    }
    if (cli.help) {
        printf("usage: %s -i <input dir> -o <output dir> [-f coordinates] [-pot] [-kin] [-tem] [-HBn] [-pdb]\n",
               argv[0]);
        return 0;
    }
    if (cli.remd) {
        fprintf(stderr, "!!ERROR!!: replica exchange runs all replicas in one process: use sremd-gb300\n");
        return 1;
    }
    const clock_t st0 = clock();
    const uint32_t seed = getenv("SDMD_DEBUG_RANDOM") ? APP_DEBUG_SEED : (uint32_t)time(NULL);
    app_run run;
    if (app_setup(&run, &cli, seed)) return 1;
    sdmd_system *sys = run.sys;
    const double old_time = sys->time;
    const int64_t old_events = app_event_total(&sys->counters);
    app_print_config(&run);
    const double old_record = app_time_estimate(&run);
    printf("\nSimulation starts...\n");
    fflush(stdout);

    sdmd_opts o;
    memset(&o, 0, sizeof o);
    o.advance = SDMD_ADVANCE_EAGER;
    o.screen = SDMD_SCREEN_FP32;
    o.threads_per_system = 128;
    sdmd_gpu *h = NULL;
    int rc;
    if ((rc = sdmd_gpu_create(sys, 1, &o, &h)) != SDMD_OK) return app_engine_fail(NULL, rc, "sdmd_gpu_create");
    if ((rc = sdmd_gpu_prepare(h, run.is_new ? 1 : 0)) != SDMD_OK) return app_engine_fail(h, rc, "sdmd_gpu_prepare");

    char timer[30];
    app_timer(timer, sizeof timer);
    if (app_start_files(&run, timer)) return 1;
    const int64_t kNoLimit = (int64_t)1 << 40;
    const int energies = cli.out_on[SDMD_OUT_POT] || cli.out_on[SDMD_OUT_KIN] || cli.out_on[SDMD_OUT_TEM];
    const clock_t st = clock();
    for (;;) {
        int32_t at = 0;
        if (run.outputrecord > 0) {
            rc = sdmd_gpu_run_to_dump(h, run.outputrecord, kNoLimit, run.p.time, &at);
        } else {   /* a new run dumps after its first executed event (any time >= 0) */
            const int64_t f0 = sys->counters.frame;
            rc = sdmd_gpu_run(h, 1, run.p.time);
            if (rc == SDMD_OK) rc = sdmd_gpu_download(h, sys, 1);
            at = rc == SDMD_OK && sys->counters.frame > f0;
        }
        if (rc != SDMD_OK) return app_engine_fail(h, rc, "sdmd_gpu_run");
        if ((rc = sdmd_gpu_download(h, sys, 1)) != SDMD_OK) return app_engine_fail(h, rc, "sdmd_gpu_download");
        if (at) {   /* SaveData for every marked file (src/SGThread.c:132-139) */
            double pot = 0, kin = 0;
            if (energies && (rc = sdmd_gpu_energies(h, &pot, &kin)) != SDMD_OK)
                return app_engine_fail(h, rc, "sdmd_gpu_energies");
            if (app_dump(&run, sys, pot, kin, timer)) return 1;
        }
        if (!at || sys->time > run.p.time) break;
    }
    const double secs = (double)(clock() - st) / CLOCKS_PER_SEC;
    app_print_stats(&sys->counters);
    app_time_record(&run, old_record, old_time, (double)(clock() - st0) / CLOCKS_PER_SEC,
                    (long)(app_event_total(&sys->counters) - old_events));
    printf("\nHost time of the loop and dumps: %.2f s, %d dumps\n", secs, run.frames);
    sdmd_gpu_destroy(h);
    app_free(&run);
    return 0;
}
