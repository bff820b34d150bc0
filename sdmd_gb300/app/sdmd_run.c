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
 * reference's (src/DMD.c:244-265).
 *
 * The random seed is time(NULL), as the reference's release build uses, or
 * 1575263273 (the reference's -DDEBUG_RANDOM seed) when SDMD_DEBUG_RANDOM is set.
 */
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include "sdmd_gpu.h"
#include "sdmd_host.h"

static const char *const kDefaultOut[SDMD_CLI_NOUT] = {"savedData.dat", "out_trj.gro", "out_pot.txt", "out_kin.txt",
                                                       "out_tem.txt",   "out_cnt.txt", "out_HBn.txt", "out_xyz.xyz",
                                                       "out_pdb.pdb",   "out_log.txt", "SysInfo.dat"};

static void out_path(char *buf, size_t len, const sdmd_cli *cli, int which) {
    const char *name = cli->out_name[which][0] ? cli->out_name[which] : kDefaultOut[which];
    snprintf(buf, len, "%s/%s", cli->savedir, name);
}

/* BackupFile / AssignName (src/DataSave.c:64-96): before an output's first write,
   an existing file of that name becomes <name>@<start time><last 4 characters> */
static void backup(const sdmd_cli *cli, int which, const char *timer) {
    const char *name = cli->out_name[which][0] ? cli->out_name[which] : kDefaultOut[which];
    char from[2400], to[2400], renamed[512];
    snprintf(from, sizeof from, "%s/%s", cli->savedir, name);
    FILE *f = fopen(from, "r");
    if (!f) return;
    fclose(f);
    const size_t len = strlen(name);
    if (len <= 4) return;
    snprintf(renamed, sizeof renamed, "%.*s@%s%s", (int)(len - 4), name, timer, name + len - 4);
    snprintf(to, sizeof to, "%s/%s", cli->savedir, renamed);
    rename(from, to);
}

static int engine_fail(sdmd_gpu *h, int rc, const char *where) {
    sdmd_error_info e;
    memset(&e, 0, sizeof e);
    if (h) sdmd_gpu_last_error(h, &e);
    fprintf(stderr, "!!ERROR!!: %s: %s (%d)", where, sdmd_gpu_strerror(rc), rc);
    if (e.code) fprintf(stderr, " at atom %d, event %lld", e.atom, (long long)e.event);
    fprintf(stderr, "\n");
    return 1;
}

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
        fprintf(stderr, "!!ERROR!!: replica exchange runs through sdmd_gpu_run_remd (one process for all replicas)\n");
        return 1;
    }
    char path[2300];
    sdmd_params p;
    snprintf(path, sizeof path, "%s/parameter.txt", cli.datadir);
    if (sdmd_read_parameters(path, &p) != SDMD_OK) {
        fprintf(stderr, "!!ERROR!!: cannot read %s\n", path);
        return 1;
    }
    const int is_new = strcmp(p.continue_mode, "new") == 0;
    if (!is_new && strcmp(p.continue_mode, "continue")) {
        fprintf(stderr, "!!ERROR!!: the simulation configuration is invalid! it only supports \"new\" or \"continue\"\n");
        return 1;
    }
    const uint32_t seed = getenv("SDMD_DEBUG_RANDOM") ? 1575263273u : (uint32_t)time(NULL);

    /* the system: built from the inputs; a continue run then takes the saved state */
    sdmd_params pb = p;
    snprintf(pb.continue_mode, sizeof pb.continue_mode, "new");
    sdmd_saved *saved = NULL;
    if (!is_new) {
        snprintf(path, sizeof path, "%s/%s", cli.savedir, cli.saved_in);   /* ReadBreakPoint reads the output folder's */
        if (sdmd_saved_read(path, &saved, err, sizeof err) != SDMD_OK) {
            fprintf(stderr, "!!ERROR!!: %s\n", err);
            return 1;
        }
        if (strcmp(p.temperature_str, "no") == 0) {   /* "no": the saved run's temperature */
            sdmd_saved_header hd;
            sdmd_saved_info(saved, &hd);
            pb.temperature = hd.temperature;
        }
    }
    sdmd_host_system *hs = NULL;
    int rc = sdmd_build_system(cli.datadir, cli.coordinate_file, &pb, cli.box_given ? cli.box : NULL, seed,
                               is_new ? 20000 : 0, &hs, err, sizeof err);
    if (rc != SDMD_OK) {
        fprintf(stderr, "!!ERROR!!: %s\n", err);
        return 1;
    }
    sdmd_system *sys = sdmd_host_view(hs);
    const char *names = sdmd_host_atom_names(hs), *resnames = sdmd_host_residue_names(hs);
    if (saved && sdmd_saved_apply(saved, sys, names, err, sizeof err) != SDMD_OK) {
        fprintf(stderr, "!!ERROR!!: %s\n", err);
        return 1;
    }
    /* the checkpoint this run writes: static records from the built system, the
       run's own Time, Dump_Rate and cut-off, and the seed the run was started with
       (a continue run keeps the one its checkpoint holds) */
    uint32_t file_seed = seed;
    if (saved) {
        sdmd_saved_header hd;
        sdmd_saved_info(saved, &hd);
        file_seed = hd.seed;
    }
    sdmd_saved *tpl = NULL;
    if (sdmd_saved_new(hs, &p, file_seed, &tpl, err, sizeof err) != SDMD_OK) {
        fprintf(stderr, "!!ERROR!!: %s\n", err);
        return 1;
    }
    sys->t_end = p.time;

    printf("\n----------------------------------------\n");
    printf("| Simulation configurations:           |\n");
    printf("| currenttime     %20.2f |\n", sys->time);
    printf("| timestep        %20.2f |\n", p.time);
    printf("| targetT         %20.2f |\n", sys->temperature);
    printf("| OutputRate      %20.2f |\n", p.dump_rate);
    printf("| CutOffRadius    %20.2f |\n", p.cutoff);
    printf("| Thermostat      %20s |\n", p.thermostat);
    printf("| WallExist       %20s |\n", p.wall_exist);
    printf("| boxsize         %6.1f %6.1f %6.1f |\n", sys->box[0], sys->box[1], sys->box[2]);
    printf("----------------------------------------\n\nSimulation starts...\n");
    fflush(stdout);

    sdmd_opts o;
    memset(&o, 0, sizeof o);
    o.advance = SDMD_ADVANCE_EAGER;
    o.screen = SDMD_SCREEN_FP32;
    o.threads_per_system = 128;
    sdmd_gpu *h = NULL;
    if ((rc = sdmd_gpu_create(sys, 1, &o, &h)) != SDMD_OK) return engine_fail(NULL, rc, "sdmd_gpu_create");
    if ((rc = sdmd_gpu_prepare(h, is_new ? 1 : 0)) != SDMD_OK) return engine_fail(h, rc, "sdmd_gpu_prepare");

    char timer[30];   /* DisplayTime (src/ToolFunctions.c:314-322) */
    {
        const time_t now = time(NULL);
        strftime(timer, sizeof timer, "%Y_%m_%d_%H_%M_%S", localtime(&now));
    }
    {   /* SaveLog in Prepare (src/SGThread.c:27-28) */
        char f[2400];
        backup(&cli, SDMD_OUT_LOG, timer);
        out_path(f, sizeof f, &cli, SDMD_OUT_LOG);
        if (sdmd_write_log(f, hs, &p, timer, sys->time, file_seed, cli.wall_dyn_size, cli.wall_dyn_rate) != SDMD_OK) {
            fprintf(stderr, "!!ERROR!!: %s\n", f);
            return 1;
        }
        if (is_new) {   /* SaveSysInfo (src/SGThread.c:36) */
            backup(&cli, SDMD_OUT_SYS, timer);
            out_path(f, sizeof f, &cli, SDMD_OUT_SYS);
            if (sdmd_write_sysinfo(f, hs) != SDMD_OK) { fprintf(stderr, "!!ERROR!!: %s\n", f); return 1; }
        }
    }
    const int64_t kNoLimit = (int64_t)1 << 40;
    double outputrecord = is_new ? 0 : sys->time + p.dump_rate;   /* src/DMD.c:31, src/SGThread.c:55 */
    int frames = 0;
    const clock_t st = clock();
    for (;;) {
        int32_t at = 0;
        if (outputrecord > 0) {
            rc = sdmd_gpu_run_to_dump(h, outputrecord, kNoLimit, p.time, &at);
        } else {   /* a new run dumps after its first executed event (any time >= 0) */
            const int64_t f0 = sys->counters.frame;
            rc = sdmd_gpu_run(h, 1, p.time);
            if (rc == SDMD_OK) rc = sdmd_gpu_download(h, sys, 1);
            at = rc == SDMD_OK && sys->counters.frame > f0;
        }
        if (rc != SDMD_OK) return engine_fail(h, rc, "sdmd_gpu_run");
        if ((rc = sdmd_gpu_download(h, sys, 1)) != SDMD_OK) return engine_fail(h, rc, "sdmd_gpu_download");
        if (at) {   /* SaveData for every marked file (src/SGThread.c:132-139) */
            const int app = frames > 0;
            char f[2400];
            if (!app) {
                static const int kMarked[] = {SDMD_OUT_TRJ, SDMD_OUT_POT, SDMD_OUT_KIN, SDMD_OUT_TEM, SDMD_OUT_CNT,
                                              SDMD_OUT_HBN, SDMD_OUT_XYZ, SDMD_OUT_SAVED};
                for (size_t q = 0; q < sizeof kMarked / sizeof kMarked[0]; q++)
                    if (kMarked[q] == SDMD_OUT_TRJ || kMarked[q] == SDMD_OUT_CNT || kMarked[q] == SDMD_OUT_SAVED ||
                        cli.out_on[kMarked[q]])
                        backup(&cli, kMarked[q], timer);
            }
            out_path(f, sizeof f, &cli, SDMD_OUT_TRJ);
            if (sdmd_write_gro(f, app, sys, names, resnames) != SDMD_OK) { fprintf(stderr, "!!ERROR!!: %s\n", f); return 1; }
            if (cli.out_on[SDMD_OUT_POT] || cli.out_on[SDMD_OUT_KIN] || cli.out_on[SDMD_OUT_TEM]) {
                double pot = 0, kin = 0;
                if ((rc = sdmd_gpu_energies(h, &pot, &kin)) != SDMD_OK) return engine_fail(h, rc, "sdmd_gpu_energies");
                if (cli.out_on[SDMD_OUT_POT]) { out_path(f, sizeof f, &cli, SDMD_OUT_POT); sdmd_write_series(f, app, sys->time, pot); }
                if (cli.out_on[SDMD_OUT_KIN]) { out_path(f, sizeof f, &cli, SDMD_OUT_KIN); sdmd_write_series(f, app, sys->time, kin); }
                if (cli.out_on[SDMD_OUT_TEM]) {   /* CalSysTem, src/ToolFunctions.c:755-757 */
                    out_path(f, sizeof f, &cli, SDMD_OUT_TEM);
                    sdmd_write_series(f, app, sys->time, 2 * kin / (3 * sys->n_atoms));
                }
            }
            out_path(f, sizeof f, &cli, SDMD_OUT_CNT);
            if (sdmd_write_cnt(f, app, sys) != SDMD_OK) { fprintf(stderr, "!!ERROR!!: %s\n", f); return 1; }
            if (cli.out_on[SDMD_OUT_HBN]) { out_path(f, sizeof f, &cli, SDMD_OUT_HBN); sdmd_write_hbn(f, app, sys); }
            if (cli.out_on[SDMD_OUT_XYZ]) { out_path(f, sizeof f, &cli, SDMD_OUT_XYZ); sdmd_write_xyz(f, app, sys, names, timer); }
            out_path(f, sizeof f, &cli, SDMD_OUT_SAVED);
            if (sdmd_saved_write(f, tpl, sys, err, sizeof err) != SDMD_OK) { fprintf(stderr, "!!ERROR!!: %s\n", err); return 1; }
            frames++;
            outputrecord += p.dump_rate;
        }
        if (!at || sys->time > p.time) break;
    }
    const double secs = (double)(clock() - st) / CLOCKS_PER_SEC;

    /* the reference's statistics block (src/DMD.c:244-265) */
    const sdmd_counters *c = &sys->counters;
    const long total = (long)(c->collision + c->bond + c->hb + c->hbneighbor + c->thermostat + c->pcc + c->wall);
    printf("\nFinished!\n\n\n");
    printf("ReCalculate times        = %li\n\n", (long)c->recal);
    printf("collision times          = %li\n", (long)c->collision);
    printf("bond times               = %li\n", (long)c->bond);
    printf("HB times                 = %li\n", (long)c->hb);
    printf("HB Neighbor times        = %li\n", (long)c->hbneighbor);
    printf("thermostat times         = %li\n", (long)c->thermostat);
    printf("PBC&CC times             = %li\n", (long)c->pcc);
    printf("Wall times               = %li\n", (long)c->wall);
    printf("CG times                 = %li\n", 0L);
    printf("percentage of thermostat = %.4f%%\n\n", total ? (float)c->thermostat / total * 100 : 0.0f);
    printf("total warning            = %li\n", (long)c->warnings);
    printf("\nHost time of the loop and dumps: %.2f s, %d dumps\n", secs, frames);
    sdmd_gpu_destroy(h);
    sdmd_host_free(hs);
    if (saved) sdmd_saved_free(saved);
    sdmd_saved_free(tpl);
    return 0;
}
