/*
 * app_common.c -- one run of the reference's set-up and its output files, shared
 * by the sDMD executable and the REMD launcher.
 */
#include "app_common.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

static const char *const kDefaultOut[SDMD_CLI_NOUT] = {"savedData.dat", "out_trj.gro", "out_pot.txt", "out_kin.txt",
                                                       "out_tem.txt",   "out_cnt.txt", "out_HBn.txt", "out_xyz.xyz",
                                                       "out_pdb.pdb",   "out_log.txt", "SysInfo.dat"};

/* AssignName (src/DataSave.c:64-76): the extra name goes before the last four
   characters of a name longer than four */
static void with_extra(char *buf, size_t len, const char *name, const char *extra) {
    const size_t n = strlen(name);
    if (!extra[0] || n <= 4) snprintf(buf, len, "%s", name);
    else snprintf(buf, len, "%.*s%s%s", (int)(n - 4), name, extra, name + n - 4);
}

static void out_name(char *buf, size_t len, const app_run *r, int which) {
    with_extra(buf, len, r->cli.out_name[which][0] ? r->cli.out_name[which] : kDefaultOut[which], r->extra);
}

void app_out_path(char *buf, size_t len, const app_run *r, int which) {
    char name[400];
    out_name(name, sizeof name, r, which);
    snprintf(buf, len, "%s/%s", r->cli.savedir, name);
}

/* BackupFile (src/DataSave.c:79-96): before an output's first write, an existing
   file of that name becomes <name>@<start time><last 4 characters> */
static void backup_name(const app_run *r, const char *name, const char *timer) {
    char from[2400], to[2400], renamed[512];
    snprintf(from, sizeof from, "%s/%s", r->cli.savedir, name);
    FILE *f = fopen(from, "r");
    if (!f) return;
    fclose(f);
    const size_t len = strlen(name);
    if (len <= 4) return;
    snprintf(renamed, sizeof renamed, "%.*s@%s%s", (int)(len - 4), name, timer, name + len - 4);
    snprintf(to, sizeof to, "%s/%s", r->cli.savedir, renamed);
    rename(from, to);
}

static void backup(const app_run *r, int which, const char *timer) {
    char name[400];
    out_name(name, sizeof name, r, which);
    backup_name(r, name, timer);
}

int app_save_re(app_run *r, double time, const char *timer) {
    char name[400], f[2400];
    with_extra(name, sizeof name, "out_REMD.txt", r->extra);
    if (!r->re_open) backup_name(r, name, timer);
    snprintf(f, sizeof f, "%s/%s", r->cli.savedir, name);
    if (sdmd_write_remd(f, r->re_open, time, r->rep.T, r->rep.num) != SDMD_OK) {
        fprintf(stderr, "!!ERROR!!: cannot write %s\n", f);
        return 1;
    }
    r->re_open = 1;
    return 0;
}

void app_timer(char *buf, size_t len) {
    const time_t now = time(NULL);
    strftime(buf, len, "%Y_%m_%d_%H_%M_%S", localtime(&now));
}

int app_engine_fail(sdmd_gpu *h, int rc, const char *where) {
    sdmd_error_info e;
    memset(&e, 0, sizeof e);
    if (h) sdmd_gpu_last_error(h, &e);
    fprintf(stderr, "!!ERROR!!: %s: %s (%d)", where, sdmd_gpu_strerror(rc), rc);
    if (e.code) fprintf(stderr, " at atom %d, event %lld", e.atom, (long long)e.event);
    fprintf(stderr, "\n");
    return 1;
}

int app_setup(app_run *r, const sdmd_cli *cli, uint32_t seed) {
    char path[2400], err[1024];
    memset(r, 0, sizeof *r);
    r->cli = *cli;
    r->seed = seed;
    snprintf(path, sizeof path, "%s/parameter.txt", cli->datadir);
    if (sdmd_read_parameters(path, &r->p) != SDMD_OK) {
        fprintf(stderr, "!!ERROR!!: cannot read %s\n", path);
        return 1;
    }
    r->is_new = strcmp(r->p.continue_mode, "new") == 0;
    if (!r->is_new && strcmp(r->p.continue_mode, "continue")) {
        fprintf(stderr, "!!ERROR!!: the simulation configuration is invalid! it only supports \"new\" or \"continue\"\n");
        return 1;
    }
    /* the system: built from the inputs; a continue run then takes the saved state */
    sdmd_params pb = r->p;
    snprintf(pb.continue_mode, sizeof pb.continue_mode, "new");
    if (cli->remd) {   /* REMDInfo from the -REMD flag (src/Initialization.c:172-211) */
        r->remd = 1;
        r->rep.port = cli->remd_port;
        r->rep.output_rate = cli->remd_rate;
        r->rep.num = cli->remd_num;
        r->rep.T = cli->remd_T;
        snprintf(r->rep.server, sizeof r->rep.server, "%.49s", cli->remd_server);
        snprintf(r->rep.extra, sizeof r->rep.extra, "%.49s", cli->remd_suffix);
        /* T(reduced) "no" keeps the replica's temperature (src/Initialization.c:531-532) */
        if (strcmp(r->p.temperature_str, "no") == 0) pb.temperature = cli->remd_T;
    }
    if (!r->is_new) {
        /* ReadBreakPoint reads the output folder's checkpoint */
        snprintf(path, sizeof path, "%s/%s", cli->savedir, cli->saved_in);
        if (sdmd_saved_read(path, &r->saved, err, sizeof err) != SDMD_OK) {
            fprintf(stderr, "!!ERROR!!: %s\n", err);
            return 1;
        }
        sdmd_saved_header hd;
        sdmd_saved_info(r->saved, &hd);
        if (strcmp(r->p.temperature_str, "no") == 0) pb.temperature = hd.temperature;   /* the saved run's */
        sdmd_replica rep;
        if (sdmd_saved_replica(r->saved, &rep) == 1) {   /* REMDInfo is the file's (src/Initialization.c:475-476) */
            r->remd = 1;
            r->rep = rep;
            pb.temperature = rep.T;
        }
    }
    if (r->remd) snprintf(r->extra, sizeof r->extra, "%s", r->rep.extra);   /* Prepare's InitializeFiles */
    int rc = sdmd_build_system(cli->datadir, cli->coordinate_file, &pb, cli->box_given ? cli->box : NULL, seed,
                               r->is_new ? 20000 : 0, &r->hs, err, sizeof err);
    if (rc != SDMD_OK) {
        fprintf(stderr, "!!ERROR!!: %s\n", err);
        return 1;
    }
    r->sys = sdmd_host_view(r->hs);
    r->names = sdmd_host_atom_names(r->hs);
    r->resnames = sdmd_host_residue_names(r->hs);
    if (r->saved && sdmd_saved_apply(r->saved, r->sys, r->names, err, sizeof err) != SDMD_OK) {
        fprintf(stderr, "!!ERROR!!: %s\n", err);
        return 1;
    }
    /* the checkpoint this run writes: static records from the built system, the
       run's own Time, Dump_Rate and cut-off, and the seed the run was started with
       (a continue run keeps the one its checkpoint holds) */
    r->file_seed = seed;
    if (r->saved) {
        sdmd_saved_header hd;
        sdmd_saved_info(r->saved, &hd);
        r->file_seed = hd.seed;
    }
    if (sdmd_saved_new(r->hs, &r->p, r->file_seed, &r->tpl, err, sizeof err) != SDMD_OK) {
        fprintf(stderr, "!!ERROR!!: %s\n", err);
        return 1;
    }
    if (r->remd) sdmd_saved_set_replica(r->tpl, &r->rep);
    r->sys->t_end = r->p.time;
    r->outputrecord = r->is_new ? 0 : r->sys->time + r->p.dump_rate;   /* src/DMD.c:31, src/SGThread.c:55 */
    return 0;
}

void app_free(app_run *r) {
    if (r->hs) sdmd_host_free(r->hs);
    if (r->saved) sdmd_saved_free(r->saved);
    if (r->tpl) sdmd_saved_free(r->tpl);
    memset(r, 0, sizeof *r);
}

void app_print_config(const app_run *r) {
    printf("\n----------------------------------------\n");
    printf("| Simulation configurations:           |\n");
    printf("| currenttime     %20.2f |\n", r->sys->time);
    printf("| timestep        %20.2f |\n", r->p.time);
    printf("| targetT         %20.2f |\n", r->sys->temperature);
    printf("| OutputRate      %20.2f |\n", r->p.dump_rate);
    printf("| CutOffRadius    %20.2f |\n", r->p.cutoff);
    printf("| Thermostat      %20s |\n", r->p.thermostat);
    printf("| WallExist       %20s |\n", r->p.wall_exist);
    printf("| boxsize         %6.1f %6.1f %6.1f |\n", r->sys->box[0], r->sys->box[1], r->sys->box[2]);
    printf("----------------------------------------\n");
}

int app_start_files(app_run *r, const char *timer) {
    char f[2400];
    backup(r, SDMD_OUT_LOG, timer);
    app_out_path(f, sizeof f, r, SDMD_OUT_LOG);
    if (sdmd_write_log_replica(f, r->hs, &r->p, timer, r->sys->time, r->file_seed, r->cli.wall_dyn_size,
                               r->cli.wall_dyn_rate, r->remd ? &r->rep : NULL) != SDMD_OK) {
        fprintf(stderr, "!!ERROR!!: %s\n", f);
        return 1;
    }
    if (r->is_new) {   /* SaveSysInfo (src/SGThread.c:36) */
        backup(r, SDMD_OUT_SYS, timer);
        app_out_path(f, sizeof f, r, SDMD_OUT_SYS);
        if (sdmd_write_sysinfo(f, r->hs) != SDMD_OK) {
            fprintf(stderr, "!!ERROR!!: %s\n", f);
            return 1;
        }
        if (r->sys->n_obst) {   /* SaveObstInfo for obstruction walls (src/SGThread.c:38) */
            char name[400];
            with_extra(name, sizeof name, "ObstInfo.dat", r->extra);
            backup_name(r, name, timer);
            snprintf(f, sizeof f, "%s/%s", r->cli.savedir, name);
            if (sdmd_write_obstinfo(f, r->hs) != SDMD_OK) {
                fprintf(stderr, "!!ERROR!!: %s\n", f);
                return 1;
            }
        }
        if (r->sys->wall) {   /* SaveWallInfo for a smooth wall (src/SGThread.c:37) */
            char name[400];
            with_extra(name, sizeof name, "WallInfo.dat", r->extra);
            backup_name(r, name, timer);
            snprintf(f, sizeof f, "%s/%s", r->cli.savedir, name);
            if (sdmd_write_wallinfo(f, r->hs) != SDMD_OK) {
                fprintf(stderr, "!!ERROR!!: %s\n", f);
                return 1;
            }
        }
    }
    return 0;
}

int app_dump(app_run *r, const sdmd_system *sys, double pot, double kin, const char *timer) {
    const sdmd_cli *cli = &r->cli;
    const int app = r->frames > 0;
    char f[2400], err[1024];
    if (!app) {
        static const int kMarked[] = {SDMD_OUT_TRJ, SDMD_OUT_POT, SDMD_OUT_KIN, SDMD_OUT_TEM,
                                      SDMD_OUT_CNT, SDMD_OUT_HBN, SDMD_OUT_XYZ, SDMD_OUT_SAVED};
        for (size_t q = 0; q < sizeof kMarked / sizeof kMarked[0]; q++)
            if (kMarked[q] == SDMD_OUT_TRJ || kMarked[q] == SDMD_OUT_CNT || kMarked[q] == SDMD_OUT_SAVED ||
                cli->out_on[kMarked[q]])
                backup(r, kMarked[q], timer);
    }
    app_out_path(f, sizeof f, r, SDMD_OUT_TRJ);
    if (sdmd_write_gro(f, app, sys, r->names, r->resnames) != SDMD_OK) goto fail;
    if (cli->out_on[SDMD_OUT_POT]) {
        app_out_path(f, sizeof f, r, SDMD_OUT_POT);
        if (sdmd_write_series(f, app, sys->time, pot) != SDMD_OK) goto fail;
    }
    if (cli->out_on[SDMD_OUT_KIN]) {
        app_out_path(f, sizeof f, r, SDMD_OUT_KIN);
        if (sdmd_write_series(f, app, sys->time, kin) != SDMD_OK) goto fail;
    }
    if (cli->out_on[SDMD_OUT_TEM]) {   /* CalSysTem, src/ToolFunctions.c:755-757 */
        app_out_path(f, sizeof f, r, SDMD_OUT_TEM);
        if (sdmd_write_series(f, app, sys->time, 2 * kin / (3 * sys->n_atoms)) != SDMD_OK) goto fail;
    }
    app_out_path(f, sizeof f, r, SDMD_OUT_CNT);
    if (sdmd_write_cnt(f, app, sys) != SDMD_OK) goto fail;
    if (cli->out_on[SDMD_OUT_HBN]) {
        app_out_path(f, sizeof f, r, SDMD_OUT_HBN);
        if (sdmd_write_hbn(f, app, sys) != SDMD_OK) goto fail;
    }
    if (cli->out_on[SDMD_OUT_XYZ]) {
        app_out_path(f, sizeof f, r, SDMD_OUT_XYZ);
        if (sdmd_write_xyz(f, app, sys, r->names, timer) != SDMD_OK) goto fail;
    }
    app_out_path(f, sizeof f, r, SDMD_OUT_SAVED);
    if (sdmd_saved_write(f, r->tpl, sys, err, sizeof err) != SDMD_OK) {
        fprintf(stderr, "!!ERROR!!: %s\n", err);
        return 1;
    }
    r->frames++;
    r->outputrecord += r->p.dump_rate;
    return 0;
fail:
    fprintf(stderr, "!!ERROR!!: cannot write %s\n", f);
    return 1;
}

int64_t app_event_total(const sdmd_counters *c) {
    return c->collision + c->bond + c->hb + c->hbneighbor + c->thermostat + c->pcc + c->wall;
}

double app_time_estimate(const app_run *r) {
    char f[2400];
    snprintf(f, sizeof f, "%s/timeEvaluation.dat", r->cli.savedir);
    FILE *t = r->is_new ? NULL : fopen(f, "rb");
    if (!t) {
        printf("Time evaluation is unavailable this time!\n");
        return 0;
    }
    double old = 0;
    if (fread(&old, sizeof old, 1, t) != 1) old = 0;
    fclose(t);
    const double est = (r->p.time - r->sys->time) / 100 * old;
    const double hours = floor(est / 3600), mins = floor((est - hours * 3600) / 60);
    printf("This simulation may take %.0lf hours %.0lf mins %.0lf sec\n", hours, mins, est - hours * 3600 - mins * 60);
    return old;
}

void app_time_record(const app_run *r, double old_record, double old_time, double seconds, long events) {
    const double hours = floor(seconds / 3600), mins = floor((seconds - hours * 3600) / 60);
    double sec = seconds - hours * 3600 - mins * 60;
    printf("\nTotal time taken: %.0f hours %.0f mins %.0f sec\n", hours, mins, sec);
    printf("Calculate event times: %li\n", events);
    sec += hours * 3600 + mins * 60;
    const double record = (sec + old_record * old_time / 100) / r->p.time * 100;
    char f[2400];
    snprintf(f, sizeof f, "%s/timeEvaluation.dat", r->cli.savedir);
    FILE *t = fopen(f, "wb");
    if (!t) return;
    fwrite(&record, sizeof record, 1, t);
    fclose(t);
}

void app_print_stats(const sdmd_counters *c) {
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
}
