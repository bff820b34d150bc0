/*
 * sremd_run.c -- the reference's REMD launcher with every replica on the GPU.
 *
 *   sremd-gb300 -f <REMDConfig.txt> -args <name> <sDMD flags ...> [-end]
 *
 * The reference runs replica exchange as separate processes: sREMD
 * (src/REMDExec.c) reads REMDConfig.txt and starts one sDMD client per replica,
 * each with the flags after -args plus "-REMD localhost <port> <T> <num> <rate>
 * <id>", and the exchange server sServer (src/Server.c) that the clients reach
 * over TCP.  Here one process holds all the replicas in one engine batch and the
 * exchange is a kernel, with the same results:
 *
 *   - each replica's command line is the launcher's: the tokens after -args (the
 *     first is the program name, as execv takes it) and the -REMD flag with the
 *     replica's reduced temperature as "%lf" text, ladder index id + 1, the
 *     ExchangeRate and the extra name id; its files carry the id
 *     (out_trj<id>.gro, savedData<id>.dat, out_REMD<id>.txt, ...);
 *   - each replica follows REMDRun (src/REMD.c:29-126): after an executed event,
 *     the dump check (currenttime >= outputrecord: every marked file, as the sDMD
 *     executable writes them) and then the exchange check (currenttime >= rate);
 *   - an exchange waits for every replica whose run has not ended, as the server's
 *     collect() waits for every open connection; then CalPotenE of each, one
 *     rearrange() pass in the clients' connection order (the launcher starts
 *     client id one second after id - 1, so that is id order), the new
 *     thermostat targets, and SaveRE's out_REMD<id>.txt line;
 *   - a replica whose run has ended leaves the exchange (its connection closes).
 *
 * Seeds: each replica's is time(NULL) + id (the launcher starts them a second
 * apart), or the reference's -DDEBUG_RANDOM seed for all of them when
 * SDMD_DEBUG_RANDOM is set; the server's is time(NULL), as the launcher passes
 * it, or SDMD_SERVER_SEED when set.  Output names given by flags get the id as
 * the default names do.  -h prints the launcher's usage.
 */
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include "app_common.h"

#define MAX_ARGS 256

static int usage(const char *me) {
    printf("Usage: %s [distribute T or not] -f [configuration file] -args [args of executable without flag -REMD]\n\n",
           me);
    printf("            -f: provide the configuration file.\n");
    printf("         -args: provide the flags and info for sDMD without -REMD, end with \"-end\"\n");
    return 0;
}

int main(int argc, const char *argv[]) {
    const clock_t st0 = clock();
    const char *config = NULL;
    const char *args[MAX_ARGS];
    int nargs = 0;
    for (int n = 1; n < argc; n++) {   /* the launcher's parse (src/REMDExec.c:52-72) */
        if (argv[n][0] != '-') continue;
        if (!strcmp(argv[n], "-h") || !strcmp(argv[n], "-help")) return usage(argv[0]);
        if (!strcmp(argv[n], "-f") && n + 1 < argc) {
            config = argv[n + 1];
        } else if (!strcmp(argv[n], "-args")) {
            int next = 1;
            while (n + next < argc && strcmp(argv[n + next], "-end")) {
                if (nargs < MAX_ARGS - 16) args[nargs++] = argv[n + next];
                next++;
            }
            n += next;
        }
    }
    if (!config || nargs < 1) {
        usage(argv[0]);
        return 1;
    }
    char err[1024];
    sdmd_remd_config *cfg = calloc(1, sizeof *cfg);
    if (!cfg || sdmd_read_remd_config(config, cfg, err, sizeof err) != SDMD_OK) {
        fprintf(stderr, "!!ERROR!!: %s\n", cfg ? err : "out of memory");
        return 1;
    }
    const int n = cfg->n_replicas;
    const int debug = getenv("SDMD_DEBUG_RANDOM") != NULL;
    const uint32_t now = (uint32_t)time(NULL);
    app_run *run = calloc((size_t)n, sizeof *run);
    sdmd_system *sys = calloc((size_t)n, sizeof *sys);
    if (!run || !sys) return 1;
    char rate_txt[32];
    snprintf(rate_txt, sizeof rate_txt, "%d", (int)cfg->exchange_time);
    for (int k = 0; k < n; k++) {
        /* the client's command line (src/REMDExec.c:112-121) */
        char port[32], T[64], num[32], id[32];
        snprintf(port, sizeof port, "%d", cfg->port);
        snprintf(T, sizeof T, "%lf", cfg->T[k]);
        snprintf(num, sizeof num, "%d", cfg->num[k]);
        snprintf(id, sizeof id, "%d", k);
        const char *cv[MAX_ARGS];
        int cn = 0;
        for (int q = 0; q < nargs; q++) cv[cn++] = args[q];
        const char *tail[] = {"-REMD", "localhost", port, T, num, rate_txt, id};
        for (size_t q = 0; q < sizeof tail / sizeof tail[0]; q++) cv[cn++] = tail[q];
        sdmd_cli cli;
        if (sdmd_parse_args(cn, cv, &cli, err, sizeof err) != SDMD_OK) {
            fprintf(stderr, "!!ERROR!!: replica %d: %s\n", k, err);
            return 1;
        }
        if (app_setup(&run[k], &cli, debug ? APP_DEBUG_SEED : now + (uint32_t)k)) return 1;
        sys[k] = *run[k].sys;   /* the engine's batch: the replicas' arrays, their scalars here */
    }
    for (int k = 1; k < n; k++)
        if (run[k].is_new != run[0].is_new) {
            fprintf(stderr, "!!ERROR!!: the replicas' checkpoints disagree on new / continue\n");
            return 1;
        }
    app_print_config(&run[0]);
    const double old_time = sys[0].time, old_record = app_time_estimate(&run[0]);
    int64_t old_events = 0;
    for (int k = 0; k < n; k++) old_events += app_event_total(&sys[k].counters);
    printf("%d replicas, exchange every %s time units\n\nSimulation starts...\n", n, rate_txt);
    fflush(stdout);

    sdmd_opts o;
    memset(&o, 0, sizeof o);
    o.advance = SDMD_ADVANCE_EAGER;
    o.screen = SDMD_SCREEN_FP32;
    o.threads_per_system = 128;
    sdmd_gpu *h = NULL;
    int rc;
    if ((rc = sdmd_gpu_create(sys, n, &o, &h)) != SDMD_OK) return app_engine_fail(NULL, rc, "sdmd_gpu_create");
    if ((rc = sdmd_gpu_prepare(h, run[0].is_new ? 1 : 0)) != SDMD_OK) return app_engine_fail(h, rc, "sdmd_gpu_prepare");
    char timer[30];
    app_timer(timer, sizeof timer);
    for (int k = 0; k < n; k++)
        if (app_start_files(&run[k], timer)) return 1;

    /* the exchange server's state: its rand() stream and each client's record */
    sdmd_remd x;
    memset(&x, 0, sizeof x);
    const char *server_seed = getenv("SDMD_SERVER_SEED");
    sdmd_rng_seed(&x.rng, server_seed ? (uint32_t)strtoul(server_seed, NULL, 10) : now);
    int32_t *num = calloc((size_t)n, sizeof *num), *at = calloc((size_t)n, sizeof *at);
    double *Tx = calloc((size_t)n, sizeof *Tx), *stop = calloc((size_t)n, sizeof *stop);
    double *pot = calloc((size_t)n, sizeof *pot), *kin = calloc((size_t)n, sizeof *kin);
    int64_t *lim = calloc((size_t)n, sizeof *lim), *rate = calloc((size_t)n, sizeof *rate);
    char *waiting = calloc((size_t)n, 1), *done = calloc((size_t)n, 1);
    if (!num || !at || !Tx || !stop || !pot || !kin || !lim || !rate || !waiting || !done) return 1;
    const int ex = (int)cfg->exchange_time;
    if (ex <= 0) {
        fprintf(stderr, "!!ERROR!!: ExchangeRate must be positive\n");
        return 1;
    }
    for (int k = 0; k < n; k++) {   /* rate = ((int)(currenttime / outputRate) + 1) * outputRate */
        if (run[k].rep.output_rate <= 0) {   /* a continue run takes it from the replica's checkpoint */
            fprintf(stderr, "!!ERROR!!: replica %d: exchange period %d must be positive\n", k, run[k].rep.output_rate);
            return 1;
        }
        rate[k] = ((int64_t)(int)(sys[k].time / run[k].rep.output_rate) + 1) * run[k].rep.output_rate;
    }
    const int64_t kNoLimit = (int64_t)1 << 40;
    int energies = 0;
    for (int k = 0; k < n; k++)
        energies |= run[k].cli.out_on[SDMD_OUT_POT] | run[k].cli.out_on[SDMD_OUT_KIN] | run[k].cli.out_on[SDMD_OUT_TEM];
    int64_t exchanges = 0;
    const clock_t st = clock();
    for (;;) {
        int alive = 0, running = 0;
        for (int k = 0; k < n; k++) {
            lim[k] = 0;
            stop[k] = 0;
            if (done[k]) continue;
            alive++;
            if (waiting[k]) continue;
            running++;
            const double next = run[k].outputrecord < (double)rate[k] ? run[k].outputrecord : (double)rate[k];
            if (next > 0) {
                stop[k] = next;
                lim[k] = kNoLimit;
            } else {
                lim[k] = 1;   /* a new run dumps after its first executed event */
            }
        }
        if (!alive) break;
        if (running) {
            if ((rc = sdmd_gpu_run_to_stops(h, stop, lim, run[0].p.time, at)) != SDMD_OK)
                return app_engine_fail(h, rc, "sdmd_gpu_run_to_stops");
            if ((rc = sdmd_gpu_download(h, sys, n)) != SDMD_OK) return app_engine_fail(h, rc, "sdmd_gpu_download");
            int any_dump = 0;
            for (int k = 0; k < n; k++)
                if (lim[k] && at[k] && sys[k].time >= run[k].outputrecord) any_dump = 1;
            if (any_dump && energies && (rc = sdmd_gpu_energies(h, pot, kin)) != SDMD_OK)
                return app_engine_fail(h, rc, "sdmd_gpu_energies");
            for (int k = 0; k < n; k++) {
                if (!lim[k]) continue;
                if (!at[k]) {   /* the run ended before the next stop */
                    done[k] = 1;
                    continue;
                }
                if (sys[k].time >= run[k].outputrecord && app_dump(&run[k], &sys[k], pot[k], kin[k], timer)) return 1;
                if (sys[k].time >= (double)rate[k]) waiting[k] = 1;
                else if (sys[k].time > run[k].p.time) done[k] = 1;
            }
            continue;
        }
        /* every replica still running waits at its exchange point */
        for (int k = 0; k < n; k++) {
            num[k] = run[k].rep.num;
            Tx[k] = done[k] ? 0 : run[k].rep.T;
        }
        x.num = num;
        x.T = Tx;
        x.E = NULL;
        if ((rc = sdmd_gpu_exchange(h, &x)) != SDMD_OK) return app_engine_fail(h, rc, "sdmd_gpu_exchange");
        exchanges++;
        for (int k = 0; k < n; k++) {
            if (!waiting[k]) continue;
            run[k].rep.num = num[k];
            run[k].rep.T = Tx[k];
            sys[k].temperature = Tx[k];   /* targetTemperature = the new T */
            sdmd_saved_set_replica(run[k].tpl, &run[k].rep);
            if (app_save_re(&run[k], sys[k].time, timer)) return 1;
            rate[k] += run[k].rep.output_rate;
            waiting[k] = 0;
            if (sys[k].time > run[k].p.time) done[k] = 1;
        }
    }
    const double secs = (double)(clock() - st) / CLOCKS_PER_SEC;
    for (int k = 0; k < n; k++) {
        printf("\nReplica %d (T = %.4f, #%d):", k, run[k].rep.T, run[k].rep.num);
        app_print_stats(&sys[k].counters);
    }
    printf("\nExchanges: %lld, pair attempts %lld, swaps %lld\n", (long long)exchanges, (long long)x.attempted,
           (long long)x.accepted);
    int64_t events = -old_events;
    for (int k = 0; k < n; k++) events += app_event_total(&sys[k].counters);
    app_time_record(&run[0], old_record, old_time, (double)(clock() - st0) / CLOCKS_PER_SEC, (long)events);
    printf("Host time of the loop, dumps and exchanges: %.2f s\n", secs);
    sdmd_gpu_destroy(h);
    for (int k = 0; k < n; k++) app_free(&run[k]);
    free(run); free(sys); free(cfg); free(num); free(at); free(Tx); free(stop); free(pot); free(kin); free(lim);
    free(rate); free(waiting); free(done);
    return 0;
}
