/*
 * cli.c -- the reference sDMD's command line and REMD configuration, read with
 * the reference's semantics, for a drop-in front end of the engine.
 *
 *   sdmd_parse_args        the flags of InputData (src/Initialization.c:63-256)
 *   sdmd_read_remd_config  REMDConfig.txt as the sREMD launcher reads it
 *                          (src/REMDExec.c:79-110), with the temperatures each
 *                          replica then receives on its -REMD command line
 */
#define _GNU_SOURCE
#include <dirent.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "sdmd_host.h"

#define BOLTZMANN 0.0019872041   /* kcal/mol/K, src/REMDExec.c:19 */

static int err(char *buf, int len, const char *fmt, ...) {
    if (buf && len > 0) {
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(buf, (size_t)len, fmt, ap);
        va_end(ap);
    }
    return SDMD_EINVAL;
}

static int is_dir(const char *p) {
    DIR *d = opendir(p);
    if (!d) return 0;
    closedir(d);
    return 1;
}

/* "-flag [name]": the name when the next argument exists and is not a flag */
static void opt_name(int argc, const char *const *argv, int i, char *dst, size_t cap) {
    if (!(i + 1 >= argc || argv[i + 1][0] == '-')) snprintf(dst, cap, "%s", argv[i + 1]);
}

static const char *const OUT_FLAGS[SDMD_CLI_NOUT] = {"-so", "-trj", "-pot", "-kin", "-tem", "-cnt",
                                                     "-HBn", "-xyz", "-pdb", "-lgf", "-sys"};

int sdmd_parse_args(int argc, const char *const *argv, sdmd_cli *c, char *errbuf, int errlen) {
    if (!c) return SDMD_EINVAL;
    memset(c, 0, sizeof(*c));
    snprintf(c->coordinate_file, sizeof c->coordinate_file, "%s", "coordinate.gro");
    snprintf(c->saved_in, sizeof c->saved_in, "%s", "savedData.dat");
    c->remd_rate = 1000;   /* REMDInfo.REMD_OutputRate's initializer (src/DMD.c:130) */
    for (int i = 1; i < argc; i++) {
        const char *a = argv[i];
        if (a[0] != '-') continue;   /* the reference looks at flags only */
        if (!strcmp(a, "-i")) {
            if (i + 1 >= argc || !is_dir(argv[i + 1]))
                return err(errbuf, errlen, "-i: please provide a valid directory for the parameter folder");
            snprintf(c->datadir, sizeof c->datadir, "%s", argv[i + 1]);
        } else if (!strcmp(a, "-o")) {
            if (i + 1 >= argc || !is_dir(argv[i + 1]))
                return err(errbuf, errlen, "-o: please provide a valid directory for the output folder");
            snprintf(c->savedir, sizeof c->savedir, "%s", argv[i + 1]);
        } else if (!strcmp(a, "-f")) {
            opt_name(argc, argv, i, c->coordinate_file, sizeof c->coordinate_file);
        } else if (!strcmp(a, "-box")) {   /* atof of the next three arguments, as the reference */
            for (int d = 0; d < 3; d++) c->box[d] = i + 1 + d < argc ? atof(argv[i + 1 + d]) : 0.0;
            c->box_given = 1;
        } else if (!strcmp(a, "-si")) {
            opt_name(argc, argv, i, c->saved_in, sizeof c->saved_in);
        } else if (!strcmp(a, "-Wsz")) {
            if (!(i + 1 >= argc || argv[i + 1][0] == '-')) c->wall_dyn_size = atof(argv[i + 1]);
        } else if (!strcmp(a, "-Wrt")) {
            if (!(i + 1 >= argc || argv[i + 1][0] == '-')) c->wall_dyn_rate = atof(argv[i + 1]);
        } else if (!strcmp(a, "-pre")) {
            c->pre_bonds = 1;
        } else if (!strcmp(a, "-npC")) {
            c->charge_no_pbc = 1;
        } else if (!strcmp(a, "-REMD")) {
            const char *what[4] = {"server name", "port number", "temperature value", "temperature sequence"};
            for (int k = 0; k < 4; k++)
                if (i + 1 + k >= argc || argv[i + 1 + k][0] == '-')
                    return err(errbuf, errlen, "-REMD: please provide a valid %s for this replica", what[k]);
            c->remd = 1;
            snprintf(c->remd_server, sizeof c->remd_server, "%s", argv[i + 1]);
            c->remd_port = atoi(argv[i + 2]);
            c->remd_T = atof(argv[i + 3]);
            c->remd_num = atoi(argv[i + 4]);
            if (!(i + 5 >= argc || argv[i + 5][0] == '-')) c->remd_rate = atoi(argv[i + 5]);
            if (!(i + 6 >= argc || argv[i + 6][0] == '-')) {
                snprintf(c->remd_suffix, sizeof c->remd_suffix, "%s", argv[i + 6]);
                snprintf(c->saved_in, sizeof c->saved_in, "savedData%s.dat", c->remd_suffix);
            }
        } else if (!strcmp(a, "-visual")) {
            c->visual = 1;   /* the OpenGL viewer: not part of this engine */
        } else if (!strcmp(a, "-h") || !strcmp(a, "-help")) {
            c->help = 1;
            return SDMD_OK;
        } else {
            static const char *const charge[SDMD_CLI_NCHARGE] = {"-arg", "-asp", "-glu", "-his", "-lys",
                                                                 "-ter", "-AlC", "-AlP", "-COM"};
            for (int k = 0; k < SDMD_CLI_NCHARGE; k++)
                if (!strcmp(a, charge[k])) c->charge[k] = 1;
            for (int k = 0; k < SDMD_CLI_NOUT; k++) {
                if (strcmp(a, OUT_FLAGS[k])) continue;
                opt_name(argc, argv, i, c->out_name[k], sizeof c->out_name[k]);
                /* -pot, -kin, -tem, -HBn and -xyz switch their output on; -pdb marks
                   the xyz output, as the reference's does (src/Initialization.c:146-151) */
                if (k == SDMD_OUT_POT || k == SDMD_OUT_KIN || k == SDMD_OUT_TEM || k == SDMD_OUT_HBN ||
                    k == SDMD_OUT_XYZ || k == SDMD_OUT_PDB)
                    c->out_on[k == SDMD_OUT_PDB ? SDMD_OUT_XYZ : k] = 1;
            }
        }
    }
    return SDMD_OK;
}

/* fscanf("%s") over a string cursor */
static int word(const char **p, char *out, size_t cap) {
    const char *s = *p;
    while (*s == ' ' || *s == '\t' || *s == '\n' || *s == '\r' || *s == '\v' || *s == '\f') s++;
    if (!*s) return 0;
    size_t n = 0;
    while (*s && !(*s == ' ' || *s == '\t' || *s == '\n' || *s == '\r' || *s == '\v' || *s == '\f')) {
        if (n + 1 < cap) out[n++] = *s;
        s++;
    }
    out[n] = 0;
    *p = s;
    return 1;
}

int sdmd_read_remd_config(const char *path, sdmd_remd_config *cfg, char *errbuf, int errlen) {
    if (!path || !cfg) return SDMD_EINVAL;
    memset(cfg, 0, sizeof(*cfg));
    FILE *f = fopen(path, "r");
    if (!f) return err(errbuf, errlen, "cannot find the configuration file at %s", path);
    char line[8192], w[256];
    /* line 1: a comment; line 2: "ReplicaNum = n" */
    if (!fgets(line, sizeof line, f) || !fgets(line, sizeof line, f)) {
        fclose(f);
        return err(errbuf, errlen, "%s: too short", path);
    }
    const char *p = line;
    if (!word(&p, w, sizeof w) || !word(&p, w, sizeof w) || !word(&p, w, sizeof w)) {
        fclose(f);
        return err(errbuf, errlen, "%s: no ReplicaNum", path);
    }
    int n = atoi(w);
    if (n <= 0 || n > SDMD_REMD_MAX_REPLICAS) {
        fclose(f);
        return err(errbuf, errlen, "%s: ReplicaNum %d outside 1..%d", path, n, SDMD_REMD_MAX_REPLICAS);
    }
    /* line 3: "Temperatures = T1 ... Tn" (K), exactly n of them */
    if (!fgets(line, sizeof line, f)) {
        fclose(f);
        return err(errbuf, errlen, "%s: no Temperatures line", path);
    }
    p = line;
    word(&p, w, sizeof w);
    word(&p, w, sizeof w);
    for (int k = 0; k < n; k++) {
        char *end;
        double t = strtod(p, &end);
        if (end == p) {
            fclose(f);
            return err(errbuf, errlen, "the number of temperatures provided is less than the number of replicas");
        }
        p = end;
        cfg->T_kelvin[k] = t;
        /* the launcher passes T * BOLTZMANN to each replica as "%lf" text and the
           replica reads it back with atof (src/REMDExec.c:98,115-118;
           src/Initialization.c:206-212): the reduced temperature has 6 decimals */
        char txt[64];
        snprintf(txt, sizeof txt, "%lf", t * BOLTZMANN);
        cfg->T[k] = atof(txt);
        cfg->num[k] = k + 1;
    }
    {
        char *end;
        strtod(p, &end);
        if (end != p) {
            fclose(f);
            return err(errbuf, errlen, "the number of temperatures provided is larger than the number of replicas");
        }
    }
    /* "SocketPort = p" and "ExchangeRate = r" (the replica reads r with atoi) */
    char rest[4096];
    size_t got = fread(rest, 1, sizeof rest - 1, f);
    rest[got] = 0;
    fclose(f);
    p = rest;
    char port[64] = "", rate[64] = "";
    if (!(word(&p, w, sizeof w) && word(&p, w, sizeof w) && word(&p, port, sizeof port) && word(&p, w, sizeof w) &&
          word(&p, w, sizeof w) && word(&p, rate, sizeof rate)))
        return err(errbuf, errlen, "%s: SocketPort / ExchangeRate missing", path);
    cfg->n_replicas = n;
    cfg->port = atoi(port);
    cfg->exchange_time = (double)atoi(rate);
    return SDMD_OK;
}
