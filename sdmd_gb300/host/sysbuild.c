/*
 * sysbuild.c -- builds an engine system (sdmd_system) from the reference's
 * inputs with the reference's semantics (see include/sdmd_host.h).
 *
 * Model-building state follows the reference's globals, but stored sparsely:
 * the dense (N+1)^2 connectionMap (src/Initialization.c:976) becomes a short
 * per-atom row of (j, bits); the linked bond/constraint lists keep the
 * reference's head-insertion order, which decides the scan order of BondTime.
 */
#include "sdmd_host.h"
#include "host_static.h"

#include <ctype.h>
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <pthread.h>

#define NT SDMD_NTYPES
#define BOND_C 1
#define CONSTR_C 2

/* ---------------------------------------------------------------------------- */
typedef struct { int j; double dmin, dmax; } bond_t;
typedef struct { int j; double dmin, dmax; int soff, sn; } cons_t;
typedef struct { int j, bits; } conn_t;

typedef struct {
    char name[8], aa[8], ext0[16], ext1[16];
    int type, aatype, protein, aanum;
    double mass, pos[3], vel[3];
    int hb_neighbor, hb_role;
    bond_t *bond; int nbond, capbond;     /* bond[0] is the list head */
    cons_t *con; int ncon, capcon;
    conn_t *conn; int nconn, capconn;
} hatom;

typedef struct { char name[8]; int type, start, end, protein; } haa;
typedef struct { int start_aa, end_aa, start_atom, end_atom; } hprot;

typedef struct { double *d, *e, *acc; int n, cap; } steppool;
typedef struct { double dmin, dmax; int soff, sn; } pairent;

struct sdmd_host_system {
    sdmd_system sys;
    /* owned arrays */
    double *mass, *x, *y, *z, *vx, *vy, *vz, *ev_time, *ev_potential;
    int32_t *protein, *aanum, *aatype, *hb_neighbor, *hb_role, *name_code;
    int32_t *bond_off, *bond_j, *con_off, *con_j, *con_step_off, *con_step_n, *conn_off, *conn_j, *conn_bits;
    double *bond_dmin, *bond_dmax, *con_dmin, *con_dmax, *con_step_d, *con_step_e, *con_step_acc;
    double *pair_dmin, *pair_dmax, *pair_step_d, *pair_step_e, *pair_step_acc;
    int32_t *pair_step_off, *pair_step_n;
    int32_t *cx, *cy, *cz, *type, *hb_bond, *hb_itype, *nb_partner, *nb_status, *nb_pnum, *ev_partner, *ev_type, *ev_sub,
        *cell_list;
    int64_t *ev_counter, *ev_pcounter;
    char *names, *resnames;
    /* the checkpoint's static records (host_static.h) */
    char *ext;
    int32_t n_aa, n_prot;
    char *aa_name;
    int32_t *aa_type, *aa_start, *aa_end, *aa_prot, *pep_start, *pep_end, *pep_aa_start, *pep_aa_end;
    double *aa_mass, *pep_mass, *charge;
    char method[20];
    double hbpot[6];
    char wall_name[8], wall_ext[32];   /* the Wall.txt record of a smooth wall */
    double wall_lib_mass;
    double sphobst[4 * SDMD_MAX_SPHOBST];
    double obst[3 * SDMD_MAX_OBST];
};

typedef struct {
    char datadir[1024], ff[20];
    const sdmd_params *p;
    hatom *atom; int n;
    haa *aa; int naa;
    hprot *prot; int nprot;
    double box[4];
    int cellnum[4];
    double cellsize[4];
    steppool conpool, pairpool;
    pairent coll[NT][NT], hb[12][NT][NT];
    double hbpot[6];   /* BB_r BB_v SS_r SS_v BS_r BS_v */
    sdmd_rng rng;
    int64_t warnings;
    int wall; int wall_type; double wall_pos[3], wall_mass;
    char wall_name[8], wall_ext[32];
    char *err; int errlen;
} B;

static int fail(B *b, const char *fmt, ...) {
    if (b->err && b->errlen > 0) {
        va_list ap; va_start(ap, fmt); vsnprintf(b->err, (size_t)b->errlen, fmt, ap); va_end(ap);
    }
    return SDMD_EINVAL;
}

/* ---- glibc rand() stream (the reference seeds it with srand(seed)) ---------- */
/* additive feedback generator r[i] = r[i-3] + r[i-31] (mod 2^32), output r >> 1,
 * seeded by the Lehmer sequence 16807^k * seed (mod 2^31 - 1), first 310 dropped */
static int32_t rng_next(sdmd_rng *r) {
    uint32_t v = (uint32_t)r->tab[r->front] + (uint32_t)r->tab[r->rear];
    r->tab[r->front] = (int32_t)v;
    int32_t out = (int32_t)((v >> 1) & 0x7fffffff);
    if (++r->front >= 31) { r->front = 0; ++r->rear; }
    else if (++r->rear >= 31) r->rear = 0;
    return out;
}
static void rng_seed(sdmd_rng *r, uint32_t seed) {
    int32_t *t = r->tab;
    t[0] = seed ? (int32_t)seed : 1;
    for (int i = 1; i < 31; i++) {
        long hi = t[i - 1] / 127773, lo = t[i - 1] % 127773;
        long w = 16807 * lo - 2836 * hi;
        if (w < 0) w += 2147483647;
        t[i] = (int32_t)w;
    }
    r->front = 3; r->rear = 0;
    for (int k = 0; k < 310; k++) rng_next(r);
}
/* the seeded stream for the other host-side files (savedata.c) */
__attribute__((visibility("hidden"))) void sdmd_host_seed_rng(sdmd_rng *r, uint32_t seed) { rng_seed(r, seed); }
static int32_t rnd(B *b) { return rng_next(&b->rng); }
static double random01(B *b) { return 0 + (double)rnd(b) / ((double)2147483647 / (1 - 0)); }
/* Maxwell_Boltzmann_Distribution (src/ToolFunctions.c:544-569) with libm log,
 * as the reference's host code calls it */
static double mb(B *b, double mean, double variance) {
    double r0, r1, s, out;
    for (;;) {
        do {
            r0 = 2 * random01(b) - 1;
            r1 = 2 * random01(b) - 1;
            s = r0 * r0 + r1 * r1;
        } while (s >= 1);
        s = sqrt(-2 * log(s) / s);
        double choose = random01(b);
        out = (choose >= 0.5) ? r0 * s : r1 * s;
        if (out != 0) break;
    }
    return out * sqrt(variance) + mean;
}

/* ---- name tables (src/Models.c) -------------------------------------------- */
static int aa_model(const char *c) {     /* AAModel, src/Models.c:65-127 */
    static const char *n[] = {"ALA", "ARG", "ASN", "ASP", "CYS", "GLN", "GLU", "GLY", "HIS", "ILE", "LEU", "LYS",
                              "MET", "PHE", "PRO", "SER", "THR", "TRP", "TYR", "VAL", "SOL", "GEL", "PHO", "PHI",
                              "RPH"};
    for (int i = 0; i < 25; i++) if (!strcmp(c, n[i])) return i + 1;
    return -1;
}
static int atom_model(const char *t) {   /* AtomModel, src/Models.c:129-206 */
    static const struct { const char *n; int v; } m[] = {
        {"OZB", 26}, {"NZB", 18}, {"CRB", 6}, {"CA", 9}, {"CA1", 10}, {"CA2", 11}, {"CA3", 12}, {"CA1P", 14},
        {"CA2P", 15}, {"CM1", 13}, {"CM1P", 16}, {"CR", 5}, {"CRN", 7}, {"CRNP", 8}, {"NCK", 21}, {"NCR", 22},
        {"NR", 23}, {"NZNP", 19}, {"NZNQ", 20}, {"NZ", 17}, {"OC", 28}, {"OW", 29}, {"OZH", 25}, {"OZ", 24},
        {"SGNP", 30}, {"SG", 31}, {"OZB_HB", 27}, {"HB", 2}, {"HO", 1}, {"HN", 1}, {"HS", 1}, {"HW", 1},
        {"H", 1}, {"H_HB", 3}, {"HB_HB", 4}, {"GEL", 32}};
    for (size_t i = 0; i < sizeof(m) / sizeof(m[0]); i++) if (!strcmp(t, m[i].n)) return m[i].v;
    return -1;
}

/* ---- small text cursor over a whole file, fscanf-like --------------------- */
typedef struct { char *buf; size_t n, at; } cur;

static int slurp(const char *path, cur *c) {
    FILE *f = fopen(path, "rb");
    if (!f) return -1;
    fseek(f, 0, SEEK_END);
    long n = ftell(f);
    fseek(f, 0, SEEK_SET);
    c->buf = malloc((size_t)n + 1);
    c->n = fread(c->buf, 1, (size_t)n, f);
    c->buf[c->n] = 0;
    c->at = 0;
    fclose(f);
    return 0;
}
static void cur_text(const char *text, cur *c) {
    c->n = strlen(text);
    c->buf = malloc(c->n + 1);
    memcpy(c->buf, text, c->n + 1);
    c->at = 0;
}
static int tok(cur *c, char *out, size_t cap) {     /* fscanf("%s") */
    while (c->at < c->n && isspace((unsigned char)c->buf[c->at])) c->at++;
    if (c->at >= c->n) return 0;
    size_t k = 0;
    while (c->at < c->n && !isspace((unsigned char)c->buf[c->at])) {
        if (k + 1 < cap) out[k++] = c->buf[c->at];
        c->at++;
    }
    out[k] = 0;
    return 1;
}
static int dbl(cur *c, double *v) {                  /* fscanf("%lf") */
    while (c->at < c->n && isspace((unsigned char)c->buf[c->at])) c->at++;
    char *end;
    double x = strtod(c->buf + c->at, &end);
    if (end == c->buf + c->at) return 0;
    c->at = (size_t)(end - c->buf);
    *v = x;
    return 1;
}
static void skipline(cur *c) {                       /* fgets */
    while (c->at < c->n && c->buf[c->at] != '\n') c->at++;
    if (c->at < c->n) c->at++;
}
static void getline_(cur *c, char *out, size_t cap) {
    size_t k = 0;
    while (c->at < c->n && c->buf[c->at] != '\n') {
        if (k + 1 < cap) out[k++] = c->buf[c->at];
        c->at++;
    }
    if (c->at < c->n) c->at++;
    out[k] = 0;
}

/* ---- parameter.txt: ReadParameter (src/Initialization.c:512-730) ----------- */
int sdmd_read_parameters(const char *path, sdmd_params *p) {
    cur c;
    if (slurp(path, &c)) return SDMD_EINVAL;
    memset(p, 0, sizeof(*p));
    char s[1024], line[4096];
    int ok = 1;
    ok &= tok(&c, s, sizeof s) && tok(&c, p->continue_mode, sizeof p->continue_mode);
    ok &= tok(&c, s, sizeof s) && dbl(&c, &p->time);
    ok &= tok(&c, s, sizeof s) && tok(&c, p->temperature_str, sizeof p->temperature_str);
    if (strcmp(p->temperature_str, "no")) p->temperature = atof(p->temperature_str);
    ok &= tok(&c, s, sizeof s) && dbl(&c, &p->dump_rate);
    ok &= tok(&c, s, sizeof s) && dbl(&c, &p->cutoff);
    ok &= tok(&c, s, sizeof s) && tok(&c, p->force_field, sizeof p->force_field);
    ok &= tok(&c, s, sizeof s) && tok(&c, p->thermostat, sizeof p->thermostat);
    ok &= tok(&c, s, sizeof s) && dbl(&c, &p->thermo_freq);
    skipline(&c);
    /* CGModel line, then three "%s%s" lines, then four free-form lines */
    getline_(&c, line, sizeof line);
    if (sscanf(line, "%1023s %15s", s, p->cg) < 2) ok = 0;
    ok &= tok(&c, s, sizeof s) && tok(&c, p->wall_exist, sizeof p->wall_exist);
    ok &= tok(&c, s, sizeof s) && tok(&c, p->wall_type, sizeof p->wall_type);
    ok &= tok(&c, s, sizeof s) && tok(&c, p->wall_dyn, sizeof p->wall_dyn);
    skipline(&c);
    char *dst[4] = {p->flow, p->obstruct, p->tunnel, p->sphobst};
    for (int k = 0; k < 4; k++) {
        getline_(&c, line, sizeof line);
        char v[32] = "";
        int pos = 0;
        if (sscanf(line, "%1023s %31s%n", s, v, &pos) < 2) ok = 0;
        snprintf(dst[k], 32, "%s", v);
        if (k == 1 && ok && strcmp(v, "no")) {
            /* the count, then an axis letter and a position per obstacle with a
               separator token between them (src/Initialization.c:634-672) */
            const int n = atoi(v);
            if (n < 0 || n > SDMD_MAX_OBST) { ok = 0; break; }
            const char *q = line + pos;
            for (int i = 0; i < 3 * n; i++) p->obst_pos[i] = -1;
            for (int i = 0; i < n && ok; i++) {
                char axis[64];
                int used = 0, dim;
                if (sscanf(q, "%63s%n", axis, &used) < 1) { ok = 0; break; }
                q += used;
                dim = axis[0] == 'x' ? 0 : axis[0] == 'y' ? 1 : axis[0] == 'z' ? 2 : -1;
                if (dim < 0 || sscanf(q, "%lf%n", &p->obst_pos[3 * i + dim], &used) < 1) { ok = 0; break; }
                q += used;
                if (i != n - 1) {
                    if (sscanf(q, "%63s%n", axis, &used) < 1) { ok = 0; break; }
                    q += used;
                }
            }
            p->n_obst = n;
        }
        if (k == 3 && ok && strcmp(v, "no")) {
            /* the count, then "x y z diameter" per obstacle with a separator token
               between them; the radius is kept (src/Initialization.c:703-724) */
            const int n = atoi(v);
            if (n < 0 || n > SDMD_MAX_SPHOBST) { ok = 0; break; }
            const char *q = line + pos;
            for (int i = 0; i < n && ok; i++) {
                double *o = &p->sphobst_xyzr[4 * i];
                int used = 0;
                if (sscanf(q, "%lf%lf%lf%lf%n", &o[0], &o[1], &o[2], &o[3], &used) < 4) { ok = 0; break; }
                o[3] /= 2;
                q += used;
                if (i != n - 1) {
                    char sep[64];
                    if (sscanf(q, "%63s%n", sep, &used) < 1) { ok = 0; break; }
                    q += used;
                }
            }
            p->n_sphobst = n;
        }
    }
    free(c.buf);
    return ok ? SDMD_OK : SDMD_EINVAL;
}

/* ---- growable per-atom lists (head insertion = reference list order) ------- */
static void bond_prepend(hatom *a, bond_t v) {
    if (a->nbond == a->capbond) { a->capbond = a->capbond ? 2 * a->capbond : 8; a->bond = realloc(a->bond, sizeof(bond_t) * a->capbond); }
    memmove(a->bond + 1, a->bond, sizeof(bond_t) * a->nbond);
    a->bond[0] = v; a->nbond++;
}
static void con_prepend(hatom *a, cons_t v) {
    if (a->ncon == a->capcon) { a->capcon = a->capcon ? 2 * a->capcon : 8; a->con = realloc(a->con, sizeof(cons_t) * a->capcon); }
    memmove(a->con + 1, a->con, sizeof(cons_t) * a->ncon);
    a->con[0] = v; a->ncon++;
}
static int *conn_at(hatom *a, int j) {
    for (int k = 0; k < a->nconn; k++) if (a->conn[k].j == j) return &a->conn[k].bits;
    if (a->nconn == a->capconn) { a->capconn = a->capconn ? 2 * a->capconn : 8; a->conn = realloc(a->conn, sizeof(conn_t) * a->capconn); }
    a->conn[a->nconn].j = j; a->conn[a->nconn].bits = 0;
    return &a->conn[a->nconn++].bits;
}
static int conn_get(const hatom *a, int j) {
    for (int k = 0; k < a->nconn; k++) if (a->conn[k].j == j) return a->conn[k].bits;
    return 0;
}
static int pool_add(steppool *p, double d, double e) {
    if (p->n == p->cap) {
        p->cap = p->cap ? 2 * p->cap : 256;
        p->d = realloc(p->d, sizeof(double) * p->cap); p->e = realloc(p->e, sizeof(double) * p->cap);
        p->acc = realloc(p->acc, sizeof(double) * p->cap);
    }
    p->d[p->n] = d; p->e[p->n] = e; p->acc[p->n] = 0;
    return p->n++;
}
/* CalAccumulatedPoten (src/ToolFunctions.c:897-919) */
static void accumulate(steppool *p, int off, int n) {
    double acc = 0;
    for (int k = 0; k < n; k++) acc += p->e[off + k];
    for (int k = 0; k < n; k++) { p->acc[off + k] = acc; acc -= p->e[off + k]; }
}

static const char *aa_name(B *b, int k) { return (k >= 1 && k <= b->naa) ? b->aa[k].name : ""; }

/* ---- .gro reading: ModifyCoordinateFile + ReadGROFile + ReadCoordinate -------- */
/* CheckValidAtom (src/Initialization.c:1311-1327), including its "O1" rule */
static int check_valid(char *name, char list[][8], int n) {
    for (int i = 0; i < n; i++) {
        if (!strcmp(name, list[i])) { strcpy(list[i], "0"); return 1; }
        if (!strcmp(name, "O1")) { strcpy(list[i], "0"); strcpy(name, "O"); return 1; }
    }
    return 0;
}
static void remove_space(char *s) {   /* RemoveSpace (src/Initialization.c:1330-1342) */
    int n = 0; char *q = s;
    while (*q == ' ') q++;
    while (*q != ' ' && *q) s[n++] = *q++;
    s[n] = 0;
}
static int read_atom_list(B *b, const char *res, char list[][8]) {
    char path[2048], t[256];
    snprintf(path, sizeof path, "%s/Library_%s/AA/%s.txt", b->datadir, b->ff, strcmp(res, "GLY") ? res : "ALA");
    cur c;
    if (slurp(path, &c)) return -1;
    skipline(&c);
    int n = 0;
    while (tok(&c, t, sizeof t) && !strcmp(t, "ATOM") && n < 20) {
        tok(&c, list[n], 8);
        n++;
        skipline(&c);
    }
    free(c.buf);
    return n;
}

static int read_gro(B *b, cur *c) {
    char line[4096], res[8], nm[8], prevres[256] = "";
    int natoms = 0, tmpint = 0, listn = 0;
    char list[20][8];
    memset(list, 0, sizeof list);
    skipline(c);
    { double v; if (!dbl(c, &v)) return fail(b, "bad .gro atom count"); natoms = (int)v; }
    skipline(c);
    int cap = natoms + 2;
    b->atom = calloc((size_t)cap + 1, sizeof(hatom));
    b->aa = calloc((size_t)natoms + 2, sizeof(haa));
    b->prot = calloc((size_t)natoms + 2, sizeof(hprot));
    int n = 0;
    double (*xyz)[3] = calloc((size_t)natoms + 2, sizeof(double[3]));
    char (*names)[8] = calloc((size_t)natoms + 2, 8);
    for (int i = 1; i <= natoms; i++) {
        getline_(c, line, sizeof line);
        /* "%i%5c%5c%s": residue number, 5-char residue name, 5-char atom name, atom number */
        char *q = line;
        while (*q == ' ' || *q == '\t') q++;
        char *end;
        long rint_ = strtol(q, &end, 0);
        if (end == q || strlen(end) < 10) { free(xyz); free(names); return fail(b, "bad .gro atom line %d", i); }
        memcpy(res, end, 5); res[5] = 0;
        memcpy(nm, end + 5, 5); nm[5] = 0;
        remove_space(res); remove_space(nm);
        char *rest = end + 10;
        while (*rest == ' ') rest++;
        while (*rest && *rest != ' ') rest++;          /* the atom number (%s) */
        int newres = (tmpint != rint_ || strcmp(res, prevres));
        if (newres) {
            if (aa_model(res) < 0) { free(xyz); free(names); return fail(b, "residue %s is not in the library", res); }
            listn = read_atom_list(b, res, list);
            if (listn < 0) { free(xyz); free(names); return fail(b, "cannot read Library_%s/AA/%s.txt", b->ff, res); }
        }
        if (check_valid(nm, list, listn)) {
            n++;
            double v[3];
            if (sscanf(rest, "%lf%lf%lf", &v[0], &v[1], &v[2]) != 3) { free(xyz); free(names); return fail(b, "bad coordinates on .gro line %d", i); }
            for (int d = 0; d < 3; d++) {
                /* the reference writes coordinate.xyz with "%16.6lf" and reads it back */
                char tmp[64];
                snprintf(tmp, sizeof tmp, "%16.6f", v[d] * 10);
                xyz[n][d] = strtod(tmp, NULL);
            }
            snprintf(names[n], 8, "%s", nm);
        }
        if (newres) {
            int k = ++b->naa;
            snprintf(b->aa[k].name, 8, "%s", res);
            b->aa[k].protein = (rint_ < tmpint || b->nprot == 0) ? b->nprot + 1 : b->nprot;
            b->aa[k - 1].end = n - 1;
            b->aa[k].start = n;
            b->aa[k].type = aa_model(res);
            if (rint_ < tmpint || b->nprot == 0) {
                int pk = ++b->nprot;
                b->prot[pk - 1].end_aa = k - 1;
                b->prot[pk].start_aa = k;
                b->prot[pk - 1].end_atom = n - 1;
                b->prot[pk].start_atom = n;
            }
            tmpint = (int)rint_;
            snprintf(prevres, sizeof prevres, "%s", res);
        }
    }
    if (!dbl(c, &b->box[1]) || !dbl(c, &b->box[2]) || !dbl(c, &b->box[3])) { free(xyz); free(names); return fail(b, "missing .gro box line"); }
    for (int d = 1; d <= 3; d++) b->box[d] *= 10;
    b->aa[b->naa].end = n;
    b->prot[b->nprot].end_aa = b->naa;
    b->prot[b->nprot].end_atom = n;
    b->n = n;
    /* ReadCoordinate (src/Initialization.c:992-1057) */
    int aanum = 1, pep = 1;
    for (int i = 1; i <= n; i++) {
        hatom *a = &b->atom[i];
        snprintf(a->name, 8, "%s", names[i]);
        memcpy(a->pos, xyz[i], sizeof a->pos);
        if (i > b->aa[aanum].end) aanum++;
        if (i > b->prot[pep].end_atom) pep++;
        a->aanum = aanum - b->prot[pep - 1].end_aa;
        a->protein = pep;
        snprintf(a->aa, 8, "%s", b->aa[aanum].name);
        a->aatype = aa_model(a->aa);
    }
    free(xyz); free(names);
    return SDMD_OK;
}

/* ---- model: ReadModel / ScanAA / Bond- and ConstrDuplicate ------------------- */
static int find_target(B *b, int k, const char *target) {   /* FindTargetAtom (:1345-1369) */
    int start, end;
    if (target[0] == '+') {
        if (k == b->naa || b->aa[k + 1].protein != b->aa[k].protein) return -1;
        start = b->aa[k + 1].start; end = b->aa[k + 1].end;
    } else {
        start = b->aa[k].start; end = b->aa[k].end;
    }
    const char *t = target[0] == '+' ? target + 1 : target;
    for (int i = start; i <= end; i++) if (i >= 1 && i <= b->n && !strcmp(b->atom[i].name, t)) return i;
    return 0;
}

static void remove_bond(hatom *a, int j) {
    for (int k = 0; k < a->nbond; k++) if (a->bond[k].j == j) {
        memmove(a->bond + k, a->bond + k + 1, sizeof(bond_t) * (a->nbond - k - 1)); a->nbond--; return;
    }
}
static void remove_con(hatom *a, int j) {
    for (int k = 0; k < a->ncon; k++) if (a->con[k].j == j) {
        memmove(a->con + k, a->con + k + 1, sizeof(cons_t) * (a->ncon - k - 1)); a->ncon--; return;
    }
}

/* FindNextBondList (src/Initialization.c:1247-1277) */
static int next_bond(B *b, int target, int self, double dmin, double dmax, int type) {
    hatom *a = &b->atom[self];
    for (int k = 0; k < a->nbond; k++) {
        if (a->bond[k].j == target) {
            if (a->bond[k].dmin != dmin || a->bond[k].dmax != dmax) {
                if (strcmp(a->aa, "PRO") && strcmp(b->atom[target].aa, "PRO")) { b->warnings++; return 0; }
                a->bond[k].dmin = dmin; a->bond[k].dmax = dmax;
            }
            return 0;
        }
    }
    bond_t v = {target, dmin, dmax};
    bond_prepend(a, v);
    if (type == 2) remove_con(a, target);
    return 1;
}

/* ConstrList (src/Initialization.c:1280-1308): reads dmin, step pairs, dmax */
static int constr_list(B *b, int target, int step, int self, cur *c, int type) {
    hatom *a = &b->atom[self];
    for (int k = 0; k < a->ncon; k++) if (a->con[k].j == target) return 0;
    cons_t v = {target, 0, 0, b->conpool.n, 0};
    dbl(c, &v.dmin); v.dmin *= v.dmin;
    for (int i = 0; i < step; i++) {
        double d = 0, e = 0;
        dbl(c, &d); dbl(c, &e);
        d *= d;
        pool_add(&b->conpool, d, e);
        v.sn++;
    }
    dbl(c, &v.dmax); v.dmax *= v.dmax;
    con_prepend(a, v);
    if (type == 2) remove_bond(a, target);
    return 1;
}

static void bond_duplicate(B *b, int k) {   /* BondDuplicate (:1372-1392) */
    for (int t = b->aa[k].start; t <= b->aa[k].end; t++) {
        int from = b->atom[t].aanum == 1 ? b->aa[k].start : b->aa[k - 1].start;
        for (int i = from; i <= b->aa[k].end; i++) {
            hatom *ai = &b->atom[i];
            for (int q = 0; q < ai->nbond; q++) {
                if (ai->bond[q].j == t) {
                    if (next_bond(b, i, t, ai->bond[q].dmin, ai->bond[q].dmax, 0)) *conn_at(&b->atom[t], i) |= BOND_C;
                    break;
                }
            }
        }
    }
}

static void constr_duplicate(B *b, int k) {   /* ConstrDuplicate (:1395-1435) */
    for (int t = b->aa[k].start; t <= b->aa[k].end; t++) {
        int from = b->atom[t].aanum == 1 ? b->aa[k].start : b->aa[k - 1].start;
        for (int i = from; i <= b->aa[k].end; i++) {
            hatom *ai = &b->atom[i];
            for (int q = 0; q < ai->ncon; q++) {
                if (ai->con[q].j != t) continue;
                int have = 0;
                hatom *at = &b->atom[t];
                for (int r = 0; r < at->ncon; r++) if (at->con[r].j == i) { have = 1; break; }
                if (have) continue;
                cons_t v = {i, ai->con[q].dmin, ai->con[q].dmax, ai->con[q].soff, ai->con[q].sn};
                con_prepend(at, v);
                *conn_at(at, i) |= CONSTR_C;
                break;
            }
        }
    }
}

static int scan_aa(B *b, int k, int type) {   /* ScanAA (src/Initialization.c:1098-1230) */
    const char *file = type == 2 ? "PRO_INTER" : type == 1 ? "ALA" : b->aa[k].name;
    char path[2048], t[256], r1[256], r2[256];
    snprintf(path, sizeof path, "%s/Library_%s/AA/%s.txt", b->datadir, b->ff, file);
    cur c;
    if (slurp(path, &c)) return fail(b, "cannot find the parameter file for amino acid %s", file);
    skipline(&c);
    int isnew = !strcmp(b->p->continue_mode, "new");
    const char *me = b->aa[k].name, *nx = aa_name(b, k + 1);
    int rc = SDMD_OK;
    while (tok(&c, t, sizeof t)) {
        if (!strcmp(t, "ATOM")) {
            if (isnew && type == 0) {
                char tn[64], e0[64], e1[64];
                double mass = 0;
                tok(&c, r1, sizeof r1);
                int num = find_target(b, k, r1);
                tok(&c, tn, sizeof tn); dbl(&c, &mass); tok(&c, e0, sizeof e0); tok(&c, e1, sizeof e1);
                if (num < 0) num = 0;
                hatom *a = &b->atom[num];
                a->mass = mass;
                snprintf(a->ext0, 16, "%.15s", e0); snprintf(a->ext1, 16, "%.15s", e1);
                a->type = atom_model(tn);
                if (a->type < 0) { rc = fail(b, "no atom type is matched to %s", tn); break; }
            } else {
                skipline(&c);
            }
        } else if (!strcmp(t, "BOND") || !strcmp(t, "ANGLE") || !strcmp(t, "INTER")) {
            tok(&c, r1, sizeof r1);
            int num = find_target(b, k, r1);
            if (num > 0) {
                double len = 0, delta = 0;
                tok(&c, r2, sizeof r2); dbl(&c, &len); dbl(&c, &delta);
                int tmp = find_target(b, k, r2);
                if (tmp == 0) {
                    if (r2[0] == 'H' || (!strcmp(nx, "GLY") && !strcmp(r2, "+CB")) ||
                        (!strcmp(me, "GLY") && !strcmp(r2, "CB")) || (!strcmp(nx, "PRO") && !strcmp(r2, "+H")))
                        continue;
                    rc = fail(b, "protein AA #%d cannot find atom %s", k, r2);
                    break;
                } else if (tmp == -1) {
                    continue;
                }
                double dmin = len * (1 - delta); dmin *= dmin;
                double dmax = len * (1 + delta); dmax *= dmax;
                if (next_bond(b, tmp, num, dmin, dmax, type)) {
                    int *bits = conn_at(&b->atom[num], tmp);
                    if (*bits & CONSTR_C) *bits ^= CONSTR_C;
                    *bits |= BOND_C;
                }
            } else if (num == 0) {
                if (r1[0] == 'H') { b->warnings++; skipline(&c); continue; }
                if (!strcmp(r1, "CB") && !strcmp(me, "GLY")) { skipline(&c); continue; }
                rc = fail(b, "cannot find atom %s in AA #%d", r1, k);
                break;
            }
        } else if (!strncmp(t, "CONSTR", 6)) {
            int nstep = t[6] - '0';
            tok(&c, r1, sizeof r1); tok(&c, r2, sizeof r2);
            int num = find_target(b, k, r1);
            if (num <= 0 && !(!strcmp(me, "GLY") && !strcmp(r1, "CB"))) { rc = fail(b, "cannot find atom %s", r1); break; }
            int tmp = find_target(b, k, r2);
            if (tmp > 0 && num > 0) {
                if (constr_list(b, tmp, nstep, num, &c, type)) {
                    int *bits = conn_at(&b->atom[num], tmp);
                    if (*bits & BOND_C) *bits ^= BOND_C;
                    *bits |= CONSTR_C;
                }
            } else if (tmp == 0) {
                if (r2[0] == 'H') continue;
                rc = fail(b, "cannot find atom %s near atom #%d", r2, num);
                break;
            }
        }
    }
    free(c.buf);
    if (rc) return rc;
    bond_duplicate(b, k);
    constr_duplicate(b, k);
    return SDMD_OK;
}

static int read_model(B *b) {   /* ReadModel (src/Initialization.c:1076-1095) */
    for (int k = 1; k <= b->naa; k++) {
        int r;
        if ((r = scan_aa(b, k, 0))) return r;
        if (!strcmp(b->aa[k].name, "GEL")) continue;
        if (strcmp(b->aa[k].name, "ALA") && strcmp(b->aa[k].name, "PRO"))
            if ((r = scan_aa(b, k, 1))) return r;
        if (!strcmp(aa_name(b, k + 1), "PRO"))
            if ((r = scan_aa(b, k, 2))) return r;
    }
    return SDMD_OK;
}

/* ---- potential tables: CreatePotentialMatrix / ReadHB ------------------------ */
static int parse_table_line(B *b, const char *line, pairent *tabs_base, int hb_class, double rate) {
    char t0[64], t1[64];
    int pos = 0;
    if (sscanf(line, "%63s%63s%n", t0, t1, &pos) < 2) return SDMD_OK;
    int a = atom_model(t0), c = atom_model(t1);
    if (a < 0 || c < 0) return fail(b, "unknown atom type in a potential table: %s %s", t0, t1);
    if (a > c) { int q = a; a = c; c = q; }
    pairent *e = tabs_base + a * NT + c;
    const char *q = line + pos;
    char *end;
    double dmin = strtod(q, &end);
    if (end == q) return fail(b, "bad potential table line: %s", line);
    e->dmin = dmin * dmin;
    q = end;
    steppool *pool = &b->pairpool;
    int first = pool->n, n = 0;
    for (;;) {
        double d = strtod(q, &end);
        if (end == q) break;
        q = end;
        double v = strtod(q, &end);
        if (end == q) return fail(b, "odd number of step values: %s", line);
        q = end;
        double ee = hb_class ? v * rate : v;
        pool_add(pool, d * d, ee);
        n++;
    }
    e->soff = first; e->sn = n;
    accumulate(pool, first, n);
    tabs_base[c * NT + a] = *e;
    return SDMD_OK;
}

static int read_tables(B *b) {
    char path[2048], line[4096];
    snprintf(path, sizeof path, "%s/Library_Ding/InteractionPotentialTable.txt", b->datadir);
    cur c;
    if (slurp(path, &c)) return fail(b, "cannot find InteractionPotentialTable.txt");
    while (c.at < c.n) {
        getline_(&c, line, sizeof line);
        if (line[0] == '#') continue;
        int r = parse_table_line(b, line, &b->coll[0][0], 0, 1.0);
        if (r) { free(c.buf); return r; }
    }
    free(c.buf);
    snprintf(path, sizeof path, "%s/Library_Ding/HBPotentialTable.txt", b->datadir);
    if (slurp(path, &c)) return fail(b, "cannot find HBPotentialTable.txt");
    char s[256];
    skipline(&c);
    tok(&c, s, sizeof s); dbl(&c, &b->hbpot[0]); dbl(&c, &b->hbpot[1]);   /* BB_r BB_v */
    tok(&c, s, sizeof s); dbl(&c, &b->hbpot[4]); dbl(&c, &b->hbpot[5]);   /* BS_r BS_v */
    tok(&c, s, sizeof s); dbl(&c, &b->hbpot[2]); dbl(&c, &b->hbpot[3]);   /* SS_r SS_v */
    while (c.at < c.n && isspace((unsigned char)c.buf[c.at])) c.at++;
    int cls = 0, flag = 0;
    while (c.at < c.n) {
        getline_(&c, line, sizeof line);
        if (line[0] == '#') { cls++; flag = 0; continue; }
        if (cls < 1 || cls > 11) { free(c.buf); return fail(b, "HB table has more than 11 classes"); }
        double rate = cls == 1 ? b->hbpot[0] : (cls <= 5 || cls == 10) ? b->hbpot[4] : b->hbpot[2];
        char t0[64], t1[64];
        if (sscanf(line, "%63s%63s", t0, t1) < 2) continue;
        int r = parse_table_line(b, line, &b->hb[cls][0][0], 1, rate);
        if (r) { free(c.buf); return r; }
        if (!flag) {
            int a = atom_model(t0), q = atom_model(t1);
            if (a > q) { int z = a; a = q; q = z; }
            b->hb[cls][0][0] = b->hb[cls][a][q];
            flag = 1;
        }
    }
    free(c.buf);
    return SDMD_OK;
}

/* HBNeighborAssign (src/Initialization.c:1672-1847) */
static void hb_neighbor_assign(B *b, int num) {
    hatom *A = b->atom;
    hatom *a = &A[num];
    int target = b->aa[b->prot[a->protein - 1].end_aa + a->aanum].end + 1;
#define BACK_TYPE(tp) do { while (target > 1 && A[--target].type != (tp)); } while (0)
#define BACK_NAME(nm) do { while (target > 1 && strcmp(A[--target].name, (nm))); } while (0)
#define SET(role) do { a->hb_neighbor = target; a->hb_role = (role); } while (0)
    const char *r = a->aa, *n = a->name;
    if (a->type == 2) { BACK_TYPE(18); SET('D'); }
    else if (a->type == 26) { BACK_TYPE(6); SET('A'); }
    else if (!strcmp(r, "HIS")) {
        if (!strcmp(n, "HD1")) { BACK_NAME("ND1"); SET('D'); }
        else if (!strcmp(n, "HE2")) { BACK_NAME("NE2"); SET('D'); }
        else if (!strcmp(n, "NE2")) { BACK_NAME("CD2"); SET('A'); }
    } else if (!strcmp(r, "TYR")) {
        if (!strcmp(n, "HH")) { BACK_NAME("OH"); SET('D'); }
        else if (!strcmp(n, "OH")) { BACK_NAME("CZ"); SET('A'); }
    } else if (!strcmp(r, "TRP")) {
        if (!strcmp(n, "HE1")) { BACK_NAME("NE1"); SET('D'); }
    } else if (!strcmp(r, "SER")) {
        if (!strcmp(n, "HG")) { BACK_NAME("OG"); SET('D'); }
        else if (!strcmp(n, "OG")) { BACK_NAME("CB"); SET('A'); }
    } else if (!strcmp(r, "THR")) {
        if (!strcmp(n, "HG1")) { BACK_NAME("OG1"); SET('D'); }
        else if (!strcmp(n, "OG1")) { BACK_NAME("CB"); SET('A'); }
    } else if (!strcmp(r, "ASN")) {
        if (!strcmp(n, "HD21") || !strcmp(n, "HD22")) { BACK_NAME("ND2"); SET('D'); }
        else if (!strcmp(n, "OD1")) { BACK_NAME("CG"); SET('A'); }
    } else if (!strcmp(r, "GLN")) {
        if (!strcmp(n, "HE21") || !strcmp(n, "HE22")) { BACK_NAME("NE2"); SET('D'); }
        else if (!strcmp(n, "OE1")) { BACK_NAME("CD"); SET('A'); }
    } else if (!strcmp(r, "LYS")) {
        if (!strcmp(n, "HZ1") || !strcmp(n, "HZ2") || !strcmp(n, "HZ3")) { BACK_NAME("NZ"); SET('D'); }
    } else if (!strcmp(r, "ARG")) {
        if (!strcmp(n, "HE")) { BACK_NAME("NE"); SET('D'); }
        else if (!strcmp(n, "HH11") || !strcmp(n, "HH12")) { BACK_NAME("NH1"); SET('D'); }
        else if (!strcmp(n, "HH21") || !strcmp(n, "HH22")) { BACK_NAME("NH2"); SET('D'); }
    } else if (!strcmp(r, "ASP")) {
        if (!strcmp(n, "OD1") || !strcmp(n, "OD2")) { BACK_NAME("CG"); SET('A'); }
    } else if (!strcmp(r, "GLU")) {
        if (!strcmp(n, "OE1") || !strcmp(n, "OE2")) { BACK_NAME("CD"); SET('A'); }
    } else if (!strcmp(r, "CYS")) {
        if (!strcmp(n, "SG")) { BACK_NAME("CB"); SET('S'); }
    }
#undef BACK_TYPE
#undef BACK_NAME
#undef SET
}

static int read_wall(B *b) {   /* ReadWall, smooth walls (src/Initialization.c:1894-1961) */
    char path[2048], s[256], name[64], tn[64], e0[64], e1[64];
    snprintf(path, sizeof path, "%s/Library_%s/Wall.txt", b->datadir, b->ff);
    cur c;
    if (slurp(path, &c)) return fail(b, "cannot find Wall.txt");
    skipline(&c);
    tok(&c, s, sizeof s); tok(&c, name, sizeof name); tok(&c, tn, sizeof tn); dbl(&c, &b->wall_mass);
    tok(&c, e0, sizeof e0); tok(&c, e1, sizeof e1);
    free(c.buf);
    memcpy(b->wall_name, name, strnlen(name, 7));
    memcpy(b->wall_ext, e0, strnlen(e0, 15));
    memcpy(b->wall_ext + 16, e1, strnlen(e1, 15));
    b->wall_type = atom_model(tn);
    if (b->wall_type < 0) return fail(b, "no atom type is matched to %s (Wall.txt)", tn);
    if (!b->wall) return SDMD_OK;
    for (int d = 0; d < 3; d++) b->wall_pos[d] = b->box[d + 1] / 2;
    if (b->wall == SDMD_WALL_PARALLEL) b->wall_pos[0] = b->wall_pos[2] = 0;
    else if (b->wall == SDMD_WALL_CYLINDER) b->wall_pos[0] = 0;
    return SDMD_OK;
}

/* GenerateVelocity (src/Initialization.c:1850-1881) */
static void generate_velocity(B *b, double temperature) {
    double com[3] = {0, 0, 0}, total = 0;
    double (*v)[3] = calloc((size_t)b->n + 1, sizeof(double[3]));
    for (int i = 1; i <= b->n; i++) {
        for (int d = 0; d < 3; d++) {
            double s = mb(b, 0, temperature / b->atom[i].mass);
            v[i][d] = s + 0.0 + 0.0;
            com[d] += v[i][d] * b->atom[i].mass;
        }
        total += b->atom[i].mass;
    }
    for (int d = 0; d < 3; d++) com[d] /= total;
    for (int i = 1; i <= b->n; i++) {
        for (int d = 0; d < 3; d++) {
            if (b->nprot == 1) v[i][d] = v[i][d] - com[d];
            b->atom[i].vel[d] = v[i][d];
        }
    }
    free(v);
}

/* SDEnergyMin (src/ToolFunctions.c:325-491): random steepest descent on bond,
 * constraint and hard-core violations, consuming rand() only for violations. */
typedef struct { int *j; double *hi, *lo, *len; int n, cap; } mlist;
static void ml_add(mlist *m, int j, double hi, double lo, double len) {
    if (m->n == m->cap) {
        m->cap = m->cap ? 2 * m->cap : 32;
        m->j = realloc(m->j, sizeof(int) * m->cap); m->hi = realloc(m->hi, sizeof(double) * m->cap);
        m->lo = realloc(m->lo, sizeof(double) * m->cap); m->len = realloc(m->len, sizeof(double) * m->cap);
    }
    m->j[m->n] = j; m->hi[m->n] = hi; m->lo[m->n] = lo; m->len[m->n] = len; m->n++;
}
static int energy_min(B *b, long stepmax) {
    int N = b->n;
    mlist *L = calloc((size_t)N + 1, sizeof(mlist));
    double (*crd)[3] = calloc((size_t)N + 1, sizeof(double[3]));
    /* neighbour search for the 12 A shell, via a coarse grid (same pairs, index order) */
    double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
    for (int i = 1; i <= N; i++)
        for (int d = 0; d < 3; d++) {
            if (b->atom[i].pos[d] < lo[d]) lo[d] = b->atom[i].pos[d];
            if (b->atom[i].pos[d] > hi[d]) hi[d] = b->atom[i].pos[d];
        }
    const double G = 12.0;
    int gn[3];
    for (int d = 0; d < 3; d++) { gn[d] = (int)((hi[d] - lo[d]) / G) + 1; if (gn[d] > 512) gn[d] = 512; }
    long ng = (long)gn[0] * gn[1] * gn[2];
    int *head = malloc(sizeof(int) * ng), *next = malloc(sizeof(int) * (N + 1)), *gi = malloc(sizeof(int) * (N + 1));
    for (long g = 0; g < ng; g++) head[g] = 0;
    for (int i = N; i >= 1; i--) {
        int c[3];
        for (int d = 0; d < 3; d++) { c[d] = (int)((b->atom[i].pos[d] - lo[d]) / G); if (c[d] >= gn[d]) c[d] = gn[d] - 1; if (c[d] < 0) c[d] = 0; }
        gi[i] = (c[2] * gn[1] + c[1]) * gn[0] + c[0];
        next[i] = head[gi[i]]; head[gi[i]] = i;
    }
    int *cand = malloc(sizeof(int) * (N + 1));
    for (int i = 1; i <= N; i++) {
        hatom *a = &b->atom[i];
        memcpy(crd[i], a->pos, sizeof(crd[i]));
        for (int q = 0; q < a->nbond; q++) {
            double h = sqrt(a->bond[q].dmax), l = sqrt(a->bond[q].dmin);
            ml_add(&L[i], a->bond[q].j, h, l, 0.5 * (h + l));
        }
        for (int q = 0; q < a->ncon; q++) {
            double h = sqrt(a->con[q].dmax), l = sqrt(a->con[q].dmin);
            ml_add(&L[i], a->con[q].j, h, l, 0.5 * (h + l));
        }
        int nc = 0;
        int c0 = gi[i] % gn[0], c1 = (gi[i] / gn[0]) % gn[1], c2 = gi[i] / (gn[0] * gn[1]);
        for (int dz = -1; dz <= 1; dz++) for (int dy = -1; dy <= 1; dy++) for (int dx = -1; dx <= 1; dx++) {
            int x = c0 + dx, y = c1 + dy, z = c2 + dz;
            if (x < 0 || y < 0 || z < 0 || x >= gn[0] || y >= gn[1] || z >= gn[2]) continue;
            for (int n = head[(z * gn[1] + y) * gn[0] + x]; n; n = next[n]) cand[nc++] = n;
        }
        /* ascending index order, as the reference's loop n = 1..N */
        for (int p = 1; p < nc; p++) { int v = cand[p], q = p - 1; while (q >= 0 && cand[q] > v) { cand[q + 1] = cand[q]; q--; } cand[q + 1] = v; }
        for (int p = 0; p < nc; p++) {
            int n = cand[p];
            double dir[3] = {b->atom[n].pos[0] - a->pos[0], b->atom[n].pos[1] - a->pos[1], b->atom[n].pos[2] - a->pos[2]};
            double l2 = dir[0] * dir[0] + dir[1] * dir[1] + dir[2] * dir[2];
            int bits = conn_get(a, n);
            if (l2 <= 144 && !(bits & BOND_C) && !(bits & CONSTR_C)) {
                int found = 0;
                for (int q = 0; q < L[i].n; q++) if (L[i].j[q] == n) { found = 1; break; }
                if (i != n && !found) {
                    int t1 = a->type, t2 = b->atom[n].type;
                    if (t1 > t2) { int z = t1; t1 = t2; t2 = z; }
                    double lo_ = sqrt(b->coll[t1][t2].dmin);
                    ml_add(&L[i], n, SDMD_INFINIT, lo_, lo_ + 0.001);
                }
            }
        }
        if (L[i].n > 510) { free(cand); return fail(b, "too many interacting atoms around atom #%d", i); }
    }
    free(cand); free(head); free(next); free(gi);
    long step = 0, total = 1;
    double factor = 0.1;
    while (total > 0) {
        for (int i = 1; i <= N; i++) {
            double ch[3] = {0, 0, 0};
            for (int q = 0; q < L[i].n; q++) {
                int j = L[i].j[q];
                double dir[3] = {crd[j][0] - crd[i][0], crd[j][1] - crd[i][1], crd[j][2] - crd[i][2]};
                double l = sqrt(dir[0] * dir[0] + dir[1] * dir[1] + dir[2] * dir[2]);
                if (l >= L[i].hi[q] || l <= L[i].lo[q]) {
                    double diff = L[i].len[q] - l;
                    double en = random01(b) * factor * diff;
                    ch[0] -= en * dir[0] / L[i].len[q];
                    ch[1] -= en * dir[1] / L[i].len[q];
                    ch[2] -= en * dir[2] / L[i].len[q];
                }
            }
            crd[i][0] += ch[0]; crd[i][1] += ch[1]; crd[i][2] += ch[2];
        }
        total = 0;
        for (int i = 1; i <= N; i++) {
            for (int q = 0; q < L[i].n; q++) {
                int j = L[i].j[q];
                if (j < i) continue;
                double dir[3] = {crd[j][0] - crd[i][0], crd[j][1] - crd[i][1], crd[j][2] - crd[i][2]};
                double l = sqrt(dir[0] * dir[0] + dir[1] * dir[1] + dir[2] * dir[2]);
                if (l >= L[i].hi[q] || l <= L[i].lo[q]) total++;
            }
            memcpy(b->atom[i].pos, crd[i], sizeof(crd[i]));
        }
        ++step;
        if (step % 1000 == 0 && factor > 0.05) factor -= 0.01;
        if (step > stepmax) break;
    }
    for (int i = 1; i <= N; i++) { free(L[i].j); free(L[i].hi); free(L[i].lo); free(L[i].len); }
    free(L); free(crd);
    return SDMD_OK;
}

/* ---- export -------------------------------------------------------------------- */
static void *zalloc(size_t n) { void *p = calloc(n ? n : 1, 1); return p; }

static int export_system(B *b, sdmd_host_system **out) {
    int N = b->n;
    size_t N1 = (size_t)N + 1;
    sdmd_host_system *h = calloc(1, sizeof(*h));
    sdmd_system *s = &h->sys;
    s->n_atoms = N;
    for (int d = 0; d < 3; d++) {
        s->cellnum[d] = b->cellnum[d + 1]; s->box[d] = b->box[d + 1]; s->cellsize[d] = b->cellsize[d + 1];
        s->wall_pos[d] = b->wall_pos[d]; s->wall_vel[d] = 0;
    }
    const sdmd_params *p = b->p;
    s->cutoff = p->cutoff;
    s->temperature = p->temperature;
    s->thermo_freq = p->thermo_freq;
    s->t_end = p->time;
    s->thermostat = strcmp(p->thermostat, "no") ? 1 : 0;
    s->wall = b->wall; s->wall_type = b->wall_type; s->wall_mass = b->wall ? b->wall_mass : 0;
    h->wall_lib_mass = b->wall_mass;   /* obstruction walls' atoms carry it too (ObstInfo.dat) */
    if (strcmp(p->obstruct, "no")) {   /* Obstruct? (src/Initialization.c:634-672) */
        s->n_obst = p->n_obst;
        memcpy(h->obst, p->obst_pos, sizeof(double) * 3 * (size_t)p->n_obst);
        s->obst = h->obst;
    }
    if (strcmp(p->sphobst, "no")) {   /* SphObst? (src/Initialization.c:703-724) */
        s->n_sphobst = p->n_sphobst;
        memcpy(h->sphobst, p->sphobst_xyzr, sizeof(double) * 4 * (size_t)p->n_sphobst);
        s->sphobst = h->sphobst;
    }
    s->hb_barrier[0] = b->hbpot[1]; s->hb_barrier[1] = b->hbpot[5]; s->hb_barrier[2] = b->hbpot[3];
#define A(name, T, cnt) h->name = zalloc(sizeof(T) * (cnt)); s->name = h->name
    A(mass, double, N1); A(protein, int32_t, N1); A(aanum, int32_t, N1); A(aatype, int32_t, N1);
    A(hb_neighbor, int32_t, N1); A(hb_role, int32_t, N1); A(name_code, int32_t, N1);
    A(x, double, N1); A(y, double, N1); A(z, double, N1); A(vx, double, N1); A(vy, double, N1); A(vz, double, N1);
    A(cx, int32_t, N1); A(cy, int32_t, N1); A(cz, int32_t, N1); A(type, int32_t, N1); A(hb_bond, int32_t, N1);
    A(hb_itype, int32_t, N1); A(nb_partner, int32_t, 4 * N1); A(nb_status, int32_t, N1); A(nb_pnum, int32_t, N1);
    A(ev_time, double, N1); A(ev_partner, int32_t, N1); A(ev_counter, int64_t, N1); A(ev_pcounter, int64_t, N1);
    A(ev_potential, double, N1); A(ev_type, int32_t, N1); A(ev_sub, int32_t, N1);
    long ncell = (long)b->cellnum[1] * b->cellnum[2] * b->cellnum[3];
    A(cell_list, int32_t, N1 + (size_t)ncell);
    A(bond_off, int32_t, N1 + 1); A(con_off, int32_t, N1 + 1); A(conn_off, int32_t, N1 + 1);
    int nb = 0, nc = 0, nn = 0;
    for (int i = 1; i <= N; i++) { nb += b->atom[i].nbond; nc += b->atom[i].ncon; nn += b->atom[i].nconn; }
    /* row 0 of the connection map: the reference's atom[0] can collect entries too */
    nn += b->atom[0].nconn;
    A(bond_j, int32_t, nb); A(bond_dmin, double, nb); A(bond_dmax, double, nb);
    A(con_j, int32_t, nc); A(con_dmin, double, nc); A(con_dmax, double, nc); A(con_step_off, int32_t, nc);
    A(con_step_n, int32_t, nc);
    A(conn_j, int32_t, nn); A(conn_bits, int32_t, nn);
    int ns = b->conpool.n;
    A(con_step_d, double, ns); A(con_step_e, double, ns); A(con_step_acc, double, ns);
    const int NT3 = SDMD_NTABLES * NT * NT;
    A(pair_dmin, double, NT3); A(pair_dmax, double, NT3); A(pair_step_off, int32_t, NT3); A(pair_step_n, int32_t, NT3);
    int np = b->pairpool.n;
    A(pair_step_d, double, np); A(pair_step_e, double, np); A(pair_step_acc, double, np);
#undef A
    h->names = zalloc(8 * N1);
    h->resnames = zalloc(8 * N1);
    s->n_bonds = nb; s->n_cons = nc; s->n_conn = nn; s->n_con_steps = ns; s->n_pair_steps = np;
    int kb = 0, kc = 0, kn = 0;
    for (int i = 0; i <= N; i++) {
        hatom *a = &b->atom[i];
        h->conn_off[i] = kn;
        /* sparse row in ascending j (lookups are by value; the order only makes rows canonical) */
        int row0 = kn;
        for (int q = 0; q < a->nconn; q++) {
            if (!a->conn[q].bits) continue;
            int jj = a->conn[q].j, bb = a->conn[q].bits, at = kn++;
            while (at > row0 && h->conn_j[at - 1] > jj) { h->conn_j[at] = h->conn_j[at - 1]; h->conn_bits[at] = h->conn_bits[at - 1]; at--; }
            h->conn_j[at] = jj; h->conn_bits[at] = bb;
        }
        if (i == 0) {
            /* the reference's atom[0] is a real struct that can pick up a mass and a
               type (FindTargetAtom returns 0 for atoms absent from a residue) */
            h->bond_off[0] = 0; h->con_off[0] = 0;
            h->mass[0] = a->mass; h->type[0] = a->type;
            h->ev_time[0] = SDMD_INFINIT; h->ev_partner[0] = SDMD_INVALID;
            continue;
        }
        h->bond_off[i] = kb;
        for (int q = 0; q < a->nbond; q++) {
            h->bond_j[kb] = a->bond[q].j; h->bond_dmin[kb] = a->bond[q].dmin; h->bond_dmax[kb] = a->bond[q].dmax; kb++;
        }
        h->con_off[i] = kc;
        for (int q = 0; q < a->ncon; q++) {
            h->con_j[kc] = a->con[q].j; h->con_dmin[kc] = a->con[q].dmin; h->con_dmax[kc] = a->con[q].dmax;
            h->con_step_off[kc] = a->con[q].soff; h->con_step_n[kc] = a->con[q].sn; kc++;
        }
        h->mass[i] = a->mass; h->protein[i] = a->protein; h->aanum[i] = a->aanum; h->aatype[i] = a->aatype;
        h->hb_neighbor[i] = a->hb_neighbor; h->hb_role[i] = a->hb_role;
        h->name_code[i] = !strcmp(a->name, "H") ? 1 : (!strcmp(a->name, "O") ? 2 : 0);
        h->x[i] = a->pos[0]; h->y[i] = a->pos[1]; h->z[i] = a->pos[2];
        h->vx[i] = a->vel[0]; h->vy[i] = a->vel[1]; h->vz[i] = a->vel[2];
        h->type[i] = a->type;
        h->ev_time[i] = SDMD_INFINIT; h->ev_partner[i] = SDMD_INVALID;
        memcpy(h->names + 8 * i, a->name, 8);
        memcpy(h->resnames + 8 * i, a->aa, 8);
    }
    h->conn_off[N + 1] = kn; h->bond_off[N + 1] = kb; h->con_off[N + 1] = kc;
    s->n_conn = kn;
    /* the checkpoint's static records: extra properties, and the residue and peptide
       tables with CalculateMass's masses (a hydrogen counts 1, src/Initialization.c
       1547-1570) */
    h->ext = zalloc(32 * N1);
    for (int i = 0; i <= N; i++) {   /* atom 0 too: it can pick up a residue's extra properties */
        memcpy(h->ext + 32 * i, b->atom[i].ext0, strnlen(b->atom[i].ext0, 15));
        memcpy(h->ext + 32 * i + 16, b->atom[i].ext1, strnlen(b->atom[i].ext1, 15));
    }
    h->n_aa = b->naa; h->n_prot = b->nprot;
    const size_t na1 = (size_t)b->naa + 1, np1 = (size_t)b->nprot + 1;
    h->aa_name = zalloc(8 * na1);
    h->aa_type = zalloc(4 * na1); h->aa_start = zalloc(4 * na1); h->aa_end = zalloc(4 * na1); h->aa_prot = zalloc(4 * na1);
    h->aa_mass = zalloc(8 * na1);
    for (int k = 1; k <= b->naa; k++) {
        memcpy(h->aa_name + 8 * k, b->aa[k].name, strnlen(b->aa[k].name, 4));
        h->aa_type[k] = b->aa[k].type; h->aa_start[k] = b->aa[k].start; h->aa_end[k] = b->aa[k].end;
        h->aa_prot[k] = b->aa[k].protein;
        for (int n = b->aa[k].start; n <= b->aa[k].end; n++)
            h->aa_mass[k] += strncmp(b->atom[n].name, "H", 1) == 0 ? 1 : b->atom[n].mass;
    }
    h->pep_start = zalloc(4 * np1); h->pep_end = zalloc(4 * np1); h->pep_aa_start = zalloc(4 * np1);
    h->pep_aa_end = zalloc(4 * np1); h->pep_mass = zalloc(8 * np1);
    for (int k = 1; k <= b->nprot; k++) {
        h->pep_start[k] = b->prot[k].start_atom; h->pep_end[k] = b->prot[k].end_atom;
        h->pep_aa_start[k] = b->prot[k].start_aa; h->pep_aa_end[k] = b->prot[k].end_aa;
        for (int n = b->prot[k].start_atom; n <= b->prot[k].end_atom; n++)
            h->pep_mass[k] += strncmp(b->atom[n].name, "H", 1) == 0 ? 1 : b->atom[n].mass;
    }
    memcpy(h->method, p->force_field, strnlen(p->force_field, sizeof h->method - 1));
    memcpy(h->hbpot, b->hbpot, sizeof h->hbpot);
    memcpy(h->wall_name, b->wall_name, sizeof h->wall_name);
    memcpy(h->wall_ext, b->wall_ext, sizeof h->wall_ext);
    /* InitializeCharge (src/Initialization.c:2092-2118) without charge-model flags:
       "+" / "-" atoms of ARG, ASP, GLU, HIS and LYS, then each peptide's first atom
       of type 18 and last of type 26 */
    h->charge = zalloc(8 * N1);
    for (int i = 1; i <= N; i++) {
        const int res = b->atom[i].aatype;
        if (res == 2 || res == 4 || res == 7 || res == 9 || res == 12) {
            if (!strcmp(b->atom[i].ext0, "+")) h->charge[i] = 1;
            else if (!strcmp(b->atom[i].ext0, "-")) h->charge[i] = -1;
        }
    }
    for (int k = 1; k <= b->nprot; k++) {
        for (int n = b->prot[k].start_atom; n <= b->prot[k].end_atom; n++)
            if (b->atom[n].type == 18) { h->charge[n] = 1; break; }
        for (int n = b->prot[k].end_atom; n >= b->prot[k].start_atom; n--)
            if (b->atom[n].type == 26) { h->charge[n] = -1; break; }
    }
    memcpy(h->con_step_d, b->conpool.d, sizeof(double) * ns);
    memcpy(h->con_step_e, b->conpool.e, sizeof(double) * ns);
    memcpy(h->con_step_acc, b->conpool.acc, sizeof(double) * ns);
    memcpy(h->pair_step_d, b->pairpool.d, sizeof(double) * np);
    memcpy(h->pair_step_e, b->pairpool.e, sizeof(double) * np);
    memcpy(h->pair_step_acc, b->pairpool.acc, sizeof(double) * np);
    for (int t = 0; t < SDMD_NTABLES; t++)
        for (int a = 0; a < NT; a++)
            for (int c = 0; c < NT; c++) {
                pairent *e = t == 0 ? &b->coll[a][c] : &b->hb[t][a][c];
                int idx = (t * NT + a) * NT + c;
                h->pair_dmin[idx] = e->dmin; h->pair_dmax[idx] = e->dmax;
                h->pair_step_off[idx] = e->soff; h->pair_step_n[idx] = e->sn;
            }
    /* LinkList("full") (src/Events.c:117-156): head insertion, atoms 1..N in order */
    for (int i = 1; i <= N; i++) {
        int c[3];
        const double pos[3] = {h->x[i], h->y[i], h->z[i]};
        for (int d = 0; d < 3; d++) {
            c[d] = (int)(pos[d] / s->cellsize[d]);
            if (c[d] == s->cellnum[d]) c[d]--;
            if (c[d] < 0 || c[d] >= s->cellnum[d]) { sdmd_host_free(h); return fail(b, "atom #%d lies outside the box after PBC", i); }
        }
        h->cx[i] = c[0]; h->cy[i] = c[1]; h->cz[i] = c[2];
        long cell = (long)c[2] * s->cellnum[0] * s->cellnum[1] + (long)c[1] * s->cellnum[0] + c[0] + 1;
        h->cell_list[i] = h->cell_list[N + cell];
        h->cell_list[N + cell] = i;
    }
    s->time = 0;
    s->rng = b->rng;
    memset(&s->counters, 0, sizeof s->counters);
    s->counters.warnings = b->warnings;
    *out = h;
    return SDMD_OK;
}

static void free_builder(B *b) {
    if (b->atom) for (int i = 0; i <= b->n + 1; i++) { free(b->atom[i].bond); free(b->atom[i].con); free(b->atom[i].conn); }
    free(b->atom); free(b->aa); free(b->prot);
    free(b->conpool.d); free(b->conpool.e); free(b->conpool.acc);
    free(b->pairpool.d); free(b->pairpool.e); free(b->pairpool.acc);
}

static int build(B *b, cur *coords, uint32_t seed, int emin, sdmd_host_system **out) {
    const sdmd_params *p = b->p;
    if (strcmp(p->continue_mode, "new")) return fail(b, "only \"new\" runs are built here (continue runs load a checkpoint)");
    if (strncmp(p->force_field, "Ding", 1)) return fail(b, "only the Ding force field is supported");
    if (strcmp(p->cg, "no") || strcmp(p->flow, "no") || strcmp(p->tunnel, "no") || strcmp(p->wall_dyn, "no"))
        return fail(b, "CG models, flow, tunnels and dynamic walls are outside the engine's scope");
    snprintf(b->ff, sizeof b->ff, "%s", p->force_field);
    b->wall = 0;
    if (strcmp(p->wall_exist, "no")) {
        if (strncmp(p->wall_exist, "smooth", 2)) return fail(b, "only smooth walls are supported");
        b->wall = p->wall_type[0] == 'p' ? SDMD_WALL_PARALLEL : p->wall_type[0] == 'c' ? SDMD_WALL_CYLINDER :
                  p->wall_type[0] == 's' ? SDMD_WALL_SPHERE : 0;
        if (!b->wall) return fail(b, "unknown wall type %s", p->wall_type);
    }
    rng_seed(&b->rng, seed);
    int r;
    if ((r = read_gro(b, coords))) return r;
    for (int d = 1; d <= 3; d++) {       /* CreateCell (src/Initialization.c:1060-1073) */
        b->cellnum[d] = (int)floor(b->box[d] / p->cutoff);
        if (b->cellnum[d] < 3) b->cellnum[d] = 3;
        b->cellsize[d] = b->box[d] / b->cellnum[d];
    }
    if ((r = read_model(b))) return r;
    if ((r = read_tables(b))) return r;
    for (int i = 1; i <= b->n; i++) hb_neighbor_assign(b, i);
    if ((b->wall || b->p->n_obst) && (r = read_wall(b))) return r;   /* obstacles are Wall.txt atoms too */
    generate_velocity(b, p->temperature);
    if (emin > 0 && (r = energy_min(b, emin))) return r;
    /* PBC("full") (src/Events.c:207-229) */
    if (b->wall != SDMD_WALL_SPHERE) {
        int dims = 3, step = 1;
        if (b->wall == SDMD_WALL_PARALLEL) step = 2;
        else if (b->wall == SDMD_WALL_CYLINDER) dims = 1;
        for (int i = 1; i <= b->n; i++)
            for (int d = 0; d < dims; d += step) {
                if (b->atom[i].pos[d] >= b->box[d + 1]) b->atom[i].pos[d] -= b->box[d + 1];
                else if (b->atom[i].pos[d] < 0) b->atom[i].pos[d] += b->box[d + 1];
            }
    }
    return export_system(b, out);
}

int sdmd_build_system(const char *datadir, const char *coord_file, const sdmd_params *p, const double *box,
                      uint32_t seed, int energy_min_steps, sdmd_host_system **out, char *errbuf, int errlen) {
    B b;
    memset(&b, 0, sizeof b);
    b.p = p; b.err = errbuf; b.errlen = errlen;
    snprintf(b.datadir, sizeof b.datadir, "%s", datadir);
    char path[2048];
    snprintf(path, sizeof path, "%s/%s", datadir, coord_file);
    const char *dot = strrchr(coord_file, '.');
    if (!dot || strcmp(dot, ".gro")) { (void)box; return fail(&b, "only .gro coordinate files are read here"); }
    cur c;
    if (slurp(path, &c)) return fail(&b, "cannot open %s", path);
    int r = build(&b, &c, seed, energy_min_steps, out);
    free(c.buf);
    free_builder(&b);
    return r;
}

int sdmd_build_system_gro_text(const char *datadir, const char *gro_text, const sdmd_params *p, uint32_t seed,
                               int energy_min_steps, sdmd_host_system **out, char *errbuf, int errlen) {
    B b;
    memset(&b, 0, sizeof b);
    b.p = p; b.err = errbuf; b.errlen = errlen;
    snprintf(b.datadir, sizeof b.datadir, "%s", datadir);
    cur c;
    cur_text(gro_text, &c);
    int r = build(&b, &c, seed, energy_min_steps, out);
    free(c.buf);
    free_builder(&b);
    return r;
}

sdmd_system *sdmd_host_view(sdmd_host_system *h) { return h ? &h->sys : NULL; }
const char *sdmd_host_atom_names(const sdmd_host_system *h) { return h ? h->names : NULL; }
const char *sdmd_host_residue_names(const sdmd_host_system *h) { return h ? h->resnames : NULL; }

void sdmd_host_static_info(const sdmd_host_system *h, sdmd_host_static *o) {
    o->n_aa = h->n_aa; o->n_prot = h->n_prot;
    o->names = h->names; o->resnames = h->resnames; o->ext = h->ext;
    o->aa_name = h->aa_name; o->aa_type = h->aa_type; o->aa_start = h->aa_start; o->aa_end = h->aa_end;
    o->aa_prot = h->aa_prot; o->aa_mass = h->aa_mass;
    o->pep_start = h->pep_start; o->pep_end = h->pep_end; o->pep_aa_start = h->pep_aa_start;
    o->pep_aa_end = h->pep_aa_end; o->pep_mass = h->pep_mass;
    o->method = h->method;
    o->mass0 = h->mass; o->type0 = h->type;
    o->hbpot = h->hbpot;
    o->charge = h->charge;
    o->wall_name = h->wall_name; o->wall_ext = h->wall_ext; o->wall_lib_mass = h->wall_lib_mass;
}

void sdmd_host_free(sdmd_host_system *h) {
    if (!h) return;
    void *ptrs[] = {h->mass, h->x, h->y, h->z, h->vx, h->vy, h->vz, h->ev_time, h->ev_potential, h->protein, h->aanum,
                    h->aatype, h->hb_neighbor, h->hb_role, h->name_code, h->bond_off, h->bond_j, h->con_off, h->con_j,
                    h->con_step_off, h->con_step_n, h->conn_off, h->conn_j, h->conn_bits, h->bond_dmin, h->bond_dmax,
                    h->con_dmin, h->con_dmax, h->con_step_d, h->con_step_e, h->con_step_acc, h->pair_dmin, h->pair_dmax,
                    h->pair_step_d, h->pair_step_e, h->pair_step_acc, h->pair_step_off, h->pair_step_n, h->cx, h->cy,
                    h->cz, h->type, h->hb_bond, h->hb_itype, h->nb_partner, h->nb_status, h->nb_pnum, h->ev_partner,
                    h->ev_type, h->ev_sub, h->cell_list, h->ev_counter, h->ev_pcounter, h->names, h->resnames,
                    h->ext, h->aa_name, h->aa_type, h->aa_start, h->aa_end, h->aa_prot, h->aa_mass, h->pep_start,
                    h->pep_end, h->pep_aa_start, h->pep_aa_end, h->pep_mass, h->charge};
    for (size_t k = 0; k < sizeof(ptrs) / sizeof(ptrs[0]); k++) free(ptrs[k]);
    free(h);
}

/* =============================================================================
 * Synthetic-workload generator: random-sequence peptides placed in a box.
 *
 * Each chain's topology comes from the same model code as above (a placeholder
 * .gro with the library's atoms is built first); atoms are then placed along
 * bonds outward from an extended backbone and relaxed against every bond,
 * angle, step-constraint and hard-core bound of the model until no bound is
 * violated.  Chains are rotated uniformly at random and translated without
 * overlap, and the result is written as .gro text (coordinates in nm with five
 * decimals), the reference's own input format.
 * ============================================================================= */
typedef struct { uint64_t s; } xrng;
static uint64_t xr_next(xrng *r) { r->s ^= r->s << 13; r->s ^= r->s >> 7; r->s ^= r->s << 17; return r->s; }
static double xr_u(xrng *r) { return (double)(xr_next(r) >> 11) * (1.0 / 9007199254740992.0); }

typedef struct { char *s; size_t n, cap; } sbuf;
static void sb_printf(sbuf *b, const char *fmt, ...) {
    va_list ap;
    for (;;) {
        va_start(ap, fmt);
        int k = vsnprintf(b->s ? b->s + b->n : NULL, b->s ? b->cap - b->n : 0, fmt, ap);
        va_end(ap);
        if (b->s && (size_t)k < b->cap - b->n) { b->n += (size_t)k; return; }
        b->cap = b->cap * 2 + (size_t)k + 1024;
        b->s = realloc(b->s, b->cap);
    }
}

/* library atom names of residue `res` as the .gro should list them */
static int residue_atoms(B *b, const char *res, int first, char names[][8]) {
    char list[20][8] = {{0}};
    int n = read_atom_list(b, res, list), m = 0;
    if (n < 0) return -1;
    for (int i = 0; i < n; i++) {
        if (!strcmp(res, "GLY") && !strcmp(list[i], "CB")) continue;   /* GLY uses ALA's list without CB */
        if (first && !strcmp(list[i], "H")) continue;                  /* the N-terminal N carries no H */
        memcpy(names[m++], list[i], 8);                                 /* tok() ends each name within 8 bytes */
    }
    return m;
}

static double dist3(const double *a, const double *c) {
    double d0 = a[0] - c[0], d1 = a[1] - c[1], d2 = a[2] - c[2];
    return sqrt(d0 * d0 + d1 * d1 + d2 * d2);
}

static void move4(double *pi, double *pj, double target, double w) {
    double d[4] = {pj[0] - pi[0], pj[1] - pi[1], pj[2] - pi[2], pj[3] - pi[3]};
    double l = sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2] + d[3] * d[3]);
    if (l < 1e-9) { d[0] = 1e-3; d[1] = 0.7e-3; d[2] = 0.3e-3; d[3] = 0; l = sqrt(1.58e-6); }
    double f = w * 0.5 * (l - target) / l;
    for (int k = 0; k < 4; k++) { pi[k] += f * d[k]; pj[k] -= f * d[k]; }
}
static double dist4(const double *a, const double *c) {
    double s = 0;
    for (int k = 0; k < 4; k++) { double d = a[k] - c[k]; s += d * d; }
    return sqrt(s);
}

/* window violation: bounds touching atoms [m0, m1], hard cores against [c0, m1] */
static double window_violation(B *b, int c0, int m0, int m1) {
    double worst = 0;
    for (int i = m0; i <= m1; i++) {
        hatom *a = &b->atom[i];
        for (int q = 0; q < a->nbond; q++) {
            int j = a->bond[q].j;
            if (j > m1) continue;
            double lo = sqrt(a->bond[q].dmin), hi = sqrt(a->bond[q].dmax), d = dist3(a->pos, b->atom[j].pos);
            double v = d < lo + 0.0004 ? lo + 0.0004 - d : (d > hi - 0.0004 ? d - hi + 0.0004 : 0);
            if (v > worst) worst = v;
        }
        for (int q = 0; q < a->ncon; q++) {
            int j = a->con[q].j;
            if (j > m1) continue;
            double lo = sqrt(a->con[q].dmin), hi = sqrt(a->con[q].dmax), d = dist3(a->pos, b->atom[j].pos);
            double v = d < lo + 0.0004 ? lo + 0.0004 - d : (d > hi - 0.0004 ? d - hi + 0.0004 : 0);
            if (v > worst) worst = v;
        }
        for (int j = c0; j <= m1; j++) {
            if (j == i || (j >= m0 && j < i)) continue;
            int bits = conn_get(&b->atom[i], j) | conn_get(&b->atom[j], i);
            if (bits & (BOND_C | CONSTR_C)) continue;
            int t1 = b->atom[i].type, t2 = b->atom[j].type;
            if (t1 > t2) { int z = t1; t1 = t2; t2 = z; }
            double dmin = sqrt(b->coll[t1][t2].dmin), d = dist3(b->atom[i].pos, b->atom[j].pos);
            if (dmin > 0 && dmin + 0.002 - d > worst) worst = dmin + 0.002 - d;
        }
    }
    return worst;
}

/* Projection relaxation in 4D of the mobile atoms [m0, m1] against the fixed
 * context [c0, m0); the 4th coordinate is then squeezed to zero while the
 * bounds keep being enforced.  Returns the window's remaining violation. */
static double relax_window(B *b, int c0, int m0, int m1, int sweeps, xrng *rng) {
    int n = m1 - c0 + 1;
    double (*P)[4] = malloc(sizeof(double[4]) * (size_t)n);
#define PP(i) P[(i) - c0]
    for (int i = c0; i <= m1; i++) {
        for (int k = 0; k < 3; k++) PP(i)[k] = b->atom[i].pos[k];
        PP(i)[3] = i >= m0 ? 2.0 * (xr_u(rng) - 0.5) : 0.0;
    }
    double res = 1e300;
    for (int sweep = 0; sweep < sweeps; sweep++) {
        int hard = sweep >= sweeps / 8;
        if (sweep >= sweeps / 4) for (int i = m0; i <= m1; i++) PP(i)[3] *= 0.9;
        for (int i = m0; i <= m1; i++) {
            hatom *a = &b->atom[i];
            for (int q = 0; q < a->nbond + a->ncon; q++) {
                int con = q >= a->nbond, j = con ? a->con[q - a->nbond].j : a->bond[q].j;
                if (j < c0 || j > m1) continue;
                double lo = sqrt(con ? a->con[q - a->nbond].dmin : a->bond[q].dmin);
                double hi = sqrt(con ? a->con[q - a->nbond].dmax : a->bond[q].dmax);
                double d = dist4(PP(i), PP(j)), target = -1;
                if (!con) { double w = hi - lo; if (d < lo + 0.25 * w || d > hi - 0.25 * w) target = 0.5 * (lo + hi); }
                else if (d < lo + 0.002) target = lo + 0.006;
                else if (d > hi - 0.002) target = hi - 0.006;
                if (target < 0) continue;
                if (j >= m0) move4(PP(i), PP(j), target, 1.0);
                else { double z[4] = {PP(j)[0], PP(j)[1], PP(j)[2], PP(j)[3]}; move4(PP(i), z, target, 2.0); }
            }
            if (!hard) continue;
            for (int j = c0; j <= m1; j++) {
                if (j == i || (j >= m0 && j < i)) continue;
                int bits = conn_get(&b->atom[i], j) | conn_get(&b->atom[j], i);
                if (bits & (BOND_C | CONSTR_C)) continue;
                int t1 = b->atom[i].type, t2 = b->atom[j].type;
                if (t1 > t2) { int z = t1; t1 = t2; t2 = z; }
                double dmin = sqrt(b->coll[t1][t2].dmin);
                if (dmin <= 0) continue;
                double d = dist4(PP(i), PP(j));
                if (d < dmin + 0.03) {
                    if (j >= m0) move4(PP(i), PP(j), dmin + 0.06, 0.5);
                    else { double z[4] = {PP(j)[0], PP(j)[1], PP(j)[2], PP(j)[3]}; move4(PP(i), z, dmin + 0.06, 1.0); }
                }
            }
        }
        if (sweep >= sweeps / 4 && (sweep & 15) == 15) {
            double w4 = 0;
            for (int i = m0; i <= m1; i++) if (fabs(PP(i)[3]) > w4) w4 = fabs(PP(i)[3]);
            if (w4 < 1e-7) {
                for (int i = m0; i <= m1; i++) for (int k = 0; k < 3; k++) b->atom[i].pos[k] = PP(i)[k];
                res = window_violation(b, c0, m0, m1);
                if (res == 0) break;
            }
        }
    }
    for (int i = m0; i <= m1; i++) for (int k = 0; k < 3; k++) b->atom[i].pos[k] = PP(i)[k];
    res = window_violation(b, c0, m0, m1);
#undef PP
    free(P);
    return res;
}

/* relaxed residue geometry in the residue's own N/CA/C frame, reused as the
   starting placement of later residues of the same type */
typedef struct { char res[8]; int first, n; char names[24][8]; double loc[24][3]; } restempl;
typedef struct { restempl t[64]; int n; } templcache;

static void frame_of(const double *N, const double *CA, const double *C, double e[3][3]) {
    double u[3], v[3];
    for (int d = 0; d < 3; d++) { u[d] = C[d] - N[d]; v[d] = CA[d] - N[d]; }
    double lu = sqrt(u[0] * u[0] + u[1] * u[1] + u[2] * u[2]);
    for (int d = 0; d < 3; d++) e[0][d] = u[d] / lu;
    double pr = v[0] * e[0][0] + v[1] * e[0][1] + v[2] * e[0][2];
    for (int d = 0; d < 3; d++) v[d] -= pr * e[0][d];
    double lv = sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    for (int d = 0; d < 3; d++) e[1][d] = v[d] / lv;
    e[2][0] = e[0][1] * e[1][2] - e[0][2] * e[1][1];
    e[2][1] = e[0][2] * e[1][0] - e[0][0] * e[1][2];
    e[2][2] = e[0][0] * e[1][1] - e[0][1] * e[1][0];
}

/* one relaxed chain; coordinates (A) and names returned in library order */
static int make_chain(const char *datadir, const char *ff, const char *seq, xrng *rng, templcache *tc, int tc_learn,
                      int *n_out, double **xyz, char (**names)[8], char (**resn)[8], int **resid, char *err, int errlen) {
    char res[64][8];
    int nres = 0;
    {
        char tmp[4096];
        snprintf(tmp, sizeof tmp, "%s", seq);
        for (char *t = strtok(tmp, " ,-"); t && nres < 64; t = strtok(NULL, " ,-")) snprintf(res[nres++], 8, "%s", t);
    }
    if (nres == 0) return SDMD_EINVAL;
    B b;
    memset(&b, 0, sizeof b);
    sdmd_params p;
    memset(&p, 0, sizeof p);
    snprintf(p.continue_mode, 20, "new"); snprintf(p.force_field, 20, "%s", ff);
    b.p = &p; b.err = err; b.errlen = errlen;
    snprintf(b.datadir, sizeof b.datadir, "%s", datadir);
    snprintf(b.ff, sizeof b.ff, "%s", ff);
    /* placeholder .gro with the right atoms */
    sbuf g = {0};
    char nm[24][8];
    int total = 0;
    for (int k = 0; k < nres; k++) total += residue_atoms(&b, res[k], k == 0, nm) > 0 ? residue_atoms(&b, res[k], k == 0, nm) : 0;
    sb_printf(&g, "placeholder\n%d\n", total);
    int serial = 0;
    for (int k = 0; k < nres; k++) {
        int m = residue_atoms(&b, res[k], k == 0, nm);
        if (m <= 0) { free(g.s); return fail(&b, "residue %s not in the library", res[k]); }
        for (int q = 0; q < m; q++)
            sb_printf(&g, "%5d%-5s%5s%5d%8.3f%8.3f%8.3f\n", k + 1, res[k], nm[q], (++serial) % 100000, 0.0, 0.0, 0.0);
    }
    sb_printf(&g, "%10.5f%10.5f%10.5f\n", 100.0, 100.0, 100.0);
    cur c;
    cur_text(g.s, &c);
    free(g.s);
    int r = read_gro(&b, &c);
    free(c.buf);
    if (!r) r = read_model(&b);
    if (!r) r = read_tables(&b);
    if (r) { free_builder(&b); return r; }
    /* residue by residue: place the new residue (backbone zigzag along +x, other
       atoms bonded outward), then relax it together with the previous residue
       against the fixed chain before them; a residue that does not relax is
       re-placed, up to 32 times */
    int N = b.n;
    int *placed = calloc((size_t)N + 1, sizeof(int));
    double best = 0;
    for (int k = 1; k <= b.naa; k++) {
        int a0 = b.aa[k].start, a1 = b.aa[k].end;
        int m0 = k > 1 ? b.aa[k - 1].start : a0;
        int c0 = k > 3 ? b.aa[k - 3].start : 1;
        double kbest = 1e300;
        double (*kpos)[3] = malloc(sizeof(double[3]) * (size_t)(a1 - m0 + 1));
        restempl *tp = NULL;
        for (int q = 0; q < tc->n; q++)
            if (!strcmp(tc->t[q].res, b.aa[k].name) && tc->t[q].first == (k == 1) && tc->t[q].n == a1 - a0 + 1) tp = &tc->t[q];
        for (int attempt = 0; attempt < 32; attempt++) {
            double s_ = ((k - 1) % 2) ? -1 : 1, x0 = 3.6 * (k - 1);
            for (int i = a0; i <= a1; i++) {
                placed[i] = 0;
                hatom *a = &b.atom[i];
                double *Pp = a->pos;
                if (!strcmp(a->name, "N")) { Pp[0] = x0; Pp[1] = 0.35 * s_; Pp[2] = 0; placed[i] = 1; }
                else if (!strcmp(a->name, "CA")) { Pp[0] = x0 + 1.2; Pp[1] = 1.0 * s_; Pp[2] = 0; placed[i] = 1; }
                else if (!strcmp(a->name, "C")) { Pp[0] = x0 + 2.4; Pp[1] = 0.35 * s_; Pp[2] = 0; placed[i] = 1; }
            }
            for (int pass = 0; pass < 32; pass++) {
                int left = 0;
                for (int i = a0; i <= a1; i++) {
                    if (placed[i]) continue;
                    hatom *a = &b.atom[i];
                    int par = 0; double len = 1.5;
                    for (int q = 0; q < a->nbond && !par; q++) {
                        int j = a->bond[q].j;
                        if (j >= a0 && j <= a1 && placed[j] && sqrt(a->bond[q].dmax) < 2.0) {
                            par = j; len = 0.5 * (sqrt(a->bond[q].dmin) + sqrt(a->bond[q].dmax));
                        }
                    }
                    if (!par) { left++; continue; }
                    double u[3] = {xr_u(rng) - 0.5, s_ * (0.6 + xr_u(rng)), (xr_u(rng) - 0.5) * 1.5};
                    double l = sqrt(u[0] * u[0] + u[1] * u[1] + u[2] * u[2]);
                    for (int d = 0; d < 3; d++) a->pos[d] = b.atom[par].pos[d] + len * u[d] / l;
                    placed[i] = 1;
                }
                if (!left) break;
            }
            for (int i = a0; i <= a1; i++)   /* anything still unplaced goes next to CA */
                if (!placed[i]) for (int d = 0; d < 3; d++) b.atom[i].pos[d] = b.atom[a0].pos[d] + 1.5 * (xr_u(rng) - 0.5);
            if (tp && attempt == 0) {        /* start from the cached geometry of this residue type */
                int iN = 0, iCA = 0, iC = 0;
                for (int i = a0; i <= a1; i++) {
                    if (!strcmp(b.atom[i].name, "N")) iN = i;
                    else if (!strcmp(b.atom[i].name, "CA")) iCA = i;
                    else if (!strcmp(b.atom[i].name, "C")) iC = i;
                }
                if (iN && iCA && iC) {
                    double e[3][3];
                    frame_of(b.atom[iN].pos, b.atom[iCA].pos, b.atom[iC].pos, e);
                    for (int i = a0; i <= a1; i++) {
                        const double *l = tp->loc[i - a0];
                        for (int d = 0; d < 3; d++)
                            b.atom[i].pos[d] = b.atom[iCA].pos[d] + l[0] * e[0][d] + l[1] * e[1][d] + l[2] * e[2][d];
                    }
                }
            }
            double v = relax_window(&b, c0, m0, a1, tp && attempt == 0 ? 600 : 3000, rng);
            if (v < kbest) { kbest = v; for (int i = m0; i <= a1; i++) memcpy(kpos[i - m0], b.atom[i].pos, sizeof(double[3])); }
            if (getenv("SDMD_RELAX_STATS")) fprintf(stderr, "res %d %s attempt %d tmpl %d v %.5f\n", k, b.aa[k].name, attempt, tp != NULL, v);
            if (v < 0.005) break;   /* mA residuals are left to the energy minimisation */
        }
        for (int i = m0; i <= a1; i++) memcpy(b.atom[i].pos, kpos[i - m0], sizeof(double[3]));
        free(kpos);
        if (kbest > best) best = kbest;
        if (tc_learn && !tp && kbest < 0.005 && tc->n < 64 && a1 - a0 + 1 <= 24) {   /* cache this residue's geometry */
            int iN = 0, iCA = 0, iC = 0;
            for (int i = a0; i <= a1; i++) {
                if (!strcmp(b.atom[i].name, "N")) iN = i;
                else if (!strcmp(b.atom[i].name, "CA")) iCA = i;
                else if (!strcmp(b.atom[i].name, "C")) iC = i;
            }
            if (iN && iCA && iC) {
                restempl *t = &tc->t[tc->n++];
                snprintf(t->res, 8, "%s", b.aa[k].name);
                t->first = (k == 1); t->n = a1 - a0 + 1;
                double e[3][3];
                frame_of(b.atom[iN].pos, b.atom[iCA].pos, b.atom[iC].pos, e);
                for (int i = a0; i <= a1; i++) {
                    double r[3] = {b.atom[i].pos[0] - b.atom[iCA].pos[0], b.atom[i].pos[1] - b.atom[iCA].pos[1],
                                   b.atom[i].pos[2] - b.atom[iCA].pos[2]};
                    for (int q = 0; q < 3; q++) t->loc[i - a0][q] = r[0] * e[q][0] + r[1] * e[q][1] + r[2] * e[q][2];
                    memcpy(t->names[i - a0], b.atom[i].name, 8);
                }
            }
        }
    }
    free(placed);
    /* residuals of a few mA are left to the energy minimisation of the build */
    if (best > 0.25) { free_builder(&b); return fail(&b, "chain %s: relaxation did not converge (%.4f A)", seq, best); }
    *n_out = N;
    *xyz = malloc(sizeof(double) * 3 * (N + 1));
    *names = malloc(8 * (size_t)(N + 1));
    *resn = malloc(8 * (size_t)(N + 1));
    *resid = malloc(sizeof(int) * (N + 1));
    for (int i = 1; i <= N; i++) {
        memcpy(*xyz + 3 * i, b.atom[i].pos, sizeof(double) * 3);
        memcpy((*names)[i], b.atom[i].name, 8);
        memcpy((*resn)[i], b.atom[i].aa, 8);
        int k = 0;
        for (int q = 1; q <= b.naa; q++) if (i >= b.aa[q].start && i <= b.aa[q].end) k = q;
        (*resid)[i] = k;
    }
    free_builder(&b);
    return SDMD_OK;
}

typedef struct {
    const char *datadir, *ff;
    const char *const *seq;
    const templcache *shared;
    int n_chains, next, failed;
    uint64_t seed;
    pthread_mutex_t mu;
    int *n; double **xyz; char (**nm)[8]; char (**rs)[8]; int **ri;
    char err[512];
} genjob;

static void *gen_worker(void *arg) {
    genjob *J = arg;
    templcache *tc = malloc(sizeof(templcache));
    for (;;) {
        pthread_mutex_lock(&J->mu);
        int c = J->failed ? J->n_chains : J->next++;
        pthread_mutex_unlock(&J->mu);
        if (c >= J->n_chains) break;
        xrng rng = {(J->seed + 0x51ed27ULL * (uint64_t)(c + 1)) * 0x9E3779B97F4A7C15ULL | 1};
        char err[512];
        *tc = *J->shared;   /* read-only templates: a chain's result does not depend on thread scheduling */
        if (make_chain(J->datadir, J->ff, J->seq[c], &rng, tc, 0, &J->n[c], &J->xyz[c], &J->nm[c], &J->rs[c], &J->ri[c], err,
                       sizeof err)) {
            pthread_mutex_lock(&J->mu);
            if (!J->failed) { J->failed = 1; snprintf(J->err, sizeof J->err, "%s", err); }
            pthread_mutex_unlock(&J->mu);
        }
    }
    free(tc);
    return NULL;
}

/* ---- compressive packing of a dense cylinder ------------------------------------
 * The chains of a dense confined workload are placed overlap-free in a longer
 * cylinder (axis x, periodic; radius D/2 about y = z = D/2), then the axis
 * shrinks to its target length by at most 1 % a step, each chain's centre moving
 * with it.  After each step the chains, kept rigid, are pushed apart: every pair
 * of atoms of two chains closer than its hard-core distance (plus a margin), and
 * every atom past the wall margin, gives its chain a push and a turn, and the
 * pushes repeat until no such contact is left.  Each chain keeps the geometry it
 * was built with. */
typedef struct { double c[3], R[9], body_r2; int a0, a1; } rchain;

static void rot_apply(const double *R, const double *v, double *o) {
    for (int k = 0; k < 3; k++) o[k] = R[3 * k] * v[0] + R[3 * k + 1] * v[1] + R[3 * k + 2] * v[2];
}

/* R <- (rotation by the small vector w) * R, re-orthonormalised */
static void rot_turn(double *R, const double *w) {
    const double th = sqrt(w[0] * w[0] + w[1] * w[1] + w[2] * w[2]);
    if (th < 1e-15) return;
    const double k[3] = {w[0] / th, w[1] / th, w[2] / th}, c = cos(th), s = sin(th), t = 1 - c;
    const double Q[9] = {t * k[0] * k[0] + c, t * k[0] * k[1] - s * k[2], t * k[0] * k[2] + s * k[1],
                         t * k[0] * k[1] + s * k[2], t * k[1] * k[1] + c, t * k[1] * k[2] - s * k[0],
                         t * k[0] * k[2] - s * k[1], t * k[1] * k[2] + s * k[0], t * k[2] * k[2] + c};
    double M[9];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) M[3 * i + j] = Q[3 * i] * R[j] + Q[3 * i + 1] * R[3 + j] + Q[3 * i + 2] * R[6 + j];
    memcpy(R, M, sizeof M);
}

/* one round of pushes, shared by the host threads: each takes a fixed range of
   atoms and sums its pushes into its own accumulators, which are added in thread
   order, so the result does not depend on scheduling */
typedef struct {
    B *b; const int *owner, *head, *next, *cell; double L, D, margin, cs;
    int i0, i1, nch; double (*acc)[7]; const rchain *ch; long contacts;
} pushjob;

static void *push_range(void *arg) {
    pushjob *J = arg;
    B *b = J->b;
    const double L = J->L, D = J->D, cs = J->cs;
    const int gx = (int)(L / cs), gy = (int)(D / cs) + 1;
    const double rw = D / 2 - J->margin;
    const rchain *ch = J->ch;
    double (*acc)[7] = J->acc;
    long contacts = 0;
    for (int i = J->i0; i < J->i1; i++) {
        hatom *a = &b->atom[i];
        const int ki = J->owner[i];
        const int c0 = J->cell[i] % gx, c1 = (J->cell[i] / gx) % gy, c2 = J->cell[i] / (gx * gy);
        for (int dz = -1; dz <= 1; dz++) for (int dy = -1; dy <= 1; dy++) for (int dx = -1; dx <= 1; dx++) {
            const int y = c1 + dy, z = c2 + dz;
            if (y < 0 || z < 0 || y >= gy || z >= gy) continue;
            const int x = (c0 + dx + gx) % gx;
            for (int j = J->head[(z * gy + y) * gx + x]; j; j = J->next[j]) {
                if (j <= i || J->owner[j] == ki) continue;
                hatom *o = &b->atom[j];
                int t1 = a->type, t2 = o->type;
                if (t1 > t2) { int t = t1; t1 = t2; t2 = t; }
                const double dmin2 = b->coll[t1][t2].dmin;
                if (dmin2 <= 0) continue;
                double v[3] = {o->pos[0] - a->pos[0], o->pos[1] - a->pos[1], o->pos[2] - a->pos[2]};
                v[0] -= L * floor(v[0] / L + 0.5);
                const double d2 = v[0] * v[0] + v[1] * v[1] + v[2] * v[2], dmin = sqrt(dmin2);
                if (d2 >= (dmin + 0.01) * (dmin + 0.01)) continue;
                contacts++;
                const double d = sqrt(d2) > 1e-9 ? sqrt(d2) : 1e-9, f = 0.5 * (dmin + 0.03 - d) / d;
                const double p[3] = {v[0] * f, v[1] * f, v[2] * f};   /* j's push; i gets -p */
                const int kj = J->owner[j];
                for (int side = 0; side < 2; side++) {
                    const int k = side ? kj : ki;
                    const double sg = side ? 1.0 : -1.0;
                    const double *q = side ? o->pos : a->pos;
                    double r[3] = {q[0] - ch[k].c[0], q[1] - ch[k].c[1], q[2] - ch[k].c[2]};
                    r[0] -= L * floor(r[0] / L + 0.5);
                    acc[k][0] += sg * p[0]; acc[k][1] += sg * p[1]; acc[k][2] += sg * p[2];
                    acc[k][3] += sg * (r[1] * p[2] - r[2] * p[1]);
                    acc[k][4] += sg * (r[2] * p[0] - r[0] * p[2]);
                    acc[k][5] += sg * (r[0] * p[1] - r[1] * p[0]);
                    acc[k][6] += 1;
                }
            }
        }
        const double ry = a->pos[1] - D / 2, rz = a->pos[2] - D / 2, rr = sqrt(ry * ry + rz * rz);
        if (rr > rw - 0.005) {   /* the wall pushes the chain inward */
            contacts++;
            const double f = (rw - 0.02 - rr) / rr, p[3] = {0, ry * f, rz * f};
            double r[3] = {a->pos[0] - ch[ki].c[0], a->pos[1] - ch[ki].c[1], a->pos[2] - ch[ki].c[2]};
            r[0] -= L * floor(r[0] / L + 0.5);
            acc[ki][1] += p[1]; acc[ki][2] += p[2];
            acc[ki][3] += r[1] * p[2] - r[2] * p[1];
            acc[ki][4] += r[2] * p[0] - r[0] * p[2];
            acc[ki][5] += r[0] * p[1] - r[1] * p[0];
            acc[ki][6] += 1;
        }
    }
    J->contacts = contacts;
    return NULL;
}

static long push_round(B *b, rchain *ch, int nch, const double *body, int *owner, double L, double D, double margin,
                       double cs, int *head, int *next, int *cell, double (*acc)[7], int nthr) {
    const int N = b->n;
    for (int k = 0; k < nch; k++)   /* atom positions from the chains' rigid motions */
        for (int i = ch[k].a0; i <= ch[k].a1; i++) {
            double *p = b->atom[i].pos;
            rot_apply(ch[k].R, body + 3 * i, p);
            for (int q = 0; q < 3; q++) p[q] += ch[k].c[q];
        }
    const int gx = (int)(L / cs), gy = (int)(D / cs) + 1;
    const double cx = L / gx;
    for (long g = 0; g < (long)gx * gy * gy; g++) head[g] = 0;
    for (int i = N; i >= 1; i--) {
        double *p = b->atom[i].pos;
        p[0] -= L * floor(p[0] / L);
        int c0 = (int)(p[0] / cx), c1 = (int)(p[1] / cs), c2 = (int)(p[2] / cs);
        c0 = c0 < 0 ? 0 : (c0 >= gx ? gx - 1 : c0);
        c1 = c1 < 0 ? 0 : (c1 >= gy ? gy - 1 : c1);
        c2 = c2 < 0 ? 0 : (c2 >= gy ? gy - 1 : c2);
        cell[i] = (c2 * gy + c1) * gx + c0;
        next[i] = head[cell[i]]; head[cell[i]] = i;
    }
    pushjob J[64];
    pthread_t th[64];
    for (int t = 0; t < nthr; t++) {
        J[t] = (pushjob){b, owner, head, next, cell, L, D, margin, cs, 1 + (int)((long)N * t / nthr),
                         1 + (int)((long)N * (t + 1) / nthr), nch, acc + (size_t)t * nch, ch, 0};
        if (t > 0) pthread_create(&th[t], NULL, push_range, &J[t]);
    }
    push_range(&J[0]);
    long contacts = J[0].contacts;
    for (int t = 1; t < nthr; t++) {
        pthread_join(th[t], NULL);
        contacts += J[t].contacts;
        for (int k = 0; k < nch; k++)
            for (int q = 0; q < 7; q++) { acc[k][q] += acc[(size_t)t * nch + k][q]; acc[(size_t)t * nch + k][q] = 0; }
    }
    for (int k = 0; k < nch; k++) {   /* the mean push moves the chain, the mean torque turns it */
        if (acc[k][6] > 0) {
            const double m = 1.0 / acc[k][6];
            for (int q = 0; q < 3; q++) ch[k].c[q] += acc[k][q] * m;
            const double w[3] = {acc[k][3] * m / ch[k].body_r2, acc[k][4] * m / ch[k].body_r2,
                                 acc[k][5] * m / ch[k].body_r2};
            rot_turn(ch[k].R, w);
        }
        for (int q = 0; q < 7; q++) acc[k][q] = 0;
    }
    return contacts;
}

static int compress_cylinder(B *b, double L0, double L1, double D, double margin) {
    const int N = b->n, nch = b->nprot;
    rchain *ch = calloc((size_t)nch, sizeof(rchain));
    double *body = malloc(sizeof(double) * 3 * (size_t)(N + 1));
    int *owner = malloc(sizeof(int) * (size_t)(N + 1));
    for (int k = 0; k < nch; k++) {   /* body frames: unwrapped about the first atom, centred */
        rchain *c = &ch[k];
        c->a0 = b->prot[k + 1].start_atom; c->a1 = b->prot[k + 1].end_atom;
        const double x0 = b->atom[c->a0].pos[0];
        double m[3] = {0, 0, 0};
        for (int i = c->a0; i <= c->a1; i++) {
            double *p = body + 3 * i;
            double dx = b->atom[i].pos[0] - x0;
            dx -= L0 * floor(dx / L0 + 0.5);
            p[0] = x0 + dx; p[1] = b->atom[i].pos[1]; p[2] = b->atom[i].pos[2];
            for (int q = 0; q < 3; q++) m[q] += p[q];
            owner[i] = k;
        }
        const double n = c->a1 - c->a0 + 1;
        double r2 = 0;
        for (int q = 0; q < 3; q++) c->c[q] = m[q] / n;
        for (int i = c->a0; i <= c->a1; i++)
            for (int q = 0; q < 3; q++) { body[3 * i + q] -= c->c[q]; r2 += body[3 * i + q] * body[3 * i + q]; }
        c->body_r2 = r2 / n + 1.0;
        for (int q = 0; q < 9; q++) c->R[q] = q % 4 == 0;
    }
    const double cs = 3.4;   /* above the largest hard-core distance plus the push margin */
    const long ncell = (long)((L0 / cs) + 2) * ((long)(D / cs) + 2) * ((long)(D / cs) + 2);
    int *head = malloc(sizeof(int) * (size_t)ncell), *next = malloc(sizeof(int) * (size_t)(N + 1)),
        *cell = malloc(sizeof(int) * (size_t)(N + 1));
    int nthr = 16;   /* a fixed partition: the packing is the same on every machine */
    {
        const char *e = getenv("SDMD_GEN_THREADS");
        if (e) nthr = atoi(e) < 1 ? 1 : (atoi(e) > 64 ? 64 : atoi(e));
    }
    double (*acc)[7] = calloc((size_t)nch * nthr, sizeof(double[7]));
    double L = L0;
    int rc = SDMD_OK;
    /* A step whose pushes do not settle within 3000 rounds is taken back: the
       chains return to the last settled packing, get a small random kick, and
       the axis shrinks by half as much (the step grows again after successes). */
    rchain *good = malloc(sizeof(rchain) * (size_t)nch);
    memcpy(good, ch, sizeof(rchain) * (size_t)nch);
    double Lgood = L, step = 0.01;
    xrng kick = {0x853c49e6748fea9bULL};
    for (;;) {
        long contacts = 1;
        int rounds = 0;
        while (contacts && rounds < 3000) {
            contacts = push_round(b, ch, nch, body, owner, L, D, margin, cs, head, next, cell, acc, nthr);
            rounds++;
        }
        if (getenv("SDMD_COMPRESS_STATS")) fprintf(stderr, "L %.3f step %.5f rounds %d contacts %ld\n", L, step, rounds, contacts);
        if (contacts) {
            if (step < 2e-4) { rc = fail(b, "compression jammed at an axis length of %.2f A (target %.2f A)", Lgood, L1); break; }
            memcpy(ch, good, sizeof(rchain) * (size_t)nch);
            L = Lgood;
            for (int k = 0; k < nch; k++) {
                for (int q = 0; q < 3; q++) ch[k].c[q] += 0.02 * (xr_u(&kick) - 0.5);
                const double w[3] = {0.004 * (xr_u(&kick) - 0.5), 0.004 * (xr_u(&kick) - 0.5), 0.004 * (xr_u(&kick) - 0.5)};
                rot_turn(ch[k].R, w);
            }
            step *= 0.5;
        } else {
            memcpy(good, ch, sizeof(rchain) * (size_t)nch);
            Lgood = L;
            if (L <= L1) break;
            if (rounds < 300 && step < 0.01) step = step * 1.5 < 0.01 ? step * 1.5 : 0.01;
        }
        const double Ln = L * (1 - step) > L1 ? L * (1 - step) : L1;
        for (int k = 0; k < nch; k++) ch[k].c[0] *= Ln / L;
        L = Ln;
    }
    free(good);
    /* whole chains (the build's energy minimisation takes plain coordinate
       differences), each with its centre inside the box */
    for (int k = 0; k < nch; k++) {
        ch[k].c[0] -= L * floor(ch[k].c[0] / L);
        for (int i = ch[k].a0; i <= ch[k].a1; i++) {
            double *p = b->atom[i].pos;
            rot_apply(ch[k].R, body + 3 * i, p);
            for (int q = 0; q < 3; q++) p[q] += ch[k].c[q];
        }
    }
    free(ch); free(body); free(owner); free(head); free(next); free(cell); free(acc);
    return rc;
}

int sdmd_generate_gro(const char *datadir, const char *ff, int n_chains, const char *const *sequences,
                      const double box[3], int wall, double margin, uint64_t seed, char **gro_out, char *err,
                      int errlen) {
    xrng rng = {seed * 0x9E3779B97F4A7C15ULL + 0x1234567ULL};
    sbuf out = {0};
    int total = 0;
    double *all = NULL;
    int nall = 0, capall = 0;
    char (*an)[8] = NULL, (*rn)[8] = NULL;
    int *rid = NULL;
    /* grid of placed atoms for overlap rejection (4 A cells); atoms of different
       chains stay 4 A apart, or 3.3 A in a cylinder (above every hard-core
       distance of the model's pair tables for peptide atoms, 3.28 A), where the density needs it */
    const double G = 4.0, clear2 = wall == SDMD_WALL_CYLINDER ? 3.3 * 3.3 : 16.0;
    /* the box the chains are placed in: the target box, or for a dense cylinder a
       longer one that the compression below brings to the target length */
    double bx[3] = {box[0], box[1], box[2]};
    int gn[3];
    int *head = NULL, *next = NULL;
    /* chains are independent: relax them on all host threads, then place them in order */
    /* residue templates, learned serially from short context chains with a fixed seed */
    templcache *shared = calloc(1, sizeof(templcache));
    {
        static const char *aa20[] = {"ALA", "ARG", "ASN", "ASP", "CYS", "GLN", "GLU", "GLY", "HIS", "ILE", "LEU", "LYS",
                                     "MET", "PHE", "PRO", "SER", "THR", "TRP", "TYR", "VAL"};
        for (int q = 0; q < 20; q++) {
            char ctx[64];
            snprintf(ctx, sizeof ctx, "%s ALA %s ALA", aa20[q], aa20[q]);
            xrng r0 = {0x2545F4914F6CDD1DULL + (uint64_t)q};
            int n = 0; double *xyz = NULL; char (*nm)[8] = NULL, (*rs)[8] = NULL; int *ri = NULL;
            char e2[256];
            if (!make_chain(datadir, ff, ctx, &r0, shared, 1, &n, &xyz, &nm, &rs, &ri, e2, sizeof e2)) {
                free(xyz); free(nm); free(rs); free(ri);
            }
        }
    }
    genjob J;
    memset(&J, 0, sizeof J);
    J.datadir = datadir; J.ff = ff; J.seq = sequences; J.n_chains = n_chains; J.seed = seed; J.shared = shared;
    pthread_mutex_init(&J.mu, NULL);
    J.n = calloc((size_t)n_chains, sizeof(int)); J.xyz = calloc((size_t)n_chains, sizeof(double *));
    J.nm = calloc((size_t)n_chains, sizeof(*J.nm)); J.rs = calloc((size_t)n_chains, sizeof(*J.rs));
    J.ri = calloc((size_t)n_chains, sizeof(int *));
    int nthr = 1;
    {
        const char *e = getenv("SDMD_GEN_THREADS");
        long ncpu = e ? atol(e) : 16;
        nthr = (int)(ncpu < 1 ? 1 : ncpu > 64 ? 64 : ncpu);
        if (nthr > n_chains) nthr = n_chains;
    }
    pthread_t th[64];
    for (int q = 0; q < nthr; q++) pthread_create(&th[q], NULL, gen_worker, &J);
    for (int q = 0; q < nthr; q++) pthread_join(th[q], NULL);
    pthread_mutex_destroy(&J.mu);
    free(shared);
    if (wall == SDMD_WALL_CYLINDER && !J.failed) {
        /* Overlap-free insertion of rigid chains stalls near 70 A^3 per atom in the
           cylinder; above 110 A^3 per atom it succeeds quickly.  Denser targets are
           placed in a cylinder stretched to that density and compressed. */
        long atoms = 0;
        for (int c = 0; c < n_chains; c++) atoms += J.n[c];
        const double ra = box[1] / 2 - margin, vol = M_PI * ra * ra * box[0];
        const double stretch = 110.0 * (double)atoms / vol;
        if (stretch > 1) bx[0] = box[0] * stretch;
    }
    for (int d = 0; d < 3; d++) gn[d] = (int)(bx[d] / G) + 1;
    long ng = (long)gn[0] * gn[1] * gn[2];
    head = malloc(sizeof(int) * ng);
    for (long q = 0; q < ng; q++) head[q] = -1;
    for (int c = 0; c < n_chains; c++) {
        int n = J.n[c]; double *xyz = J.xyz[c]; char (*nm)[8] = J.nm[c], (*rs)[8] = J.rs[c]; int *ri = J.ri[c];
        if (J.failed) {
            for (int q = 0; q < n_chains; q++) { free(J.xyz[q]); free(J.nm[q]); free(J.rs[q]); free(J.ri[q]); }
            free(J.n); free(J.xyz); free(J.nm); free(J.rs); free(J.ri);
            free(head); free(all); free(an); free(rn); free(rid); free(next); free(out.s);
            snprintf(err, (size_t)errlen, "%s", J.err);
            return SDMD_EINVAL;
        }
        /* centre */
        double cm[3] = {0, 0, 0};
        for (int i = 1; i <= n; i++) for (int d = 0; d < 3; d++) cm[d] += xyz[3 * i + d] / n;
        for (int i = 1; i <= n; i++) for (int d = 0; d < 3; d++) xyz[3 * i + d] -= cm[d];
        int ok = 0;
        double *tr = malloc(sizeof(double) * 3 * (n + 1));
        /* inside a cylinder the chains lie along its (periodic) x axis: their longest
           extent (the principal axis of their positions) is turned onto x first, and
           each attempt turns them about x by a random angle */
        double A[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
        if (wall == SDMD_WALL_CYLINDER) {
            double Cv[9] = {0};
            for (int i = 1; i <= n; i++)
                for (int a = 0; a < 3; a++)
                    for (int b = 0; b < 3; b++) Cv[3 * a + b] += xyz[3 * i + a] * xyz[3 * i + b];
            double e[3] = {1, 0.5, 0.25};
            for (int it = 0; it < 200; it++) {   /* power iteration: the largest-variance direction */
                double f[3];
                for (int a = 0; a < 3; a++) f[a] = Cv[3 * a] * e[0] + Cv[3 * a + 1] * e[1] + Cv[3 * a + 2] * e[2];
                double nf = sqrt(f[0] * f[0] + f[1] * f[1] + f[2] * f[2]);
                if (!(nf > 0)) break;
                for (int a = 0; a < 3; a++) e[a] = f[a] / nf;
            }
            /* rows of A: e, and two unit vectors orthogonal to it */
            double u[3] = {fabs(e[0]) < 0.9 ? 1.0 : 0.0, fabs(e[0]) < 0.9 ? 0.0 : 1.0, 0.0};
            double w[3] = {e[1] * u[2] - e[2] * u[1], e[2] * u[0] - e[0] * u[2], e[0] * u[1] - e[1] * u[0]};
            double nw = sqrt(w[0] * w[0] + w[1] * w[1] + w[2] * w[2]);
            for (int a = 0; a < 3; a++) w[a] /= nw;
            double v[3] = {w[1] * e[2] - w[2] * e[1], w[2] * e[0] - w[0] * e[2], w[0] * e[1] - w[1] * e[0]};
            for (int a = 0; a < 3; a++) { A[a] = e[a]; A[3 + a] = v[a]; A[6 + a] = w[a]; }
        }
        for (int attempt = 0; attempt < 20000 && !ok; attempt++) {
            double R[9];
            double t[3] = {xr_u(&rng) * bx[0], xr_u(&rng) * bx[1], xr_u(&rng) * bx[2]};
            if (wall == SDMD_WALL_CYLINDER) {   /* R = (turn about x by phi) * A */
                const double ph = 2 * M_PI * xr_u(&rng), c = cos(ph), sn = sin(ph);
                const double Rx[9] = {1, 0, 0, 0, c, -sn, 0, sn, c};
                for (int a = 0; a < 3; a++)
                    for (int b = 0; b < 3; b++)
                        R[3 * a + b] = Rx[3 * a] * A[b] + Rx[3 * a + 1] * A[3 + b] + Rx[3 * a + 2] * A[6 + b];
                /* the centre within the cylinder's cross-section, uniform over the disc */
                const double rr = (bx[1] / 2 - margin) * sqrt(xr_u(&rng)), th = 2 * M_PI * xr_u(&rng);
                t[1] = bx[1] / 2 + rr * cos(th);
                t[2] = bx[2] / 2 + rr * sin(th);
            } else {   /* uniform rotation from a random unit quaternion */
                double u1 = xr_u(&rng), u2 = xr_u(&rng), u3 = xr_u(&rng);
                double qa = sqrt(1 - u1) * sin(2 * M_PI * u2), qb = sqrt(1 - u1) * cos(2 * M_PI * u2);
                double qc = sqrt(u1) * sin(2 * M_PI * u3), qd = sqrt(u1) * cos(2 * M_PI * u3);
                const double Q[9] = {1 - 2 * (qc * qc + qd * qd), 2 * (qb * qc - qa * qd), 2 * (qb * qd + qa * qc),
                                     2 * (qb * qc + qa * qd), 1 - 2 * (qb * qb + qd * qd), 2 * (qc * qd - qa * qb),
                                     2 * (qb * qd - qa * qc), 2 * (qc * qd + qa * qb), 1 - 2 * (qb * qb + qc * qc)};
                memcpy(R, Q, sizeof R);
            }
            ok = 1;
            for (int i = 1; i <= n && ok; i++) {
                const double *p = xyz + 3 * i;
                for (int d = 0; d < 3; d++) tr[3 * i + d] = R[3 * d] * p[0] + R[3 * d + 1] * p[1] + R[3 * d + 2] * p[2] + t[d];
                double *q = tr + 3 * i;
                if (wall == SDMD_WALL_CYLINDER) {
                    double ry = q[1] - bx[1] / 2, rz = q[2] - bx[2] / 2;
                    if (sqrt(ry * ry + rz * rz) > bx[1] / 2 - margin) { ok = 0; break; }
                    q[0] = fmod(q[0], bx[0]);   /* the axis is periodic */
                    if (q[0] < 0) q[0] += bx[0];
                } else {
                    /* periodic box: the build wraps every atom once (PBC "full"), so stay
                       within one box length of the primary cell */
                    for (int d = 0; d < 3; d++) if (q[d] < -bx[d] || q[d] >= 2 * bx[d]) ok = 0;
                }
                if (!ok) break;
                int gc[3];
                for (int d = 0; d < 3; d++) {
                    double w = fmod(q[d], bx[d]); if (w < 0) w += bx[d];
                    gc[d] = (int)(w / G); if (gc[d] >= gn[d]) gc[d] = gn[d] - 1; if (gc[d] < 0) gc[d] = 0;
                }
                for (int dz = -1; dz <= 1 && ok; dz++) for (int dy = -1; dy <= 1 && ok; dy++) for (int dx = -1; dx <= 1 && ok; dx++) {
                    int x = gc[0] + dx, y = gc[1] + dy, z = gc[2] + dz;
                    if (x < 0 || y < 0 || z < 0 || x >= gn[0] || y >= gn[1] || z >= gn[2]) continue;
                    for (int a = head[((long)z * gn[1] + y) * gn[0] + x]; a >= 0; a = next[a]) {
                        double dd = 0;
                        for (int d = 0; d < 3; d++) {   /* minimum image */
                            double v = q[d] - all[3 * a + d];
                            v -= bx[d] * floor(v / bx[d] + 0.5);
                            dd += v * v;
                        }
                        if (dd < clear2) { ok = 0; break; }
                    }
                }
            }
        }
        if (!ok) {
            for (int q = c; q < n_chains; q++) { free(J.xyz[q]); free(J.nm[q]); free(J.rs[q]); free(J.ri[q]); }
            free(J.n); free(J.xyz); free(J.nm); free(J.rs); free(J.ri);
            free(tr); free(head); free(all); free(an); free(rn); free(rid); free(next); free(out.s);
            snprintf(err, (size_t)errlen, "could not place chain %d without overlap", c);
            return SDMD_EINVAL;
        }
        if (nall + n + 1 > capall) {
            capall = 2 * (nall + n + 1);
            all = realloc(all, sizeof(double) * 3 * capall); next = realloc(next, sizeof(int) * capall);
            an = realloc(an, 8 * (size_t)capall); rn = realloc(rn, 8 * (size_t)capall); rid = realloc(rid, sizeof(int) * capall);
        }
        for (int i = 1; i <= n; i++) {
            int a = nall++;
            memcpy(all + 3 * a, tr + 3 * i, sizeof(double) * 3);
            memcpy(an[a], nm[i], 8); memcpy(rn[a], rs[i], 8);
            rid[a] = ri[i];   /* residue numbers restart at 1 in every chain */
            const double *q = all + 3 * a;
            int gc[3];
            for (int d = 0; d < 3; d++) {
                double w = fmod(q[d], bx[d]); if (w < 0) w += bx[d];
                gc[d] = (int)(w / G); if (gc[d] >= gn[d]) gc[d] = gn[d] - 1; if (gc[d] < 0) gc[d] = 0;
            }
            long cell = ((long)gc[2] * gn[1] + gc[1]) * gn[0] + gc[0];
            next[a] = head[cell]; head[cell] = a;
        }
        total += n;
        free(tr); free(xyz); free(nm); free(rs); free(ri);
    }
    free(J.n); free(J.xyz); free(J.nm); free(J.rs); free(J.ri);
    free(head); free(next);
    /* residue numbers restart at 1 for every chain: the reader starts a new
       protein when the residue number decreases (src/Initialization.c:946) */
    for (int pass = 0; pass < 2; pass++) {
        const double *bb = pass == 0 ? bx : box;
        sb_printf(&out, "generated peptides\n%d\n", total);
        for (int a = 0; a < nall; a++) {
            sb_printf(&out, "%5d%-5s%5s%5d%10.5f%10.5f%10.5f\n", rid[a] % 100000, rn[a], an[a], (a + 1) % 100000,
                      all[3 * a] / 10, all[3 * a + 1] / 10, all[3 * a + 2] / 10);
        }
        sb_printf(&out, "%10.5f%10.5f%10.5f\n", bb[0] / 10, bb[1] / 10, bb[2] / 10);
        if (pass == 1 || bx[0] <= box[0]) break;
        /* the stretched placement, read back with the model's bounds, compressed to
           the target length, and written again */
        B b;
        memset(&b, 0, sizeof b);
        sdmd_params p;
        memset(&p, 0, sizeof p);
        snprintf(p.continue_mode, 20, "new"); snprintf(p.force_field, 20, "%s", ff);
        b.p = &p; b.err = err; b.errlen = errlen;
        snprintf(b.datadir, sizeof b.datadir, "%s", datadir);
        snprintf(b.ff, sizeof b.ff, "%s", ff);
        cur c;
        cur_text(out.s, &c);
        int r = read_gro(&b, &c);
        free(c.buf);
        if (!r) r = read_model(&b);
        if (!r) r = read_tables(&b);
        if (!r && b.n != nall) r = fail(&b, "generated system has %d atoms, expected %d", b.n, nall);
        if (!r) r = compress_cylinder(&b, bx[0], box[0], box[1], margin);
        if (!r) for (int a = 0; a < nall; a++) memcpy(all + 3 * a, b.atom[a + 1].pos, sizeof(double) * 3);
        free_builder(&b);
        out.n = 0;
        if (r) {
            free(all); free(an); free(rn); free(rid); free(out.s);
            return r;
        }
    }
    free(all); free(an); free(rn); free(rid);
    *gro_out = out.s;
    return SDMD_OK;
}

void sdmd_free_text(char *p) { free(p); }
