/*
 * sdmd_oracle.c -- CPU restatement of the reference sDMD event loop.
 *
 * TEST INFRASTRUCTURE ONLY (see sdmd_oracle.h): tests/, smoke() and bench.py's
 * cpu_baseline leg use it as the checker; the product never links it.
 *
 * Each function names the reference function and file:line it restates.  The
 * floating-point expressions keep the reference's association order, and the
 * file must be compiled with -ffp-contract=off so no multiply-add is fused.
 */
#include "sdmd_oracle.h"

#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define NT SDMD_NTYPES
#define ZERO SDMD_ZERO
#define INFINIT SDMD_INFINIT
#define INVALID SDMD_INVALID

/* 27-cell scan order: the reference's atomList.x/y/z (src/DMD.c:117-121). */
static const int NBX[27] = {0, 1, 0, 0, 0, 1, 1, 1, -1, 0, 0, 0, -1, -1, -1, 0, 0, 1, -1, 1, -1, -1, -1, 1, 1, 1, -1};
static const int NBY[27] = {0, 0, 1, 0, 1, 0, 1, 1, 0, -1, 0, -1, 0, -1, -1, -1, 1, 0, 0, -1, 1, -1, 1, -1, 1, -1, 1};
static const int NBZ[27] = {0, 0, 0, 1, 1, 1, 0, 1, 0, 0, -1, -1, -1, 0, -1, 1, -1, -1, 1, 0, 0, 1, -1, -1, -1, 1, 1};

enum { K_COLLISION, K_CONSTRAINT, K_HB, K_NEIGHBOR };

typedef struct {
    int err;
    int err_atom;
} ostat;

static ostat G;   /* error latch of the current call (single-threaded checker) */

static void fail(int code, int atom) {
    if (!G.err) { G.err = code; G.err_atom = atom; }
}

/* ------------------------------------------------------------------------- */
/* glibc rand(): additive feedback generator r[i] = r[i-3] + r[i-31] (mod 2^32), */
/* output r >> 1 (degree 31, separation 3).                                     */
int32_t oracle_rand(sdmd_rng *r) {
    uint32_t v = (uint32_t)r->tab[r->front] + (uint32_t)r->tab[r->rear];
    r->tab[r->front] = (int32_t)v;
    int32_t out = (int32_t)((v >> 1) & 0x7fffffff);
    if (++r->front >= 31) { r->front = 0; ++r->rear; }
    else if (++r->rear >= 31) r->rear = 0;
    return out;
}

/* RandomValue(0, 1) = 0 + (double)rand() / ((double)RAND_MAX / 1)  (src/ToolFunctions.c:517-522) */
static double rv01(sdmd_rng *r) {
    return 0 + (double)oracle_rand(r) / ((double)2147483647 / (1 - 0));
}

/* ---- correctly rounded natural log (double-double evaluation) -------------- */
/* log(x) = e*ln2 + 2*atanh(f), f = (m-1)/(m+1), m in [sqrt(1/2), sqrt(2)).     */
/* Every step is an exact error-free transform or a double-double operation      */
/* accurate to ~2^-104, so rounding the result to double is correct except when  */
/* the exact logarithm lies within ~2^-100 relative of a rounding midpoint.      */
typedef struct { double hi, lo; } dd;

static dd two_sum(double a, double b) {
    dd r; double s = a + b; double bb = s - a;
    r.hi = s; r.lo = (a - (s - bb)) + (b - bb); return r;
}
static dd quick_two_sum(double a, double b) {
    dd r; double s = a + b; r.hi = s; r.lo = b - (s - a); return r;
}
static void split(double a, double *hi, double *lo) {
    double t = 134217729.0 * a;   /* 2^27 + 1 */
    *hi = t - (t - a); *lo = a - *hi;
}
static dd two_prod(double a, double b) {
    double ah, al, bh, bl; dd r;
    r.hi = a * b;
    split(a, &ah, &al); split(b, &bh, &bl);
    r.lo = ((ah * bh - r.hi) + ah * bl + al * bh) + al * bl;
    return r;
}
static dd dd_add(dd a, dd b) {
    dd s = two_sum(a.hi, b.hi), t = two_sum(a.lo, b.lo);
    s.lo += t.hi; s = quick_two_sum(s.hi, s.lo); s.lo += t.lo; return quick_two_sum(s.hi, s.lo);
}
static dd dd_mul(dd a, dd b) {
    dd p = two_prod(a.hi, b.hi);
    p.lo += a.hi * b.lo + a.lo * b.hi;
    return quick_two_sum(p.hi, p.lo);
}
static dd dd_div_d(double n, dd d) {   /* n / d */
    double q1 = n / d.hi;
    dd p = dd_mul((dd){q1, 0.0}, d);
    dd r = dd_add((dd){n, 0.0}, (dd){-p.hi, -p.lo});
    double q2 = r.hi / d.hi;
    return quick_two_sum(q1, q2);
}
/* 1/(2k+1) as double-double, k = 0..21 */
static dd inv_odd(int k) {
    double n = (double)(2 * k + 1);
    double h = 1.0 / n;
    dd p = two_prod(h, n);                 /* h*n exactly */
    double rem = (1.0 - p.hi) - p.lo;      /* exact */
    return quick_two_sum(h, rem / n);
}

double oracle_log(double x) {
    if (!(x > 0)) return x == 0 ? -HUGE_VAL : NAN;
    if (isinf(x)) return x;
    int e;
    double m = frexp(x, &e);            /* x = m * 2^e, m in [0.5, 1) */
    m *= 2.0; e -= 1;                   /* m in [1, 2) */
    if (m > 1.4142135623730951) { m *= 0.5; e += 1; }
    double num = m - 1.0;               /* exact */
    dd den = two_sum(m, 1.0);
    dd f = dd_div_d(num, den);
    dd z = dd_mul(f, f);
    /* tail k = 21..11 in double, head k = 10..0 in double-double (Horner) */
    double t = 1.0 / 43.0;
    for (int k = 20; k >= 11; k--) t = t * z.hi + 1.0 / (double)(2 * k + 1);
    dd acc = {t, 0.0};
    for (int k = 10; k >= 0; k--) acc = dd_add(dd_mul(acc, z), inv_odd(k));
    dd lm = dd_mul(f, acc);
    lm.hi *= 2.0; lm.lo *= 2.0;
    const dd LN2 = {0x1.62e42fefa39efp-1, 0x1.abc9e3b39803fp-56};
    dd el = dd_add(two_prod((double)e, LN2.hi), (dd){(double)e * LN2.lo, 0.0});
    dd r = dd_add(el, lm);
    return r.hi + r.lo;
}

/* Maxwell_Boltzmann_Distribution (src/ToolFunctions.c:544-569): polar Box-Muller
 * with rejection, then a coin flip picks one of the two normals. */
double oracle_mb(sdmd_rng *r, double mean, double variance) {
    double a, b, s, out;
    for (;;) {
        do {
            a = 2 * rv01(r) - 1;
            b = 2 * rv01(r) - 1;
            s = a * a + b * b;
        } while (s >= 1);
        s = sqrt(-2 * oracle_log(s) / s);
        double choose = rv01(r);
        out = (choose >= 0.5) ? a * s : b * s;
        if (out != 0) break;
    }
    return out * sqrt(variance) + mean;
}

/* ------------------------------------------------------------------------- */
static inline int cell_lin(const sdmd_system *s, int cx, int cy, int cz) {
    return cz * s->cellnum[0] * s->cellnum[1] + cy * s->cellnum[0] + cx + 1;
}

/* head of neighbour cell k of atom i (wrap of src/TimePrediction.c:62-75) */
static int nb_head(const sdmd_system *s, int i, int k) {
    int c[3] = {s->cx[i] + NBX[k], s->cy[i] + NBY[k], s->cz[i] + NBZ[k]};
    for (int d = 0; d < 3; d++) {
        if (c[d] < 0) c[d] = s->cellnum[d] - 1;
        else if (c[d] >= s->cellnum[d]) c[d] = 0;
    }
    return s->cell_list[s->n_atoms + cell_lin(s, c[0], c[1], c[2])];
}

/* AtomTypeChange (src/ToolFunctions.c:233-270) */
static int type_change(int t, int to_hb) {
    if (to_hb) { if (t == 1) return 3; if (t == 2) return 4; if (t == 26) return 27; }
    else { if (t == 3) return 1; if (t == 4) return 2; if (t == 27) return 26; }
    return t;
}

static inline int tab_idx(int t, int a, int b) { return (t * NT + a) * NT + b; }

/* RightPair (src/ToolFunctions.c:278-292): collision table entry, falling back to
 * the pre-HB types.  Returns -1 when none has dmin > 0. */
static int right_pair(const sdmd_system *s, int t1, int t2, int nofallback) {
    if (s->pair_dmin[tab_idx(0, t1, t2)] > 0) return tab_idx(0, t1, t2);
    if (nofallback) return -1;
    int r;
    if ((r = right_pair(s, type_change(t1, 0), t2, 1)) >= 0) return r;
    if ((r = right_pair(s, t1, type_change(t2, 0), 1)) >= 0) return r;
    return right_pair(s, type_change(t1, 0), type_change(t2, 0), 1);
}

/* HBModel (src/Models.c:212-290): HB class 1..11, -1 for "no HB", 0 = fatal. */
static int hb_model(const sdmd_system *s, int a1, int a2) {
    if (s->hb_role[a1] == 'A' || s->hb_role[a1] == 'S') { int t = a1; a1 = a2; a2 = t; }
    int t1 = type_change(s->type[a1], 0), t2 = type_change(s->type[a2], 0);
    int aa2 = s->aatype[a2];
    if (t1 == 2 && t2 == 26) return 1;
    if (t1 == 2) {
        switch (aa2) {
            case 4: case 7: return 2;
            case 16: case 17: case 19: return 3;
            case 9: return 4;
            case 5: return 10;
            case 3: case 6: return -1;
            default: break;
        }
    } else if (t2 == 26) {
        return 5;
    } else if (t1 == 31 && t2 == 31) {
        return 9;
    } else if (t1 == 1) {
        switch (aa2) {
            case 4: case 7: return 6;
            case 16: case 17: case 19: return 7;
            case 9: return 8;
            case 3: case 6: return 11;
            default: break;
        }
    }
    fail(SDMD_EHBMAP, a1);
    return 0;
}

/* HBBarrier (src/Events.c:1097-1119) */
static double hb_barrier(const sdmd_system *s, int a1, int a2) {
    if (s->hb_role[a1] == 'A' || s->hb_role[a1] == 'S') { int t = a1; a1 = a2; a2 = t; }
    int t1 = type_change(s->type[a1], 0), t2 = type_change(s->type[a2], 0);
    if (t1 == 2 && t2 == 26) return s->hb_barrier[0];
    if (t1 != 2 && t2 != 26) return s->hb_barrier[2];
    return s->hb_barrier[1];
}

static int conn_bits(const sdmd_system *s, int i, int j) {
    for (int k = s->conn_off[i]; k < s->conn_off[i + 1]; k++)
        if (s->conn_j[k] == j) return s->conn_bits[k];
    return 0;
}

/* FindElemInList(neighborPartner, j, -1, -1, 0) (src/ToolFunctions.c:1062-1087):
 * 1-based scan of the zero-terminated list (at most 4 entries held). */
static int nb_has(const sdmd_system *s, int i, int j) {
    for (int k = 0; k < 4; k++) {
        int v = s->nb_partner[4 * i + k];
        if (v == 0) return 0;
        if (v == j) return k + 1;
    }
    return 0;
}

/* FindPair (src/ToolFunctions.c:39-224).  `a1`/`a2` are atom ids; for a wall pair
 * a2 is 0 and wall_type2 is its type.  Returns coreorShell (-1, 0, 1). */
typedef struct { double lo, up, lopot, uppot, acc; } pairlim;

static int find_pair(sdmd_system *s, int a1, int a2, int kind, double direction, double distance2,
                     pairlim *o, int hbpartner, int type_change_dir, int wall_type2) {
    int cs = -1;
    double dir = direction < 0 ? 1 : -1;
    double tol = dir * ZERO;
    double dmin, dmax;
    const double *sd, *se, *sa;
    int sn;
    if (kind == K_CONSTRAINT) {
        int k;
        for (k = s->con_off[a1]; k < s->con_off[a1 + 1]; k++) if (s->con_j[k] == a2) break;
        if (k == s->con_off[a1 + 1]) { fail(SDMD_EUNSUPPORTED, a1); return -1; }
        dmin = s->con_dmin[k]; dmax = s->con_dmax[k]; sn = s->con_step_n[k];
        sd = s->con_step_d + s->con_step_off[k]; se = s->con_step_e + s->con_step_off[k];
        sa = s->con_step_acc + s->con_step_off[k];
    } else {
        int e;
        if (kind == K_COLLISION) {
            int t1 = s->type[a1];
            if (type_change_dir == 1) t1 = type_change(t1, 1);
            else if (type_change_dir == -1) t1 = type_change(t1, 0);
            int t2 = a2 ? s->type[a2] : wall_type2;
            e = right_pair(s, t1, t2, 0);
            if (e < 0) { fail(SDMD_EUNSUPPORTED, a1); return -1; }   /* NULL entry in the reference */
        } else if (kind == K_HB) {
            e = tab_idx(hb_model(s, a1, a2), 0, 0);
        } else {   /* K_NEIGHBOR */
            int tn = hb_model(s, a2, hbpartner);
            e = tab_idx(tn, type_change(s->type[a1], 0), type_change(s->type[a2], 0));
        }
        dmin = s->pair_dmin[e]; dmax = s->pair_dmax[e]; sn = s->pair_step_n[e];
        sd = s->pair_step_d + s->pair_step_off[e]; se = s->pair_step_e + s->pair_step_off[e];
        sa = s->pair_step_acc + s->pair_step_off[e];
    }
    int flag = (sn == 0);
    if (dmin == 0) { fail(SDMD_EUNSUPPORTED, a1); return -1; }
    int a1bond = a1 ? s->hb_bond[a1] : 0, a2bond = a2 ? s->hb_bond[a2] : 0;
    int warn = !(kind == K_NEIGHBOR && a2bond == 0) && !(kind == K_HB && a1bond == 0);
    if (distance2 < dmin - ZERO) {
        o->lo = INFINIT; o->up = INFINIT; o->acc = INFINIT; o->lopot = 0; o->uppot = 0;
        if (warn) s->counters.warnings++;
        return cs;
    }
    o->lo = dmin; o->lopot = 0;
    for (int q = 0; q < sn && sd[q] != 0; q++) {
        if (distance2 < sd[q] + tol) {
            o->up = sd[q]; o->uppot = -1 * se[q]; o->acc = sa[q];
            if (q == 0) return 0;
            if (kind == K_HB && q == sn - 1 && a1bond > 0) return 1;
            if (kind == K_NEIGHBOR && q == sn - 1 && a2bond > 0) { o->uppot = 0; return 1; }
            return cs;
        }
        o->lo = sd[q]; o->lopot = se[q];
    }
    if (kind == K_HB && a1bond > 0) s->counters.warnings++;
    if (dmax > 0) {
        if (distance2 < dmax + ZERO) {
            o->up = dmax; o->uppot = 0; o->acc = 0;
            cs = 1;
            if (flag == 1 && dir == 1) cs = 0;
            return cs;
        }
        o->lo = INFINIT; o->up = INFINIT; o->acc = INFINIT; o->lopot = 0; o->uppot = 0;
        if (warn) s->counters.warnings++;
    } else {
        o->up = INFINIT; o->uppot = INFINIT; o->acc = INFINIT;
        return 1;
    }
    return cs;
}

/* ---- pair kinematics: PBCShift + CalculateParameters ----------------------- */
/* (src/ToolFunctions.c:801-817, src/TimePrediction.c:1081-1090)                 */
typedef struct { double r2, b, v2; double rx, ry, rz; } kin;

static void pair_kin(const sdmd_system *s, int i, int j, kin *k) {
    const int ci[3] = {s->cx[i], s->cy[i], s->cz[i]}, cj[3] = {s->cx[j], s->cy[j], s->cz[j]};
    double sh[3];
    for (int d = 0; d < 3; d++) {
        sh[d] = 0;
        if (ci[d] != cj[d]) {
            if (ci[d] == 0 && cj[d] == s->cellnum[d] - 1) sh[d] = -1 * s->box[d];
            else if (ci[d] == s->cellnum[d] - 1 && cj[d] == 0) sh[d] = s->box[d];
        }
    }
    double rx = s->x[i] - (s->x[j] + sh[0]);
    double ry = s->y[i] - (s->y[j] + sh[1]);
    double rz = s->z[i] - (s->z[j] + sh[2]);
    double vx = s->vx[i] - s->vx[j], vy = s->vy[i] - s->vy[j], vz = s->vz[i] - s->vz[j];
    k->rx = rx; k->ry = ry; k->rz = rz;
    k->r2 = rx * rx + ry * ry + rz * rz;
    k->b = rx * vx + ry * vy + rz * vz;
    k->v2 = vx * vx + vy * vy + vz * vz;
}

/* CalculateDisc / CalculateTime (src/TimePrediction.c:1092-1099) */
static inline double disc(const kin *k, double shortlim) { return k->b * k->b - k->v2 * (k->r2 - shortlim); }
static inline double root(const kin *k, int stime, double d2) {
    return (-1 * k->b + stime * sqrt(k->b * k->b - k->v2 * (k->r2 - d2))) / k->v2;
}

/* ---- running minimum: JobAssign / CheckDuplication -------------------------- */
/* (src/TimePrediction.c:1140-1158, 1101-1117)                                   */
typedef struct { double time, potential; int sub; } cand;

static int job_assign(sdmd_system *s, int i, int j, const cand *c, int type) {
    if (c->time > 0 && s->ev_time[i] > c->time) {
        s->ev_potential[i] = c->potential;
        s->ev_sub[i] = c->sub;
        s->ev_time[i] = c->time;
        s->ev_type[i] = type;
        if (j) { s->ev_partner[i] = j; s->ev_pcounter[i] = s->ev_counter[j]; }
        else s->ev_partner[i] = INVALID;
        return 1;
    }
    return 0;
}

static int check_dup(sdmd_system *s, int i, int j, int type) {
    if (s->ev_partner[j] == i && s->ev_type[j] == type && s->ev_pcounter[j] == s->ev_counter[i] &&
        s->ev_time[i] > s->ev_time[j]) {
        s->ev_partner[i] = j;
        s->ev_potential[i] = s->ev_potential[j];
        s->ev_sub[i] = s->ev_sub[j];
        s->ev_time[i] = s->ev_time[j];
        s->ev_type[i] = type;
        s->ev_pcounter[i] = s->ev_counter[j];
        return 1;
    }
    return 0;
}

/* ---- prediction ------------------------------------------------------------ */
/* BondTime (src/TimePrediction.c:186-295) */
static void bond_time(sdmd_system *s, int i) {
    cand c = {INFINIT, 0, SDMD_SUB_INVALID};
    for (int q = s->bond_off[i]; q < s->bond_off[i + 1]; q++) {
        int j = s->bond_j[q];
        if (check_dup(s, i, j, SDMD_EV_BOND)) continue;
        double lng = s->bond_dmax[q], sht = s->bond_dmin[q];
        kin k; pair_kin(s, i, j, &k);
        if (k.r2 - lng > ZERO) {
            if (k.b >= 0) {
                c.sub = SDMD_SUB_WELL_BOUNCE; c.time = 1e-16 * i * j;
                job_assign(s, i, j, &c, SDMD_EV_BOND);
                continue;
            }
        } else if (sht - k.r2 > ZERO) {
            if (k.b < 0) {
                c.sub = SDMD_SUB_CORE; c.time = 1e-16 * i * j;
                job_assign(s, i, j, &c, SDMD_EV_BOND);
                continue;
            }
        }
        int st; double d2;
        if (k.b < 0 && disc(&k, sht) > 0) { st = -1; d2 = sht; c.sub = SDMD_SUB_CORE; }
        else { st = 1; d2 = lng; c.sub = SDMD_SUB_WELL_BOUNCE; }
        c.time = root(&k, st, d2);
        if (c.time < 0) c.time = INFINIT;
        job_assign(s, i, j, &c, SDMD_EV_BOND);
    }
}

/* CollisionTime (src/TimePrediction.c:44-183) */
static void collision_time(sdmd_system *s, int i) {
    cand c = {INFINIT, 0, SDMD_SUB_INVALID};
    double cut = s->cutoff * 0.90; cut *= cut;
    for (int kc = 0; kc < 27; kc++) {
        for (int j = nb_head(s, i, kc); j; j = s->cell_list[j]) {
            if (i == j) continue;
            if (check_dup(s, i, j, SDMD_EV_COLLISION)) continue;
            int bits = conn_bits(s, i, j);
            if ((bits & 1) || s->hb_bond[i] == j || nb_has(s, i, j)) continue;
            kin k; pair_kin(s, i, j, &k);
            if (!(k.r2 <= cut)) continue;
            pairlim L; int cs;
            int constrained = bits & 2;
            if (constrained) {
                cs = find_pair(s, i, j, K_CONSTRAINT, k.b, k.r2, &L, 0, 0, 0);
            } else {
                cs = find_pair(s, i, j, K_COLLISION, k.b, k.r2, &L, 0, 0, 0);
                if (L.lopot == 0 && L.uppot == 0) continue;
            }
            int st; double d2;
            if (k.b < 0 && disc(&k, L.lo) > 0) {
                st = -1; d2 = L.lo; c.potential = L.lopot;
                c.sub = (cs == 0) ? SDMD_SUB_CORE : SDMD_SUB_TBD_CAPTURE;
            } else {
                st = 1; d2 = L.up; c.potential = L.uppot;
                if (constrained) c.sub = (cs == 1) ? SDMD_SUB_WELL_BOUNCE : SDMD_SUB_TBD_ESCAPE;
                else {
                    if (cs == 1) continue;
                    c.sub = SDMD_SUB_TBD_ESCAPE;
                }
            }
            c.time = root(&k, st, d2);
            job_assign(s, i, j, &c, SDMD_EV_COLLISION);
        }
    }
}

/* PBCandCrossCellTime (src/TimePrediction.c:598-632) */
static void pcc_time(sdmd_system *s, int i) {
    cand c = {INFINIT, 0, SDMD_SUB_INVALID};
    const double pos[3] = {s->x[i], s->y[i], s->z[i]}, v[3] = {s->vx[i], s->vy[i], s->vz[i]};
    const int ci[3] = {s->cx[i], s->cy[i], s->cz[i]};
    for (int d = 0; d < 3; d++) {
        double lo = ci[d] * s->cellsize[d], hi = (ci[d] + 1) * s->cellsize[d], t;
        if (v[d] > 0) {
            t = (hi - pos[d] + ZERO) / v[d];
            if (c.time > t && t > 0) c.time = t;
        } else if (v[d] < 0) {
            t = (lo - pos[d] - ZERO) / v[d];
            if (c.time > t && t > 0) c.time = t;
        }
    }
    job_assign(s, i, 0, &c, SDMD_EV_PCC);
}

/* ThermostatTime (src/TimePrediction.c:582-595) */
static void thermostat_time(sdmd_system *s, int i) {
    if (!s->thermostat) return;
    cand c = {INFINIT, 0, SDMD_SUB_INVALID};
    double t = oracle_mb(&s->rng, 0, 1);
    c.time = s->thermo_freq * (t < 0 ? -t : t);
    job_assign(s, i, 0, &c, SDMD_EV_THERMOSTAT);
}

/* CheckPairMatch (src/TimePrediction.c:1119-1138) */
static int pair_match(sdmd_system *s, int i, int j) {
    int t = hb_model(s, i, j);
    if (t < 0) return -1;
    int ti = s->type[i], tj = s->type[j];
    if (s->pair_step_n[tab_idx(t, ti, tj)] == 0) return -1;
    int ni = type_change(s->type[s->hb_neighbor[i]], 0), nj = type_change(s->type[s->hb_neighbor[j]], 0);
    if (s->pair_step_n[tab_idx(t, ti, nj)] == 0 || s->pair_step_n[tab_idx(t, tj, ni)] == 0) return -1;
    return 0;
}

static inline int hb_pair_ok(const sdmd_system *s, int i, int j) {
    int ri = s->hb_role[i], rj = s->hb_role[j];
    return (ri == 'A' && rj == 'D') || (ri == 'D' && rj == 'A') ||
           (ri == 'S' && s->type[j] == 2) || (rj == 'S' && s->type[i] == 2) ||
           (ri == 'S' && rj == 'S');
}

/* HBTime (src/TimePrediction.c:298-483) */
static void hb_time(sdmd_system *s, int i) {
    cand c = {INFINIT, 0, SDMD_SUB_INVALID};
    if (s->hb_itype[i] == SDMD_HB_SKIP) { s->hb_itype[i] = SDMD_HB_NOEVENT; return; }
    s->hb_itype[i] = SDMD_HB_NOEVENT;
    if (s->hb_bond[i] > 0) {
        int j = s->hb_bond[i];
        if (check_dup(s, i, j, SDMD_EV_HB)) return;
        kin k; pair_kin(s, i, j, &k);
        pairlim L;
        int cs = find_pair(s, i, j, K_HB, k.b, k.r2, &L, 0, 0, 0);
        int st; double d2;
        if (k.b < 0 && disc(&k, L.lo) > 0) {
            st = -1; d2 = L.lo; c.potential = L.lopot;
            c.sub = (cs == 0) ? SDMD_SUB_CORE : SDMD_SUB_TBD_CAPTURE;
        } else {
            st = 1; d2 = L.up; c.potential = L.uppot;
            c.sub = (cs == 1) ? SDMD_SUB_TBD_HBBREAK : SDMD_SUB_TBD_ESCAPE;
        }
        c.time = root(&k, st, d2);
        if (c.time < 0) c.time = INFINIT;
        job_assign(s, i, j, &c, SDMD_EV_HB);
    } else if (i != 0 && (s->hb_role[i] == 'A' || s->hb_role[i] == 'D' || s->hb_role[i] == 'S') &&
               s->hb_bond[i] == 0) {
        double cut = s->cutoff * 0.90; cut *= cut;
        for (int kc = 0; kc < 27; kc++) {
            for (int j = nb_head(s, i, kc); j; j = s->cell_list[j]) {
                if (!(i != j && hb_pair_ok(s, i, j) && s->hb_bond[j] == 0 &&
                      ((s->protein[i] == s->protein[j] && abs(s->aanum[i] - s->aanum[j]) >= 4) ||
                       s->protein[i] != s->protein[j])))
                    continue;
                if (check_dup(s, i, j, SDMD_EV_HB)) continue;
                kin k; pair_kin(s, i, j, &k);
                if (!(k.r2 <= cut)) continue;
                if (pair_match(s, i, j) < 0) continue;
                pairlim L;
                int cs = find_pair(s, i, j, K_HB, k.b, k.r2, &L, 0, 0, 0);
                if (!(k.b < 0 && cs == 1 && disc(&k, L.lo) > 0)) continue;
                c.potential = L.lopot; c.sub = SDMD_SUB_TBD_HBFORM;
                c.time = root(&k, -1, L.lo);
                if (c.time < 0) c.time = INFINIT;
                job_assign(s, i, j, &c, SDMD_EV_HB);
            }
        }
    }
}

/* HBNeighborTime (src/TimePrediction.c:486-579) */
static void hbnb_time(sdmd_system *s, int i) {
    cand c = {INFINIT, 0, SDMD_SUB_INVALID};
    int flag = 0;
    for (int n = 1; n <= s->nb_status[i]; n++) {
        int j = s->nb_partner[4 * i + n - 1];
        if (flag == 0) s->nb_pnum[i] = n;
        if (check_dup(s, i, j, SDMD_EV_HBNEIGHBOR)) { s->nb_pnum[i] = n; flag = 1; continue; }
        kin k; pair_kin(s, i, j, &k);
        int host, nbr, hpart;
        int ri = s->hb_role[i];
        if ((ri == 'A' || ri == 'D' || ri == 'S') && s->hb_bond[i] && s->hb_neighbor[s->hb_bond[i]] == j) {
            host = i; nbr = j; hpart = s->hb_bond[i];
        } else {
            host = j; nbr = i; hpart = s->hb_bond[j];
        }
        pairlim L;
        int cs = find_pair(s, nbr, host, K_NEIGHBOR, k.b, k.r2, &L, hpart, 0, 0);
        int st; double d2;
        if (k.b < 0 && disc(&k, L.lo) > 0) {
            st = -1; d2 = L.lo; c.potential = L.lopot;
            c.sub = (cs == 0) ? SDMD_SUB_CORE : SDMD_SUB_TBD_CAPTURE;
        } else {
            st = 1; d2 = L.up; c.potential = L.uppot;
            c.sub = (cs == 1) ? SDMD_SUB_WELL_BOUNCE : SDMD_SUB_TBD_ESCAPE;
        }
        c.time = root(&k, st, d2);
        if (c.time < 0) c.time = INFINIT;
        if (job_assign(s, i, j, &c, SDMD_EV_HBNEIGHBOR)) { s->nb_pnum[i] = n; flag = 1; }
    }
}

/* WallTime, smooth walls (src/TimePrediction.c:635-737) */
static void wall_time(sdmd_system *s, int i) {
recal:;
    cand c = {INFINIT, 0, SDMD_SUB_INVALID};
    double p[3] = {s->x[i], s->y[i], s->z[i]}, v[3] = {s->vx[i], s->vy[i], s->vz[i]};
    if (s->wall == SDMD_WALL_PARALLEL) { p[0] = p[2] = 0; v[0] = v[2] = 0; }
    else if (s->wall == SDMD_WALL_CYLINDER) { p[0] = 0; v[0] = 0; }
    kin k;
    k.rx = p[0] - s->wall_pos[0]; k.ry = p[1] - s->wall_pos[1]; k.rz = p[2] - s->wall_pos[2];
    double vx = v[0] - s->wall_vel[0], vy = v[1] - s->wall_vel[1], vz = v[2] - s->wall_vel[2];
    k.r2 = k.rx * k.rx + k.ry * k.ry + k.rz * k.rz;
    k.b = k.rx * vx + k.ry * vy + k.rz * vz;
    k.v2 = vx * vx + vy * vy + vz * vz;
    double L2 = s->box[1];
    double dist2 = L2 * L2 * 0.25 + k.r2 - L2 * sqrt(k.r2);
    pairlim L;
    int cs = find_pair(s, i, 0, K_COLLISION, -1 * k.b, dist2, &L, 0, 0, s->wall_type);
    if (L.lopot == 0 && L.uppot == 0) {
        if (s->wall_dyn) {   /* the moving wall passed the atom: widen the box, predict again
                                (src/TimePrediction.c:674-697) */
            s->wall_dyn_touch++;
            if (s->wall == SDMD_WALL_PARALLEL) {
                s->box[1] += s->wall_dyn_step;
            } else if (s->wall == SDMD_WALL_CYLINDER) {
                s->box[1] += s->wall_dyn_step; s->box[2] += s->wall_dyn_step;
            } else if (s->wall == SDMD_WALL_SPHERE) {
                s->box[0] += s->wall_dyn_step; s->box[1] += s->wall_dyn_step; s->box[2] += s->wall_dyn_step;
            }
            if (s->box[1] > s->wall_dyn_orig_box[1]) { fail(SDMD_EWALL, i); return; }
            goto recal;
        }
        fail(SDMD_EWALL, i);
        return;
    }
    int st; double d2;
    if (k.b < 0 && disc(&k, L.lo) > 0) {
        if (cs == 1) return;
        c.sub = SDMD_SUB_TBD_CAPTURE;
        st = -1; d2 = L2 * L2 * 0.25 + L.up - L2 * sqrt(L.up); c.potential = L.uppot;
    } else {
        c.sub = (cs == 0) ? SDMD_SUB_WELL_BOUNCE : SDMD_SUB_TBD_ESCAPE;
        st = 1; d2 = L2 * L2 * 0.25 + L.lo - L2 * sqrt(L.lo); c.potential = L.lopot;
    }
    c.time = root(&k, st, d2);
    if (c.time < 0) c.time = INFINIT;
    job_assign(s, i, 0, &c, SDMD_EV_WALL);
}

/* ObstTime (src/TimePrediction.c:740-829): for each plane n across axis d, the
 * axis component alone (the others zeroed, as the reference zeroes them) against
 * the potential steps of the pair (atom type, wall type); the partner becomes
 * -d - 10 n when that plane gives the new earliest event. */
static void obst_time(sdmd_system *s, int i) {
    const double p[3] = {s->x[i], s->y[i], s->z[i]}, v[3] = {s->vx[i], s->vy[i], s->vz[i]};
    for (int n = 0; n < s->n_obst; n++) {
        for (int dim = 0; dim < 3; dim++) {
            const double pos = s->obst[3 * n + dim];
            if (pos < 0) continue;
            double pi[3] = {0, 0, 0}, pj[3] = {0, 0, 0}, vi[3] = {0, 0, 0}, vj[3] = {0, 0, 0};
            pi[dim] = p[dim]; pj[dim] = pos; vi[dim] = v[dim];
            kin k;
            k.rx = pi[0] - pj[0]; k.ry = pi[1] - pj[1]; k.rz = pi[2] - pj[2];
            const double wx = vi[0] - vj[0], wy = vi[1] - vj[1], wz = vi[2] - vj[2];
            k.r2 = k.rx * k.rx + k.ry * k.ry + k.rz * k.rz;
            k.b = k.rx * wx + k.ry * wy + k.rz * wz;
            k.v2 = wx * wx + wy * wy + wz * wz;
            pairlim L;
            const int cs = find_pair(s, i, 0, K_COLLISION, k.b, k.r2, &L, 0, 0, s->wall_type);
            if (L.lopot == 0 && L.uppot == 0) continue;   /* inside the holes */
            cand c = {INFINIT, 0, SDMD_SUB_INVALID};
            int st; double d2;
            if (k.b < 0) {
                c.sub = cs == 0 ? SDMD_SUB_CORE : SDMD_SUB_TBD_CAPTURE;
                st = -1; d2 = L.lo; c.potential = L.lopot;
            } else {
                if (cs == 1) continue;
                c.sub = SDMD_SUB_TBD_ESCAPE;
                st = 1; d2 = L.up; c.potential = L.uppot;
            }
            c.time = root(&k, st, d2);
            if (c.time < 0) { fail(SDMD_ENEGTIME, i); return; }
            if (job_assign(s, i, 0, &c, SDMD_EV_OBST)) s->ev_partner[i] = -(dim + 1) - 10 * n;
        }
    }
}

/* SphObstTime (src/TimePrediction.c:1020-1071): a core collision with each fixed
 * sphere the atom approaches (absolute coordinates, no periodic image); the event's
 * partner becomes -1000 n when obstacle n gives the new earliest event. */
static void sphobst_time(sdmd_system *s, int i) {
    for (int n = 0; n < s->n_sphobst; n++) {
        const double *o = s->sphobst + 4 * n;
        kin k;
        k.rx = s->x[i] - o[0]; k.ry = s->y[i] - o[1]; k.rz = s->z[i] - o[2];
        const double vx = s->vx[i] - 0.0, vy = s->vy[i] - 0.0, vz = s->vz[i] - 0.0;
        k.r2 = k.rx * k.rx + k.ry * k.ry + k.rz * k.rz;
        k.b = k.rx * vx + k.ry * vy + k.rz * vz;
        k.v2 = vx * vx + vy * vy + vz * vz;
        const double lo = o[3] * o[3];
        if (!(k.b < 0 && disc(&k, lo) > 0)) continue;
        cand c = {INFINIT, 0, SDMD_SUB_CORE};
        c.time = root(&k, -1, lo);
        if (c.time < 0) { fail(SDMD_ENEGTIME, i); return; }
        if (job_assign(s, i, 0, &c, SDMD_EV_SPHOBST)) s->ev_partner[i] = -1000 * n;
    }
}

/* Predict (src/SGThread.c:158-211) with ResetTarget (src/ToolFunctions.c:504-514) */
static void predict(sdmd_system *s, const int *list, int n) {
    for (int q = 0; q < n; q++) {
        int i = list[q];
        s->ev_type[i] = SDMD_EV_INVALID; s->ev_time[i] = INFINIT; s->ev_partner[i] = INVALID;
    }
    for (int q = 0; q < n && !G.err; q++) {
        int i = list[q];
        bond_time(s, i);
        collision_time(s, i);
        pcc_time(s, i);
        thermostat_time(s, i);
        hb_time(s, i);
        hbnb_time(s, i);
        if (s->wall) wall_time(s, i);
        if (s->n_obst) obst_time(s, i);
        if (s->n_sphobst) sphobst_time(s, i);
    }
}

int oracle_predict_all(sdmd_system *s) {
    G.err = 0;
    int *list = malloc(sizeof(int) * (s->n_atoms + 1));
    for (int i = 0; i < s->n_atoms; i++) list[i] = i + 1;
    predict(s, list, s->n_atoms);
    free(list);
    return G.err;
}

/* ---- events ------------------------------------------------------------------ */
/* HBEnergyChange (src/Events.c:1027-1095).  Note the reference keeps `accumPoten`
 * across candidates, so a skipped HB neighbour adds the previous candidate's value. */
static double hb_energy_change(sdmd_system *s, int t, int skip, int to_hb) {
    double cut = s->cutoff * s->cutoff, energy = 0, acc = 0;
    for (int kc = 0; kc < 27; kc++) {
        for (int j = nb_head(s, t, kc); j; j = s->cell_list[j]) {
            int bits = conn_bits(s, t, j);
            if (!(t != j && !(bits & 1) && !(bits & 2) && j != skip)) continue;
            kin k; pair_kin(s, t, j, &k);
            if (k.r2 <= cut) {
                pairlim L;
                if (!to_hb) {
                    find_pair(s, t, j, K_COLLISION, 0, k.r2, &L, 0, -1, 0); acc = L.acc;
                } else if (j != s->hb_neighbor[skip]) {
                    find_pair(s, t, j, K_COLLISION, 0, k.r2, &L, 0, 1, 0); acc = L.acc;
                }
                if (acc == INFINIT) acc = 0;
                energy += acc;
            }
        }
    }
    return energy;
}

/* position of atom a imaged next to atom t by cell indices (src/Events.c:815-823) */
static void imaged(const sdmd_system *s, int t, int a, double p[3]) {
    const int ct[3] = {s->cx[t], s->cy[t], s->cz[t]}, ca[3] = {s->cx[a], s->cy[a], s->cz[a]};
    p[0] = s->x[a]; p[1] = s->y[a]; p[2] = s->z[a];
    for (int d = 0; d < 3; d++) {
        if (ct[d] != ca[d]) {
            if (ct[d] == 0 && ca[d] == s->cellnum[d] - 1) p[d] -= s->box[d];
            else if (ct[d] == s->cellnum[d] - 1 && ca[d] == 0) p[d] += s->box[d];
        }
    }
}

/* InteractionEvent (src/Events.c:798-1024) */
static void interaction_event(sdmd_system *s, int t, int p, int ni, int nj) {
    double pi[3] = {s->x[t], s->y[t], s->z[t]}, pj[3];
    imaged(s, t, p, pj);
    double r[3] = {pi[0] - pj[0], pi[1] - pj[1], pi[2] - pj[2]};
    double v[3] = {s->vx[t] - s->vx[p], s->vy[t] - s->vy[p], s->vz[t] - s->vz[p]};
    double d2 = r[0] * r[0] + r[1] * r[1] + r[2] * r[2];
    double b = r[0] * v[0] + r[1] * v[1] + r[2] * v[2];
    double mt = s->mass[t], mp = s->mass[p];
    double mu = mt * mp / (mt + mp);
    double pot = s->ev_potential[t];
    int sv = 0;
    if (s->ev_type[t] == SDMD_EV_HB && (s->ev_sub[t] == SDMD_SUB_TBD_HBFORM || s->ev_sub[t] == SDMD_SUB_TBD_HBBREAK)) {
        int form = s->ev_sub[t] == SDMD_SUB_TBD_HBFORM;
        if ((nb_has(s, t, nj) || nb_has(s, p, ni)) && form) { s->hb_itype[t] = SDMD_HB_SKIP; return; }
        double pni[3], pnj[3];
        imaged(s, t, ni, pni);
        imaged(s, t, nj, pnj);
        double rci[3] = {pi[0] - pnj[0], pi[1] - pnj[1], pi[2] - pnj[2]};
        double rcj[3] = {pj[0] - pni[0], pj[1] - pni[1], pj[2] - pni[2]};
        double rni2 = rci[0] * rci[0] + rci[1] * rci[1] + rci[2] * rci[2];
        double rnj2 = rcj[0] * rcj[0] + rcj[1] * rcj[1] + rcj[2] * rcj[2];
        double acc[6];
        acc[0] = hb_energy_change(s, t, p, 0);
        acc[1] = hb_energy_change(s, p, t, 0);
        acc[2] = hb_energy_change(s, t, p, 1);
        acc[3] = hb_energy_change(s, p, t, 1);
        pairlim L;
        find_pair(s, nj, t, K_NEIGHBOR, 0, rni2, &L, p, 0, 0); acc[4] = L.acc;
        find_pair(s, ni, p, K_NEIGHBOR, 0, rnj2, &L, t, 0, 0); acc[5] = L.acc;
        if (form) {
            pot -= hb_barrier(s, t, p);
            pot += (acc[2] - acc[0] + acc[3] - acc[1] + acc[4] + acc[5]);
        } else {
            pot += hb_barrier(s, t, p);
            pot += (acc[0] - acc[2] + acc[1] - acc[3] - acc[4] - acc[5]);
        }
        if (pot < -0.5 * INFINIT && !form) { s->hb_itype[t] = SDMD_HB_SKIP; return; }
        if (pot > 0.5 * INFINIT && form) { s->hb_itype[t] = SDMD_HB_SKIP; return; }
        if (b * b - 2 * d2 * pot / mu > 0) {
            if (form) { s->ev_sub[t] = SDMD_SUB_WELL_CAPTURE; s->hb_itype[t] = SDMD_HB_FORM; }
            else { s->ev_sub[t] = SDMD_SUB_WELL_ESCAPE; s->hb_itype[t] = SDMD_HB_BREAK; }
        } else {
            if (form) { s->hb_itype[t] = SDMD_HB_SKIP; return; }
            pot = 0; s->ev_sub[t] = SDMD_SUB_WELL_BOUNCE; s->hb_itype[t] = SDMD_HB_NOEVENT;
        }
    }
    switch (s->ev_sub[t]) {
        case SDMD_SUB_CORE: sv = 1; pot = 0; break;
        case SDMD_SUB_WELL_BOUNCE: sv = b < 0 ? 1 : -1; pot = 0; break;
        case SDMD_SUB_WELL_CAPTURE: sv = -1; break;
        case SDMD_SUB_WELL_ESCAPE: sv = b < 0 ? -1 : 1; break;
        case SDMD_SUB_TBD_CAPTURE:
            if (b * b - 2 * d2 * pot / mu <= 0) { pot = 0; sv = 1; } else sv = -1;
            break;
        case SDMD_SUB_TBD_ESCAPE:
            if (b * b - 2 * d2 * pot / mu <= 0) { pot = 0; sv = b < 0 ? 1 : -1; }
            else sv = b < 0 ? -1 : 1;
            break;
        default: fail(SDMD_EEVENTTYPE, t); return;
    }
    double phi = (-1 * b + sv * sqrt((b * b - 2 * d2 * pot / mu))) / ((mt + mp) * d2);
    if (isnan(phi)) { fail(SDMD_ENAN, t); return; }
    double ft = mp * phi, fp = mt * phi;
    s->vx[t] = s->vx[t] + ft * r[0]; s->vy[t] = s->vy[t] + ft * r[1]; s->vz[t] = s->vz[t] + ft * r[2];
    s->vx[p] = s->vx[p] - fp * r[0]; s->vy[p] = s->vy[p] - fp * r[1]; s->vz[p] = s->vz[p] - fp * r[2];
}

/* ListRefresh(target, list, 1, 4) (src/ToolFunctions.c:572-597) */
static void nb_remove(sdmd_system *s, int a, int value) {
    int32_t *l = s->nb_partner + 4 * a;   /* l[k-1] is neighborPartner[k] */
    int i = nb_has(s, a, value);
    if (!i) return;
    int n = i + 1;
    while (n <= 4 && l[n - 1] != 0) { l[i - 1] = l[n - 1]; i++; n++; }
    l[i - 1] = 0;
}

static void nb_append(sdmd_system *s, int a, int value) {
    int k = ++s->nb_status[a];
    if (k > 4) { fail(SDMD_ECAPACITY, a); return; }
    s->nb_partner[4 * a + k - 1] = value;
}

static int alpha_hb(const sdmd_system *s, int i, int j) {
    return s->protein[i] == s->protein[j] &&
           ((s->name_code[i] == 1 && s->name_code[j] == 2 && s->aanum[j] == s->aanum[i] - 4) ||
            (s->name_code[i] == 2 && s->name_code[j] == 1 && s->aanum[i] == s->aanum[j] - 4));
}

/* HBEvent (src/Events.c:275-393) */
static void hb_event(sdmd_system *s, int i, int j, int ni, int nj) {
    int nbi = s->hb_neighbor[i], nbj = s->hb_neighbor[j];
    if (s->hb_itype[i] == SDMD_HB_FORM) {
        if (nb_has(s, i, nbj) || nb_has(s, nbj, i) || nb_has(s, j, nbi) || nb_has(s, nbi, j)) {
            fail(SDMD_EHBMAP, i); return;
        }
        s->hb_bond[i] = j; s->hb_bond[j] = i;
        s->type[i] = type_change(s->type[i], 1); s->type[j] = type_change(s->type[j], 1);
        nb_append(s, i, nbj);
        nb_append(s, j, nbi);
        nb_append(s, ni, j);
        nb_append(s, nj, i);
        if (alpha_hb(s, i, j)) s->counters.alpha_hb_formed++;
        s->counters.hb_formed++;
    } else if (s->hb_itype[i] == SDMD_HB_BREAK) {
        s->hb_bond[i] = 0; s->hb_bond[j] = 0;
        s->type[i] = type_change(s->type[i], 0); s->type[j] = type_change(s->type[j], 0);
        --s->nb_status[i]; nb_remove(s, i, nbj);
        --s->nb_status[j]; nb_remove(s, j, nbi);
        --s->nb_status[ni]; nb_remove(s, ni, j);
        --s->nb_status[nj]; nb_remove(s, nj, i);
        if (alpha_hb(s, i, j)) s->counters.alpha_hb_formed--;
        s->counters.hb_formed--;
        if (s->counters.hb_formed < s->counters.alpha_hb_formed) s->counters.warnings++;
    }
}

/* ThermostatEvent, Andersen (src/Events.c:396-420) */
static void thermostat_event(sdmd_system *s, int t) {
    double sp[3];
    for (int d = 0; d < 3; d++) {
        do { sp[d] = oracle_mb(&s->rng, 0, s->temperature / s->mass[t]); } while (sp[d] == 0);
    }
    s->vx[t] = sp[0]; s->vy[t] = sp[1]; s->vz[t] = sp[2];
}

/* PBC("part") + LinkList("part") via PBCandCrossCellEvent (src/Events.c:248-272,
 * 207-245, 158-200) */
static void pcc_event(sdmd_system *s, int t) {
    int old[3] = {s->cx[t], s->cy[t], s->cz[t]};
    double *pos[3] = {&s->x[t], &s->y[t], &s->z[t]};
    for (int d = 0; d < 3; d++) {
        if (old[d] == 0 || old[d] == s->cellnum[d] - 1) {
            if (s->wall != SDMD_WALL_SPHERE) {
                int dims = 3, step = 1;
                if (s->wall == SDMD_WALL_PARALLEL) step = 2;
                else if (s->wall == SDMD_WALL_CYLINDER) dims = 1;
                for (int n = 0; n < dims; n += step) {
                    if (*pos[n] >= s->box[n]) *pos[n] -= s->box[n];
                    else if (*pos[n] < 0) *pos[n] += s->box[n];
                }
            }
            break;
        }
    }
    int N = s->n_atoms;
    int oldc = cell_lin(s, old[0], old[1], old[2]);
    int nc[3];
    for (int d = 0; d < 3; d++) {
        nc[d] = (int)(*pos[d] / s->cellsize[d]);
        if (nc[d] == s->cellnum[d]) nc[d]--;
    }
    s->cx[t] = nc[0]; s->cy[t] = nc[1]; s->cz[t] = nc[2];
    int newc = cell_lin(s, nc[0], nc[1], nc[2]);
    int *L = s->cell_list;
    int at = oldc + N, guard = 0;
    if (L[at] == 0) { fail(SDMD_ELINK, t); return; }
    while (L[at] != t) {
        at = L[at];
        if (at == 0 || ++guard > N) { fail(SDMD_ELINK, t); return; }
    }
    L[at] = L[t];
    L[t] = L[newc + N];
    L[newc + N] = t;
}

/* WallEvent, smooth walls (src/Events.c:423-499) */
static void wall_event(sdmd_system *s, int t) {
    double p[3] = {s->x[t], s->y[t], s->z[t]}, v[3] = {s->vx[t], s->vy[t], s->vz[t]};
    if (s->wall == SDMD_WALL_PARALLEL) { p[0] = p[2] = 0; v[0] = v[2] = 0; }
    else if (s->wall == SDMD_WALL_CYLINDER) { p[0] = 0; v[0] = 0; }
    double r[3] = {p[0] - s->wall_pos[0], p[1] - s->wall_pos[1], p[2] - s->wall_pos[2]};
    double w[3] = {v[0] - s->wall_vel[0], v[1] - s->wall_vel[1], v[2] - s->wall_vel[2]};
    double d2 = r[0] * r[0] + r[1] * r[1] + r[2] * r[2];
    double b = r[0] * w[0] + r[1] * w[1] + r[2] * w[2];
    double mu = s->mass[t], pot = s->ev_potential[t];
    int sv;
    switch (s->ev_sub[t]) {
        case SDMD_SUB_WELL_BOUNCE: sv = -1; pot = 0; break;
        case SDMD_SUB_TBD_CAPTURE:
            if (b * b - 2 * d2 * pot / mu <= 0) { pot = 0; sv = 1; } else sv = -1;
            break;
        case SDMD_SUB_TBD_ESCAPE:
            if (b * b - 2 * d2 * pot / mu <= 0) { pot = 0; sv = -1; } else sv = 1;
            break;
        default: fail(SDMD_EEVENTTYPE, t); return;
    }
    double phi = (-1 * b + sv * sqrt(b * b - 2 * d2 * pot / s->mass[t])) / d2;
    if (isnan(phi)) { fail(SDMD_ENAN, t); return; }
    s->vx[t] = s->vx[t] + phi * r[0]; s->vy[t] = s->vy[t] + phi * r[1]; s->vz[t] = s->vz[t] + phi * r[2];
}

/* ObstEvent (src/Events.c:543-617): plane -partner / 10 across axis -partner % 10 */
static void obst_event(sdmd_system *s, int t) {
    const int part = s->ev_partner[t];
    const int n = part / -10, dim = (part * -1) % 10;
    if (n < 0 || n >= s->n_obst || dim < 1 || dim > 3) { fail(SDMD_EEVENTTYPE, t); return; }
    double pi[3] = {0, 0, 0}, pj[3] = {0, 0, 0}, vi[3] = {0, 0, 0}, vj[3] = {0, 0, 0};
    pi[dim - 1] = dim == 1 ? s->x[t] : dim == 2 ? s->y[t] : s->z[t];
    vi[dim - 1] = dim == 1 ? s->vx[t] : dim == 2 ? s->vy[t] : s->vz[t];
    pj[dim - 1] = s->obst[3 * n + dim - 1];
    const double r[3] = {pi[0] - pj[0], pi[1] - pj[1], pi[2] - pj[2]};
    const double w[3] = {vi[0] - vj[0], vi[1] - vj[1], vi[2] - vj[2]};
    const double d2 = r[0] * r[0] + r[1] * r[1] + r[2] * r[2];
    const double b = r[0] * w[0] + r[1] * w[1] + r[2] * w[2];
    const double mu = s->mass[t];
    double pot = s->ev_potential[t];
    int sv;
    switch (s->ev_sub[t]) {
        case SDMD_SUB_CORE: sv = 1; pot = 0; break;
        case SDMD_SUB_TBD_CAPTURE:
            if (b * b - 2 * d2 * pot / mu <= 0) { pot = 0; sv = 1; } else sv = -1;
            break;
        case SDMD_SUB_TBD_ESCAPE:
            if (b * b - 2 * d2 * pot / mu <= 0) { pot = 0; sv = -1; } else sv = 1;
            break;
        default: fail(SDMD_EEVENTTYPE, t); return;
    }
    const double phi = (-1 * b + sv * sqrt(b * b - 2 * d2 * pot / s->mass[t])) / d2;
    if (isnan(phi)) { fail(SDMD_ENAN, t); return; }
    s->vx[t] = s->vx[t] + phi * r[0]; s->vy[t] = s->vy[t] + phi * r[1]; s->vz[t] = s->vz[t] + phi * r[2];
}

/* SphObstEvent (src/Events.c:752-795): the core bounce off fixed sphere
 * -partner / 1000 */
static void sphobst_event(sdmd_system *s, int t) {
    const int n = s->ev_partner[t] / -1000;
    if (n < 0 || n >= s->n_sphobst || s->ev_sub[t] != SDMD_SUB_CORE) { fail(SDMD_EEVENTTYPE, t); return; }
    const double *o = s->sphobst + 4 * n;
    double r[3] = {s->x[t] - o[0], s->y[t] - o[1], s->z[t] - o[2]};
    double w[3] = {s->vx[t] - 0.0, s->vy[t] - 0.0, s->vz[t] - 0.0};
    double d2 = r[0] * r[0] + r[1] * r[1] + r[2] * r[2];
    double b = r[0] * w[0] + r[1] * w[1] + r[2] * w[2];
    const double pot = 0;
    const int sv = 1;
    double phi = (-1 * b + sv * sqrt(b * b - 2 * d2 * pot / s->mass[t])) / d2;
    if (isnan(phi)) { fail(SDMD_ENAN, t); return; }
    s->vx[t] = s->vx[t] + phi * r[0]; s->vy[t] = s->vy[t] + phi * r[1]; s->vz[t] = s->vz[t] + phi * r[2];
}

/* DoWallDyn (src/Events.c:502-541), after each executed event: once per time
 * unit the wall moves by sign * step (a pulse turns at its extremes), the atoms
 * heading for the wall have their events invalidated, and a compression or an
 * expansion that is complete stops. */
static void do_wall_dyn(sdmd_system *s) {
    if (!(s->time >= s->wall_dyn_cur_time)) return;
    const double *o = s->wall_dyn_orig_box;
    if (s->wall_dyn == 3) {
        if ((o[1] - s->box[1] >= s->wall_dyn_size) || (o[1] == s->box[1])) {
            s->wall_dyn_sign *= -1;
            s->wall_dyn_touch = 0;
        } else if (fabs(s->box[1] + (int)(s->time / s->wall_dyn_rate + 1) * s->wall_dyn_size -
                        (s->time - 1) * s->wall_dyn_step - o[1]) <= s->wall_dyn_step &&
                   s->wall_dyn_touch >= 5) {
            s->wall_dyn_sign *= -1;
            s->wall_dyn_touch = 0;
        }
    }
    s->wall_dyn_cur_time += 1;
    if (s->wall == SDMD_WALL_PARALLEL) {
        s->box[1] += s->wall_dyn_sign * s->wall_dyn_step;
    } else if (s->wall == SDMD_WALL_CYLINDER) {
        s->box[1] += s->wall_dyn_sign * s->wall_dyn_step;
        s->box[2] += s->wall_dyn_sign * s->wall_dyn_step;
    } else if (s->wall == SDMD_WALL_SPHERE) {
        s->box[0] += s->wall_dyn_sign * s->wall_dyn_step;
        s->box[1] += s->wall_dyn_sign * s->wall_dyn_step;
        s->box[2] += s->wall_dyn_sign * s->wall_dyn_step;
    }
    for (int i = 1; i <= s->n_atoms; i++)
        if (s->ev_type[i] == SDMD_EV_WALL) s->ev_counter[i]++;
    if ((o[1] - s->box[1] >= s->wall_dyn_size && s->wall_dyn == 1) ||
        (o[1] - s->box[1] <= s->wall_dyn_step && s->wall_dyn == 2))
        s->wall_dyn = 0;
}

/* DoEvent (src/Events.c:25-114) */
static void do_event(sdmd_system *s, int t, int p) {
    switch (s->ev_type[t]) {
        case SDMD_EV_COLLISION: interaction_event(s, t, p, 0, 0); s->counters.collision++; break;
        case SDMD_EV_BOND: interaction_event(s, t, p, 0, 0); s->counters.bond++; break;
        case SDMD_EV_HBNEIGHBOR: interaction_event(s, t, p, 0, 0); s->counters.hbneighbor++; break;
        case SDMD_EV_HB: {
            int ni = s->hb_neighbor[t], nj = s->hb_neighbor[p];
            interaction_event(s, t, p, ni, nj);
            if (!G.err) hb_event(s, t, p, ni, nj);
            s->counters.hb++;
        } break;
        case SDMD_EV_THERMOSTAT: thermostat_event(s, t); s->counters.thermostat++; break;
        case SDMD_EV_PCC: pcc_event(s, t); s->counters.pcc++; break;
        case SDMD_EV_WALL: wall_event(s, t); s->counters.wall++; break;
        case SDMD_EV_OBST: obst_event(s, t); s->counters.wall++; break;         /* walleventsum */
        case SDMD_EV_SPHOBST: sphobst_event(s, t); s->counters.wall++; break;   /* walleventsum */
        default: fail(SDMD_EEVENTTYPE, t); break;
    }
}

/* ---- complete-binary-tree event queue (src/CBT.c) ------------------------------ */
struct oracle_loop {
    sdmd_system *s;
    int32_t *node, *leaf;
    int32_t count;
};

static void cbt_update(oracle_loop *L, int a) {   /* UpdateCBTRun, src/CBT.c:56-83 */
    const double *tm = L->s->ev_time;
    int f;
    for (f = L->leaf[a] / 2; f > 0; f /= 2) {
        if (L->node[f] != a) break;
        int l = L->node[2 * f], r = L->node[2 * f + 1];
        L->node[f] = tm[l] < tm[r] ? l : r;
    }
    for (; f > 0; f /= 2) {
        int old = L->node[f], l = L->node[2 * f], r = L->node[2 * f + 1];
        L->node[f] = tm[l] < tm[r] ? l : r;
        if (L->node[f] == old) return;
    }
}

static void cbt_insert(oracle_loop *L, int a) {   /* InsertCBTRun, src/CBT.c:86-105 */
    if (L->count == 0) { L->node[1] = a; L->count++; return; }
    int i = L->node[L->count];
    L->node[2 * L->count] = i;
    L->node[2 * L->count + 1] = a;
    L->leaf[i] = 2 * L->count;
    L->leaf[a] = 2 * L->count + 1;
    L->count++;
    cbt_update(L, i);
}

oracle_loop *oracle_loop_create(sdmd_system *s) {
    oracle_loop *L = calloc(1, sizeof(*L));
    L->s = s;
    L->node = calloc(2 * (size_t)s->n_atoms + 2, sizeof(int32_t));
    L->leaf = calloc((size_t)s->n_atoms + 2, sizeof(int32_t));
    for (int i = 1; i <= s->n_atoms; i++) cbt_insert(L, i);
    return L;
}

void oracle_loop_destroy(oracle_loop *L) {
    if (!L) return;
    free(L->node); free(L->leaf); free(L);
}

int oracle_cbt(oracle_loop *L, int32_t *node, int32_t *leaf) {
    memcpy(node, L->node, sizeof(int32_t) * 2 * L->s->n_atoms);
    memcpy(leaf, L->leaf, sizeof(int32_t) * (L->s->n_atoms + 1));
    return 0;
}

/* ---- the loop: SingleThreadRun (src/SGThread.c:67-155); with stop_time > 0 it also
 * stops after the first executed event at time >= stop_time, REMDRun's exchange
 * point (src/REMD.c:97) ---------------------------------------------------------- */
static int run_loop(oracle_loop *L, int64_t max_events, double t_end, double stop_time,
                    sdmd_trace_rec *trace, int64_t trace_cap, int64_t *n_pops) {
    sdmd_system *s = L->s;
    G.err = 0;
    int N = s->n_atoms;
    int64_t start = s->counters.frame, pops = 0;
    int at_stop = 0;
    while (s->time <= t_end && s->counters.frame - start < max_events && !at_stop) {
        /* AssignJob (src/SGThread.c:237-259) */
        int t = L->node[1];
        double dt = s->ev_time[t];
        int p = s->ev_partner[t] > 0 ? s->ev_partner[t] : 0;
        int rec_partner = s->ev_partner[t], rec_type = s->ev_type[t], rec_sub = s->ev_sub[t];
        /* UpdateData + TimeForward (src/ToolFunctions.c:23-36) */
        for (int i = 1; i <= N; i++) {
            s->x[i] += s->vx[i] * dt;
            s->y[i] += s->vy[i] * dt;
            s->z[i] += s->vz[i] * dt;
        }
        for (int i = 1; i <= N; i++) s->ev_time[i] -= dt;
        s->time += dt;
        /* HazardCheck (src/SGThread.c:215-235) */
        int hazard = p > 0 && s->ev_pcounter[t] < s->ev_counter[p];
        int list[2] = {t, p};
        int n = 1;
        if (!hazard) {
            s->counters.frame++;
            do_event(s, t, p);
            if (G.err) break;
            s->ev_counter[t]++;
            if (p) { s->ev_counter[p]++; n = 2; }
            if (stop_time > 0 && s->time >= stop_time) at_stop = 1;
        } else {
            s->counters.recal++;
        }
        predict(s, list, n);
        for (int q = 0; q < n; q++) cbt_update(L, list[q]);
        if (!hazard && s->wall_dyn) do_wall_dyn(s);
        if (trace && pops < trace_cap) {
            sdmd_trace_rec *r = &trace[pops];
            memset(r, 0, sizeof(*r));
            r->target = t; r->partner = rec_partner; r->type = rec_type; r->sub = rec_sub;
            r->executed = !hazard; r->hb_itype_after = s->hb_itype[t];
            r->dt = dt; r->time_now = s->time;
            r->vt[0] = s->vx[t]; r->vt[1] = s->vy[t]; r->vt[2] = s->vz[t];
            r->t_new_time = s->ev_time[t]; r->t_new_partner = s->ev_partner[t]; r->t_new_type = s->ev_type[t];
            if (p) {
                r->vp[0] = s->vx[p]; r->vp[1] = s->vy[p]; r->vp[2] = s->vz[p];
                r->p_new_time = s->ev_time[p]; r->p_new_partner = s->ev_partner[p]; r->p_new_type = s->ev_type[p];
            }
        }
        pops++;
        if (G.err) break;
    }
    if (n_pops) *n_pops = pops;
    return G.err;
}

int oracle_run(oracle_loop *L, int64_t max_events, double t_end,
               sdmd_trace_rec *trace, int64_t trace_cap, int64_t *n_pops) {
    return run_loop(L, max_events, t_end, 0, trace, trace_cap, n_pops);
}

int oracle_run_until(oracle_loop *L, double t_end, double stop_time, int64_t *n_pops) {
    return run_loop(L, INT64_MAX, t_end, stop_time, NULL, 0, n_pops);
}

/* ---- observables ------------------------------------------------------------- */
/* CalKinetE with no flow (src/ToolFunctions.c:626-656) */
double oracle_kinetic_energy(const sdmd_system *s) {
    double tke = 0;
    for (int i = 1; i <= s->n_atoms; i++) {
        double tx = s->vx[i] - 0, ty = s->vy[i] - 0, tz = s->vz[i] - 0;
        double t0 = tx * tx + ty * ty + tz * tz;
        tke += 0.5 * s->mass[i] * t0;
    }
    return tke;
}

/* CalPotenE (src/ToolFunctions.c:659-752): each pair once (pair > i) within the
 * cutoff; HB pairs add their accumulated HB step energy minus the barrier. */
static double poten(sdmd_system *s, int keep_warnings);
double oracle_potential_energy(const sdmd_system *sc) { return poten((sdmd_system *)sc, 0); }
/* CalPotenE as REMDRun calls it (src/REMD.c:98): FindPair's warnings stay counted */
double oracle_potential_energy_counted(sdmd_system *s) { return poten(s, 1); }

static double poten(sdmd_system *s, int keep_warnings) {
    int64_t w = s->counters.warnings;
    double tpe = 0;
    int N = s->n_atoms;
    for (int i = 1; i <= N; i++) {
        for (int kc = 0; kc < 27; kc++) {
            int c[3] = {s->cx[i] + NBX[kc], s->cy[i] + NBY[kc], s->cz[i] + NBZ[kc]};
            double sh[3];
            for (int d = 0; d < 3; d++) {
                sh[d] = 0;
                if (c[d] < 0) { c[d] = s->cellnum[d] - 1; sh[d] = -1 * s->box[d]; }
                else if (c[d] >= s->cellnum[d]) { c[d] = 0; sh[d] = s->box[d]; }
            }
            for (int pj = s->cell_list[N + cell_lin(s, c[0], c[1], c[2])]; pj; pj = s->cell_list[pj]) {
                if (pj <= i) continue;
                double rx = s->x[i] - (s->x[pj] + sh[0]), ry = s->y[i] - (s->y[pj] + sh[1]),
                       rz = s->z[i] - (s->z[pj] + sh[2]);
                double d2 = rx * rx + ry * ry + rz * rz;
                int bits = conn_bits(s, i, pj);
                if (!(d2 <= s->cutoff * s->cutoff && !(bits & 1))) continue;
                int ai = i, aj = pj, kind, hbp = 0;
                if (s->hb_bond[ai] == aj) { kind = K_HB; tpe -= hb_barrier(s, ai, aj); }
                else if (bits & 2) kind = K_CONSTRAINT;
                else if (nb_has(s, ai, aj)) {
                    if (s->hb_neighbor[s->hb_bond[ai]] == aj) { int q = ai; ai = aj; aj = q; }
                    hbp = s->hb_bond[aj];
                    kind = K_NEIGHBOR;
                } else kind = K_COLLISION;
                double wx = s->vx[ai] - s->vx[aj], wy = s->vy[ai] - s->vy[aj], wz = s->vz[ai] - s->vz[aj];
                double dirn = rx * wx + ry * wy + rz * wz;
                pairlim L;
                L.acc = 0;
                find_pair(s, ai, aj, kind, dirn, d2, &L, hbp, 0, 0);
                if (L.acc < INFINIT / 2) tpe += L.acc;
            }
        }
    }
    if (!keep_warnings) s->counters.warnings = w;
    return tpe;
}

/* ---- REMD exchange sweep (src/Server.c:145-192) ------------------------------ */
void oracle_remd_rearrange(int32_t n, int32_t *num, double *T, const double *E, sdmd_rng *rng) {
    for (int i = 0; i < n; i++) {
        if (!T[i]) continue;
        for (int j = 0; j < n; j++) {
            if (!T[j]) continue;
            if (num[i] == num[j] + 1 || (num[i] == 1 && num[j] == 2)) {
                double b1 = 1 / T[i], b2 = 1 / T[j];
                double dE = (b1 - b2) * (E[j] - E[i]);
                if (dE <= 0.0 || (0 + (double)oracle_rand(rng) / ((double)2147483647 / (1 - 0))) < exp(-1 * dE)) {
                    int tn = num[i]; num[i] = num[j]; num[j] = tn;
                    double tt = T[i]; T[i] = T[j]; T[j] = tt;
                }
                break;
            }
        }
    }
}
