/*
 * writers.c -- the reference's text outputs (SaveData, src/DataSave.c), written
 * from an engine state (an sdmd_system as sdmd_gpu_download fills it).
 *
 * Each call appends one frame to the named file (or starts it, append == 0), in
 * the reference's exact format: the trajectory (SaveGRO :616-640, SavePDB
 * :588-613), the connection map (SaveConnectionMap :218-233), the hydrogen-bond
 * counts (SaveHB :205-216), the xyz trajectory (SaveXYZ :488-505) and the
 * one-number-per-dump series of potential and
 * kinetic energy and temperature (SavePot / SaveKin / SaveTemp :235-278).  The
 * energies are the caller's (sdmd_gpu_energies computes the reference's
 * CalPotenE / CalKinetE on the device); the writer only formats them.
 *
 * Atom and residue names come as 8-byte records (entry i at i*8), as
 * sdmd_host_atom_names / sdmd_host_residue_names return them.
 */
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "sdmd_host.h"
#include "host_static.h"

#define BOND_CONNECT 0x01       /* connection-map bits (src/DMD.h:59-63) */
#define CONSTRAINT_CONNECT 0x02
#define HB_CONNECT 0x04
#define NEIGHBOR_CONNECT 0x08

static FILE *open_out(const char *path, int append) { return path ? fopen(path, append ? "a" : "w") : NULL; }

static int close_out(FILE *f) { return fclose(f) == 0 ? SDMD_OK : SDMD_EINVAL; }

/* a name record as the reference prints it: at most 7 characters, NUL-terminated */
static const char *name8(const char *names, int i, char *buf) {
    memcpy(buf, names + 8 * (size_t)i, 8);
    buf[7] = 0;
    return buf;
}

int sdmd_write_gro(const char *path, int append, const sdmd_system *s, const char *names8, const char *resnames8) {
    if (!s || !names8 || !resnames8) return SDMD_EINVAL;
    FILE *f = open_out(path, append);
    if (!f) return SDMD_EINVAL;
    char a[8], r[8];
    fprintf(f, "model\n");
    fprintf(f, "%5i\n", s->n_atoms);
    for (int i = 1; i <= s->n_atoms; i++)
        fprintf(f, "%5i%-5s%5s%5i%8.3f%8.3f%8.3f%10.4f%10.4f%10.4f\n", s->aanum[i], name8(resnames8, i, r),
                name8(names8, i, a), i, s->x[i] / 10, s->y[i] / 10, s->z[i] / 10, s->vx[i], s->vy[i], s->vz[i]);
    fprintf(f, "%10.5f%10.5f%10.5f\n", s->box[0] / 10, s->box[1] / 10, s->box[2] / 10);
    return close_out(f);
}

int sdmd_write_xyz(const char *path, int append, const sdmd_system *s, const char *names8, const char *timer) {
    if (!s || !names8) return SDMD_EINVAL;
    FILE *f = open_out(path, append);
    if (!f) return SDMD_EINVAL;
    char a[8];
    fprintf(f, "%i\n", s->n_atoms);
    fprintf(f, "Model %s\n", timer ? timer : "");
    for (int i = 1; i <= s->n_atoms; i++)
        fprintf(f, "%-8s%16.6lf%16.6lf%16.6lf\n", name8(names8, i, a), s->x[i], s->y[i], s->z[i]);
    return close_out(f);
}

int sdmd_write_pdb(const char *path, int append, const sdmd_system *s, const char *names8, const char *resnames8) {
    if (!s || !names8 || !resnames8) return SDMD_EINVAL;
    FILE *f = open_out(path, append);
    if (!f) return SDMD_EINVAL;
    char a[8], r[8];
    fprintf(f, "TITLE     I have tried to minimize the energy!\n");
    fprintf(f, "REMARK    THIS IS A SIMULATION BOX\n");
    fprintf(f, "CRYST1%9.3lf%9.3lf%9.3lf  90.00  90.00  90.00 P 1           1\n", s->box[0], s->box[1], s->box[2]);
    for (int i = 1; i <= s->n_atoms; i++) {
        name8(names8, i, a);
        /* the chain letter: peptide 1 is 'A' (the reference adds '0' to 'A' - '1') */
        const char chain = (char)(s->protein[i] + 'A' - '1' + '0');
        fprintf(f, "ATOM  %5i  %-4s%3s %c%4i    %8.3lf%8.3lf%8.3lf%6.2lf%6.2lf           %c\n", i, a,
                name8(resnames8, i, r), chain, s->aanum[i], s->x[i], s->y[i], s->z[i], 1.0, 0.0, a[0]);
    }
    fprintf(f, "TER\n");
    fprintf(f, "ENDMDL\n");
    return close_out(f);
}

static int cmp_int(const void *a, const void *b) {
    const int x = *(const int *)a, y = *(const int *)b;
    return (x > y) - (x < y);
}

/* The connection map of the state: the static BOND/CONSTRAINT bits of the sparse
   rows, and for every formed hydrogen bond i -> j (hb_bond) the bits HBEvent sets:
   map[i][j] |= HB, map[i][nb(j)] |= NEIGHBOR, map[nb(j)][i] |= NEIGHBOR, with nb(j)
   j's HB neighbour (src/Events.c:320-325). */
int sdmd_write_cnt(const char *path, int append, const sdmd_system *s) {
    if (!s) return SDMD_EINVAL;
    const int N = s->n_atoms;
    /* the HB-derived entries as (row, column, bits) triples */
    int cap = 16, n_hb = 0;
    int (*hb)[3] = malloc(sizeof(int[3]) * (size_t)cap);
    if (!hb) return SDMD_ENOMEM;
    for (int i = 1; i <= N; i++) {
        const int j = s->hb_bond[i];
        if (j <= 0 || j > N) continue;
        const int nj = s->hb_neighbor[j];
        if (n_hb + 3 > cap) {
            cap *= 2;
            int (*g)[3] = realloc(hb, sizeof(int[3]) * (size_t)cap);
            if (!g) { free(hb); return SDMD_ENOMEM; }
            hb = g;
        }
        hb[n_hb][0] = i; hb[n_hb][1] = j; hb[n_hb][2] = HB_CONNECT; n_hb++;
        if (nj > 0 && nj <= N) {
            hb[n_hb][0] = i; hb[n_hb][1] = nj; hb[n_hb][2] = NEIGHBOR_CONNECT; n_hb++;
            hb[n_hb][0] = nj; hb[n_hb][1] = i; hb[n_hb][2] = NEIGHBOR_CONNECT; n_hb++;
        }
    }
    FILE *f = open_out(path, append);
    if (!f) { free(hb); return SDMD_EINVAL; }
    int *cols = malloc(sizeof(int) * ((size_t)N + 2));
    int32_t *bits = calloc((size_t)N + 2, sizeof(int32_t));
    if (!cols || !bits) { fclose(f); free(hb); free(cols); free(bits); return SDMD_ENOMEM; }
    fprintf(f, "Frame=%.2lf\n", s->time);
    for (int i = 1; i <= N; i++) {
        int nc = 0;
        for (int q = s->conn_off[i]; q < s->conn_off[i + 1]; q++) {
            const int n = s->conn_j[q];
            if (n < 1 || n > N) continue;
            if (!bits[n]) cols[nc++] = n;
            bits[n] |= s->conn_bits[q] & (BOND_CONNECT | CONSTRAINT_CONNECT);
        }
        for (int k = 0; k < n_hb; k++) {
            if (hb[k][0] != i) continue;
            const int n = hb[k][1];
            if (!bits[n]) cols[nc++] = n;
            bits[n] |= hb[k][2];
        }
        qsort(cols, (size_t)nc, sizeof(int), cmp_int);
        for (int k = 0; k < nc; k++) {
            if (bits[cols[k]] > 0) fprintf(f, "%i %i ", cols[k], bits[cols[k]]);
            bits[cols[k]] = 0;
        }
        fprintf(f, "\n");
    }
    free(hb); free(cols); free(bits);
    return close_out(f);
}

int sdmd_write_hbn(const char *path, int append, const sdmd_system *s) {
    if (!s) return SDMD_EINVAL;
    FILE *f = open_out(path, append);
    if (!f) return SDMD_EINVAL;
    fprintf(f, "%5.2lf%10i%10i\n", s->time, s->counters.hb_formed, s->counters.alpha_hb_formed);
    return close_out(f);
}

/* ---- SysInfo.dat (SaveSysInfo, src/DataSave.c:280-331) ----------------------------
 * The reference's records as it lays them out (LP64), pointer fields included: a
 * reader follows its lists while the stored pointer is non-NULL (the analysis
 * tools' SystemInformation.c), so a list continues exactly where the reference's
 * pointer was non-NULL.  The addresses themselves are the writing process's; here
 * a present link is written as 1. */
typedef struct { int32_t atomNum, proteinNum, aminoacidNum; } si_seq;
typedef struct {
    char name[8], extraProperty[2][16], nameofAA[8];
    int32_t num, typeofAtom, typeofAA;
    double charge, mass, color[3];
    si_seq sequence;
    uint64_t bond, constr;
} si_property;
typedef struct { int32_t connection; double dmin; uint64_t step; double dmax; uint64_t next; } si_constr;
typedef struct { double d, e, accumulated; uint64_t next; } si_step;
typedef struct { int32_t bondConnection, neighbor; char role; int32_t interactionType; } si_hb;
typedef struct { char nameofAA[5]; int32_t type, startAtomNum, endAtomNum, proteinNum; double mass; } si_aa;
typedef struct { int32_t startAtomNum, endAtomNum, startAANum, endAANum; double mass; } si_pep;
_Static_assert(sizeof(si_property) == 136, "PropertyStr layout");
_Static_assert(sizeof(si_constr) == 40, "ConstraintStr layout");
_Static_assert(sizeof(si_step) == 32, "StepPotenStr layout");
_Static_assert(sizeof(si_hb) == 16, "HBStr layout");
_Static_assert(sizeof(si_aa) == 32, "AAStr layout");
_Static_assert(sizeof(si_pep) == 24, "PepStr layout");

#define NATOMTYPE 32   /* src/DMD.h:29: the tables SaveSysInfo writes are [NATOMTYPE][NATOMTYPE] */

static int write_steps(FILE *f, const double *d, const double *e, const double *acc, int off, int n) {
    int ok = 1;
    for (int q = 0; q < n; q++) {
        si_step st;
        memset(&st, 0, sizeof st);
        st.d = d[off + q]; st.e = e[off + q]; st.accumulated = acc[off + q]; st.next = q + 1 < n;
        ok &= fwrite(&st, sizeof st, 1, f) == 1;
    }
    return ok;
}

/* one pair-table entry (a ConstraintStr of potentialPairCollision / potentialPairHB) */
static int write_pair_entry(FILE *f, const sdmd_system *s, int table, int a, int c) {
    si_constr e;
    memset(&e, 0, sizeof e);
    int off = 0, n = 0;
    if (table >= 0) {
        const int idx = (table * SDMD_NTYPES + a) * SDMD_NTYPES + c;
        e.dmin = s->pair_dmin[idx]; e.dmax = s->pair_dmax[idx];
        off = s->pair_step_off[idx]; n = s->pair_step_n[idx];
        e.step = n > 0;
    }
    return fwrite(&e, sizeof e, 1, f) == 1 && write_steps(f, s->pair_step_d, s->pair_step_e, s->pair_step_acc, off, n);
}

int sdmd_write_sysinfo(const char *path, const sdmd_host_system *h) {
    if (!path || !h) return SDMD_EINVAL;
    const sdmd_system *s = sdmd_host_view((sdmd_host_system *)h);
    sdmd_host_static st;
    sdmd_host_static_info(h, &st);
    FILE *f = fopen(path, "wb");
    if (!f) return SDMD_EINVAL;
    const int N = s->n_atoms;
    int ok = fwrite(&s->n_atoms, 4, 1, f) == 1 && fwrite(&st.n_prot, 4, 1, f) == 1 && fwrite(&st.n_aa, 4, 1, f) == 1;
    for (int k = 0; ok && k <= st.n_aa; k++) {
        si_aa a;
        memset(&a, 0, sizeof a);
        if (k > 0) {
            memcpy(a.nameofAA, st.aa_name + 8 * (size_t)k, 4);
            a.type = st.aa_type[k]; a.startAtomNum = st.aa_start[k]; a.endAtomNum = st.aa_end[k];
            a.proteinNum = st.aa_prot[k]; a.mass = st.aa_mass[k];
        }
        ok = fwrite(&a, sizeof a, 1, f) == 1;
    }
    for (int k = 0; ok && k <= st.n_prot; k++) {
        si_pep p;
        memset(&p, 0, sizeof p);
        if (k > 0) {
            p.startAtomNum = st.pep_start[k]; p.endAtomNum = st.pep_end[k];
            p.startAANum = st.pep_aa_start[k]; p.endAANum = st.pep_aa_end[k]; p.mass = st.pep_mass[k];
        }
        ok = fwrite(&p, sizeof p, 1, f) == 1;
    }
    for (int i = 0; ok && i <= N; i++) {
        si_property P;
        memset(&P, 0, sizeof P);
        memcpy(P.extraProperty, st.ext + 32 * (size_t)i, 32);
        P.mass = s->mass[i]; P.typeofAtom = s->type[i];
        const int nb = s->bond_off[i + 1] - s->bond_off[i], nc = s->con_off[i + 1] - s->con_off[i];
        if (i > 0) {
            memcpy(P.name, st.names + 8 * (size_t)i, 8);
            P.name[7] = 0;
            memcpy(P.nameofAA, st.resnames + 8 * (size_t)i, 8);
            P.nameofAA[7] = 0;
            P.num = i; P.typeofAA = s->aatype[i]; P.charge = st.charge[i];
            P.sequence.atomNum = i; P.sequence.proteinNum = s->protein[i]; P.sequence.aminoacidNum = s->aanum[i];
            P.bond = nb > 0; P.constr = nc > 0;
        }
        ok = fwrite(&P, sizeof P, 1, f) == 1;
        for (int q = 0; ok && i > 0 && q < nc; q++) {   /* the constraint list, in list order */
            const int k = s->con_off[i] + q;
            si_constr e;
            memset(&e, 0, sizeof e);
            e.connection = s->con_j[k]; e.dmin = s->con_dmin[k]; e.dmax = s->con_dmax[k];
            e.step = s->con_step_n[k] > 0; e.next = q + 1 < nc;
            ok = fwrite(&e, sizeof e, 1, f) == 1 &&
                 write_steps(f, s->con_step_d, s->con_step_e, s->con_step_acc, s->con_step_off[k], s->con_step_n[k]);
        }
        si_hb hb;
        memset(&hb, 0, sizeof hb);
        if (i > 0) {
            hb.bondConnection = s->hb_bond[i]; hb.neighbor = s->hb_neighbor[i];
            hb.role = (char)s->hb_role[i]; hb.interactionType = s->hb_itype[i];
        }
        ok = ok && fwrite(&hb, sizeof hb, 1, f) == 1;
    }
    ok = ok && fwrite(st.hbpot, 8, 6, f) == 6;
    for (int a = 0; ok && a < NATOMTYPE; a++)
        for (int c = 0; ok && c < NATOMTYPE; c++) ok = write_pair_entry(f, s, 0, a, c);
    /* potentialPairHB[0..10] (SaveSysInfo's loop, src/DataSave.c:314-327): table 0
       is never filled, so it is written empty */
    for (int t = 0; ok && t < 11; t++)
        for (int a = 0; ok && a < NATOMTYPE; a++)
            for (int c = 0; ok && c < NATOMTYPE; c++) ok = write_pair_entry(f, s, t == 0 ? -1 : t, a, c);
    if (fclose(f) != 0) ok = 0;
    return ok ? SDMD_OK : SDMD_EINVAL;
}

/* SaveLog (src/DataSave.c:333-462) for the engine's configurations: no coarse
   graining, flow, obstruction, tunnel or column obstacle, no dynamic wall */
int sdmd_write_log(const char *path, const sdmd_host_system *h, const sdmd_params *p, const char *timer,
                   double old_time, uint32_t seed, double wall_dyn_size, double wall_dyn_rate) {
    return sdmd_write_log_replica(path, h, p, timer, old_time, seed, wall_dyn_size, wall_dyn_rate, NULL);
}

int sdmd_write_log_replica(const char *path, const sdmd_host_system *h, const sdmd_params *p, const char *timer,
                           double old_time, uint32_t seed, double wall_dyn_size, double wall_dyn_rate,
                           const sdmd_replica *r) {
    if (!path || !h || !p) return SDMD_EINVAL;
    const sdmd_system *s = sdmd_host_view((sdmd_host_system *)h);
    sdmd_host_static st;
    sdmd_host_static_info(h, &st);
    FILE *f = fopen(path, "w");
    if (!f) return SDMD_EINVAL;
    fprintf(f, "#Log file at %s\n", timer ? timer : "");
    fprintf(f, "System:\n");
    fprintf(f, "Protein Num         = %i\n", st.n_prot);
    fprintf(f, "Protein Seq         = \n");
    for (int k = 1; k <= st.n_prot; k++) {
        fprintf(f, "                    ");
        for (int n = st.pep_aa_start[k]; n <= st.pep_aa_end[k]; n++) fprintf(f, "%5s", st.aa_name + 8 * (size_t)n);
        fprintf(f, "\n");
    }
    fprintf(f, "OldTime             = %-5.2lf\n", old_time);
    fprintf(f, "TargetTime          = %-5.2lf\n", p->time);
    fprintf(f, "TargetTemperature   = %-5.2lf\n", s->temperature);
    fprintf(f, "OutputRate          = %-5.2lf\n", p->dump_rate);
    fprintf(f, "CutOffR             = %-5.2lf\n", p->cutoff);
    fprintf(f, "Method              = %s\n", p->force_field);
    fprintf(f, "ThermostatType      = %s\n", p->thermostat);
    fprintf(f, "ThermostatParameter = %-5.3lf\n", p->thermo_freq);
    fprintf(f, "CGModel             = %s, %s\n", p->cg, p->cg);
    fprintf(f, "WallExist           = %s\n", p->wall_exist);
    fprintf(f, "WallType            = %s\n", p->wall_type);
    fprintf(f, "WallDyn             = %s\n", p->wall_dyn);
    fprintf(f, "WallDynSize         = %-5.2lf\n", wall_dyn_size);
    fprintf(f, "WallDynRate         = %-5.2lf\n", wall_dyn_rate);
    fprintf(f, "OrigBoxSize         = CurtBoxSize\n");
    fprintf(f, "CurtBoxSize         = %-8.2lf%-8.2lf%-8.2lf\n", s->box[0], s->box[1], s->box[2]);
    fprintf(f, "FlowType            = %-5i\n", 0);
    fprintf(f, "                      No flow.\n");
    fprintf(f, "Obstruct            = %-5i\n", (int)p->n_obst);   /* obstObj.num */
    if (!p->n_obst) {
        fprintf(f, "                      No obstruction.\n");
    } else {
        fprintf(f, "ObstructionPosition = ");
        for (int i = 0; i < p->n_obst; i++) {
            const double *o = &p->obst_pos[3 * i];
            fprintf(f, "%.1lf%5.1lf%5.1lf", o[0], o[1], o[2]);
            if (i < p->n_obst - 1) fprintf(f, ", ");
        }
        fprintf(f, "\n");
    }
    fprintf(f, "Tunnel              = %-5i\n", 0);
    fprintf(f, "                      No tunnel.\n");
    const int columns = strcmp(p->sphobst, "no") != 0;   /* SphObstObj.mark */
    fprintf(f, "ColumnObstacles     = %-5i\n", columns);
    if (!columns) {
        fprintf(f, "                      No column.\n");
    } else {
        fprintf(f, "ColumnInfo          =");
        for (int i = 0; i < p->n_sphobst; i++) {
            const double *o = &p->sphobst_xyzr[4 * i];
            fprintf(f, "%-8.2lf%-8.2lf%-8.2lf%-8.2lf\n", o[0], o[1], o[2], o[3] * 2);
            if (i < p->n_sphobst - 1) fprintf(f, ", ");
        }
        fprintf(f, "\n");
    }
    fprintf(f, "RandomSeed          = %i\n", (int)seed);
    /* REMDInfo: the -REMD flag's values, else its initializer (src/DMD.c:126-132) */
    fprintf(f, "REMDPortNum         = %i\n", r ? (int)r->port : -1);
    fprintf(f, "REMDTemperature     = %.2lf\n", r ? r->T : -1.0);
    fprintf(f, "REMDTempSeq         = %i\n", r ? (int)r->num : -1);
    fprintf(f, "REMDOutputRate      = %i\n", r ? (int)r->output_rate : 1000);
    fprintf(f, "REMDServerName      = %.50s\n", r ? r->server : "");
    fprintf(f, "REMDExtraName       = %.50s\n", r ? r->extra : "");
    fprintf(f, "\n");
    return close_out(f);
}

int sdmd_write_series(const char *path, int append, double time, double value) {
    FILE *f = open_out(path, append);
    if (!f) return SDMD_EINVAL;
    fprintf(f, "%5.2lf    %10.4lf\n", time, value);
    return close_out(f);
}

/* SaveRE (src/DataSave.c:687-700): written after each exchange, while the
   replica's temperature is valid */
int sdmd_write_remd(const char *path, int append, double time, double T, int32_t num) {
    FILE *f = open_out(path, append);
    if (!f) return SDMD_EINVAL;
    if (T > 0) fprintf(f, "%5.2f %8.4lf %2i\n", time, T, (int)num);
    return close_out(f);
}
