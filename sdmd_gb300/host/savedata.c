/*
 * savedata.c -- the reference's checkpoint file, savedData.dat, read and written
 * from an engine system.
 *
 * The file is a raw dump of the reference's globals and structs in its own
 * order (SaveDAT, src/DataSave.c:512-585; read back by ReadBreakPoint,
 * src/Initialization.c:360-509).  The record types below mirror the reference's
 * structs member for member (src/DMD.h:231-466) so that the LP64 compiler lays
 * them out the same way on x86-64 and aarch64 (PropertyStr 136 bytes,
 * DynamicStr 176, AAStr 32, PepStr 24, REMDStr 128).
 *
 * Reading keeps every record of the file; sdmd_saved_apply writes the state a
 * continue run starts from into a system built from the same inputs, and
 * sdmd_saved_write writes an engine system's state in the file's layout, with the
 * static records (atom properties, residue and peptide tables, the dense
 * connection map's BOND/CONSTRAINT bits, parameters) of a file read before.
 */
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "sdmd_host.h"
#include "host_static.h"

typedef struct { int32_t atomNum, proteinNum, aminoacidNum; } sv_seq;
typedef struct {
    char name[8];
    char extraProperty[2][16];
    char nameofAA[8];
    int32_t num, typeofAtom, typeofAA;
    double charge, mass, color[3];
    sv_seq sequence;
    void *bond, *constr;          /* pointers of the writing process: ignored on reading */
} sv_property;
typedef struct { int32_t bondConnection, neighbor; char role; int32_t interactionType; } sv_hb;
typedef struct { int32_t neighborPartner[5], partnerNum, neighborStatus; } sv_hbnb;
typedef struct {
    int32_t partner;
    long counter, partnerCounter;
    double time, potential;
    int32_t eventType, subEventType;
} sv_event;
typedef struct {
    int32_t cellIndex[4];
    double coordinate[4], velocity[4];
    sv_hb HB;
    sv_hbnb HBNeighbor;
    sv_event event;
} sv_dynamic;
typedef struct { char nameofAA[5]; int32_t type, startAtomNum, endAtomNum, proteinNum; double mass; } sv_aa;
typedef struct { int32_t startAtomNum, endAtomNum, startAANum, endAANum; double mass; } sv_pep;
typedef struct { int32_t num; double T; } sv_remdT;
typedef struct {
    int32_t flag, REMD_PortNum, REMD_OutputRate;
    char REMD_ServerName[50], REMD_ExtraName[50];
    sv_remdT REMD_Temperature;
} sv_remd;

_Static_assert(sizeof(sv_property) == 136, "PropertyStr layout");
_Static_assert(sizeof(sv_dynamic) == 176, "DynamicStr layout");
_Static_assert(sizeof(sv_aa) == 32, "AAStr layout");
_Static_assert(sizeof(sv_pep) == 24, "PepStr layout");
_Static_assert(sizeof(sv_remd) == 128, "REMDStr layout");
_Static_assert(sizeof(long) == 8, "LP64");

void sdmd_host_seed_rng(sdmd_rng *r, uint32_t seed);   /* sysbuild.c: srand(seed)'s stream */

#define HB_CONNECT 0x04         /* connection-map bits (src/DMD.h:59-63) */
#define NEIGHBOR_CONNECT 0x08

struct sdmd_saved {
    int32_t atomnum, numofprotein, totalAminoAcids;
    int32_t *cmap;              /* (N+1)^2 */
    long frame;
    double timestep, currenttime, cutoffr, temperature, outputrate;
    char method[20];
    double box[4];
    sv_aa *aa;
    sv_pep *pep;
    sv_property *prop;
    sv_dynamic *dyn;
    int32_t wd_sign, wd_touch;
    double wd_curTime, wd_origBox[4];
    long ev[7];                 /* collision, HB, bond, HB-neighbour, thermostat, PCC, wall */
    int32_t cellnum[4];
    int32_t *celllist;
    double cellsize[4];
    int32_t hb_formed, alpha_hb_formed;
    uint32_t seed;
    sv_remd remd;
};

static int fail(char *err, int len, const char *msg, const char *path) {
    if (err && len > 0) snprintf(err, (size_t)len, "%s: %s", path ? path : "", msg);
    return SDMD_EINVAL;
}

void sdmd_saved_free(sdmd_saved *s) {
    if (!s) return;
    free(s->cmap); free(s->aa); free(s->pep); free(s->prop); free(s->dyn); free(s->celllist);
    free(s);
}

/* The template of a new run's checkpoint, from the system the host library built:
   every static record as the reference's set-up leaves it (ReadCoordinate's
   property fields, CalculateMass's residue and peptide masses, the connection
   map's BOND / CONSTRAINT bits, zeroed padding, no pointers), the parameters, and
   the seed; dynamic fields come from the state at each write. */
int sdmd_saved_new(const sdmd_host_system *h, const sdmd_params *p, uint32_t seed, sdmd_saved **out, char *err,
                   int errlen) {
    if (!h || !p || !out) return SDMD_EINVAL;
    const sdmd_system *sys = sdmd_host_view((sdmd_host_system *)h);
    sdmd_host_static st;
    sdmd_host_static_info(h, &st);
    const int N = sys->n_atoms;
    const size_t N1 = (size_t)N + 1;
    sdmd_saved *s = calloc(1, sizeof *s);
    if (!s) return SDMD_ENOMEM;
    s->atomnum = N; s->numofprotein = st.n_prot; s->totalAminoAcids = st.n_aa;
    s->cmap = calloc(N1 * N1, sizeof(int32_t));
    s->aa = calloc((size_t)st.n_aa + 1, sizeof(sv_aa));
    s->pep = calloc((size_t)st.n_prot + 1, sizeof(sv_pep));
    s->prop = calloc(N1, sizeof(sv_property));
    s->dyn = calloc(N1, sizeof(sv_dynamic));
    if (!s->cmap || !s->aa || !s->pep || !s->prop || !s->dyn) { sdmd_saved_free(s); return SDMD_ENOMEM; }
    for (int i = 0; i <= N; i++)
        for (int q = sys->conn_off[i]; q < sys->conn_off[i + 1]; q++)
            s->cmap[(size_t)i * N1 + sys->conn_j[q]] = sys->conn_bits[q];
    s->timestep = p->time; s->cutoffr = p->cutoff; s->temperature = p->temperature; s->outputrate = p->dump_rate;
    memcpy(s->method, st.method, sizeof s->method);
    for (int d = 0; d < 3; d++) {
        s->box[d + 1] = sys->box[d]; s->cellnum[d + 1] = sys->cellnum[d]; s->cellsize[d + 1] = sys->cellsize[d];
    }
    for (int k = 1; k <= st.n_aa; k++) {
        memcpy(s->aa[k].nameofAA, st.aa_name + 8 * k, 4);
        s->aa[k].type = st.aa_type[k]; s->aa[k].startAtomNum = st.aa_start[k]; s->aa[k].endAtomNum = st.aa_end[k];
        s->aa[k].proteinNum = st.aa_prot[k]; s->aa[k].mass = st.aa_mass[k];
    }
    for (int k = 1; k <= st.n_prot; k++) {
        s->pep[k].startAtomNum = st.pep_start[k]; s->pep[k].endAtomNum = st.pep_end[k];
        s->pep[k].startAANum = st.pep_aa_start[k]; s->pep[k].endAANum = st.pep_aa_end[k];
        s->pep[k].mass = st.pep_mass[k];
    }
    s->prop[0].mass = st.mass0[0];
    s->prop[0].typeofAtom = st.type0[0];
    memcpy(s->prop[0].extraProperty, st.ext, 32);
    s->dyn[0].event.partner = SDMD_INVALID;   /* atom 0's event as initialised */
    s->dyn[0].event.time = SDMD_INFINIT;
    for (int i = 1; i <= N; i++) {
        sv_property *P = &s->prop[i];
        memcpy(P->name, st.names + 8 * (size_t)i, 8);
        P->name[7] = 0;
        memcpy(P->extraProperty, st.ext + 32 * (size_t)i, 32);
        memcpy(P->nameofAA, st.resnames + 8 * (size_t)i, 8);
        P->nameofAA[7] = 0;
        P->num = i; P->typeofAtom = sys->type[i]; P->typeofAA = sys->aatype[i]; P->mass = sys->mass[i];
        P->sequence.atomNum = i; P->sequence.proteinNum = sys->protein[i]; P->sequence.aminoacidNum = sys->aanum[i];
        s->dyn[i].HB.neighbor = sys->hb_neighbor[i];
        s->dyn[i].HB.role = (char)sys->hb_role[i];
        P->charge = st.charge[i];
    }
    s->cellnum[0] = N + sys->cellnum[0] * sys->cellnum[1] * sys->cellnum[2] + 1;   /* src/Initialization.c:1068 */
    s->seed = seed;
    sdmd_saved_set_replica(s, NULL);   /* a run without -REMD */
    *out = s;
    (void)err; (void)errlen;
    return SDMD_OK;
}

/* SaveWallInfo (src/DataSave.c:280-292): the smooth wall's atom record as ReadWall
   builds it (src/Initialization.c:1907-1931) -- its Wall.txt name, extra
   properties and mass, the atom type it names, residue "Wall", the position from
   the box, an invalid event -- the rest zero, as calloc leaves it */
int sdmd_write_wallinfo(const char *path, const sdmd_host_system *h) {
    if (!path || !h) return SDMD_EINVAL;
    const sdmd_system *sys = sdmd_host_view((sdmd_host_system *)h);
    if (!sys->wall) return SDMD_EINVAL;
    sdmd_host_static st;
    sdmd_host_static_info(h, &st);
    sv_property P;
    sv_dynamic D;
    memset(&P, 0, sizeof P);
    memset(&D, 0, sizeof D);
    memcpy(P.name, st.wall_name, 8);
    memcpy(P.extraProperty, st.wall_ext, 32);
    memcpy(P.nameofAA, "Wall", 5);
    P.typeofAtom = sys->wall_type;
    P.mass = sys->wall_mass;
    for (int d = 0; d < 3; d++) D.coordinate[d + 1] = sys->wall_pos[d];
    D.event.partner = SDMD_INVALID;
    D.event.subEventType = SDMD_SUB_INVALID;
    D.event.eventType = SDMD_EV_INVALID;
    FILE *f = fopen(path, "wb");
    if (!f) return SDMD_EINVAL;
    const int ok = fwrite(&P, sizeof P, 1, f) == 1 && fwrite(&D, sizeof D, 1, f) == 1;
    return fclose(f) == 0 && ok ? SDMD_OK : SDMD_EINVAL;
}

/* SaveObstInfo (src/DataSave.c:294-308): each obstruction wall's atom record as
   the reference builds it (src/Initialization.c:1981-2013) -- the Wall.txt name,
   extra properties and mass, the atom type it names, residue "Wall", the plane's
   position[1..3] (-1 off its axis), an invalid event -- the rest zero */
int sdmd_write_obstinfo(const char *path, const sdmd_host_system *h) {
    if (!path || !h) return SDMD_EINVAL;
    const sdmd_system *sys = sdmd_host_view((sdmd_host_system *)h);
    if (!sys->n_obst) return SDMD_EINVAL;
    sdmd_host_static st;
    sdmd_host_static_info(h, &st);
    FILE *f = fopen(path, "wb");
    if (!f) return SDMD_EINVAL;
    int ok = 1;
    for (int n = 0; n < sys->n_obst; n++) {
        sv_property P;
        sv_dynamic D;
        memset(&P, 0, sizeof P);
        memset(&D, 0, sizeof D);
        memcpy(P.name, st.wall_name, 8);
        memcpy(P.extraProperty, st.wall_ext, 32);
        memcpy(P.nameofAA, "Wall", 5);
        P.typeofAtom = sys->wall_type;
        P.mass = st.wall_lib_mass;
        for (int d = 0; d < 3; d++) D.coordinate[d + 1] = sys->obst[3 * n + d];
        D.event.partner = SDMD_INVALID;
        D.event.subEventType = SDMD_SUB_INVALID;
        D.event.eventType = SDMD_EV_INVALID;
        ok &= fwrite(&P, sizeof P, 1, f) == 1 && fwrite(&D, sizeof D, 1, f) == 1;
    }
    return fclose(f) == 0 && ok ? SDMD_OK : SDMD_EINVAL;
}

int sdmd_saved_set_replica(sdmd_saved *s, const sdmd_replica *r) {
    if (!s) return SDMD_EINVAL;
    memset(&s->remd, 0, sizeof s->remd);
    if (!r) {   /* REMDInfo's initializer (src/DMD.c:126-132) */
        s->remd.REMD_PortNum = -1;
        s->remd.REMD_OutputRate = 1000;
        s->remd.REMD_Temperature.num = -1;
        s->remd.REMD_Temperature.T = -1;
        return SDMD_OK;
    }
    s->remd.flag = 1;
    s->remd.REMD_PortNum = r->port;
    s->remd.REMD_OutputRate = r->output_rate;
    /* the names as sprintf leaves them in the zeroed global: text, then zeros */
    memcpy(s->remd.REMD_ServerName, r->server, strnlen(r->server, sizeof s->remd.REMD_ServerName - 1));
    memcpy(s->remd.REMD_ExtraName, r->extra, strnlen(r->extra, sizeof s->remd.REMD_ExtraName - 1));
    s->remd.REMD_Temperature.num = r->num;
    s->remd.REMD_Temperature.T = r->T;
    return SDMD_OK;
}

int sdmd_saved_replica(const sdmd_saved *s, sdmd_replica *out) {
    if (!s || !out) return SDMD_EINVAL;
    memset(out, 0, sizeof *out);
    out->port = s->remd.REMD_PortNum;
    out->output_rate = s->remd.REMD_OutputRate;
    out->num = s->remd.REMD_Temperature.num;
    out->T = s->remd.REMD_Temperature.T;
    memcpy(out->server, s->remd.REMD_ServerName, sizeof out->server);
    memcpy(out->extra, s->remd.REMD_ExtraName, sizeof out->extra);
    out->server[sizeof out->server - 1] = out->extra[sizeof out->extra - 1] = 0;
    return s->remd.flag ? 1 : 0;
}

#define RD(ptr, size, n) (fread((ptr), (size), (size_t)(n), f) == (size_t)(n))

int sdmd_saved_read(const char *path, sdmd_saved **out, char *err, int errlen) {
    if (!path || !out) return SDMD_EINVAL;
    FILE *f = fopen(path, "rb");
    if (!f) return fail(err, errlen, "cannot open", path);
    sdmd_saved *s = calloc(1, sizeof *s);
    int ok = s && RD(&s->atomnum, 4, 1) && RD(&s->numofprotein, 4, 1) && RD(&s->totalAminoAcids, 4, 1);
    if (ok) ok = s->atomnum > 0 && s->atomnum < (1 << 26) && s->numofprotein >= 0 && s->totalAminoAcids >= 0;
    if (ok) {
        const size_t N1 = (size_t)s->atomnum + 1;
        s->cmap = malloc(sizeof(int32_t) * N1 * N1);
        s->aa = calloc((size_t)s->totalAminoAcids + 1, sizeof(sv_aa));
        s->pep = calloc((size_t)s->numofprotein + 1, sizeof(sv_pep));
        s->prop = calloc(N1, sizeof(sv_property));
        s->dyn = calloc(N1, sizeof(sv_dynamic));
        ok = s->cmap && s->aa && s->pep && s->prop && s->dyn && RD(s->cmap, 4, N1 * N1) && RD(&s->frame, 8, 1) &&
             RD(&s->timestep, 8, 1) && RD(&s->currenttime, 8, 1) && RD(&s->cutoffr, 8, 1) &&
             RD(&s->temperature, 8, 1) && RD(&s->outputrate, 8, 1) && RD(s->method, 1, 20) && RD(s->box, 8, 4) &&
             RD(s->aa, sizeof(sv_aa), s->totalAminoAcids + 1) && RD(s->pep, sizeof(sv_pep), s->numofprotein + 1);
        for (size_t i = 0; ok && i < N1; i++)
            ok = RD(&s->prop[i], sizeof(sv_property), 1) && RD(&s->dyn[i], sizeof(sv_dynamic), 1);
        ok = ok && RD(&s->wd_sign, 4, 1) && RD(&s->wd_touch, 4, 1) && RD(&s->wd_curTime, 8, 1) &&
             RD(s->wd_origBox, 8, 4) && RD(s->ev, 8, 7) && RD(s->cellnum, 4, 4);
        if (ok) {
            const long long nc = (long long)s->cellnum[1] * s->cellnum[2] * s->cellnum[3];
            ok = s->cellnum[1] > 0 && s->cellnum[2] > 0 && s->cellnum[3] > 0 && nc < (1LL << 31);
            if (ok) {
                s->celllist = malloc(sizeof(int32_t) * (N1 + (size_t)nc));
                ok = s->celllist && RD(s->celllist, 4, N1 + (size_t)nc);
            }
        }
        ok = ok && RD(s->cellsize, 8, 4) && RD(&s->hb_formed, 4, 1) && RD(&s->alpha_hb_formed, 4, 1) &&
             RD(&s->seed, 4, 1) && RD(&s->remd, sizeof(sv_remd), 1);
    }
    fclose(f);
    if (!ok) {
        sdmd_saved_free(s);
        return fail(err, errlen, "truncated or not a savedData.dat of this layout", path);
    }
    *out = s;
    return SDMD_OK;
}

int sdmd_saved_info(const sdmd_saved *s, sdmd_saved_header *h) {
    if (!s || !h) return SDMD_EINVAL;
    memset(h, 0, sizeof *h);
    h->atomnum = s->atomnum;
    h->frame = s->frame;
    h->timestep = s->timestep;
    h->currenttime = s->currenttime;
    h->temperature = s->temperature;
    h->outputrate = s->outputrate;
    h->seed = s->seed;
    h->remd_flag = s->remd.flag;
    h->remd_T = s->remd.REMD_Temperature.T;
    for (int d = 0; d < 3; d++) { h->box[d] = s->box[d + 1]; h->cellnum[d] = s->cellnum[d + 1]; }
    memcpy(h->method, s->method, 20);
    h->method[19] = 0;
    return SDMD_OK;
}

int sdmd_saved_apply(const sdmd_saved *sv, sdmd_system *s, const char *names8, char *err, int errlen) {
    if (!sv || !s) return SDMD_EINVAL;
    const int N = sv->atomnum;
    if (s->n_atoms != N) return fail(err, errlen, "atom count differs from the system's", NULL);
    for (int d = 0; d < 3; d++)
        if (s->cellnum[d] != sv->cellnum[d + 1]) return fail(err, errlen, "cell grid differs from the system's", NULL);
    if (names8)
        for (int i = 1; i <= N; i++)
            if (strncmp(names8 + 8 * i, sv->prop[i].name, 8)) return fail(err, errlen, "atom names differ", NULL);
    for (int i = 1; i <= N; i++) {
        const sv_dynamic *D = &sv->dyn[i];
        s->x[i] = D->coordinate[1]; s->y[i] = D->coordinate[2]; s->z[i] = D->coordinate[3];
        s->vx[i] = D->velocity[1]; s->vy[i] = D->velocity[2]; s->vz[i] = D->velocity[3];
        s->cx[i] = D->cellIndex[1]; s->cy[i] = D->cellIndex[2]; s->cz[i] = D->cellIndex[3];
        s->type[i] = sv->prop[i].typeofAtom;
        s->hb_bond[i] = D->HB.bondConnection;
        s->hb_itype[i] = D->HB.interactionType;
        for (int q = 0; q < 4; q++) s->nb_partner[4 * i + q] = D->HBNeighbor.neighborPartner[q + 1];
        s->nb_status[i] = D->HBNeighbor.neighborStatus;
        s->nb_pnum[i] = D->HBNeighbor.partnerNum;
        s->ev_time[i] = D->event.time;
        s->ev_partner[i] = D->event.partner;
        s->ev_counter[i] = D->event.counter;
        s->ev_pcounter[i] = D->event.partnerCounter;
        s->ev_potential[i] = D->event.potential;
        s->ev_type[i] = D->event.eventType;
        s->ev_sub[i] = D->event.subEventType;
    }
    const size_t ncell = (size_t)sv->cellnum[1] * sv->cellnum[2] * sv->cellnum[3];
    memcpy(s->cell_list, sv->celllist, sizeof(int32_t) * ((size_t)N + 1 + ncell));
    s->time = sv->currenttime;
    /* ReadBreakPoint restarts rand() from the saved seed (src/Initialization.c:472-473);
       the counters it does not store start again at zero */
    sdmd_host_seed_rng(&s->rng, sv->seed);
    memset(&s->counters, 0, sizeof s->counters);
    s->counters.frame = sv->frame;
    s->counters.collision = sv->ev[0]; s->counters.hb = sv->ev[1]; s->counters.bond = sv->ev[2];
    s->counters.hbneighbor = sv->ev[3]; s->counters.thermostat = sv->ev[4]; s->counters.pcc = sv->ev[5];
    s->counters.wall = sv->ev[6];
    s->counters.hb_formed = sv->hb_formed;
    s->counters.alpha_hb_formed = sv->alpha_hb_formed;
    if (sv->remd.flag) s->temperature = sv->remd.REMD_Temperature.T;
    return SDMD_OK;
}

#define WR(ptr, size, n) (fwrite((ptr), (size), (size_t)(n), f) == (size_t)(n))

int sdmd_saved_write(const char *path, const sdmd_saved *tpl, const sdmd_system *s, char *err, int errlen) {
    if (!path || !tpl || !s) return SDMD_EINVAL;
    const int N = tpl->atomnum;
    if (s->n_atoms != N) return fail(err, errlen, "atom count differs from the template's", path);
    for (int d = 0; d < 3; d++)
        if (s->cellnum[d] != tpl->cellnum[d + 1]) return fail(err, errlen, "cell grid differs from the template's", path);
    const size_t N1 = (size_t)N + 1;
    /* the connection map: the template's bits without HB / NEIGHBOR, then those of
       the system's formed hydrogen bonds as HBEvent keeps them (src/Events.c:320-325) */
    int32_t *cmap = malloc(sizeof(int32_t) * N1 * N1);
    if (!cmap) return SDMD_ENOMEM;
    for (size_t k = 0; k < N1 * N1; k++) cmap[k] = tpl->cmap[k] & ~(HB_CONNECT | NEIGHBOR_CONNECT);
    for (int i = 1; i <= N; i++) {
        const int j = s->hb_bond[i];
        if (j <= 0 || j > N) continue;
        const int nj = tpl->dyn[j].HB.neighbor;
        cmap[(size_t)i * N1 + j] |= HB_CONNECT;
        cmap[(size_t)i * N1 + nj] |= NEIGHBOR_CONNECT;
        cmap[(size_t)nj * N1 + i] |= NEIGHBOR_CONNECT;
    }
    FILE *f = fopen(path, "wb");
    if (!f) { free(cmap); return fail(err, errlen, "cannot open for writing", path); }
    const long frame = (long)s->counters.frame;
    const double temperature = s->temperature;
    int ok = WR(&tpl->atomnum, 4, 1) && WR(&tpl->numofprotein, 4, 1) && WR(&tpl->totalAminoAcids, 4, 1) &&
             WR(cmap, 4, N1 * N1) && WR(&frame, 8, 1) && WR(&tpl->timestep, 8, 1) && WR(&s->time, 8, 1) &&
             WR(&tpl->cutoffr, 8, 1) && WR(&temperature, 8, 1) && WR(&tpl->outputrate, 8, 1) &&
             WR(tpl->method, 1, 20) && WR(tpl->box, 8, 4) && WR(tpl->aa, sizeof(sv_aa), tpl->totalAminoAcids + 1) &&
             WR(tpl->pep, sizeof(sv_pep), tpl->numofprotein + 1);
    free(cmap);
    for (int i = 0; ok && i <= N; i++) {
        sv_property P = tpl->prop[i];
        sv_dynamic D = tpl->dyn[i];     /* padding and the unused [0] entries as the template has them */
        if (i > 0) {
            P.typeofAtom = s->type[i];
            D.coordinate[1] = s->x[i]; D.coordinate[2] = s->y[i]; D.coordinate[3] = s->z[i];
            D.velocity[1] = s->vx[i]; D.velocity[2] = s->vy[i]; D.velocity[3] = s->vz[i];
            D.cellIndex[1] = s->cx[i]; D.cellIndex[2] = s->cy[i]; D.cellIndex[3] = s->cz[i];
            D.HB.bondConnection = s->hb_bond[i];
            D.HB.interactionType = s->hb_itype[i];
            for (int q = 0; q < 4; q++) D.HBNeighbor.neighborPartner[q + 1] = s->nb_partner[4 * i + q];
            D.HBNeighbor.neighborStatus = s->nb_status[i];
            D.HBNeighbor.partnerNum = s->nb_pnum[i];
            D.event.partner = s->ev_partner[i];
            D.event.counter = (long)s->ev_counter[i];
            D.event.partnerCounter = (long)s->ev_pcounter[i];
            D.event.time = s->ev_time[i];
            D.event.potential = s->ev_potential[i];
            D.event.eventType = s->ev_type[i];
            D.event.subEventType = s->ev_sub[i];
        }
        ok = WR(&P, sizeof P, 1) && WR(&D, sizeof D, 1);
    }
    const long ev[7] = {(long)s->counters.collision, (long)s->counters.hb, (long)s->counters.bond,
                        (long)s->counters.hbneighbor, (long)s->counters.thermostat, (long)s->counters.pcc,
                        (long)s->counters.wall};
    const size_t ncell = (size_t)tpl->cellnum[1] * tpl->cellnum[2] * tpl->cellnum[3];
    const int32_t hbf = s->counters.hb_formed, ahf = s->counters.alpha_hb_formed;
    ok = ok && WR(&tpl->wd_sign, 4, 1) && WR(&tpl->wd_touch, 4, 1) && WR(&tpl->wd_curTime, 8, 1) &&
         WR(tpl->wd_origBox, 8, 4) && WR(ev, 8, 7) && WR(tpl->cellnum, 4, 4) && WR(s->cell_list, 4, N1 + ncell) &&
         WR(tpl->cellsize, 8, 4) && WR(&hbf, 4, 1) && WR(&ahf, 4, 1) && WR(&tpl->seed, 4, 1) &&
         WR(&tpl->remd, sizeof(sv_remd), 1);
    if (fclose(f) != 0) ok = 0;
    return ok ? SDMD_OK : fail(err, errlen, "write failed", path);
}
