/*
 * sdmd_ref_bridge.c -- the reference's globals <-> an engine sdmd_system.
 *
 * Compiled inside the reference (gcc -I<sDMD>/src -I<this repo>/include): it
 * includes the reference's DMD.h and reads its data structures as they are
 * (src/DMD.h:231-466): 1-based atom[] with PropertyStr / DynamicStr, the linked
 * bond and constraint lists, the (N+1)^2 connectionMap, the pair tables
 * potentialPairCollision / potentialPairHB, the celllist array.
 */
#include "DMD.h"
#include "sdmd_bridge.h"

#include <stdint.h>
#include <stdlib.h>
#include <string.h>

struct sdmd_bridge {
    void *blocks[64];
    int n, failed;
};

/* zeroed arrays owned by the bridge; a failed allocation is remembered and checked
   before the arrays are written */
static void *take(sdmd_bridge *b, size_t bytes) {
    void *p = b->n < 64 ? calloc(1, bytes ? bytes : 1) : NULL;
    if (p) b->blocks[b->n++] = p;
    else b->failed = 1;
    return p;
}

void sdmd_bridge_free(sdmd_bridge *b) {
    if (!b) return;
    for (int k = 0; k < b->n; k++) free(b->blocks[k]);
    free(b);
}

/* glibc keeps rand()'s TYPE_3 table behind a header word 5 * rear + 3; initstate()
   returns the previous state with that header written, setstate() switches to a
   buffer in the same format */
#define GLIBC_MAX_TYPES 5
#define GLIBC_TYPE_3 3
static int32_t g_rand_buf[32];

int sdmd_bridge_get_rand(sdmd_rng *r) {
    static int32_t tmp[32];
    int32_t *prev = (int32_t *)initstate(1, (char *)tmp, sizeof tmp);
    if (!prev) return SDMD_EINVAL;
    const int32_t head = prev[0];
    if (head % GLIBC_MAX_TYPES != GLIBC_TYPE_3) { setstate((char *)prev); return SDMD_EUNSUPPORTED; }
    for (int k = 0; k < 31; k++) r->tab[k] = prev[1 + k];
    r->rear = head / GLIBC_MAX_TYPES;
    r->front = (r->rear + 3) % 31;
    setstate((char *)prev);
    return SDMD_OK;
}

int sdmd_bridge_set_rand(const sdmd_rng *r) {
    if (r->rear < 0 || r->rear >= 31 || r->front != (r->rear + 3) % 31) return SDMD_EINVAL;
    g_rand_buf[0] = GLIBC_MAX_TYPES * r->rear + GLIBC_TYPE_3;
    for (int k = 0; k < 31; k++) g_rand_buf[1 + k] = r->tab[k];
    return setstate((char *)g_rand_buf) ? SDMD_OK : SDMD_EINVAL;
}

static int name_code(const char *name) { return !strcmp(name, "H") ? 1 : (!strcmp(name, "O") ? 2 : 0); }

int sdmd_bridge_fill(sdmd_system *s, sdmd_bridge **owner) {
    if (!s || !owner) return SDMD_EINVAL;
    const int N = atomnum;
    const size_t N1 = (size_t)N + 1;
    for (int i = 1; i <= N; i++)
        if (!strcmp(atom[i].property->extraProperty[1], "_CONS")) return SDMD_EUNSUPPORTED;
    int wall_kind = SDMD_WALL_NONE;
    if (!strcmp(wallExist, "smooth")) {
        if (!strcmp(wallType, "parallel")) wall_kind = SDMD_WALL_PARALLEL;
        else if (!strcmp(wallType, "cylinder")) wall_kind = SDMD_WALL_CYLINDER;
        else if (!strcmp(wallType, "sphere")) wall_kind = SDMD_WALL_SPHERE;
        else return SDMD_EUNSUPPORTED;
    } else if (strcmp(wallExist, "no")) {
        return SDMD_EUNSUPPORTED;
    }
    /* outside the engine: tunnels (and so obstructions with holes), flow, CG models,
       dynamic walls */
    if (tunlObj.mark || flow.mark || CG.mark || strcmp(wallDyn.mark, "no") ||
        (SphObstObj.mark && (SphObstObj.num < 0 || SphObstObj.num > SDMD_MAX_SPHOBST)) ||
        (obstObj.mark && (obstObj.num < 0 || obstObj.num > SDMD_MAX_OBST)))
        return SDMD_EUNSUPPORTED;
    sdmd_bridge *b = calloc(1, sizeof *b);
    if (!b) return SDMD_ENOMEM;
    memset(s, 0, sizeof *s);
    s->n_atoms = N;
    for (int d = 0; d < 3; d++) {
        s->cellnum[d] = cellnum[d + 1];
        s->box[d] = boxDimension[d + 1];
        s->cellsize[d] = cellsize[d + 1];
    }
    s->cutoff = cutoffr;
    s->temperature = targetTemperature;
    s->thermo_freq = thermoF;
    s->t_end = timestep;
    s->thermostat = strcmp(thermostatType, "no") ? 1 : 0;
    s->wall = wall_kind;
    if (wall_kind != SDMD_WALL_NONE) {
        for (int d = 0; d < 3; d++) {
            s->wall_pos[d] = wall[0].dynamic->coordinate[d + 1];
            s->wall_vel[d] = wall[0].dynamic->velocity[d + 1];
        }
        s->wall_type = wall[0].property->typeofAtom;
        s->wall_mass = wall[0].property->mass;
    }
    s->hb_barrier[0] = HBPotential.BB_v;
    s->hb_barrier[1] = HBPotential.BS_v;
    s->hb_barrier[2] = HBPotential.SS_v;

#define T(type, n) ((type *)take(b, sizeof(type) * (size_t)(n)))
    if (obstObj.mark && obstObj.num > 0) {   /* obstruction walls: position[1..3] each */
        double *ob = T(double, 3 * (size_t)obstObj.num);
        for (int k = 0; k < obstObj.num; k++)
            for (int d = 0; d < 3; d++) ob[3 * k + d] = obstObj.position[k][d + 1];
        s->n_obst = obstObj.num;
        s->obst = ob;
        if (wall_kind == SDMD_WALL_NONE) s->wall_type = obstObj.obst[0].property->typeofAtom;
    }
    if (SphObstObj.mark) {   /* spherical obstacles: x, y, z, radius each */
        double *sph = T(double, 4 * (size_t)SphObstObj.num);
        for (int k = 0; k < SphObstObj.num; k++) {
            for (int d = 0; d < 3; d++) sph[4 * k + d] = SphObstObj.position[k][d + 1];
            sph[4 * k + 3] = SphObstObj.radius[k];
        }
        s->n_sphobst = SphObstObj.num;
        s->sphobst = sph;
    }
    double *mass = T(double, N1);
    int32_t *protein = T(int32_t, N1), *aanum = T(int32_t, N1), *aatype = T(int32_t, N1);
    int32_t *hb_neighbor = T(int32_t, N1), *hb_role = T(int32_t, N1), *ncode = T(int32_t, N1);
    double *x = T(double, N1), *y = T(double, N1), *z = T(double, N1);
    double *vx = T(double, N1), *vy = T(double, N1), *vz = T(double, N1);
    int32_t *cx = T(int32_t, N1), *cy = T(int32_t, N1), *cz = T(int32_t, N1), *type = T(int32_t, N1);
    int32_t *hb_bond = T(int32_t, N1), *hb_itype = T(int32_t, N1), *nbp = T(int32_t, 4 * N1);
    int32_t *nbs = T(int32_t, N1), *nbn = T(int32_t, N1);
    double *ev_time = T(double, N1), *ev_pot = T(double, N1);
    int32_t *ev_partner = T(int32_t, N1), *ev_type = T(int32_t, N1), *ev_sub = T(int32_t, N1);
    int64_t *ev_counter = T(int64_t, N1), *ev_pcounter = T(int64_t, N1);
    const long ncell = (long)cellnum[1] * cellnum[2] * cellnum[3];
    int32_t *cell_list = T(int32_t, N1 + (size_t)ncell);
    if (b->failed) { sdmd_bridge_free(b); return SDMD_ENOMEM; }
    for (int i = 0; i <= N; i++) {
        const struct PropertyStr *P = atom[i].property;
        const struct DynamicStr *D = atom[i].dynamic;
        mass[i] = P->mass;
        type[i] = P->typeofAtom;
        ev_time[i] = D->event.time;
        ev_partner[i] = D->event.partner;
        if (i == 0) continue;   /* atom 0 is unused by the loop; its mass and type are kept */
        protein[i] = P->sequence.proteinNum;
        aanum[i] = P->sequence.aminoacidNum;
        aatype[i] = P->typeofAA;
        hb_neighbor[i] = D->HB.neighbor;
        hb_role[i] = D->HB.role;
        ncode[i] = name_code(P->name);
        x[i] = D->coordinate[1]; y[i] = D->coordinate[2]; z[i] = D->coordinate[3];
        vx[i] = D->velocity[1]; vy[i] = D->velocity[2]; vz[i] = D->velocity[3];
        cx[i] = D->cellIndex[1]; cy[i] = D->cellIndex[2]; cz[i] = D->cellIndex[3];
        hb_bond[i] = D->HB.bondConnection;
        hb_itype[i] = (int32_t)D->HB.interactionType;
        for (int q = 0; q < 4; q++) nbp[4 * i + q] = D->HBNeighbor.neighborPartner[q + 1];
        nbs[i] = D->HBNeighbor.neighborStatus;
        nbn[i] = D->HBNeighbor.partnerNum;
        ev_counter[i] = D->event.counter;
        ev_pcounter[i] = D->event.partnerCounter;
        ev_pot[i] = D->event.potential;
        ev_type[i] = (int32_t)D->event.eventType;
        ev_sub[i] = (int32_t)D->event.subEventType;
    }
    memcpy(cell_list, celllist, sizeof(int32_t) * (N1 + (size_t)ncell));

    /* bond and constraint lists in linked-list order, CSR over atoms */
    int nb = 0, nc = 0, ns = 0;
    for (int i = 1; i <= N; i++) {
        for (const struct ConstraintStr *c = atom[i].property->bond; c; c = c->next) nb++;
        for (const struct ConstraintStr *c = atom[i].property->constr; c; c = c->next) {
            nc++;
            for (const struct StepPotenStr *st = c->step; st; st = st->next) ns++;
        }
    }
    int32_t *bond_off = T(int32_t, N1 + 1), *bond_j = T(int32_t, nb);
    double *bond_dmin = T(double, nb), *bond_dmax = T(double, nb);
    int32_t *con_off = T(int32_t, N1 + 1), *con_j = T(int32_t, nc), *con_so = T(int32_t, nc), *con_sn = T(int32_t, nc);
    double *con_dmin = T(double, nc), *con_dmax = T(double, nc);
    double *csd = T(double, ns), *cse = T(double, ns), *csa = T(double, ns);
    if (b->failed) { sdmd_bridge_free(b); return SDMD_ENOMEM; }
    int kb = 0, kc = 0, ks = 0;
    for (int i = 1; i <= N; i++) {
        bond_off[i] = kb;
        for (const struct ConstraintStr *c = atom[i].property->bond; c; c = c->next) {
            bond_j[kb] = c->connection; bond_dmin[kb] = c->dmin; bond_dmax[kb] = c->dmax; kb++;
        }
        con_off[i] = kc;
        for (const struct ConstraintStr *c = atom[i].property->constr; c; c = c->next) {
            con_j[kc] = c->connection; con_dmin[kc] = c->dmin; con_dmax[kc] = c->dmax;
            con_so[kc] = ks; con_sn[kc] = 0;
            for (const struct StepPotenStr *st = c->step; st; st = st->next) {
                csd[ks] = st->d; cse[ks] = st->e; csa[ks] = st->accumulated; ks++; con_sn[kc]++;
            }
            kc++;
        }
    }
    bond_off[N + 1] = kb; con_off[N + 1] = kc;

    /* BOND / CONSTRAINT bits of the dense connection map as sparse rows (rows 0..N,
       ascending partner) */
    long nn = 0;
    for (int i = 0; i <= N; i++)
        for (int j = 0; j <= N; j++)
            if (connectionMap[i][j] & (BOND_CONNECT | CONSTRAINT_CONNECT)) nn++;
    int32_t *conn_off = T(int32_t, N1 + 1), *conn_j = T(int32_t, nn), *conn_bits = T(int32_t, nn);
    if (b->failed) { sdmd_bridge_free(b); return SDMD_ENOMEM; }
    long kn = 0;
    for (int i = 0; i <= N; i++) {
        conn_off[i] = (int32_t)kn;
        for (int j = 0; j <= N; j++) {
            const int bits = connectionMap[i][j] & (BOND_CONNECT | CONSTRAINT_CONNECT);
            if (bits) { conn_j[kn] = j; conn_bits[kn] = bits; kn++; }
        }
    }
    conn_off[N + 1] = (int32_t)kn;

    /* pair tables: table 0 potentialPairCollision, 1..11 potentialPairHB */
    const int NTY = NATOMTYPE + 1;
    const size_t NT3 = (size_t)SDMD_NTABLES * SDMD_NTYPES * SDMD_NTYPES;
    long np = 0;
    for (int t = 0; t < SDMD_NTABLES; t++)
        for (int a = 0; a < NTY; a++)
            for (int c = 0; c < NTY; c++) {
                const struct ConstraintStr *e = t == 0 ? &potentialPairCollision[a][c] : &potentialPairHB[t][a][c];
                for (const struct StepPotenStr *st = e->step; st; st = st->next) np++;
            }
    double *pdmin = T(double, NT3), *pdmax = T(double, NT3);
    int32_t *pso = T(int32_t, NT3), *psn = T(int32_t, NT3);
    double *psd = T(double, np), *pse = T(double, np), *psa = T(double, np);
    if (b->failed) { sdmd_bridge_free(b); return SDMD_ENOMEM; }
    long kp = 0;
    for (int t = 0; t < SDMD_NTABLES; t++)
        for (int a = 0; a < NTY; a++)
            for (int c = 0; c < NTY; c++) {
                const struct ConstraintStr *e = t == 0 ? &potentialPairCollision[a][c] : &potentialPairHB[t][a][c];
                const size_t idx = ((size_t)t * NTY + a) * NTY + c;
                pdmin[idx] = e->dmin; pdmax[idx] = e->dmax; pso[idx] = (int32_t)kp; psn[idx] = 0;
                for (const struct StepPotenStr *st = e->step; st; st = st->next) {
                    psd[kp] = st->d; pse[kp] = st->e; psa[kp] = st->accumulated; kp++; psn[idx]++;
                }
            }
#undef T
    s->n_bonds = nb; s->n_cons = nc; s->n_con_steps = ns; s->n_conn = (int32_t)kn; s->n_pair_steps = (int32_t)np;
    s->mass = mass; s->protein = protein; s->aanum = aanum; s->aatype = aatype;
    s->hb_neighbor = hb_neighbor; s->hb_role = hb_role; s->name_code = ncode;
    s->bond_off = bond_off; s->bond_j = bond_j; s->bond_dmin = bond_dmin; s->bond_dmax = bond_dmax;
    s->con_off = con_off; s->con_j = con_j; s->con_step_off = con_so; s->con_step_n = con_sn;
    s->con_dmin = con_dmin; s->con_dmax = con_dmax; s->con_step_d = csd; s->con_step_e = cse; s->con_step_acc = csa;
    s->conn_off = conn_off; s->conn_j = conn_j; s->conn_bits = conn_bits;
    s->pair_dmin = pdmin; s->pair_dmax = pdmax; s->pair_step_off = pso; s->pair_step_n = psn;
    s->pair_step_d = psd; s->pair_step_e = pse; s->pair_step_acc = psa;
    s->x = x; s->y = y; s->z = z; s->vx = vx; s->vy = vy; s->vz = vz;
    s->cx = cx; s->cy = cy; s->cz = cz; s->type = type;
    s->hb_bond = hb_bond; s->hb_itype = hb_itype; s->nb_partner = nbp; s->nb_status = nbs; s->nb_pnum = nbn;
    s->ev_time = ev_time; s->ev_partner = ev_partner; s->ev_counter = ev_counter; s->ev_pcounter = ev_pcounter;
    s->ev_potential = ev_pot; s->ev_type = ev_type; s->ev_sub = ev_sub;
    s->cell_list = cell_list;
    s->time = currenttime;
    s->counters.frame = frame;
    s->counters.recal = countReCal;
    s->counters.collision = collisioneventsum;
    s->counters.bond = bondeventsum;
    s->counters.hb = HBeventsum;
    s->counters.hbneighbor = HBNeighboreventsum;
    s->counters.thermostat = thermostateventsum;
    s->counters.pcc = pbcandcrosseventsum;
    s->counters.wall = walleventsum;
    s->counters.warnings = warningsum;
    s->counters.hb_formed = HBnumformed;
    s->counters.alpha_hb_formed = alphaHBformed;
    int r = sdmd_bridge_get_rand(&s->rng);
    if (r) { sdmd_bridge_free(b); return r; }
    *owner = b;
    return SDMD_OK;
}

/* the HB / NEIGHBOR bits HBEvent keeps for a formed bond i - j (src/Events.c:320-325) */
static void hb_bits(int i, int j, int on) {
    const int ni = atom[i].dynamic->HB.neighbor, nj = atom[j].dynamic->HB.neighbor;
    if (on) {
        connectionMap[i][j] |= HB_CONNECT; connectionMap[j][i] |= HB_CONNECT;
        connectionMap[i][nj] |= NEIGHBOR_CONNECT; connectionMap[nj][i] |= NEIGHBOR_CONNECT;
        connectionMap[j][ni] |= NEIGHBOR_CONNECT; connectionMap[ni][j] |= NEIGHBOR_CONNECT;
    } else {
        connectionMap[i][j] &= ~HB_CONNECT; connectionMap[j][i] &= ~HB_CONNECT;
        connectionMap[i][nj] &= ~NEIGHBOR_CONNECT; connectionMap[nj][i] &= ~NEIGHBOR_CONNECT;
        connectionMap[j][ni] &= ~NEIGHBOR_CONNECT; connectionMap[ni][j] &= ~NEIGHBOR_CONNECT;
    }
}

int sdmd_bridge_readback(const sdmd_system *s) {
    if (!s || s->n_atoms != atomnum) return SDMD_EINVAL;
    if (s->cellnum[0] != cellnum[1] || s->cellnum[1] != cellnum[2] || s->cellnum[2] != cellnum[3]) return SDMD_EINVAL;
    const int N = atomnum;
    /* the bits of the bonds formed now are cleared, then those of the new state set */
    for (int i = 1; i <= N; i++) {
        const int j = atom[i].dynamic->HB.bondConnection;
        if (j > 0 && j <= N) hb_bits(i, j, 0);
    }
    for (int i = 1; i <= N; i++) {
        struct DynamicStr *D = atom[i].dynamic;
        D->coordinate[1] = s->x[i]; D->coordinate[2] = s->y[i]; D->coordinate[3] = s->z[i];
        D->velocity[1] = s->vx[i]; D->velocity[2] = s->vy[i]; D->velocity[3] = s->vz[i];
        D->cellIndex[1] = s->cx[i]; D->cellIndex[2] = s->cy[i]; D->cellIndex[3] = s->cz[i];
        atom[i].property->typeofAtom = s->type[i];
        D->HB.bondConnection = s->hb_bond[i];
        D->HB.interactionType = (enum EHBEventType)s->hb_itype[i];
        for (int q = 0; q < 4; q++) D->HBNeighbor.neighborPartner[q + 1] = s->nb_partner[4 * i + q];
        D->HBNeighbor.neighborStatus = s->nb_status[i];
        D->HBNeighbor.partnerNum = s->nb_pnum[i];
        D->event.time = s->ev_time[i];
        D->event.partner = s->ev_partner[i];
        D->event.counter = (long)s->ev_counter[i];
        D->event.partnerCounter = (long)s->ev_pcounter[i];
        D->event.potential = s->ev_potential[i];
        D->event.eventType = (enum EEventType)s->ev_type[i];
        D->event.subEventType = (enum EInteractionType)s->ev_sub[i];
    }
    for (int i = 1; i <= N; i++) {
        const int j = s->hb_bond[i];
        if (j > 0 && j <= N) hb_bits(i, j, 1);
    }
    const long ncell = (long)cellnum[1] * cellnum[2] * cellnum[3];
    memcpy(celllist, s->cell_list, sizeof(int) * ((size_t)N + 1 + (size_t)ncell));
    currenttime = s->time;
    frame = s->counters.frame;
    countReCal = s->counters.recal;
    collisioneventsum = s->counters.collision;
    bondeventsum = s->counters.bond;
    HBeventsum = s->counters.hb;
    HBNeighboreventsum = s->counters.hbneighbor;
    thermostateventsum = s->counters.thermostat;
    pbcandcrosseventsum = s->counters.pcc;
    walleventsum = s->counters.wall;
    warningsum = s->counters.warnings;
    HBnumformed = s->counters.hb_formed;
    alphaHBformed = s->counters.alpha_hb_formed;
    return sdmd_bridge_set_rand(&s->rng);
}
