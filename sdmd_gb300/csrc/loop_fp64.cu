// loop_fp64.cu -- exact FP64 event loop: one CTA per system.
//
// Restates SingleThreadRun (src/SGThread.c:67-155) with Predict
// (src/SGThread.c:158-211), DoEvent (src/Events.c:25-114) and the CBT
// (src/CBT.c) on the GPU.  Per pop the CTA
//   1. pops the tree root (AssignJob, src/SGThread.c:237-259),
//   2. advances every atom and every event time (UpdateData/TimeForward,
//      src/ToolFunctions.c:23-36) -- all threads,
//   3. checks the hazard and executes the event -- thread 0,
//   4. predicts the target (and partner): the bonded, 27-cell collision and HB
//      candidates are gathered and evaluated by all threads, then thread 0 folds
//      them into the running minimum in the reference's scan order, which
//      reproduces JobAssign's strict "<" and CheckDuplication exactly,
//   5. repairs the tree (UpdateCBTRun, src/CBT.c:56-83) -- thread 0.
// Compiled with -fmad=false: bit-identical to the reference's FP64 results.
#include "dev.cuh"
#include "engine.h"

namespace sdmd {

// slot flags
enum : int32_t { F_DUP = 1, F_FRESH = 2 };

__host__ __device__ inline size_t al16(size_t b) { return (b + 15) & ~size_t(15); }

struct Slots {
    int32_t *j, *info;      // info: flags | sub << 8 | warnings << 16
    double *t, *tdup, *pot;
};

struct Blk {                 // block-uniform scalars in shared memory
    int32_t err, err_atom;
    int32_t nnb;
    int32_t hbmode;          // 0 skip HB, 1 bonded, 2 scan
    int64_t warn;
};

__device__ inline void set_err(Blk &B, int code, int atom) {
    if (B.err == 0) { B.err = code; B.err_atom = atom; }
}

// Helper-block side of the eager advance: wait for the next published pop, then
// x += v dt and t -= dt (UpdateData / TimeForward, src/ToolFunctions.c:23-36) for
// this block's slice of atoms, except the pop's target and partner, which the
// system's own block advances itself.  Every wait is bounded.
__device__ __noinline__ void helper_body(const DSys *systems, int n_systems) {
    const int b = blockIdx.x - n_systems, nh = gridDim.x - n_systems;
    const int s = b % n_systems, h = b / n_systems;
    const int H = (nh - s + n_systems - 1) / n_systems;    // helpers of system s
    const DSys &G = systems[s];
    const int n = G.n;
    const int a0 = 1 + (int)((long long)h * n / H), a1 = 1 + (int)((long long)(h + 1) * n / H);
    double *x = G.x, *y = G.y, *z = G.z, *et = G.ev_time;
    const double *vx = G.vx, *vy = G.vy, *vz = G.vz;
    Adv *A = G.adv;
    __shared__ double s_dt;
    __shared__ int32_t s_t, s_p, s_go;
    unsigned long long seen = 0;
    for (;;) {
        if (threadIdx.x == 0) {
            unsigned long long q;
            const unsigned long long t0 = gtimer();
            int go = 1;
            while ((q = ld_acquire(&A->seq)) == seen) {
                if (gtimer() - t0 > ADV_WAIT_NS) { atomicExch(&A->herr, 1); go = 0; break; }
                __nanosleep(100);
            }
            if (go && q == ADV_STOP) go = 0;
            if (go) {
                seen = q;
                s_dt = *(volatile double *)&A->dt;
                s_t = *(volatile int32_t *)&A->t;
                s_p = *(volatile int32_t *)&A->p;
            }
            s_go = go;
        }
        __syncthreads();
        if (!s_go) break;
        const double dt = s_dt;
        const int t = s_t, p = s_p;
        for (int i = a0 + threadIdx.x; i < a1; i += blockDim.x) {
            if (i == t || i == p) continue;
            x[i] += vx[i] * dt;
            y[i] += vy[i] * dt;
            z[i] += vz[i] * dt;
            et[i] -= dt;
        }
        __syncthreads();
        if (threadIdx.x == 0) red_release_add(&A->done, 1ull);
    }
}

// the system's block: publish this pop to the helpers
__device__ __forceinline__ void adv_publish(DSys &S, int t, int p, double dt) {
    Adv *A = S.adv;
    *(volatile double *)&A->dt = dt;
    *(volatile int32_t *)&A->t = t;
    *(volatile int32_t *)&A->p = p;
    S.adv_seq++;
    st_release(&A->seq, S.adv_seq);
}
// the system's block: wait until every helper advanced the last published pop
__device__ __noinline__ void adv_wait(const DSys &S, Blk &B) {
    const unsigned long long want = S.adv_seq * (unsigned long long)S.adv_h;
    const unsigned long long t0 = gtimer();
    while (ld_acquire(&S.adv->done) < want) {
        if (gtimer() - t0 > ADV_WAIT_NS) { set_err(B, SDMD_ETIMEOUT, 0); return; }
        __nanosleep(20);
    }
}

// lazy mode: bring the target t and the partner p (when > 0) to the current time
// before they change, x += v * (now - tloc) per axis.  Lanes 0..5 of warp 0 take
// one (atom, axis) each: the six independent FP64 chains share warp-instructions.
__device__ inline void sync_pair_warp0(const DSys &S, int t, int p) {
    const int l = threadIdx.x;
    if (!S.lazy || l >= 6) return;
    const int a = l < 3 ? t : p, d = l % 3;
    if (a > 0) {
        double *X = d == 0 ? S.x : (d == 1 ? S.y : S.z);
        const double *V = d == 0 ? S.vx : (d == 1 ? S.vy : S.vz);
        const double dt = S.now - S.tloc[a];
        X[a] = X[a] + V[a] * dt;
    }
    __syncwarp(0x3fu);                                 // every axis has read the old tloc
    if (d == 0 && a > 0) S.tloc[a] = S.now;
    __syncwarp(0x3fu);
}

// ---------------------------------------------------------------------------
// gather the 27-cell neighbourhood of atom i into nbj[] in scan order
// (27 cells in src/DMD.c:117-121 order, each list head-first: src/TimePrediction.c:60-80)
__device__ void gather(const DSys &S, int i, int32_t *nbj, int32_t *cnt, Blk &B) {
    int tid = threadIdx.x;
    int head = 0, c = 0, cell = 0;
    if (tid < 27) {
        cell = nb_cell(S, i, tid);
        if (S.cell_arr) c = S.cell_cnt[cell];   // screened path: per-cell arrays
        else {
            head = S.cell_list[S.n + cell];
            for (int a = head; a; a = S.cell_list[a]) {
                if (++c > S.n) break;   // a corrupted (cyclic) list cannot spin forever
            }
        }
        cnt[tid] = c;
    }
    __syncthreads();
    if (tid == 0) {
        int tot = 0;
        for (int k = 0; k < 27; k++) { int v = cnt[k]; cnt[k] = tot; tot += v; }
        if (tot > S.nbcap) { set_err(B, SDMD_ECAPACITY, i); tot = 0; }
        B.nnb = tot;
    }
    __syncthreads();
    if (tid < 27 && B.err == 0) {
        int o = cnt[tid], m = 0;
        if (S.cell_arr) {
            const int32_t *arr = S.cell_arr + (size_t)cell * S.maxc;
            for (; m < c; m++) nbj[o + m] = arr[c - 1 - m];
        } else {
            for (int a = head; a && m < c; a = S.cell_list[a]) nbj[o + m++] = a;
        }
    }
    __syncthreads();
}

// ---- candidate evaluation (all threads) -------------------------------------
__device__ inline void put(Slots &L, int k, int j, int info, double t, double tdup, double pot) {
    L.j[k] = j; L.info[k] = info; L.t[k] = t; L.tdup[k] = tdup; L.pot[k] = pot;
}

// BondTime, one bond (src/TimePrediction.c:217-293)
__device__ void eval_bond(const DSys &S, int i, int q, Slots &L, int k, int *bad) {
    int j = S.bond_j[q];
    int info = 0;
    double tdup = 0;
    if (j < S.dup_limit && S.ev_partner[j] == i && S.ev_type[j] == SDMD_EV_BOND && S.ev_pcounter[j] == S.ev_counter[i]) {
        info |= F_DUP; tdup = S.ev_time[j];
    }
    double lng = S.bond_dmax[q], sht = S.bond_dmin[q];
    Kin kk; pair_kin(S, i, j, kk);
    int sub; double t;
    if (kk.r2 - lng > ZERO && kk.b >= 0) { sub = SDMD_SUB_WELL_BOUNCE; t = 1e-16 * i * j; }
    else if (!(kk.r2 - lng > ZERO) && sht - kk.r2 > ZERO && kk.b < 0) { sub = SDMD_SUB_CORE; t = 1e-16 * i * j; }
    else {
        int st; double d2;
        if (kk.b < 0 && disc(kk, sht) > 0) { st = -1; d2 = sht; sub = SDMD_SUB_CORE; }
        else { st = 1; d2 = lng; sub = SDMD_SUB_WELL_BOUNCE; }
        t = root(kk, st, d2);
        if (t < 0) t = INFINIT;
    }
    put(L, k, j, info | F_FRESH | (sub << 8), t, tdup, 0.0);
}

// CollisionTime, one candidate j (src/TimePrediction.c:78-179)
__device__ void eval_collision(const DSys &S, int i, int j, double cut, Slots &L, int k, int *bad) {
    int info = 0, warn = 0, sub = SDMD_SUB_INVALID;
    double tdup = 0, t = 0, pot = 0;
    if (j == i) { put(L, k, j, -1, 0, 0, 0); return; }   // -1: not a candidate at all
    if (j < S.dup_limit && S.ev_partner[j] == i && S.ev_type[j] == SDMD_EV_COLLISION && S.ev_pcounter[j] == S.ev_counter[i]) {
        info |= F_DUP; tdup = S.ev_time[j];
    }
    int bits = conn_bits(S, i, j);
    if (!((bits & 1) || S.hb_bond[i] == j || nb_has(S, i, j))) {
        Kin kk; pair_kin(S, i, j, kk);
        if (kk.r2 <= cut) {
            Lim o; int cs; bool go = true;
            int constrained = bits & 2;
            if (constrained) {
                cs = find_pair(S, i, j, K_CONSTRAINT, kk.b, kk.r2, o, 0, 0, 0, &warn, bad);
            } else {
                cs = find_pair(S, i, j, K_COLLISION, kk.b, kk.r2, o, 0, 0, 0, &warn, bad);
                if (o.lopot == 0 && o.uppot == 0) go = false;
            }
            if (go) {
                int st; double d2;
                if (kk.b < 0 && disc(kk, o.lo) > 0) {
                    st = -1; d2 = o.lo; pot = o.lopot;
                    sub = (cs == 0) ? SDMD_SUB_CORE : SDMD_SUB_TBD_CAPTURE;
                } else {
                    st = 1; d2 = o.up; pot = o.uppot;
                    if (constrained) sub = (cs == 1) ? SDMD_SUB_WELL_BOUNCE : SDMD_SUB_TBD_ESCAPE;
                    else if (cs == 1) go = false;
                    else sub = SDMD_SUB_TBD_ESCAPE;
                }
                if (go) { t = root(kk, st, d2); info |= F_FRESH; }
            }
        }
    }
    put(L, k, j, info | (sub << 8) | (warn << 16), t, tdup, pot);
}

__device__ inline bool hb_pair_ok(const DSys &S, int i, int j) {
    int ri = S.hb_role[i], rj = S.hb_role[j];
    return (ri == 'A' && rj == 'D') || (ri == 'D' && rj == 'A') ||
           (ri == 'S' && S.type[j] == 2) || (rj == 'S' && S.type[i] == 2) || (ri == 'S' && rj == 'S');
}

// CheckPairMatch (src/TimePrediction.c:1119-1138)
__device__ int pair_match(const DSys &S, int i, int j, int *bad) {
    int t = hb_model(S, i, j, bad);
    if (t < 0) return -1;
    int ti = S.type[i], tj = S.type[j];
    if (S.pair_step_n[tab_idx(t, ti, tj)] == 0) return -1;
    int ni = type_change(S.type[S.hb_neighbor[i]], 0), nj = type_change(S.type[S.hb_neighbor[j]], 0);
    if (S.pair_step_n[tab_idx(t, ti, nj)] == 0 || S.pair_step_n[tab_idx(t, tj, ni)] == 0) return -1;
    return 0;
}

// HBTime, unbonded scan over one candidate (src/TimePrediction.c:398-479)
__device__ void eval_hb_scan(const DSys &S, int i, int j, double cut, Slots &L, int k, int *bad) {
    if (!(i != j && hb_pair_ok(S, i, j) && S.hb_bond[j] == 0 &&
          ((S.protein[i] == S.protein[j] && abs(S.aanum[i] - S.aanum[j]) >= 4) || S.protein[i] != S.protein[j]))) {
        put(L, k, j, -1, 0, 0, 0);
        return;
    }
    int info = 0, warn = 0;
    double tdup = 0, t = 0, pot = 0;
    if (j < S.dup_limit && S.ev_partner[j] == i && S.ev_type[j] == SDMD_EV_HB && S.ev_pcounter[j] == S.ev_counter[i]) {
        info |= F_DUP; tdup = S.ev_time[j];
    }
    Kin kk; pair_kin(S, i, j, kk);
    if (kk.r2 <= cut && pair_match(S, i, j, bad) >= 0) {
        Lim o;
        int cs = find_pair(S, i, j, K_HB, kk.b, kk.r2, o, 0, 0, 0, &warn, bad);
        if (kk.b < 0 && cs == 1 && disc(kk, o.lo) > 0) {
            pot = o.lopot;
            t = root(kk, -1, o.lo);
            if (t < 0) t = INFINIT;
            info |= F_FRESH;
        }
    }
    put(L, k, j, info | (SDMD_SUB_TBD_HBFORM << 8) | (warn << 16), t, tdup, pot);
}

// ---- running minimum (thread 0): JobAssign + CheckDuplication ---------------
// (src/TimePrediction.c:1140-1158, 1101-1117).  The atom's running event lives in
// thread 0's registers during a prediction and is stored once at the end.
struct Cur {
    long long key;          // tkey(time)
    double time, potential;
    int32_t partner, type, sub;
    int64_t pcounter;
};
__device__ inline void cur_load(const DSys &S, int i, Cur &c) {
    c.time = S.ev_time[i]; c.key = tkey(c.time); c.potential = S.ev_potential[i];
    c.partner = S.ev_partner[i]; c.type = S.ev_type[i]; c.sub = S.ev_sub[i]; c.pcounter = S.ev_pcounter[i];
}
__device__ inline void cur_store(const DSys &S, int i, const Cur &c) {
    S.ev_time[i] = c.time; S.ev_potential[i] = c.potential; S.ev_partner[i] = c.partner;
    S.ev_type[i] = c.type; S.ev_sub[i] = c.sub; S.ev_pcounter[i] = c.pcounter;
}
__device__ inline bool job_assign(const DSys &S, Cur &c, int j, double t, double pot, int sub, int type) {
    if (tkey(t) <= 0) return false;
    if (S.lazy) t = S.now + t;          // lazy mode keeps absolute event times
    const long long kt = tkey(t);
    if (c.key > kt) {
        c.potential = pot; c.sub = sub; c.time = t; c.key = kt; c.type = type;
        if (j) { c.partner = j; c.pcounter = S.ev_counter[j]; }
        else c.partner = INVALID;
        return true;
    }
    return false;
}
__device__ inline bool dup_assign(const DSys &S, Cur &c, int j, double tdup, int type) {
    const long long kt = tkey(tdup);
    if (c.key > kt) {
        c.partner = j; c.potential = S.ev_potential[j]; c.sub = S.ev_sub[j];
        c.time = tdup; c.key = kt; c.type = type; c.pcounter = S.ev_counter[j];
        return true;
    }
    return false;
}
__device__ void resolve(const DSys &S, Cur &c, const Slots &L, int n, int type, Blk &B) {
    for (int k = 0; k < n; k++) {
        int info = L.info[k];
        if (info < 0) continue;
        int j = L.j[k];
        if ((info & F_DUP) && dup_assign(S, c, j, L.tdup[k], type)) continue;
        B.warn += (info >> 16) & 0xff;
        if (info & F_FRESH) job_assign(S, c, j, L.t[k], L.pot[k], (info >> 8) & 0xff, type);
    }
}

// ---- scalar predictions (thread 0) -----------------------------------------
// PBCandCrossCellTime (src/TimePrediction.c:598-632): the face-crossing time of
// one dimension (computed by three threads at once; FP64 divisions are slow)
__device__ double pcc_face(const DSys &S, int i, int d) {
    const double pos = d == 0 ? S.x[i] : d == 1 ? S.y[i] : S.z[i];
    const double v = d == 0 ? S.vx[i] : d == 1 ? S.vy[i] : S.vz[i];
    const int ci = d == 0 ? S.cx[i] : d == 1 ? S.cy[i] : S.cz[i];
    double lo = ci * S.cs[d], hi = (ci + 1) * S.cs[d];
    if (v > 0) return (hi - pos + ZERO) / v;
    if (v < 0) return (lo - pos - ZERO) / v;
    return -1.0;   // no crossing in this dimension
}
__device__ void pcc_time(const DSys &S, Cur &c, const double *face) {
    double best = INFINIT;
    for (int d = 0; d < 3; d++) {
        double t = face[d];
        if (tkey(best) > tkey(t) && tkey(t) > 0) best = t;
    }
    job_assign(S, c, 0, best, 0, SDMD_SUB_INVALID, SDMD_EV_PCC);
}

// ThermostatTime (src/TimePrediction.c:582-595)
__device__ inline double take_sample(const DSys &S, DScal &C, Blk &B) {
    if (C.smp_used >= C.smp_avail) { set_err(B, SDMD_ETIMEOUT, 0); return 1.0; }   // the loop pauses before this
    return S.smp[C.smp_used++];
}

// ThermostatTime (src/TimePrediction.c:582-595): MB(0, 1) = the sample * sqrt(1) + 0
__device__ __noinline__ void thermostat_time(const DSys &S, Cur &c, DScal &C, Blk &B) {
    if (!S.thermostat) return;
    double t = take_sample(S, C, B) * sqrt(1.0) + 0;
    job_assign(S, c, 0, S.thermo_freq * (t < 0 ? -t : t), 0, SDMD_SUB_INVALID, SDMD_EV_THERMOSTAT);
}

// HBTime for an HB-bonded atom (src/TimePrediction.c:329-387)
__device__ __noinline__ void hb_bonded(const DSys &S, int i, Cur &c, Blk &B, int *bad) {
    int j = S.hb_bond[i];
    if (j < S.dup_limit && S.ev_partner[j] == i && S.ev_type[j] == SDMD_EV_HB && S.ev_pcounter[j] == S.ev_counter[i] &&
        dup_assign(S, c, j, S.ev_time[j], SDMD_EV_HB))
        return;
    Kin kk; pair_kin(S, i, j, kk);
    Lim o; int warn = 0;
    int cs = find_pair(S, i, j, K_HB, kk.b, kk.r2, o, 0, 0, 0, &warn, bad);
    B.warn += warn;
    int st, sub; double d2, pot;
    if (kk.b < 0 && disc(kk, o.lo) > 0) {
        st = -1; d2 = o.lo; pot = o.lopot; sub = (cs == 0) ? SDMD_SUB_CORE : SDMD_SUB_TBD_CAPTURE;
    } else {
        st = 1; d2 = o.up; pot = o.uppot; sub = (cs == 1) ? SDMD_SUB_TBD_HBBREAK : SDMD_SUB_TBD_ESCAPE;
    }
    double t = root(kk, st, d2);
    if (t < 0) t = INFINIT;
    job_assign(S, c, j, t, pot, sub, SDMD_EV_HB);
}

// HBNeighborTime (src/TimePrediction.c:486-579)
__device__ __noinline__ void hbnb_time(const DSys &S, int i, Cur &c, Blk &B, int *bad) {
    int flag = 0;
    for (int n = 1; n <= S.nb_status[i]; n++) {
        int j = S.nb_partner[4 * i + n - 1];
        if (flag == 0) S.nb_pnum[i] = n;
        if (j < S.dup_limit && S.ev_partner[j] == i && S.ev_type[j] == SDMD_EV_HBNEIGHBOR && S.ev_pcounter[j] == S.ev_counter[i] &&
            dup_assign(S, c, j, S.ev_time[j], SDMD_EV_HBNEIGHBOR)) {
            S.nb_pnum[i] = n; flag = 1; continue;
        }
        Kin kk; pair_kin(S, i, j, kk);
        int host, nbr, hpart, ri = S.hb_role[i];
        if ((ri == 'A' || ri == 'D' || ri == 'S') && S.hb_bond[i] && S.hb_neighbor[S.hb_bond[i]] == j) {
            host = i; nbr = j; hpart = S.hb_bond[i];
        } else {
            host = j; nbr = i; hpart = S.hb_bond[j];
        }
        Lim o; int warn = 0;
        int cs = find_pair(S, nbr, host, K_NEIGHBOR, kk.b, kk.r2, o, hpart, 0, 0, &warn, bad);
        B.warn += warn;
        int st, sub; double d2, pot;
        if (kk.b < 0 && disc(kk, o.lo) > 0) {
            st = -1; d2 = o.lo; pot = o.lopot; sub = (cs == 0) ? SDMD_SUB_CORE : SDMD_SUB_TBD_CAPTURE;
        } else {
            st = 1; d2 = o.up; pot = o.uppot; sub = (cs == 1) ? SDMD_SUB_WELL_BOUNCE : SDMD_SUB_TBD_ESCAPE;
        }
        double t = root(kk, st, d2);
        if (t < 0) t = INFINIT;
        if (job_assign(S, c, j, t, pot, sub, SDMD_EV_HBNEIGHBOR)) { S.nb_pnum[i] = n; flag = 1; }
    }
}

// WallTime, smooth walls (src/TimePrediction.c:635-737)
__device__ __noinline__ void wall_time(const DSys &S, int i, Cur &c, Blk &B, int *bad) {
    double p[3] = {S.x[i], S.y[i], S.z[i]}, v[3] = {S.vx[i], S.vy[i], S.vz[i]};
    if (S.wall == SDMD_WALL_PARALLEL) { p[0] = p[2] = 0; v[0] = v[2] = 0; }
    else if (S.wall == SDMD_WALL_CYLINDER) { p[0] = 0; v[0] = 0; }
    Kin k;
    k.rx = p[0] - S.wall_pos[0]; k.ry = p[1] - S.wall_pos[1]; k.rz = p[2] - S.wall_pos[2];
    double vx = v[0] - S.wall_vel[0], vy = v[1] - S.wall_vel[1], vz = v[2] - S.wall_vel[2];
    k.r2 = k.rx * k.rx + k.ry * k.ry + k.rz * k.rz;
    k.b = k.rx * vx + k.ry * vy + k.rz * vz;
    k.v2 = vx * vx + vy * vy + vz * vz;
    double L2 = S.box[1];
    double dist2 = L2 * L2 * 0.25 + k.r2 - L2 * sqrt(k.r2);
    Lim o; int warn = 0;
    int cs = find_pair(S, i, 0, K_COLLISION, -1 * k.b, dist2, o, 0, 0, S.wall_type, &warn, bad);
    B.warn += warn;
    if (o.lopot == 0 && o.uppot == 0) { set_err(B, SDMD_EWALL, i); return; }
    int st, sub; double d2, pot;
    if (k.b < 0 && disc(k, o.lo) > 0) {
        if (cs == 1) return;
        sub = SDMD_SUB_TBD_CAPTURE; st = -1;
        d2 = L2 * L2 * 0.25 + o.up - L2 * sqrt(o.up); pot = o.uppot;
    } else {
        sub = (cs == 0) ? SDMD_SUB_WELL_BOUNCE : SDMD_SUB_TBD_ESCAPE; st = 1;
        d2 = L2 * L2 * 0.25 + o.lo - L2 * sqrt(o.lo); pot = o.lopot;
    }
    double t = root(k, st, d2);
    if (t < 0) t = INFINIT;
    job_assign(S, c, 0, t, pot, sub, SDMD_EV_WALL);
}

// ObstTime, obstruction walls (src/TimePrediction.c:740-829): for each plane n
// across axis d, the axis component alone (the others zeroed, as the reference
// zeroes them) against the potential steps of the pair (atom type, wall type);
// the partner becomes -d - 10 n when that plane gives the new earliest event
__device__ __noinline__ void obst_time(const DSys &S, int i, Cur &c, Blk &B, int *bad) {
    const double p[3] = {S.x[i], S.y[i], S.z[i]}, v[3] = {S.vx[i], S.vy[i], S.vz[i]};
    for (int n = 0; n < S.n_obst; n++) {
        for (int dim = 0; dim < 3; dim++) {
            const double pos = S.obst[3 * n + dim];
            if (pos < 0) continue;
            double pi[3] = {0, 0, 0}, pj[3] = {0, 0, 0}, vi[3] = {0, 0, 0}, vj[3] = {0, 0, 0};
            pi[dim] = p[dim]; pj[dim] = pos; vi[dim] = v[dim];
            Kin k;
            k.rx = pi[0] - pj[0]; k.ry = pi[1] - pj[1]; k.rz = pi[2] - pj[2];
            const double wx = vi[0] - vj[0], wy = vi[1] - vj[1], wz = vi[2] - vj[2];
            k.r2 = k.rx * k.rx + k.ry * k.ry + k.rz * k.rz;
            k.b = k.rx * wx + k.ry * wy + k.rz * wz;
            k.v2 = wx * wx + wy * wy + wz * wz;
            Lim o; int warn = 0;
            const int cs = find_pair(S, i, 0, K_COLLISION, k.b, k.r2, o, 0, 0, S.wall_type, &warn, bad);
            B.warn += warn;
            if (o.lopot == 0 && o.uppot == 0) continue;   // inside the holes
            int st, sub; double d2, pot;
            if (k.b < 0) {   // approaching
                sub = cs == 0 ? SDMD_SUB_CORE : SDMD_SUB_TBD_CAPTURE;
                st = -1; d2 = o.lo; pot = o.lopot;
            } else {         // leaving
                if (cs == 1) continue;
                sub = SDMD_SUB_TBD_ESCAPE;
                st = 1; d2 = o.up; pot = o.uppot;
            }
            const double t = root(k, st, d2);
            if (t < 0) { set_err(B, SDMD_ENEGTIME, i); return; }
            if (!(t > 0)) continue;   // no root (NaN): JobAssign's time > 0 test fails
            if (job_assign(S, c, 0, t, pot, sub, SDMD_EV_OBST)) c.partner = -(dim + 1) - 10 * n;
        }
    }
}

// SphObstTime, spherical obstacles (src/TimePrediction.c:1020-1071): a core
// collision with each fixed sphere the atom approaches (absolute coordinates, no
// periodic image); the partner becomes -1000 n when obstacle n gives the new
// earliest event
__device__ __noinline__ void sphobst_time(const DSys &S, int i, Cur &c, Blk &B) {
    for (int n = 0; n < S.n_sph; n++) {
        const double *o = S.sph + 4 * n;
        Kin k;
        k.rx = S.x[i] - o[0]; k.ry = S.y[i] - o[1]; k.rz = S.z[i] - o[2];
        const double vx = S.vx[i] - 0.0, vy = S.vy[i] - 0.0, vz = S.vz[i] - 0.0;
        k.r2 = k.rx * k.rx + k.ry * k.ry + k.rz * k.rz;
        k.b = k.rx * vx + k.ry * vy + k.rz * vz;
        k.v2 = vx * vx + vy * vy + vz * vz;
        const double lo = o[3] * o[3];
        if (!(k.b < 0 && disc(k, lo) > 0)) continue;
        const double t = root(k, -1, lo);
        if (t < 0) { set_err(B, SDMD_ENEGTIME, i); return; }
        if (job_assign(S, c, 0, t, 0.0, SDMD_SUB_CORE, SDMD_EV_SPHOBST)) c.partner = -1000 * n;
    }
}

// ---- Predict for one atom (ResetTarget already applied) ---------------------
struct Shm {
    int32_t *nbj, *cnt;
    Slots L;
    double *face;    // 3 PCC face times
};

__device__ __noinline__ void predict_atom(const DSys &S, int i, Shm &M, Blk &B, DScal &C) {
    const int tid = threadIdx.x, T = blockDim.x;
    int bad = 0;
    Cur c;
    if (tid == 0) cur_load(S, i, c);
    double cut = S.cutoff * 0.90; cut *= cut;
    // BondTime
    int b0 = S.bond_off[i], nb = S.bond_off[i + 1] - b0;
    if (nb > (S.nbcap > 64 ? S.nbcap : 64)) {   // slot capacity
        if (tid == 0) set_err(B, SDMD_ECAPACITY, i);
        __syncthreads();
        return;
    }
    for (int k = tid; k < nb; k += T) eval_bond(S, i, b0 + k, M.L, k, &bad);
    __syncthreads();
    if (tid == 0) resolve(S, c, M.L, nb, SDMD_EV_BOND, B);
    // CollisionTime over the gathered 27-cell neighbourhood
    gather(S, i, M.nbj, M.cnt, B);
    int nn = B.nnb;
    for (int k = tid; k < nn; k += T) eval_collision(S, i, M.nbj[k], cut, M.L, k, &bad);
    if (tid < 3) M.face[tid] = pcc_face(S, i, tid);
    __syncthreads();
    if (tid == 0) {
        resolve(S, c, M.L, nn, SDMD_EV_COLLISION, B);
        pcc_time(S, c, M.face);
        thermostat_time(S, c, C, B);
        // HBTime prologue: one-shot HBSkip suppression (src/TimePrediction.c:309-327)
        int mode;
        if (S.hb_itype[i] == SDMD_HB_SKIP) mode = 0;
        else if (S.hb_bond[i] > 0) mode = 1;
        else {
            int r = S.hb_role[i];
            mode = (r == 'A' || r == 'D' || r == 'S') ? 2 : 0;
        }
        S.hb_itype[i] = SDMD_HB_NOEVENT;
        B.hbmode = mode;
        if (mode == 1) hb_bonded(S, i, c, B, &bad);
    }
    __syncthreads();
    if (B.hbmode == 2) {
        for (int k = tid; k < nn; k += T) eval_hb_scan(S, i, M.nbj[k], cut, M.L, k, &bad);
        __syncthreads();
        if (tid == 0) resolve(S, c, M.L, nn, SDMD_EV_HB, B);
    }
    if (tid == 0) {
        hbnb_time(S, i, c, B, &bad);
        if (S.wall) wall_time(S, i, c, B, &bad);
        if (S.n_obst) obst_time(S, i, c, B, &bad);
        if (S.n_sph) sphobst_time(S, i, c, B);
        cur_store(S, i, c);
    }
    if (bad) set_err(B, SDMD_EHBMAP, i);
    __syncthreads();
}

// ---- events (thread 0) -------------------------------------------------------
__device__ void imaged(const DSys &S, int t, int a, double p[3]) {
    const int ct[3] = {S.cx[t], S.cy[t], S.cz[t]}, ca[3] = {S.cx[a], S.cy[a], S.cz[a]};
    p[0] = lzx(S, S.x, S.vx, a); p[1] = lzx(S, S.y, S.vy, a); p[2] = lzx(S, S.z, S.vz, a);
    for (int d = 0; d < 3; d++) {
        if (ct[d] != ca[d]) {
            if (ct[d] == 0 && ca[d] == S.cn[d] - 1) p[d] -= S.box[d];
            else if (ct[d] == S.cn[d] - 1 && ca[d] == 0) p[d] += S.box[d];
        }
    }
}

// HBEnergyChange (src/Events.c:1027-1095); `acc` carries over between candidates
// exactly as the reference's local does.
__device__ double hb_energy_change(const DSys &S, int t, int skip, int to_hb, Blk &B, int *bad) {
    double cut = S.cutoff * S.cutoff, energy = 0, acc = 0;
    auto visit = [&](int j) {
        int bits = conn_bits(S, t, j);
        if (!(t != j && !(bits & 1) && !(bits & 2) && j != skip)) return;
        Kin k; pair_kin(S, t, j, k);
        if (k.r2 <= cut) {
            Lim o; int warn = 0;
            if (!to_hb) { find_pair(S, t, j, K_COLLISION, 0, k.r2, o, 0, -1, 0, &warn, bad); acc = o.acc; }
            else if (j != S.hb_neighbor[skip]) { find_pair(S, t, j, K_COLLISION, 0, k.r2, o, 0, 1, 0, &warn, bad); acc = o.acc; }
            B.warn += warn;
            if (acc == INFINIT) acc = 0;
            energy += acc;
        }
    };
    for (int kc = 0; kc < 27; kc++) {
        const int cell = nb_cell(S, t, kc);
        if (S.cell_arr) {   // screened path: the per-cell arrays, newest first (the list's order)
            const int32_t *arr = S.cell_arr + (size_t)cell * S.maxc;
            for (int m = S.cell_cnt[cell] - 1; m >= 0; m--) visit(arr[m]);
        } else {
            int guard = 0;
            for (int j = S.cell_list[S.n + cell]; j && guard <= S.n; j = S.cell_list[j], guard++) visit(j);
        }
    }
    return energy;
}

// InteractionEvent (src/Events.c:798-1024)
__device__ void interaction_event(const DSys &S, int t, int p, int ni, int nj, Blk &B, int *bad) {
    double pi[3] = {S.x[t], S.y[t], S.z[t]}, pj[3];
    imaged(S, t, p, pj);
    double r[3] = {pi[0] - pj[0], pi[1] - pj[1], pi[2] - pj[2]};
    double v[3] = {S.vx[t] - S.vx[p], S.vy[t] - S.vy[p], S.vz[t] - S.vz[p]};
    double d2 = r[0] * r[0] + r[1] * r[1] + r[2] * r[2];
    double b = r[0] * v[0] + r[1] * v[1] + r[2] * v[2];
    double mt = S.mass[t], mp = S.mass[p];
    double mu = mt * mp / (mt + mp);
    double pot = S.ev_potential[t];
    int sv = 0;
    if (S.ev_type[t] == SDMD_EV_HB && (S.ev_sub[t] == SDMD_SUB_TBD_HBFORM || S.ev_sub[t] == SDMD_SUB_TBD_HBBREAK)) {
        bool form = S.ev_sub[t] == SDMD_SUB_TBD_HBFORM;
        if ((nb_has(S, t, nj) || nb_has(S, p, ni)) && form) { S.hb_itype[t] = SDMD_HB_SKIP; return; }
        double pni[3], pnj[3];
        imaged(S, t, ni, pni);
        imaged(S, t, nj, pnj);
        double rci[3] = {pi[0] - pnj[0], pi[1] - pnj[1], pi[2] - pnj[2]};
        double rcj[3] = {pj[0] - pni[0], pj[1] - pni[1], pj[2] - pni[2]};
        double rni2 = rci[0] * rci[0] + rci[1] * rci[1] + rci[2] * rci[2];
        double rnj2 = rcj[0] * rcj[0] + rcj[1] * rcj[1] + rcj[2] * rcj[2];
        double acc[6];
        acc[0] = hb_energy_change(S, t, p, 0, B, bad);
        acc[1] = hb_energy_change(S, p, t, 0, B, bad);
        acc[2] = hb_energy_change(S, t, p, 1, B, bad);
        acc[3] = hb_energy_change(S, p, t, 1, B, bad);
        Lim o; int warn = 0;
        find_pair(S, nj, t, K_NEIGHBOR, 0, rni2, o, p, 0, 0, &warn, bad); acc[4] = o.acc;
        find_pair(S, ni, p, K_NEIGHBOR, 0, rnj2, o, t, 0, 0, &warn, bad); acc[5] = o.acc;
        B.warn += warn;
        if (form) {
            pot -= hb_barrier(S, t, p);
            pot += (acc[2] - acc[0] + acc[3] - acc[1] + acc[4] + acc[5]);
        } else {
            pot += hb_barrier(S, t, p);
            pot += (acc[0] - acc[2] + acc[1] - acc[3] - acc[4] - acc[5]);
        }
        if (pot < -0.5 * INFINIT && !form) { S.hb_itype[t] = SDMD_HB_SKIP; return; }
        if (pot > 0.5 * INFINIT && form) { S.hb_itype[t] = SDMD_HB_SKIP; return; }
        if (b * b - 2 * d2 * pot / mu > 0) {
            if (form) { S.ev_sub[t] = SDMD_SUB_WELL_CAPTURE; S.hb_itype[t] = SDMD_HB_FORM; }
            else { S.ev_sub[t] = SDMD_SUB_WELL_ESCAPE; S.hb_itype[t] = SDMD_HB_BREAK; }
        } else {
            if (form) { S.hb_itype[t] = SDMD_HB_SKIP; return; }
            pot = 0; S.ev_sub[t] = SDMD_SUB_WELL_BOUNCE; S.hb_itype[t] = SDMD_HB_NOEVENT;
        }
    }
    switch (S.ev_sub[t]) {
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
        default: set_err(B, SDMD_EEVENTTYPE, t); return;
    }
    double phi = (-1 * b + sv * sqrt((b * b - 2 * d2 * pot / mu))) / ((mt + mp) * d2);
    if (isnan(phi)) { set_err(B, SDMD_ENAN, t); return; }
    double ft = mp * phi, fp = mt * phi;
    S.vx[t] = S.vx[t] + ft * r[0]; S.vy[t] = S.vy[t] + ft * r[1]; S.vz[t] = S.vz[t] + ft * r[2];
    S.vx[p] = S.vx[p] - fp * r[0]; S.vy[p] = S.vy[p] - fp * r[1]; S.vz[p] = S.vz[p] - fp * r[2];
}

// ListRefresh (src/ToolFunctions.c:572-597) and neighbour-list append
__device__ void nb_remove(const DSys &S, int a, int value) {
    int32_t *l = S.nb_partner + 4 * a;
    int i = nb_has(S, a, value);
    if (!i) return;
    int n = i + 1;
    while (n <= 4 && l[n - 1] != 0) { l[i - 1] = l[n - 1]; i++; n++; }
    l[i - 1] = 0;
}
__device__ void nb_append(const DSys &S, int a, int value, Blk &B) {
    int k = ++S.nb_status[a];
    if (k > 4) { set_err(B, SDMD_ECAPACITY, a); return; }
    S.nb_partner[4 * a + k - 1] = value;
}
__device__ inline bool alpha_hb(const DSys &S, int i, int j) {
    return S.protein[i] == S.protein[j] &&
           ((S.name_code[i] == 1 && S.name_code[j] == 2 && S.aanum[j] == S.aanum[i] - 4) ||
            (S.name_code[i] == 2 && S.name_code[j] == 1 && S.aanum[i] == S.aanum[j] - 4));
}

// HBEvent (src/Events.c:275-393)
__device__ void hb_event(const DSys &S, DScal &C, int i, int j, int ni, int nj, Blk &B) {
    int nbi = S.hb_neighbor[i], nbj = S.hb_neighbor[j];
    if (S.hb_itype[i] == SDMD_HB_FORM) {
        if (nb_has(S, i, nbj) || nb_has(S, nbj, i) || nb_has(S, j, nbi) || nb_has(S, nbi, j)) {
            set_err(B, SDMD_EHBMAP, i); return;
        }
        S.hb_bond[i] = j; S.hb_bond[j] = i;
        S.type[i] = type_change(S.type[i], 1); S.type[j] = type_change(S.type[j], 1);
        nb_append(S, i, nbj, B); nb_append(S, j, nbi, B); nb_append(S, ni, j, B); nb_append(S, nj, i, B);
        if (alpha_hb(S, i, j)) C.c.alpha_hb_formed++;
        C.c.hb_formed++;
    } else if (S.hb_itype[i] == SDMD_HB_BREAK) {
        S.hb_bond[i] = 0; S.hb_bond[j] = 0;
        S.type[i] = type_change(S.type[i], 0); S.type[j] = type_change(S.type[j], 0);
        --S.nb_status[i]; nb_remove(S, i, nbj);
        --S.nb_status[j]; nb_remove(S, j, nbi);
        --S.nb_status[ni]; nb_remove(S, ni, j);
        --S.nb_status[nj]; nb_remove(S, nj, i);
        if (alpha_hb(S, i, j)) C.c.alpha_hb_formed--;
        C.c.hb_formed--;
        if (C.c.hb_formed < C.c.alpha_hb_formed) C.c.warnings++;
    }
}

// ThermostatEvent, Andersen (src/Events.c:396-420)
__device__ void thermostat_event(const DSys &S, int t, DScal &C, Blk &B) {
    double sp[3];
    for (int d = 0; d < 3; d++) {
        sp[d] = take_sample(S, C, B) * sqrt(S.temperature / S.mass[t]) + 0;
        if (sp[d] == 0) { set_err(B, SDMD_ETIMEOUT, t); return; }   // a Box-Muller value is never exactly 0
    }
    S.vx[t] = sp[0]; S.vy[t] = sp[1]; S.vz[t] = sp[2];
}

// PBCandCrossCellEvent with PBC("part") and LinkList("part")
// (src/Events.c:248-272, 207-245, 158-200)
__device__ void pcc_event(const DSys &S, int t, Blk &B, int32_t *moved = nullptr) {
    int old[3] = {S.cx[t], S.cy[t], S.cz[t]};
    double pos[3] = {S.x[t], S.y[t], S.z[t]};
    for (int d = 0; d < 3; d++) {
        if (old[d] == 0 || old[d] == S.cn[d] - 1) {
            if (S.wall != SDMD_WALL_SPHERE) {
                int dims = 3, step = 1;
                if (S.wall == SDMD_WALL_PARALLEL) step = 2;
                else if (S.wall == SDMD_WALL_CYLINDER) dims = 1;
                for (int n = 0; n < dims; n += step) {
                    if (pos[n] >= S.box[n]) pos[n] -= S.box[n];
                    else if (pos[n] < 0) pos[n] += S.box[n];
                }
            }
            break;
        }
    }
    S.x[t] = pos[0]; S.y[t] = pos[1]; S.z[t] = pos[2];
    int N = S.n, oldc = cell_lin(S, old[0], old[1], old[2]);
    int nc[3];
    for (int d = 0; d < 3; d++) {
        nc[d] = (int)(pos[d] / S.cs[d]);
        if (nc[d] == S.cn[d]) nc[d]--;
    }
    S.cx[t] = nc[0]; S.cy[t] = nc[1]; S.cz[t] = nc[2];
    if (nc[0] < 0 || nc[1] < 0 || nc[2] < 0 || nc[0] >= S.cn[0] || nc[1] >= S.cn[1] || nc[2] >= S.cn[2]) {
        set_err(B, SDMD_ELINK, t); return;
    }
    int newc = cell_lin(S, nc[0], nc[1], nc[2]);
    if (moved) {   // the screened path keeps per-cell arrays: the move is applied by a warp
        moved[0] = t; moved[1] = oldc; moved[2] = newc;
        return;
    }
    int32_t *L = S.cell_list;
    int at = oldc + N, guard = 0;
    if (L[at] == 0) { set_err(B, SDMD_ELINK, t); return; }
    while (L[at] != t) {
        at = L[at];
        if (at == 0 || ++guard > N) { set_err(B, SDMD_ELINK, t); return; }
    }
    L[at] = L[t];
    L[t] = L[newc + N];
    L[newc + N] = t;
}

// WallEvent, smooth walls (src/Events.c:423-499)
__device__ void wall_event(const DSys &S, int t, Blk &B) {
    double p[3] = {S.x[t], S.y[t], S.z[t]}, v[3] = {S.vx[t], S.vy[t], S.vz[t]};
    if (S.wall == SDMD_WALL_PARALLEL) { p[0] = p[2] = 0; v[0] = v[2] = 0; }
    else if (S.wall == SDMD_WALL_CYLINDER) { p[0] = 0; v[0] = 0; }
    double r[3] = {p[0] - S.wall_pos[0], p[1] - S.wall_pos[1], p[2] - S.wall_pos[2]};
    double w[3] = {v[0] - S.wall_vel[0], v[1] - S.wall_vel[1], v[2] - S.wall_vel[2]};
    double d2 = r[0] * r[0] + r[1] * r[1] + r[2] * r[2];
    double b = r[0] * w[0] + r[1] * w[1] + r[2] * w[2];
    double mu = S.mass[t], pot = S.ev_potential[t];
    int sv;
    switch (S.ev_sub[t]) {
        case SDMD_SUB_WELL_BOUNCE: sv = -1; pot = 0; break;
        case SDMD_SUB_TBD_CAPTURE: if (b * b - 2 * d2 * pot / mu <= 0) { pot = 0; sv = 1; } else sv = -1; break;
        case SDMD_SUB_TBD_ESCAPE: if (b * b - 2 * d2 * pot / mu <= 0) { pot = 0; sv = -1; } else sv = 1; break;
        default: set_err(B, SDMD_EEVENTTYPE, t); return;
    }
    double phi = (-1 * b + sv * sqrt(b * b - 2 * d2 * pot / S.mass[t])) / d2;
    if (isnan(phi)) { set_err(B, SDMD_ENAN, t); return; }
    S.vx[t] = S.vx[t] + phi * r[0]; S.vy[t] = S.vy[t] + phi * r[1]; S.vz[t] = S.vz[t] + phi * r[2];
}

// ObstEvent (src/Events.c:543-617): plane -partner / 10 across axis -partner % 10
__device__ void obst_event(const DSys &S, int t, Blk &B) {
    const int part = S.ev_partner[t];
    const int n = part / -10, dim = (part * -1) % 10;
    if (n < 0 || n >= S.n_obst || dim < 1 || dim > 3) { set_err(B, SDMD_EEVENTTYPE, t); return; }
    double pi[3] = {0, 0, 0}, pj[3] = {0, 0, 0}, vi[3] = {0, 0, 0}, vj[3] = {0, 0, 0};
    pi[dim - 1] = dim == 1 ? S.x[t] : dim == 2 ? S.y[t] : S.z[t];
    vi[dim - 1] = dim == 1 ? S.vx[t] : dim == 2 ? S.vy[t] : S.vz[t];
    pj[dim - 1] = S.obst[3 * n + dim - 1];
    const double r[3] = {pi[0] - pj[0], pi[1] - pj[1], pi[2] - pj[2]};
    const double w[3] = {vi[0] - vj[0], vi[1] - vj[1], vi[2] - vj[2]};
    const double d2 = r[0] * r[0] + r[1] * r[1] + r[2] * r[2];
    const double b = r[0] * w[0] + r[1] * w[1] + r[2] * w[2];
    const double mu = S.mass[t];
    double pot = S.ev_potential[t];
    int sv;
    switch (S.ev_sub[t]) {
        case SDMD_SUB_CORE: sv = 1; pot = 0; break;
        case SDMD_SUB_TBD_CAPTURE: if (b * b - 2 * d2 * pot / mu <= 0) { pot = 0; sv = 1; } else sv = -1; break;
        case SDMD_SUB_TBD_ESCAPE: if (b * b - 2 * d2 * pot / mu <= 0) { pot = 0; sv = -1; } else sv = 1; break;
        default: set_err(B, SDMD_EEVENTTYPE, t); return;
    }
    const double phi = (-1 * b + sv * sqrt(b * b - 2 * d2 * pot / S.mass[t])) / d2;
    if (isnan(phi)) { set_err(B, SDMD_ENAN, t); return; }
    S.vx[t] = S.vx[t] + phi * r[0]; S.vy[t] = S.vy[t] + phi * r[1]; S.vz[t] = S.vz[t] + phi * r[2];
}

// SphObstEvent (src/Events.c:752-795): the core bounce off fixed sphere -partner / 1000
__device__ void sphobst_event(const DSys &S, int t, Blk &B) {
    const int n = S.ev_partner[t] / -1000;
    if (n < 0 || n >= S.n_sph || S.ev_sub[t] != SDMD_SUB_CORE) { set_err(B, SDMD_EEVENTTYPE, t); return; }
    const double *o = S.sph + 4 * n;
    const double r[3] = {S.x[t] - o[0], S.y[t] - o[1], S.z[t] - o[2]};
    const double w[3] = {S.vx[t] - 0.0, S.vy[t] - 0.0, S.vz[t] - 0.0};
    const double d2 = r[0] * r[0] + r[1] * r[1] + r[2] * r[2];
    const double b = r[0] * w[0] + r[1] * w[1] + r[2] * w[2];
    const double pot = 0;
    const int sv = 1;
    const double phi = (-1 * b + sv * sqrt(b * b - 2 * d2 * pot / S.mass[t])) / d2;
    if (isnan(phi)) { set_err(B, SDMD_ENAN, t); return; }
    S.vx[t] = S.vx[t] + phi * r[0]; S.vy[t] = S.vy[t] + phi * r[1]; S.vz[t] = S.vz[t] + phi * r[2];
}

// DoEvent (src/Events.c:25-114)
__device__ void do_event(const DSys &S, DScal &C, int t, int p, Blk &B, int32_t *moved = nullptr) {
    int bad = 0;
    switch (S.ev_type[t]) {
        case SDMD_EV_COLLISION: interaction_event(S, t, p, 0, 0, B, &bad); C.c.collision++; break;
        case SDMD_EV_BOND: interaction_event(S, t, p, 0, 0, B, &bad); C.c.bond++; break;
        case SDMD_EV_HBNEIGHBOR: interaction_event(S, t, p, 0, 0, B, &bad); C.c.hbneighbor++; break;
        case SDMD_EV_HB: {
            int ni = S.hb_neighbor[t], nj = S.hb_neighbor[p];
            interaction_event(S, t, p, ni, nj, B, &bad);
            if (!B.err) hb_event(S, C, t, p, ni, nj, B);
            C.c.hb++;
        } break;
        case SDMD_EV_THERMOSTAT: thermostat_event(S, t, C, B); C.c.thermostat++; break;
        case SDMD_EV_PCC: pcc_event(S, t, B, moved); C.c.pcc++; break;
        case SDMD_EV_WALL: wall_event(S, t, B); C.c.wall++; break;
        case SDMD_EV_OBST: obst_event(S, t, B); C.c.wall++; break;         // walleventsum
        case SDMD_EV_SPHOBST: sphobst_event(S, t, B); C.c.wall++; break;   // walleventsum
        default: set_err(B, SDMD_EEVENTTYPE, t); break;
    }
    if (bad) set_err(B, SDMD_EHBMAP, t);
}

// one pop's trace record (a real call: tracing is off in timed runs)
__device__ __noinline__ void record_trace(const DSys &S, const DScal &C, int t, int p, int partner, int type, int sub,
                                          int executed, double dt) {
    sdmd_trace_rec &r = S.trace[C.pops % S.trace_cap];
    r.target = t; r.partner = partner; r.type = type; r.sub = sub;
    r.executed = executed; r.hb_itype_after = S.hb_itype[t];
    r.t_new_partner = S.ev_partner[t]; r.t_new_type = S.ev_type[t];
    r.p_new_partner = p ? S.ev_partner[p] : 0; r.p_new_type = p ? S.ev_type[p] : 0;
    r.system = blockIdx.x; r.pad = 0;
    r.dt = dt; r.time_now = C.time;
    r.vt[0] = S.vx[t]; r.vt[1] = S.vy[t]; r.vt[2] = S.vz[t];
    r.vp[0] = p ? S.vx[p] : 0; r.vp[1] = p ? S.vy[p] : 0; r.vp[2] = p ? S.vz[p] : 0;
    r.t_new_time = S.ev_time[t]; r.p_new_time = p ? S.ev_time[p] : 0;
}

// ---- CBT (src/CBT.c) -----------------------------------------------------------
__device__ void cbt_update(const DSys &S, int a) {   // UpdateCBTRun, src/CBT.c:56-83
    int32_t *node = S.cbt_node;
    const int32_t *leaf = S.cbt_leaf;
    const double *tm = S.ev_time;
    int f;
    for (f = leaf[a] / 2; f > 0; f /= 2) {
        if (node[f] != a) break;
        int l = node[2 * f], r = node[2 * f + 1];
        node[f] = tkey(tm[l]) < tkey(tm[r]) ? l : r;
    }
    for (; f > 0; f /= 2) {
        int old = node[f], l = node[2 * f], r = node[2 * f + 1];
        node[f] = tkey(tm[l]) < tkey(tm[r]) ? l : r;
        if (node[f] == old) return;
    }
}
__device__ void cbt_build(const DSys &S) {            // CreateCBT, src/CBT.c:16-30
    int32_t *node = S.cbt_node, *leaf = S.cbt_leaf;
    int count = 0;
    for (int a = 1; a <= S.n; a++) {
        if (count == 0) { node[1] = a; count = 1; continue; }
        int i = node[count];
        node[2 * count] = i; node[2 * count + 1] = a;
        leaf[i] = 2 * count; leaf[a] = 2 * count + 1;
        count++;
        cbt_update(S, i);
    }
}

// ---- kernels ---------------------------------------------------------------------
__host__ __device__ inline size_t fp64_smem_bytes_dev(int nbcap) {
    int cap = nbcap > 64 ? nbcap : 64;
    return al16((size_t)(cap * 3 + 4) * sizeof(double) + (size_t)(2 * cap + nbcap + 32) * sizeof(int32_t));
}

__device__ inline void carve(Shm &M, int nbcap) {
    extern __shared__ __align__(16) unsigned char smem[];
    int cap = nbcap > 64 ? nbcap : 64;
    double *d = reinterpret_cast<double *>(smem);
    M.L.t = d; M.L.tdup = d + cap; M.L.pot = d + 2 * cap;
    M.face = d + 3 * cap;
    int32_t *ip = reinterpret_cast<int32_t *>(d + 3 * cap + 4);
    M.L.j = ip; M.L.info = ip + cap; M.nbj = ip + 2 * cap; M.cnt = ip + 2 * cap + nbcap;
}

}  // namespace sdmd
#include "screen.cuh"
#include "sweep_par.cuh"
namespace sdmd {

// ---- whole-system staging in shared memory ------------------------------------
// A small system's per-atom arrays, topology, cell list and event tree are copied
// into shared memory at kernel start; the block's DSys pointers are redirected to
// the copies (generic addressing makes every device function work unchanged),
// and the mutable arrays are written back at the end.  Shared-memory latency is
// ~30 cycles against ~300-600 for L2.
struct Stager {
    unsigned char *p;
    bool copy;
    template <class T> __device__ T *take(const T *src, size_t count) {
        size_t a = (reinterpret_cast<size_t>(p) + 15) & ~size_t(15);
        T *dst = reinterpret_cast<T *>(a);
        p = reinterpret_cast<unsigned char *>(dst + count);
        if (copy && src)
            for (size_t k = threadIdx.x; k < count; k += blockDim.x) dst[k] = src[k];
        return dst;
    }
};

size_t staged_state_bytes(int n, int ncell, int nb, int nc, int ncs, int nconn) {
    size_t N1 = (size_t)n + 1, t = 0;
    t += al16(N1 * 8) * 10;                                  // mass, x..vz, ev_time, ev_potential, tloc
    t += al16(N1 * 4) * 17;                                  // 6 static + 11 dynamic int arrays
    t += al16(4 * N1 * 4);                                   // nb_partner
    t += al16(N1 * 8) * 2;                                   // ev_counter, ev_pcounter
    t += al16((N1 + 1) * 4) * 3;                             // bond/con/conn offsets
    t += al16((size_t)nb * 4) + 2 * al16((size_t)nb * 8);
    t += 3 * al16((size_t)nc * 4) + 2 * al16((size_t)nc * 8) + 3 * al16((size_t)ncs * 8);
    t += 2 * al16((size_t)nconn * 4);
    t += al16((N1 + (size_t)ncell) * 4);                     // cell list
    t += al16((2 * N1 + 2) * 4) + al16((N1 + 1) * 4);        // tree
    return t + 64;
}

// stage (copy == true) or locate (copy == false) the state after the slot buffers
__device__ __noinline__ void stage_state(DSys &S, const DSys &G, unsigned char *base, bool copy) {
    Stager st{base, copy};
    size_t N1 = (size_t)G.n + 1;
    DSys L = G;
    L.mass = st.take(G.mass, N1);
    L.x = st.take(G.x, N1); L.y = st.take(G.y, N1); L.z = st.take(G.z, N1);
    L.vx = st.take(G.vx, N1); L.vy = st.take(G.vy, N1); L.vz = st.take(G.vz, N1);
    L.ev_time = st.take(G.ev_time, N1); L.ev_potential = st.take(G.ev_potential, N1);
    if (G.lazy) L.tloc = st.take(G.tloc, N1);
    L.protein = st.take(G.protein, N1); L.aanum = st.take(G.aanum, N1); L.aatype = st.take(G.aatype, N1);
    L.hb_neighbor = st.take(G.hb_neighbor, N1); L.hb_role = st.take(G.hb_role, N1);
    L.name_code = st.take(G.name_code, N1);
    L.cx = st.take(G.cx, N1); L.cy = st.take(G.cy, N1); L.cz = st.take(G.cz, N1);
    L.type = st.take(G.type, N1); L.hb_bond = st.take(G.hb_bond, N1); L.hb_itype = st.take(G.hb_itype, N1);
    L.nb_status = st.take(G.nb_status, N1); L.nb_pnum = st.take(G.nb_pnum, N1);
    L.ev_partner = st.take(G.ev_partner, N1); L.ev_type = st.take(G.ev_type, N1); L.ev_sub = st.take(G.ev_sub, N1);
    L.nb_partner = st.take(G.nb_partner, 4 * N1);
    L.ev_counter = st.take(G.ev_counter, N1); L.ev_pcounter = st.take(G.ev_pcounter, N1);
    L.bond_off = st.take(G.bond_off, N1 + 1); L.con_off = st.take(G.con_off, N1 + 1);
    L.conn_off = st.take(G.conn_off, N1 + 1);
    L.bond_j = st.take(G.bond_j, (size_t)G.n_bonds);
    L.bond_dmin = st.take(G.bond_dmin, (size_t)G.n_bonds); L.bond_dmax = st.take(G.bond_dmax, (size_t)G.n_bonds);
    L.con_j = st.take(G.con_j, (size_t)G.n_cons); L.con_step_off = st.take(G.con_step_off, (size_t)G.n_cons);
    L.con_step_n = st.take(G.con_step_n, (size_t)G.n_cons);
    L.con_dmin = st.take(G.con_dmin, (size_t)G.n_cons); L.con_dmax = st.take(G.con_dmax, (size_t)G.n_cons);
    L.con_step_d = st.take(G.con_step_d, (size_t)G.n_con_steps);
    L.con_step_e = st.take(G.con_step_e, (size_t)G.n_con_steps);
    L.con_step_acc = st.take(G.con_step_acc, (size_t)G.n_con_steps);
    L.conn_j = st.take(G.conn_j, (size_t)G.n_conn); L.conn_bits = st.take(G.conn_bits, (size_t)G.n_conn);
    L.cell_list = st.take(G.cell_list, N1 + (size_t)G.ncell);
    L.cbt_node = st.take(G.cbt_node, 2 * N1 + 2); L.cbt_leaf = st.take(G.cbt_leaf, N1 + 1);
    __syncthreads();
    if (threadIdx.x == 0) S = L;
    __syncthreads();
}

// write the mutable staged arrays back to global memory
__device__ __noinline__ void unstage_state(const DSys &S, const DSys &G) {
    size_t N1 = (size_t)G.n + 1;
    for (size_t k = threadIdx.x; k < N1; k += blockDim.x) {
        G.x[k] = S.x[k]; G.y[k] = S.y[k]; G.z[k] = S.z[k];
        G.vx[k] = S.vx[k]; G.vy[k] = S.vy[k]; G.vz[k] = S.vz[k];
        G.ev_time[k] = S.ev_time[k]; G.ev_potential[k] = S.ev_potential[k];
        if (G.lazy) G.tloc[k] = S.tloc[k];
        G.cx[k] = S.cx[k]; G.cy[k] = S.cy[k]; G.cz[k] = S.cz[k];
        G.type[k] = S.type[k]; G.hb_bond[k] = S.hb_bond[k]; G.hb_itype[k] = S.hb_itype[k];
        G.nb_status[k] = S.nb_status[k]; G.nb_pnum[k] = S.nb_pnum[k];
        G.ev_partner[k] = S.ev_partner[k]; G.ev_type[k] = S.ev_type[k]; G.ev_sub[k] = S.ev_sub[k];
        G.ev_counter[k] = S.ev_counter[k]; G.ev_pcounter[k] = S.ev_pcounter[k];
        for (int q = 0; q < 4; q++) G.nb_partner[4 * k + q] = S.nb_partner[4 * k + q];
    }
    for (size_t k = threadIdx.x; k < N1 + (size_t)G.ncell; k += blockDim.x) G.cell_list[k] = S.cell_list[k];
    for (size_t k = threadIdx.x; k < 2 * N1 + 2; k += blockDim.x) G.cbt_node[k] = S.cbt_node[k];
    for (size_t k = threadIdx.x; k < N1 + 1; k += blockDim.x) G.cbt_leaf[k] = S.cbt_leaf[k];
}

size_t fp64_smem_bytes(int nbcap) { return fp64_smem_bytes_dev(nbcap); }

// Full-rebuild sweep: ResetTarget + Predict over 1..N (src/SGThread.c:47-52), then
// CreateCBT.  With full == 0 only the tree is built (continue mode).  SCR selects
// the FP32-screened prediction (identical results).
template <bool SCR>
__device__ __forceinline__ void sweep_body(const DSys *systems, int full, DSys &S, Blk &B, DScal &C, PairScal &PS) {
    if (threadIdx.x == 0) S = systems[blockIdx.x];
    if (threadIdx.x == 0) { B.err = 0; B.warn = 0; C = *S.sc; S.now = C.time; }
    __syncthreads();
    if (C.err) return;
    Shm M;
    ShmS MS;
    if constexpr (SCR) carve_screen(MS, S.nbcap); else carve(M, S.nbcap);
    if constexpr (SCR) {
        cells_from_list(S, B);
        __syncthreads();
        stage_rp(S);
    }
    if (full) {
        if (S.thermostat && C.smp_avail < S.n) {   // one sample per predicted atom
            if (threadIdx.x == 0) { S.sc->err = SDMD_ECAPACITY; S.sc->err_atom = 0; }
            return;
        }
        for (int i = 1 + threadIdx.x; i <= S.n; i += blockDim.x) {
            S.ev_type[i] = SDMD_EV_INVALID; S.ev_time[i] = INFINIT; S.ev_partner[i] = INVALID;
        }
        __syncthreads();
        for (int i = 1; i <= S.n && B.err == 0; i++) {
            if constexpr (SCR) predict_two(S, i, 0, MS, PS, B, C);
            else predict_atom(S, i, M, B, C);
        }
    }
    if (threadIdx.x == 0) {
        if (B.err == 0) cbt_build(S);
        C.c.warnings += B.warn;
        C.cbt_built = 1;
        if (B.err) { C.err = B.err; C.err_atom = B.err_atom; C.err_event = C.c.frame; }
        *S.sc = C;
    }
}

__global__ void sweep_kernel_fp64(const DSys *systems, int full) {
    __shared__ DSys S;
    __shared__ Blk B;
    __shared__ DScal C;
    __shared__ PairScal PS;
    sweep_body<false>(systems, full, S, B, C, PS);
}
__global__ void sweep_kernel_screen(const DSys *systems, int full) {
    __shared__ DSys S;
    __shared__ Blk B;
    __shared__ DScal C;
    __shared__ PairScal PS;
    sweep_body<true>(systems, full, S, B, C, PS);
}

// The event loop (src/SGThread.c:75-151)
template <bool SCR>
__device__ __forceinline__ void loop_body(const DSys *systems, double t_end_override, int staged, DSys &S, DSys &G,
                                          Blk &B, DScal &C, PairScal &PS, int n_chain = 0) {
    if (threadIdx.x == 0) {
        S = systems[blockIdx.x];
        G = S;
        // a launch of n_chain system blocks plus helper blocks (helper_body): the
        // helpers numbered b = s, s + n_chain, ... advance system s's other atoms
        const int nh = n_chain > 0 ? (int)gridDim.x - n_chain : 0;
        S.adv_h = nh > 0 ? (nh - (int)blockIdx.x + n_chain - 1) / n_chain : 0;
        S.adv_on = S.adv_h > 0 && !S.lazy && S.adv != nullptr;
        S.adv_seq = 0;
    }
    const int tid = threadIdx.x, T = blockDim.x;
    __shared__ int32_t sh_t, sh_p, sh_exec, sh_go;
    __shared__ double sh_dt;
    __shared__ int32_t rec_partner, rec_type, rec_sub;
    __shared__ int32_t sh_move[3], sh_cells_ok, sh_rebase;
    // the records' epoch T0 moves to the current time every 4N pops, so that the
    // interval of now - T0 stays about one mean free flight wide (thread 0's copies)
    int64_t rebase_at = 0, rec_pop0 = 0;
    if (tid == 0) {
        B.err = 0; B.warn = 0; C = *S.sc;
        if (!C.cbt_built && !C.err) { C.err = SDMD_EINVAL; C.err_atom = 0; *S.sc = C; }   // prepare() first
        rebase_at = C.pops + 4 * (int64_t)S.n;
        rec_pop0 = C.pops;
    }
    __syncthreads();
    if (C.err) {
        if (tid == 0 && S.adv_h > 0) st_release(&S.adv->seq, ADV_STOP);
        return;
    }
    Shm M;
    ShmS MS;
    if constexpr (SCR) carve_screen(MS, S.nbcap); else carve(M, S.nbcap);
    if (staged) {
        extern __shared__ __align__(16) unsigned char smem_all[];
        stage_state(S, G, smem_all + (SCR ? screen_smem_bytes_dev(S.nbcap) : fp64_smem_bytes_dev(S.nbcap)), true);
    }
    if constexpr (SCR) {
        cells_from_list(S, B);
        __syncthreads();
        if (tid == 0) sh_cells_ok = B.err == 0;
        stage_rp(S);
        if (S.shr) {   // interval records of every atom for this launch (epoch T0 = now)
            if (tid == 0) {
                S.T0 = C.time;
                S.T0f = __double2float_ru(C.time);
                if (!S.lazy) S.now = C.time;   // eager: the records hold the positions at the clock's value
            }
            __syncthreads();
            for (int k = 1 + tid; k <= S.n; k += T)
                for (int w = 0; w < 4; w++) shadow_word(S, k, w);
            __syncthreads();
            if (tid == 0) { S.shadow_ok = 1; shadow_now(S); }
            __syncthreads();
        }
    }
    const double t_end = t_end_override > 0 ? t_end_override : S.t_end;
    const int64_t stop_at = C.target_frame;
    // denied pops do not advance `frame`; bound the pops so that no input can spin forever
    // (a run without an event limit, stop_at near INT64_MAX, gets 2^40 pops)
    const int64_t left = stop_at - C.c.frame;
    const int64_t pop_limit = C.pops + (left > (int64_t(1) << 34) ? int64_t(1) << 40 : 64 * left + 1000000);
    for (;;) {
        if (tid == 0) {
            if (C.pops >= pop_limit) set_err(B, SDMD_ETIMEOUT, 0);
            int go = (C.time <= t_end) && (C.c.frame < stop_at) && B.err == 0 && !C.at_stop;
            // a pop consumes at most 5 samples (2 predictions + a thermostat event)
            if (go && S.thermostat && C.smp_avail - C.smp_used < 5) { C.paused = 1; go = 0; }
            sh_go = go;
            if (go) {
                const int t = S.cbt_node[1];
                // the popped event's fields into registers before any shared store
                const double tev = S.ev_time[t];
                const int rp = S.ev_partner[t], rt = S.ev_type[t], rs = S.ev_sub[t];
                rec_partner = rp; rec_type = rt; rec_sub = rs;
                sh_t = t;
                if (S.lazy) {   // absolute event times: the clock jumps to the event
                    sh_dt = tev - C.time;
                    S.now = tev;
                    sh_rebase = 0;
                    if (S.shadow_ok) {
                        if (C.pops >= rebase_at) { S.T0 = S.now; rebase_at = C.pops + 4 * (int64_t)S.n; sh_rebase = 1; }
                        shadow_now(S);
                    }
                } else {
                    sh_dt = tev;
                    sh_rebase = 0;
                    // eager: records are rewritten from the positions before this pop's
                    // advance, which belong to the clock's current value
                    if (S.shadow_ok && C.pops >= rebase_at) {
                        S.T0 = C.time; S.T0f = __double2float_ru(C.time); S.now = C.time;
                        rebase_at = C.pops + 4 * (int64_t)S.n; rec_pop0 = C.pops; sh_rebase = 1;
                    }
                    // the helpers start on this pop at once (after the records, when they are rebuilt)
                    if (S.adv_on && !sh_rebase) adv_publish(S, t, rp > 0 ? rp : 0, tev);
                }
                sh_p = rp > 0 ? rp : 0;
            }
        }
        __syncthreads();
        if (!sh_go) break;
        if constexpr (SCR) {
            if (S.shadow_ok && sh_rebase) {   // every record against the new epoch
                for (int k = 1 + tid; k <= S.n; k += T)
                    for (int w = 0; w < 4; w++) shadow_word(S, k, w);
                __syncthreads();
                if (tid == 0 && S.adv_on) adv_publish(S, sh_t, sh_p, sh_dt);
            }
        }
        const double dt = sh_dt;
        const int t = sh_t, p = sh_p;
        if (!S.lazy) {
            if (S.adv_on) {   // the helpers advance the rest; lanes 0-7 take t's and p's x, y, z, time
                if (tid < 8) {
                    const int a = tid < 4 ? t : p, d = tid & 3;
                    if (a > 0) {
                        if (d == 3) S.ev_time[a] -= dt;
                        else {
                            double *X = d == 0 ? S.x : (d == 1 ? S.y : S.z);
                            const double *V = d == 0 ? S.vx : (d == 1 ? S.vy : S.vz);
                            X[a] += V[a] * dt;
                        }
                    }
                }
                if (tid < 32) __syncwarp();
            } else {
                for (int i = 1 + tid; i <= S.n; i += T) {      // UpdateData + TimeForward
                    S.x[i] += S.vx[i] * dt;
                    S.y[i] += S.vy[i] * dt;
                    S.z[i] += S.vz[i] * dt;
                    S.ev_time[i] -= dt;
                }
                __syncthreads();
            }
        }
        sync_pair_warp0(S, t, p);
        if (tid == 0) {
            if (S.lazy) C.time = S.now;
            else {
                C.time += dt;
                S.now = C.time;
                if (S.shadow_ok) {
                    // A record written at the clock value tr bounds x(tr) + v (now - tr).
                    // The reference's position is x(tr) advanced by m separately rounded
                    // steps x += v dt_k, and its clock also rounds at every step, so the
                    // two differ by at most 2u m (|v| |now| + max|x|) per axis
                    // (u = 2^-53), for the m <= pops - rec_pop0 + 1 pops since tr.
                    shadow_now(S);
                    const float m = (float)(C.pops - rec_pop0 + 1);
                    const float c = __fmul_ru(m, 0x1p-51f);
                    S.mxa = __fmul_ru(c, S.xmax32);
                    S.mxb = __fmul_ru(c, __fadd_ru(S.nhi, S.T0f));
                }
            }
            int hazard = p > 0 && S.ev_pcounter[t] < S.ev_counter[p];   // HazardCheck
            sh_exec = !hazard;
            sh_move[0] = 0;
            if (!hazard) {
                C.c.frame++;
                // an HB event rescans the target's neighbourhood: every atom must be current
                if (S.adv_on && S.ev_type[t] == SDMD_EV_HB) adv_wait(S, B);
                do_event(S, C, t, p, B, SCR ? sh_move : nullptr);
                S.ev_counter[t]++;
                if (p) S.ev_counter[p]++;
                // REMDRun's exchange point (src/REMD.c:97): after an executed event at time >= rate
                if (C.stop_time > 0 && C.time >= C.stop_time) C.at_stop = 1;
            } else {
                C.c.recal++;
            }
            // ResetTarget for the renew list
            S.ev_type[t] = SDMD_EV_INVALID; S.ev_time[t] = INFINIT; S.ev_partner[t] = INVALID;
            if (!hazard && p) { S.ev_type[p] = SDMD_EV_INVALID; S.ev_time[p] = INFINIT; S.ev_partner[p] = INVALID; }
        }
        __syncthreads();
        if constexpr (SCR) {
            if (sh_move[0]) {   // a PCC event moved t between cells: update the cell arrays
                if (tid < 32) cell_move_warp(S, sh_move[0], sh_move[1], sh_move[2], B);
                __syncthreads();
            }
        }
        if (B.err) break;
        if constexpr (SCR) {
            // a denied event still brought p's position to now: its record follows
            // (predict_two refreshes the atoms it predicts)
            if (S.shadow_ok && !sh_exec && p && tid < 4) shadow_word(S, p, tid);
            const bool t_tree = predict_two(S, t, sh_exec ? p : 0, MS, PS, B, C);
            if (tid < 32 && B.err == 0) {
                if (!t_tree) cbt_update_warp(S, t);
                if (sh_exec && p) cbt_update_warp(S, p, t_tree);
            }
        } else {
            predict_atom(S, t, M, B, C);
            if (sh_exec && p && B.err == 0) predict_atom(S, p, M, B, C);
            if (tid == 0) {
                cbt_update(S, t);
                if (sh_exec && p) cbt_update(S, p);
            }
        }
        if (tid == 0) {
            if (S.trace_cap > 0) record_trace(S, C, t, p, rec_partner, rec_type, rec_sub, sh_exec, dt);
            C.pops++;
        }
        __syncthreads();
    }
    if (tid == 0 && S.adv_h > 0) st_release(&S.adv->seq, ADV_STOP);   // the helpers stop
    if constexpr (SCR) {
        __syncthreads();
        if (sh_cells_ok) cells_to_list(S);
    }
    if (staged) {
        __syncthreads();
        unstage_state(S, G);
    }
    if (tid == 0) {
        C.c.warnings += B.warn;
        if (B.err) { C.err = B.err; C.err_atom = B.err_atom; C.err_event = C.c.frame; }
        *G.sc = C;
    }
}

__global__ void loop_kernel_fp64(const DSys *systems, double t_end_override, int staged) {
    __shared__ DSys S, G;   // G: the global-memory view (write-back target when staged)
    __shared__ Blk B;
    __shared__ DScal C;
    __shared__ PairScal PS;
    loop_body<false>(systems, t_end_override, staged, S, G, B, C, PS);
}
__global__ void loop_kernel_screen(const DSys *systems, double t_end_override, int staged) {
    __shared__ DSys S, G;
    __shared__ Blk B;
    __shared__ DScal C;
    __shared__ PairScal PS;
    loop_body<true>(systems, t_end_override, staged, S, G, B, C, PS);
}

// The same loop built for at most 128 registers a thread (up to 256 threads, two
// CTAs per SM): for batches with more systems than the full build keeps resident,
// where registers, not shared memory, bound the CTAs per SM.
__global__ void __launch_bounds__(256, 2) loop_kernel_screen_r128(const DSys *systems, double t_end_override,
                                                                   int staged) {
    __shared__ DSys S, G;
    __shared__ Blk B;
    __shared__ DScal C;
    __shared__ PairScal PS;
    loop_body<true>(systems, t_end_override, staged, S, G, B, C, PS);
}

__global__ void loop_kernel_screen_coop(const DSys *systems, double t_end_override, int n_chain) {
    __shared__ DSys S, G;
    __shared__ Blk B;
    __shared__ DScal C;
    __shared__ PairScal PS;
    if ((int)blockIdx.x >= n_chain) {
        helper_body(systems, n_chain);
        return;
    }
    loop_body<true>(systems, t_end_override, 0, S, G, B, C, PS, n_chain);
}

// The same launch built for 512 threads a block (at most 128 registers a thread):
// dense systems, whose hundreds of candidates per atom then take half the screen
// passes.
__global__ void __launch_bounds__(512, 1) loop_kernel_screen_coop512(const DSys *systems, double t_end_override,
                                                                     int n_chain) {
    __shared__ DSys S, G;
    __shared__ Blk B;
    __shared__ DScal C;
    __shared__ PairScal PS;
    if ((int)blockIdx.x >= n_chain) {
        helper_body(systems, n_chain);
        return;
    }
    loop_body<true>(systems, t_end_override, 0, S, G, B, C, PS, n_chain);
}

size_t screen_smem_bytes(int nbcap) { return screen_smem_bytes_dev(nbcap); }
size_t verify_smem_bytes(int nbcap, int warps) { return verify_warp_bytes(nbcap) * (size_t)warps; }

}  // namespace sdmd

namespace sdmd {
// lazy mode entry: positions are valid now, event times become absolute
__global__ void lazy_enter_kernel(const DSys *systems) {
    const DSys &S = systems[blockIdx.x];
    double T = S.sc->time;
    for (int i = 1 + threadIdx.x; i <= S.n; i += blockDim.x) {
        S.tloc[i] = T;
        S.ev_time[i] = S.ev_time[i] + T;
    }
}
}  // namespace sdmd
