// dev.cuh -- device-side system view and the physics of one event loop step.
//
// Every function restates a reference routine (file:line given) in FP64 with the
// reference's association order.  The translation unit is compiled with
// -fmad=false so that no multiply-add is contracted: results are bit-identical
// to the reference's x86-64 -O2 build, which has no FMA contraction either.
#pragma once
#include <cstdint>
#include "sdmd_gpu.h"

namespace sdmd {

constexpr double ZERO = SDMD_ZERO;
constexpr double INFINIT = SDMD_INFINIT;
constexpr int INVALID = SDMD_INVALID;
constexpr int NT = SDMD_NTYPES;

// per-system scalars living in device memory
struct DScal {
    double time;
    sdmd_rng rng;            // rand() state after every consumed draw
    sdmd_counters c;
    int32_t err, err_atom;
    int64_t err_event;
    int64_t pops;            // total pops (trace ring position)
    int32_t cbt_built;
    int32_t paused;          // 1: the loop stopped because its normal-sample batch ran low
    sdmd_rng rng0;           // state at the start of the current sample batch
    int64_t smp_avail, smp_used;
    int64_t target_frame;    // the run stops once c.frame reaches it
    int32_t sw_nflag;        // parallel sweep: atoms left for the in-order re-prediction
    int32_t at_stop;         // the loop stopped at stop_time (replica exchange)
    double stop_time;        // > 0: stop after the first executed event with time >= stop_time
};

// Eager advance by helper blocks (large systems, one cooperative launch).  The
// system's own block publishes each pop (seq, dt, target, partner) with a release
// store; the helper blocks advance every other atom (UpdateData / TimeForward,
// src/ToolFunctions.c:23-36) and count their completions in `done` with release
// adds.  The two groups of fields sit on separate 128-byte lines.
constexpr unsigned long long ADV_STOP = ~0ull;
struct __align__(128) Adv {
    unsigned long long seq;   // pops published so far; ADV_STOP ends the helpers
    double dt;
    int32_t t, p;
    int32_t herr;             // set by a helper whose wait for the next pop ran out
    int32_t pad0[25];
    unsigned long long done;  // helper completions, all pops together
    int32_t pad1[30];
};

__device__ __forceinline__ unsigned long long ld_acquire(const unsigned long long *p) {
    unsigned long long v;
    asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release(unsigned long long *p, unsigned long long v) {
    asm volatile("st.release.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ void red_release_add(unsigned long long *p, unsigned long long v) {
    asm volatile("red.release.gpu.global.add.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ unsigned long long gtimer() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
constexpr unsigned long long ADV_WAIT_NS = 2000000000ull;   // 2 s without progress ends a wait

// one system's device arrays (all 1-based per-atom arrays, entry 0 unused)
struct DSys {
    int32_t n, ncell;
    int32_t cn[3];
    int32_t thermostat, wall, wall_type;
    double box[3], cs[3], cutoff, temperature, thermo_freq, t_end;
    double wall_pos[3], wall_vel[3], hb_barrier[3];
    int32_t n_sph;                 // spherical obstacles: x, y, z, radius each
    const double *sph;
    int32_t n_obst;                // obstruction walls: position[1..3] each, -1 off their axis
    const double *obst;
    // static
    const double *mass;
    const int32_t *protein, *aanum, *aatype, *hb_neighbor, *hb_role, *name_code;
    const int32_t *bond_off, *bond_j;
    const double *bond_dmin, *bond_dmax;
    const int32_t *con_off, *con_j, *con_step_off, *con_step_n;
    const double *con_dmin, *con_dmax, *con_step_d, *con_step_e, *con_step_acc;
    const int32_t *conn_off, *conn_j, *conn_bits;
    const double *pair_dmin, *pair_dmax;
    const int32_t *pair_step_off, *pair_step_n;
    const double *pair_step_d, *pair_step_e, *pair_step_acc;
    // dynamic
    double *x, *y, *z, *vx, *vy, *vz;
    int32_t *cx, *cy, *cz, *type, *hb_bond, *hb_itype, *nb_partner, *nb_status, *nb_pnum;
    double *ev_time;
    int32_t *ev_partner;
    int64_t *ev_counter, *ev_pcounter;
    double *ev_potential;
    int32_t *ev_type, *ev_sub;
    int32_t *cell_list;
    int32_t *cbt_node, *cbt_leaf;
    DScal *sc;
    sdmd_trace_rec *trace;
    int32_t trace_cap;
    int32_t nbcap;           // capacity of the gathered 27-cell neighbour list
    // precomputed standard-normal samples of the rand() stream (see samples.cu)
    double *smp;             // sample values, consumed in order
    int32_t *smp_raw;        // 3 rand() outputs per sample (a, b, coin)
    int64_t *smp_cum;        // rand() calls consumed up to and including sample k
    int32_t smp_cap;
    int32_t n_bonds, n_cons, n_con_steps, n_conn;
    // lazy free flight: positions are valid at tloc[i]; event times are absolute
    double *tloc;
    int32_t lazy, pad3;
    double now;              // the current time while a block works on this system
    // FP32 screen: float brackets [lo, hi] around FP64 thresholds and limits
    // (built on the host, see api.cu).  Per pair-table entry 8 floats:
    // fl(dmin - ZERO), fl(dmax + ZERO), dmin, dmax; per pooled step 6 floats:
    // fl(d + ZERO), fl(d - ZERO), d; constraints as pair entries / steps; per bond
    // 4 floats: dmin, dmax.
    const float *pair_thr32, *pair_step32, *con_thr32, *con_step32, *bond32;
    float cut32[2], zero32[2], box32[6];
    int32_t screen, pad4;
    // exact refine: the same FP64 thresholds as ordered integer keys (tkey), so a
    // comparison costs an integer compare instead of an FP64 add and compare.
    // Per pair entry / constraint 2 keys: fl(dmin - ZERO), fl(dmax + ZERO); per
    // pooled step 2 keys: fl(d + ZERO), fl(d - ZERO).
    const long long *pair_key, *pair_stepkey, *con_key, *con_stepkey;
    long long cut_key;               // tkey((0.9 cutoff)^2)
    // connection-map bits of atom i for partners i-64 .. i+63: [base, 4 BOND
    // words, 4 CONSTRAINT words]; base < 0 when the row does not fit the window
    const int32_t *conn_win;
    // screened path: per-cell atom arrays, the cell lists in insertion order (the
    // reference's list head is the last entry); authoritative inside the screened
    // kernels, which rebuild cell_list from them before they return
    int32_t *cell_cnt, *cell_arr;
    int32_t maxc;
    // CheckDuplication only considers partners j < dup_limit: INT32_MAX in the event
    // loop; the parallel full-rebuild sweep lowers it (0 while every atom is
    // predicted at once, i while atom i is re-predicted in atom order)
    int32_t dup_limit;
    // the CBT leaf layout CreateCBT produces for N atoms (it depends on N only)
    const int32_t *cbt_leaf0;
    // parallel full-rebuild sweep scratch: pre-sweep HB interaction type, and the
    // atoms whose adopted duplicate differs from their own fresh offer
    int32_t *sw_hbit, *sw_flag, *sw_warn;
    // RightPair (src/ToolFunctions.c:278-292) of every type pair, resolved on the
    // host: the table-0 entry of (t1, t2), or -1 (33 x 33)
    const int16_t *rp_idx;
    // per atom i: the constraint of i with partner i-64 .. i+63 as an offset into
    // i's constraint list (first occurrence), -1 for none; con_ok[i] = 0 when a
    // partner lies outside the window (the list is then searched)
    const int8_t *con_win, *con_ok;
    // screened path: per atom a 64-byte record of outward-rounded FP32 intervals --
    // {x, y}, {z, vx}, {vy, vz}, {tr - T0, packed cell} -- so that a candidate's
    // position interval costs FP32 work only; valid while shadow_ok.  tr is the
    // time the record's position belongs to: tloc in lazy mode, the clock value of
    // the pop that wrote the record in eager mode.  [nlo, nhi] holds now - T0 for
    // the event being predicted.
    float4 *shr;
    double T0;
    int32_t shadow_ok;
    float nlo, nhi;
    // eager mode: the record bounds x(tr) + v (now - tr), while the position the
    // reference's step-by-step advance reaches differs from it by the rounding of
    // the pops since tr.  Per axis that is at most mxa + mxb |v| (see loop_body);
    // xmax32 bounds |x| for every atom (4 times the largest box edge).
    float mxa, mxb, xmax32;
    float T0f;                // an upper bound of T0 as a float (eager mode)
    // eager mode with helper blocks: adv_on in the block's copy while they run,
    // adv_h of them advance this system, adv_seq pops published so far
    Adv *adv;
    int32_t adv_on, adv_h;
    unsigned long long adv_seq;
};

// position component of atom j at the current time (lazy mode extrapolates)
__device__ __forceinline__ double lzx(const DSys &S, const double *x, const double *v, int j) {
    return S.lazy ? x[j] + v[j] * (S.now - S.tloc[j]) : x[j];
}

// Total order on doubles as a signed 64-bit key (equal keys for +0.0 and -0.0):
// FP64 compares cost as much as FP64 arithmetic on this part, integer compares
// do not.
__device__ __forceinline__ long long tkey(double d) {
    long long b = __double_as_longlong(d);
    return b >= 0 ? b : -(b & 0x7fffffffffffffffLL);
}

// 27-cell scan order of the reference (src/DMD.c:117-121)
__constant__ int8_t c_nbx[27] = {0, 1, 0, 0, 0, 1, 1, 1, -1, 0, 0, 0, -1, -1, -1, 0, 0, 1, -1, 1, -1, -1, -1, 1, 1, 1, -1};
__constant__ int8_t c_nby[27] = {0, 0, 1, 0, 1, 0, 1, 1, 0, -1, 0, -1, 0, -1, -1, -1, 1, 0, 0, -1, 1, -1, 1, -1, 1, -1, 1};
__constant__ int8_t c_nbz[27] = {0, 0, 0, 1, 1, 1, 0, 1, 0, 0, -1, -1, -1, 0, -1, 1, -1, -1, 1, 0, 0, 1, -1, -1, -1, 1, 1};

enum { K_COLLISION = 0, K_CONSTRAINT = 1, K_HB = 2, K_NEIGHBOR = 3 };

// ---------------------------------------------------------------------------
// glibc-compatible rand(): additive feedback r[i] = r[i-3] + r[i-31] mod 2^32,
// output r >> 1 (TYPE_3: degree 31, separation 3).
__device__ inline int32_t rng_next(sdmd_rng &r) {
    uint32_t v = (uint32_t)r.tab[r.front] + (uint32_t)r.tab[r.rear];
    r.tab[r.front] = (int32_t)v;
    int32_t out = (int32_t)((v >> 1) & 0x7fffffffu);
    if (++r.front >= 31) { r.front = 0; ++r.rear; }
    else if (++r.rear >= 31) r.rear = 0;
    return out;
}
// RandomValue(0, 1) (src/ToolFunctions.c:517-522)
__device__ inline double rv01(sdmd_rng &r) { return 0 + (double)rng_next(r) / ((double)2147483647 / (1 - 0)); }

// ---- correctly rounded log: double-double evaluation of e*ln2 + 2*atanh(f) ----
struct dd { double hi, lo; };
__device__ inline dd two_sum(double a, double b) {
    double s = a + b, bb = s - a;
    return {s, (a - (s - bb)) + (b - bb)};
}
__device__ inline dd quick_two_sum(double a, double b) { double s = a + b; return {s, b - (s - a)}; }
__device__ inline dd two_prod(double a, double b) { double p = a * b; return {p, fma(a, b, -p)}; }  // exact
__device__ inline dd dd_add(dd a, dd b) {
    dd s = two_sum(a.hi, b.hi), t = two_sum(a.lo, b.lo);
    s.lo += t.hi; s = quick_two_sum(s.hi, s.lo); s.lo += t.lo;
    return quick_two_sum(s.hi, s.lo);
}
__device__ inline dd dd_mul(dd a, dd b) {
    dd p = two_prod(a.hi, b.hi);
    p.lo += a.hi * b.lo + a.lo * b.hi;
    return quick_two_sum(p.hi, p.lo);
}
__device__ inline dd inv_odd(int k) {
    double n = (double)(2 * k + 1), h = 1.0 / n;
    dd p = two_prod(h, n);
    double rem = (1.0 - p.hi) - p.lo;
    return quick_two_sum(h, rem / n);
}
// natural log for normal x > 0 (the Box-Muller argument lies in (0, 1))
__device__ inline double cr_log(double x) {
    long long bits = __double_as_longlong(x);
    int e = (int)((bits >> 52) & 0x7ff) - 1023;
    double m = __longlong_as_double((bits & 0x000fffffffffffffLL) | 0x3ff0000000000000LL);  // [1, 2)
    if (m > 1.4142135623730951) { m *= 0.5; e += 1; }
    double num = m - 1.0;
    dd den = two_sum(m, 1.0);
    double q1 = num / den.hi;
    dd p = dd_mul({q1, 0.0}, den);
    dd rr = dd_add({num, 0.0}, {-p.hi, -p.lo});
    dd f = quick_two_sum(q1, rr.hi / den.hi);
    dd z = dd_mul(f, f);
    double t = 1.0 / 43.0;
    for (int k = 20; k >= 11; k--) t = t * z.hi + 1.0 / (double)(2 * k + 1);
    dd acc = {t, 0.0};
    for (int k = 10; k >= 0; k--) acc = dd_add(dd_mul(acc, z), inv_odd(k));
    dd lm = dd_mul(f, acc);
    lm.hi *= 2.0; lm.lo *= 2.0;
    const dd LN2 = {0x1.62e42fefa39efp-1, 0x1.abc9e3b39803fp-56};
    dd el = dd_add(two_prod((double)e, LN2.hi), {(double)e * LN2.lo, 0.0});
    dd r = dd_add(el, lm);
    return r.hi + r.lo;
}
// 1/n in double-double (n > 0)
__device__ inline dd dd_inv(int n) {
    double nd = (double)n, h = 1.0 / nd;
    dd p = two_prod(h, nd);
    double rem = (1.0 - p.hi) - p.lo;
    return quick_two_sum(h, rem / nd);
}
// e^x (the replica-exchange test, src/Server.c:169): x = k ln2 + r with the
// reduction in double-double (|r| <= ln2/2), e^r by its Taylor series in Horner
// form in double-double, then 2^k.  Correctly rounded unless e^x lies within about
// 2^-100 relative of a rounding boundary; results in the subnormal range are
// rounded twice.
__device__ inline double cr_exp(double x) {
    if (x != x) return x;
    if (x > 709.782712893384) return __longlong_as_double(0x7ff0000000000000LL);
    if (x < -745.2) return 0.0;
    const double kd = rint(x * 1.4426950408889634);
    const dd LN2 = {0x1.62e42fefa39efp-1, 0x1.abc9e3b39803fp-56};
    dd kl = dd_add(two_prod(kd, LN2.hi), {kd * LN2.lo, 0.0});
    dd r = dd_add({x, 0.0}, {-kl.hi, -kl.lo});
    dd acc = {1.0, 0.0};
    for (int n = 22; n >= 1; n--) acc = dd_add({1.0, 0.0}, dd_mul(dd_mul(r, dd_inv(n)), acc));
    return ldexp(acc.hi + acc.lo, (int)kd);
}

// Maxwell_Boltzmann_Distribution (src/ToolFunctions.c:544-569).  The rejection
// loops are bounded: a healthy stream accepts with probability pi/4 per attempt,
// so 4096 consecutive rejections only happen for a degenerate (e.g. all-zero)
// RNG state; *bad is then set and 0 returned instead of spinning.
__device__ inline double mb_draw(sdmd_rng &r, double mean, double variance, int *bad) {
    double a, b, s, out = 0;
    for (int outer = 0; outer < 64; outer++) {
        int tries = 0;
        do {
            a = 2 * rv01(r) - 1;
            b = 2 * rv01(r) - 1;
            s = a * a + b * b;
        } while (s >= 1 && ++tries < 4096);
        if (s >= 1) { *bad = 1; return 0; }
        s = sqrt(-2 * cr_log(s) / s);
        double choose = rv01(r);
        out = (choose >= 0.5) ? a * s : b * s;
        if (out != 0) return out * sqrt(variance) + mean;
    }
    *bad = 1;
    return 0;
}

// ---------------------------------------------------------------------------
__device__ inline int cell_lin(const DSys &S, int cx, int cy, int cz) {
    return cz * S.cn[0] * S.cn[1] + cy * S.cn[0] + cx + 1;
}
__device__ inline int nb_cell(const DSys &S, int i, int k) {
    int c0 = S.cx[i] + c_nbx[k], c1 = S.cy[i] + c_nby[k], c2 = S.cz[i] + c_nbz[k];
    if (c0 < 0) c0 = S.cn[0] - 1; else if (c0 >= S.cn[0]) c0 = 0;
    if (c1 < 0) c1 = S.cn[1] - 1; else if (c1 >= S.cn[1]) c1 = 0;
    if (c2 < 0) c2 = S.cn[2] - 1; else if (c2 >= S.cn[2]) c2 = 0;
    return cell_lin(S, c0, c1, c2);
}

// AtomTypeChange (src/ToolFunctions.c:233-270)
__device__ inline int type_change(int t, int to_hb) {
    if (to_hb) { if (t == 1) return 3; if (t == 2) return 4; if (t == 26) return 27; }
    else { if (t == 3) return 1; if (t == 4) return 2; if (t == 27) return 26; }
    return t;
}
__device__ inline int tab_idx(int t, int a, int b) { return (t * NT + a) * NT + b; }

// RightPair (src/ToolFunctions.c:278-292), unrolled recursion
__device__ inline int right_pair(const DSys &S, int t1, int t2) {
    if (S.pair_dmin[tab_idx(0, t1, t2)] > 0) return tab_idx(0, t1, t2);
    int a = type_change(t1, 0), b = type_change(t2, 0);
    if (S.pair_dmin[tab_idx(0, a, t2)] > 0) return tab_idx(0, a, t2);
    if (S.pair_dmin[tab_idx(0, t1, b)] > 0) return tab_idx(0, t1, b);
    if (S.pair_dmin[tab_idx(0, a, b)] > 0) return tab_idx(0, a, b);
    return -1;
}

// HBModel (src/Models.c:212-290): class 1..11, -1 "no HB", 0 (with *bad) fatal
__device__ inline int hb_model(const DSys &S, int a1, int a2, int *bad) {
    if (S.hb_role[a1] == 'A' || S.hb_role[a1] == 'S') { int t = a1; a1 = a2; a2 = t; }
    int t1 = type_change(S.type[a1], 0), t2 = type_change(S.type[a2], 0);
    int aa2 = S.aatype[a2];
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
    *bad = 1;
    return 0;
}

// HBBarrier (src/Events.c:1097-1119)
__device__ inline double hb_barrier(const DSys &S, int a1, int a2) {
    if (S.hb_role[a1] == 'A' || S.hb_role[a1] == 'S') { int t = a1; a1 = a2; a2 = t; }
    int t1 = type_change(S.type[a1], 0), t2 = type_change(S.type[a2], 0);
    if (t1 == 2 && t2 == 26) return S.hb_barrier[0];
    if (t1 != 2 && t2 != 26) return S.hb_barrier[2];
    return S.hb_barrier[1];
}

__device__ inline int conn_bits(const DSys &S, int i, int j) {
    for (int k = S.conn_off[i], e = S.conn_off[i + 1]; k < e; k++)
        if (S.conn_j[k] == j) return S.conn_bits[k];
    return 0;
}

// FindElemInList(neighborPartner, j, -1, -1, 0) (src/ToolFunctions.c:1062-1087)
__device__ inline int nb_has(const DSys &S, int i, int j) {
    const int32_t *l = S.nb_partner + 4 * i;
    for (int k = 0; k < 4; k++) {
        int v = l[k];
        if (v == 0) return 0;
        if (v == j) return k + 1;
    }
    return 0;
}

struct Lim { double lo, up, lopot, uppot, acc; };

// FindPair (src/ToolFunctions.c:39-224).  Returns coreorShell; *warn counts the
// reference's warningsum increments; *bad flags a fatal table miss.
__device__ inline int find_pair(const DSys &S, int a1, int a2, int kind, double direction, double distance2,
                                Lim &o, int hbpartner, int tc, int wall_type2, int *warn, int *bad) {
    int cs = -1;
    double dir = direction < 0 ? 1 : -1;
    double tol = dir * ZERO;
    double dmin, dmax;
    const double *sd, *se, *sa;
    int sn;
    if (kind == K_CONSTRAINT) {
        int k = S.con_off[a1], e = S.con_off[a1 + 1];
        for (; k < e; k++) if (S.con_j[k] == a2) break;
        if (k == e) { *bad = 1; return -1; }
        dmin = S.con_dmin[k]; dmax = S.con_dmax[k]; sn = S.con_step_n[k];
        int so = S.con_step_off[k];
        sd = S.con_step_d + so; se = S.con_step_e + so; sa = S.con_step_acc + so;
    } else {
        int e;
        if (kind == K_COLLISION) {
            int t1 = S.type[a1];
            if (tc == 1) t1 = type_change(t1, 1);
            else if (tc == -1) t1 = type_change(t1, 0);
            int t2 = a2 ? S.type[a2] : wall_type2;
            e = right_pair(S, t1, t2);
            if (e < 0) { *bad = 1; return -1; }
        } else if (kind == K_HB) {
            int tn = hb_model(S, a1, a2, bad);
            if (tn < 0) { *bad = 1; tn = 0; }   // the reference indexes table -1 here; refuse instead
            e = tab_idx(tn, 0, 0);
        } else {
            int tn = hb_model(S, a2, hbpartner, bad);
            if (tn < 0) { *bad = 1; tn = 0; }
            e = tab_idx(tn, type_change(S.type[a1], 0), type_change(S.type[a2], 0));
        }
        dmin = S.pair_dmin[e]; dmax = S.pair_dmax[e]; sn = S.pair_step_n[e];
        int so = S.pair_step_off[e];
        sd = S.pair_step_d + so; se = S.pair_step_e + so; sa = S.pair_step_acc + so;
    }
    int flag = (sn == 0);
    if (dmin == 0) { *bad = 1; return -1; }
    int a1bond = a1 ? S.hb_bond[a1] : 0, a2bond = a2 ? S.hb_bond[a2] : 0;
    int warnable = !(kind == K_NEIGHBOR && a2bond == 0) && !(kind == K_HB && a1bond == 0);
    if (distance2 < dmin - ZERO) {
        o.lo = INFINIT; o.up = INFINIT; o.acc = INFINIT; o.lopot = 0; o.uppot = 0;
        if (warnable) ++*warn;
        return cs;
    }
    o.lo = dmin; o.lopot = 0;
    for (int q = 0; q < sn; q++) {
        double d = sd[q];
        if (d == 0) break;
        if (distance2 < d + tol) {
            o.up = d; o.uppot = -1 * se[q]; o.acc = sa[q];
            if (q == 0) return 0;
            if (kind == K_HB && q == sn - 1 && a1bond > 0) return 1;
            if (kind == K_NEIGHBOR && q == sn - 1 && a2bond > 0) { o.uppot = 0; return 1; }
            return cs;
        }
        o.lo = d; o.lopot = se[q];
    }
    if (kind == K_HB && a1bond > 0) ++*warn;
    if (dmax > 0) {
        if (distance2 < dmax + ZERO) {
            o.up = dmax; o.uppot = 0; o.acc = 0;
            cs = 1;
            if (flag == 1 && dir == 1) cs = 0;
            return cs;
        }
        o.lo = INFINIT; o.up = INFINIT; o.acc = INFINIT; o.lopot = 0; o.uppot = 0;
        if (warnable) ++*warn;
    } else {
        o.up = INFINIT; o.uppot = INFINIT; o.acc = INFINIT;
        return 1;
    }
    return cs;
}

struct Kin { double r2, b, v2, rx, ry, rz; };

// PBCShift + CalculateParameters (src/ToolFunctions.c:801-817, src/TimePrediction.c:1081-1090)
__device__ inline void pair_kin(const DSys &S, int i, int j, Kin &k) {
    const int ci[3] = {S.cx[i], S.cy[i], S.cz[i]}, cj[3] = {S.cx[j], S.cy[j], S.cz[j]};
    double sh[3];
#pragma unroll
    for (int d = 0; d < 3; d++) {
        sh[d] = 0;
        if (ci[d] != cj[d]) {
            if (ci[d] == 0 && cj[d] == S.cn[d] - 1) sh[d] = -1 * S.box[d];
            else if (ci[d] == S.cn[d] - 1 && cj[d] == 0) sh[d] = S.box[d];
        }
    }
    double rx = lzx(S, S.x, S.vx, i) - (lzx(S, S.x, S.vx, j) + sh[0]);
    double ry = lzx(S, S.y, S.vy, i) - (lzx(S, S.y, S.vy, j) + sh[1]);
    double rz = lzx(S, S.z, S.vz, i) - (lzx(S, S.z, S.vz, j) + sh[2]);
    double vx = S.vx[i] - S.vx[j], vy = S.vy[i] - S.vy[j], vz = S.vz[i] - S.vz[j];
    k.rx = rx; k.ry = ry; k.rz = rz;
    k.r2 = rx * rx + ry * ry + rz * rz;
    k.b = rx * vx + ry * vy + rz * vz;
    k.v2 = vx * vx + vy * vy + vz * vz;
}

// CalculateDisc / CalculateTime (src/TimePrediction.c:1092-1099)
__device__ inline double disc(const Kin &k, double shortlim) { return k.b * k.b - k.v2 * (k.r2 - shortlim); }
__device__ inline double root(const Kin &k, int st, double d2) {
    return (-1 * k.b + st * sqrt(k.b * k.b - k.v2 * (k.r2 - d2))) / k.v2;
}

}  // namespace sdmd
