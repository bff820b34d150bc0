// screen.cuh -- FP32 interval screen + lane-packed FP64 refine for Predict.
//
// Included at the end of loop_fp64.cu: it reuses that file's exact FP64 pieces
// (eval_bond / eval_collision / eval_hb_scan, the fold helpers, the events).
//
// Why: on GB300 a warp issues one FP64 instruction per ~64 cycles whatever its
// active mask, while FP32 issues ~50x faster.  Evaluating every 27-cell
// candidate in FP64 therefore costs ~100 FP64 warp-instructions per warp pass.
//
// How, with results identical to the exact path:
//   1. every candidate of the target (and of the partner) is screened in FP32
//      with outward-rounded intervals that follow the reference's FP64
//      operation sequence step by step (rounding is monotone, so every FP64
//      intermediate lies inside its interval).  The screen decides each
//      branch of CollisionTime / BondTime / HBTime / FindPair with certainty
//      or marks the candidate "refine";
//   2. U = the smallest upper time bound over bond and collision offers that
//      are certainly made: the bond/collision part of the fold ends at or below
//      U.  Offers whose lower bound exceeds U' = max(U, every duplicate time)
//      can neither be a running-minimum record of the fold nor change the
//      outcome of a duplicate check, so they are dropped (their warning counts
//      are certain and still added);
//   3. the remaining candidates (typically 1-4 per atom) are recomputed
//      exactly with the FP64 code of the plain path, packed into lanes: the
//      FP64 cost is per warp instruction, so one pass covers up to 32 of them;
//   4. thread 0 folds the refined offers in the reference's scan order
//      (JobAssign's strict "<", CheckDuplication), exactly as the plain path.
#pragma once

namespace sdmd {

// ---- outward-rounded FP32 intervals ----------------------------------------------
struct Iv { float lo, hi; };

__device__ __forceinline__ float f_dn(float x) {   // next float toward -inf
    if (x > 0.f) return __uint_as_float(__float_as_uint(x) - 1u);
    if (x == 0.f) return -0x1p-149f;
    if (isinf(x)) return x;
    return __uint_as_float(__float_as_uint(x) + 1u);
}
__device__ __forceinline__ float f_up(float x) {   // next float toward +inf
    if (x < 0.f) return __uint_as_float(__float_as_uint(x) - 1u);
    if (x == 0.f) return 0x1p-149f;
    if (isinf(x)) return x;
    return __uint_as_float(__float_as_uint(x) + 1u);
}
// a double as an interval: round to nearest, widen by the worst rounding error
__device__ __forceinline__ Iv ivd(double d) {
    float m = __double2float_rn(d);
    float e = __fmaf_ru(fabsf(m), 0x1p-24f, 0x1p-149f);
    return {__fsub_rd(m, e), __fadd_ru(m, e)};
}
__device__ __forceinline__ Iv ivc(float lo, float hi) { return {lo, hi}; }
__device__ __forceinline__ Iv iadd(Iv a, Iv b) { return {__fadd_rd(a.lo, b.lo), __fadd_ru(a.hi, b.hi)}; }
__device__ __forceinline__ Iv isub(Iv a, Iv b) { return {__fsub_rd(a.lo, b.hi), __fsub_ru(a.hi, b.lo)}; }
__device__ __forceinline__ Iv ineg(Iv a) { return {-a.hi, -a.lo}; }
__device__ __forceinline__ Iv imul(Iv a, Iv b) {
    float l1 = __fmul_rd(a.lo, b.lo), l2 = __fmul_rd(a.lo, b.hi), l3 = __fmul_rd(a.hi, b.lo), l4 = __fmul_rd(a.hi, b.hi);
    float h1 = __fmul_ru(a.lo, b.lo), h2 = __fmul_ru(a.lo, b.hi), h3 = __fmul_ru(a.hi, b.lo), h4 = __fmul_ru(a.hi, b.hi);
    return {fminf(fminf(l1, l2), fminf(l3, l4)), fmaxf(fmaxf(h1, h2), fmaxf(h3, h4))};
}
__device__ __forceinline__ Iv isqr(Iv a) {
    if (a.lo >= 0.f) return {__fmul_rd(a.lo, a.lo), __fmul_ru(a.hi, a.hi)};
    if (a.hi <= 0.f) return {__fmul_rd(a.hi, a.hi), __fmul_ru(a.lo, a.lo)};
    return {0.f, fmaxf(__fmul_ru(a.lo, a.lo), __fmul_ru(a.hi, a.hi))};
}
// sqrt of an interval with a.lo >= 0 (IEEE round-to-nearest, stepped outward)
__device__ __forceinline__ Iv isqrt(Iv a) {
    float lo = a.lo > 0.f ? f_dn(__fsqrt_rn(a.lo)) : 0.f;
    return {lo > 0.f ? lo : 0.f, f_up(__fsqrt_rn(a.hi))};
}
// a / b with b.lo > 0 (IEEE round-to-nearest quotients, stepped outward)
__device__ __forceinline__ Iv idiv(Iv a, Iv b) {
    float ql, qh;
    if (a.lo >= 0.f) { ql = __fdiv_rn(a.lo, b.hi); qh = __fdiv_rn(a.hi, b.lo); }
    else if (a.hi <= 0.f) { ql = __fdiv_rn(a.lo, b.lo); qh = __fdiv_rn(a.hi, b.hi); }
    else { ql = __fdiv_rn(a.lo, b.lo); qh = __fdiv_rn(a.hi, b.lo); }
    return {f_dn(ql), f_up(qh)};
}
// is the FP64 value inside `a` below the FP64 threshold bracketed by thr[0..1]?
// 1 certainly, 0 certainly not, 2 undecided (also for NaN)
__device__ __forceinline__ int lt3(Iv a, const float *thr) {
    if (a.hi < thr[0]) return 1;
    if (a.lo >= thr[1]) return 0;
    return 2;
}
__device__ __forceinline__ bool dbl_is_zero(double d) { return (__double_as_longlong(d) << 1) == 0; }
__device__ __forceinline__ bool dbl_pos(double d) { return __double_as_longlong(d) > 0; }   // d > 0 (no NaN in tables)

// ---- positions and pair kinematics as intervals ---------------------------------
struct PIv { Iv x[3], v[3]; int c[3]; };

// the FP64 position lzx() would produce, and the velocity, of atom j
__device__ __forceinline__ void atom_piv(const DSys &S, int j, PIv &P) {
    const double *X[3] = {S.x, S.y, S.z}, *V[3] = {S.vx, S.vy, S.vz};
    Iv dti{0.f, 0.f};
    if (S.lazy) dti = ivd(S.now - S.tloc[j]);
#pragma unroll
    for (int d = 0; d < 3; d++) {
        Iv xv = ivd(X[d][j]), vv = ivd(V[d][j]);
        P.v[d] = vv;
        P.x[d] = S.lazy ? iadd(xv, imul(vv, dti)) : xv;
    }
    P.c[0] = S.cx[j]; P.c[1] = S.cy[j]; P.c[2] = S.cz[j];
}

struct KIv { Iv r2, b, v2; };

// pair_kin() as intervals: r = r_i - (r_j + shift), v = v_i - v_j, r2, b, v2
__device__ __forceinline__ void kin_iv(const DSys &S, const PIv &I, const PIv &J, KIv &k) {
    Iv r[3], v[3];
#pragma unroll
    for (int d = 0; d < 3; d++) {
        Iv xj = J.x[d];
        if (I.c[d] != J.c[d]) {
            if (I.c[d] == 0 && J.c[d] == S.cn[d] - 1) xj = iadd(xj, ineg(ivc(S.box32[2 * d], S.box32[2 * d + 1])));
            else if (I.c[d] == S.cn[d] - 1 && J.c[d] == 0) xj = iadd(xj, ivc(S.box32[2 * d], S.box32[2 * d + 1]));
        }
        r[d] = isub(I.x[d], xj);
        v[d] = isub(I.v[d], J.v[d]);
    }
    k.r2 = iadd(iadd(isqr(r[0]), isqr(r[1])), isqr(r[2]));
    k.b = iadd(iadd(imul(r[0], v[0]), imul(r[1], v[1])), imul(r[2], v[2]));
    k.v2 = iadd(iadd(isqr(v[0]), isqr(v[1])), isqr(v[2]));
}
__device__ __forceinline__ Iv disc_iv(const KIv &k, Iv d2) { return isub(isqr(k.b), imul(k.v2, isub(k.r2, d2))); }
// root(): (-1*b + st*sqrt(b*b - v2*(r2 - d2))) / v2; ok = false when undecidable
__device__ __forceinline__ Iv root_iv(const KIv &k, int st, Iv d2, bool &ok) {
    Iv D = disc_iv(k, d2);
    ok = D.lo >= 0.f && k.v2.lo > 0.f && D.hi < INFINITY;
    if (!ok) return {0.f, 0.f};
    Iv s = isqrt(D);
    Iv num = iadd(ineg(k.b), st > 0 ? s : ineg(s));
    Iv t = idiv(num, k.v2);
    ok = t.lo <= t.hi;   // false for NaN
    return t;
}

// ---- screen verdicts ----------------------------------------------------------
enum : int { SC_NONE = 0, SC_OFFER = 1, SC_REFINE = 2 };
struct Verdict { int st, warn, dup; Iv t; };

__device__ __forceinline__ int bsign3(Iv b) { return b.hi < 0.f ? 1 : (b.lo >= 0.f ? 0 : 2); }   // 1: b < 0

// FindPair as a screen: which step bracket r2 falls in, certain or not.
struct FPs { int cs, warn; bool lopot0, uppot0, inf; Iv lo, up; };
__device__ bool fp_screen(const DSys &S, int a1, int a2, int kind, int neg, Iv r2, FPs &o) {
    const float *thr, *stp;
    const double *se;
    double dmin, dmax;
    int sn;
    if (kind == K_CONSTRAINT) {
        int k = S.con_off[a1], e = S.con_off[a1 + 1];
        for (; k < e; k++) if (S.con_j[k] == a2) break;
        if (k == e) return false;
        thr = S.con_thr32 + 8 * k; dmin = S.con_dmin[k]; dmax = S.con_dmax[k]; sn = S.con_step_n[k];
        int so = S.con_step_off[k];
        stp = S.con_step32 + 6 * so; se = S.con_step_e + so;
    } else {
        int e;
        if (kind == K_COLLISION) {
            int t1 = S.type[a1], t2 = S.type[a2];
            if (dbl_pos(S.pair_dmin[tab_idx(0, t1, t2)])) e = tab_idx(0, t1, t2);
            else {
                int a = type_change(t1, 0), b = type_change(t2, 0);
                if (dbl_pos(S.pair_dmin[tab_idx(0, a, t2)])) e = tab_idx(0, a, t2);
                else if (dbl_pos(S.pair_dmin[tab_idx(0, t1, b)])) e = tab_idx(0, t1, b);
                else if (dbl_pos(S.pair_dmin[tab_idx(0, a, b)])) e = tab_idx(0, a, b);
                else return false;
            }
        } else {   // K_HB
            int bad = 0;
            int tn = hb_model(S, a1, a2, &bad);
            if (tn < 0 || bad) return false;
            e = tab_idx(tn, 0, 0);
        }
        thr = S.pair_thr32 + 8 * e; dmin = S.pair_dmin[e]; dmax = S.pair_dmax[e]; sn = S.pair_step_n[e];
        int so = S.pair_step_off[e];
        stp = S.pair_step32 + 6 * so; se = S.pair_step_e + so;
    }
    if (dbl_is_zero(dmin)) return false;
    const int a1bond = a1 ? S.hb_bond[a1] : 0;
    const bool warnable = !(kind == K_HB && a1bond == 0);
    o.warn = 0; o.inf = false; o.cs = -1;
    if (lt3(r2, thr + 0) != 0) return false;        // inside dmin - ZERO (or undecided): rare, exact path
    o.lo = ivc(thr[4], thr[5]); o.lopot0 = true;
    const int col = neg ? 0 : 2;                    // fl(d + ZERO) when approaching, fl(d - ZERO) otherwise
    for (int q = 0; q < sn; q++) {
        const float *p = stp + 6 * q;
        if (p[4] == 0.f && p[5] == 0.f) break;      // d == 0 ends the list
        int c = lt3(r2, p + col);
        if (c == 2) return false;
        if (c == 1) {
            o.up = ivc(p[4], p[5]); o.uppot0 = dbl_is_zero(se[q]);
            if (q == 0) { o.cs = 0; return true; }
            if (kind == K_HB && q == sn - 1 && a1bond > 0) { o.cs = 1; return true; }
            return true;
        }
        o.lo = ivc(p[4], p[5]); o.lopot0 = dbl_is_zero(se[q]);
    }
    if (kind == K_HB && a1bond > 0) o.warn++;
    if (dbl_pos(dmax)) {
        int c = lt3(r2, thr + 2);
        if (c == 2) return false;
        if (c == 1) {
            o.up = ivc(thr[6], thr[7]); o.uppot0 = true; o.cs = 1;
            if (sn == 0 && neg) o.cs = 0;
            return true;
        }
        o.lo = o.up = ivc(1e8f, 1e8f); o.lopot0 = o.uppot0 = true; o.inf = true;
        if (warnable) o.warn++;
        return true;
    }
    o.up = ivc(1e8f, 1e8f); o.uppot0 = false; o.cs = 1;
    return true;
}

// BondTime for one bond (eval_bond's branches)
__device__ void screen_bond(const DSys &S, int i, int q, const PIv &I, Verdict &v, int always_refine) {
    v.warn = 0; v.dup = 0;
    int j = S.bond_j[q];
    if (S.ev_partner[j] == i && S.ev_type[j] == SDMD_EV_BOND && S.ev_pcounter[j] == S.ev_counter[i]) {
        v.st = SC_REFINE; v.dup = 1; return;
    }
    if (always_refine) { v.st = SC_REFINE; return; }
    PIv J; atom_piv(S, j, J);
    KIv k; kin_iv(S, I, J, k);
    const float *bb = S.bond32 + 4 * q;
    Iv sht = ivc(bb[0], bb[1]), lng = ivc(bb[2], bb[3]);
    v.st = SC_REFINE;
    int neg = bsign3(k.b);
    if (neg == 2) return;
    Iv dl = isub(k.r2, lng);                           // r2 - lng > ZERO ?
    int c1 = dl.lo > S.zero32[1] ? 1 : (dl.hi <= S.zero32[0] ? 0 : 2);
    if (c1 == 2 || (c1 == 1 && !neg)) return;          // undecided, or the self-correcting pseudo-time
    if (c1 == 0) {
        Iv ds = isub(sht, k.r2);                       // sht - r2 > ZERO ?
        int c3 = ds.lo > S.zero32[1] ? 1 : (ds.hi <= S.zero32[0] ? 0 : 2);
        if (c3 == 2 || (c3 == 1 && neg)) return;
    }
    int st = 1; Iv d2 = lng;
    if (neg) {
        Iv D = disc_iv(k, sht);
        if (D.lo > 0.f) { st = -1; d2 = sht; }
        else if (!(D.hi <= 0.f)) return;
    }
    bool ok;
    Iv t = root_iv(k, st, d2, ok);
    if (!ok) return;
    if (t.hi < 0.f) { v.st = SC_OFFER; v.t = ivc(1e8f, 1e8f); return; }   // t < 0 -> INFINIT
    if (t.lo > 0.f) { v.st = SC_OFFER; v.t = t; }
}

// CollisionTime for one candidate (eval_collision's branches); st NONE also
// covers "not a candidate"
__device__ void screen_coll(const DSys &S, int i, int j, const PIv &I, Verdict &v, int always_refine) {
    v.warn = 0; v.dup = 0; v.st = SC_NONE;
    if (j == i) return;
    if (S.ev_partner[j] == i && S.ev_type[j] == SDMD_EV_COLLISION && S.ev_pcounter[j] == S.ev_counter[i]) {
        v.st = SC_REFINE; v.dup = 1; return;
    }
    if (always_refine) { v.st = SC_REFINE; return; }
    int bits = conn_bits(S, i, j);
    if ((bits & 1) || S.hb_bond[i] == j || nb_has(S, i, j)) return;
    PIv J; atom_piv(S, j, J);
    KIv k; kin_iv(S, I, J, k);
    if (k.r2.lo > S.cut32[1]) return;                  // certainly beyond the scan radius
    v.st = SC_REFINE;
    if (!(k.r2.hi <= S.cut32[0])) return;
    int neg = bsign3(k.b);
    if (neg == 2) return;
    const int constrained = bits & 2;
    FPs o;
    if (!fp_screen(S, i, j, constrained ? K_CONSTRAINT : K_COLLISION, neg, k.r2, o)) return;
    if (!constrained && o.lopot0 && o.uppot0) { v.st = SC_NONE; v.warn = o.warn; return; }
    if (o.inf) return;                                 // constraint beyond its outer limit: exact path
    int st = 1; Iv d2 = o.up;
    if (neg) {
        Iv D = disc_iv(k, o.lo);
        if (D.lo > 0.f) { st = -1; d2 = o.lo; }
        else if (!(D.hi <= 0.f)) return;
    }
    if (st == 1 && !constrained && o.cs == 1) { v.st = SC_NONE; v.warn = o.warn; return; }
    bool ok;
    Iv t = root_iv(k, st, d2, ok);
    if (!ok) return;
    if (t.lo > 0.f) { v.st = SC_OFFER; v.t = t; v.warn = o.warn; }
    else if (t.hi <= 0.f) { v.st = SC_NONE; v.warn = o.warn; }   // JobAssign rejects t <= 0
}

// HBTime's scan over one candidate (eval_hb_scan's branches)
__device__ void screen_hbs(const DSys &S, int i, int j, const PIv &I, Verdict &v, int always_refine) {
    v.warn = 0; v.dup = 0; v.st = SC_NONE;
    if (!(i != j && hb_pair_ok(S, i, j) && S.hb_bond[j] == 0 &&
          ((S.protein[i] == S.protein[j] && abs(S.aanum[i] - S.aanum[j]) >= 4) || S.protein[i] != S.protein[j])))
        return;
    if (S.ev_partner[j] == i && S.ev_type[j] == SDMD_EV_HB && S.ev_pcounter[j] == S.ev_counter[i]) {
        v.st = SC_REFINE; v.dup = 1; return;
    }
    v.st = SC_REFINE;
    if (always_refine) return;
    PIv J; atom_piv(S, j, J);
    KIv k; kin_iv(S, I, J, k);
    if (k.r2.lo > S.cut32[1]) { v.st = SC_NONE; return; }
    if (!(k.r2.hi <= S.cut32[0])) return;
    int bad = 0;
    int pm = pair_match(S, i, j, &bad);
    if (bad) return;
    if (pm < 0) { v.st = SC_NONE; return; }
    int neg = bsign3(k.b);
    if (neg == 2) return;
    FPs o;
    if (!fp_screen(S, i, j, K_HB, neg, k.r2, o)) return;
    if (o.inf) return;
    if (!(neg && o.cs == 1)) { v.st = SC_NONE; v.warn = o.warn; return; }
    Iv D = disc_iv(k, o.lo);
    if (D.hi <= 0.f) { v.st = SC_NONE; v.warn = o.warn; return; }
    if (!(D.lo > 0.f)) return;
    bool ok;
    Iv t = root_iv(k, -1, o.lo, ok);
    if (!ok) return;
    if (t.hi < 0.f) { v.st = SC_OFFER; v.t = ivc(1e8f, 1e8f); v.warn = o.warn; return; }
    if (t.lo > 0.f) { v.st = SC_OFFER; v.t = t; v.warn = o.warn; }
}

// ---- HB-bonded partner: the fresh part of hb_bonded(), evaluated by a lane ------
struct HbbOut { double t, pot; int sub, warn, bad; };
__device__ void hbb_fresh(const DSys &S, int i, HbbOut &r) {
    int j = S.hb_bond[i];
    Kin kk; pair_kin(S, i, j, kk);
    Lim o; int warn = 0, bad = 0;
    int cs = find_pair(S, i, j, K_HB, kk.b, kk.r2, o, 0, 0, 0, &warn, &bad);
    int st, sub; double d2, pot;
    if (kk.b < 0 && disc(kk, o.lo) > 0) {
        st = -1; d2 = o.lo; pot = o.lopot; sub = (cs == 0) ? SDMD_SUB_CORE : SDMD_SUB_TBD_CAPTURE;
    } else {
        st = 1; d2 = o.up; pot = o.uppot; sub = (cs == 1) ? SDMD_SUB_TBD_HBBREAK : SDMD_SUB_TBD_ESCAPE;
    }
    double t = root(kk, st, d2);
    if (t < 0) t = INFINIT;
    r.t = t; r.pot = pot; r.sub = sub; r.warn = warn; r.bad = bad;
}

// ---- warp helpers ----------------------------------------------------------------
// gather atom i's 27-cell neighbourhood into nbj[] in scan order with one warp
__device__ int gather_warp(const DSys &S, int i, int32_t *nbj, int nbcap, int *overflow) {
    const int lane = threadIdx.x & 31;
    int head = 0, c = 0;
    if (lane < 27) {
        head = S.cell_list[S.n + nb_cell(S, i, lane)];
        for (int a = head; a; a = S.cell_list[a]) {
            if (++c > S.n) break;
        }
    }
    int incl = c;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += y;
    }
    int tot = __shfl_sync(0xffffffffu, incl, 31);
    if (tot > nbcap) { *overflow = 1; return 0; }
    if (lane < 27) {
        int off = incl - c, m = 0;
        for (int a = head; a && m < c; a = S.cell_list[a]) nbj[off + m++] = a;
    }
    __syncwarp();
    return tot;
}

// UpdateCBTRun (src/CBT.c:56-83) for leaf atom a, by one warp.  The sequential
// repair walks up from a's leaf: while the node still names a it is recomputed;
// after that each node is recomputed and the walk stops at the first node whose
// value did not change.  Every recomputed value is the winner of the path value
// below and the sibling node (ties go to the right child), i.e. a prefix minimum
// over (key, rightness) of a and the siblings, which the warp scans in parallel.
__device__ void cbt_update_warp(const DSys &S, int a) {
    const int lane = threadIdx.x & 31;
    int32_t *node = S.cbt_node;
    const double *tm = S.ev_time;
    const int lf = S.cbt_leaf[a];
    int depth = 31 - __clz(lf);                 // number of internal levels above the leaf
    const bool on = lane < depth;
    long long key = 0x7fffffffffffffffLL;
    int pos = 0, id = a, old = 0, f = 0;
    if (on) {
        f = lf >> (lane + 1);
        int c = lf >> lane;
        int s = node[c ^ 1];
        old = node[f];
        key = tkey(tm[s]);
        id = s;
        pos = (c & 1) ? -(lane + 1) : (lane + 1);   // sibling left (negative) or right of the path
    }
    // lane 0 also holds a itself (position 0): combine a with the level-0 sibling
    long long ka = tkey(tm[a]);
    if (lane == 0 && on) {
        if (ka < key || (ka == key && 0 > pos)) { key = ka; id = a; pos = 0; }
    }
    // inclusive prefix minimum over lanes by (key asc, pos desc)
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        long long k2 = __shfl_up_sync(0xffffffffu, key, o);
        int p2 = __shfl_up_sync(0xffffffffu, pos, o);
        int i2 = __shfl_up_sync(0xffffffffu, id, o);
        if (lane >= o && on && (k2 < key || (k2 == key && p2 > pos))) { key = k2; pos = p2; id = i2; }
    }
    unsigned not_a = __ballot_sync(0xffffffffu, on && old != a);
    int first = not_a ? __ffs(not_a) - 1 : depth;   // levels below `first` are the phase that follows a
    unsigned stop = __ballot_sync(0xffffffffu, on && lane >= first && id == old);
    int last = stop ? __ffs(stop) - 1 : depth - 1;
    if (on && lane <= last && id != old) node[f] = id;
    __syncwarp();
}

// ---- the two-atom screened Predict -------------------------------------------------
constexpr int RC = 64;            // refined candidates per atom before the plain path takes over

struct ShmS {
    Shm F;                        // the plain path's buffers (used when more than RC candidates need FP64)
    int32_t *nbj[2];
    uint8_t *stat[2];             // verdict | warnings << 2, per entry
    float *tlo[2];                // lower time bound of an offer
    uint32_t *mask[2];            // entries to refine
    int32_t *rl[2];               // refined entries in scan order
    Slots R[2];                   // their exact FP64 results
    double *face;                 // PCC face times, 3 per atom
};

struct PairScal {                 // per-atom block scalars of one two-atom prediction
    int i[2], nb[2], nn[2], mode[2], E[2], rn[2], over[2], warn_excl[2];
    unsigned u_key[2], dup_key[2];
    float uprime[2], nowf;
    PIv P[2];
    HbbOut hbb[2];
};

__host__ __device__ inline size_t screen_ecap(int nbcap) { return 64 + 2 * (size_t)nbcap; }
__host__ __device__ inline size_t screen_smem_bytes_dev(int nbcap) {
    size_t ecap = screen_ecap(nbcap), words = (ecap + 31) / 32;
    size_t b = fp64_smem_bytes_dev(nbcap);
    b += al16(2 * (size_t)nbcap * 4) + al16(2 * ecap) + al16(2 * ecap * 4) + al16(2 * words * 4);
    b += al16(2 * RC * 4) + 2 * (2 * al16(RC * 4) + 3 * al16(RC * 8)) + al16(6 * 8);
    return al16(b);
}
__device__ inline void carve_screen(ShmS &M, int nbcap) {
    extern __shared__ __align__(16) unsigned char smem[];
    carve(M.F, nbcap);
    unsigned char *p = smem + fp64_smem_bytes_dev(nbcap);
    auto take = [&p](size_t bytes) { unsigned char *r = p; p += al16(bytes); return r; };
    size_t ecap = screen_ecap(nbcap), words = (ecap + 31) / 32;
    int32_t *nbj = (int32_t *)take(2 * (size_t)nbcap * 4);
    uint8_t *st = (uint8_t *)take(2 * ecap);
    float *tl = (float *)take(2 * ecap * 4);
    uint32_t *mk = (uint32_t *)take(2 * words * 4);
    int32_t *rl = (int32_t *)take(2 * RC * 4);
    for (int a = 0; a < 2; a++) {
        M.nbj[a] = nbj + a * nbcap; M.stat[a] = st + a * ecap; M.tlo[a] = tl + a * ecap;
        M.mask[a] = mk + a * words; M.rl[a] = rl + a * RC;
        M.R[a].j = (int32_t *)take(RC * 4); M.R[a].info = (int32_t *)take(RC * 4);
        M.R[a].t = (double *)take(RC * 8); M.R[a].tdup = (double *)take(RC * 8); M.R[a].pot = (double *)take(RC * 8);
    }
    M.face = (double *)take(6 * 8);
}

// order-preserving map of floats onto unsigned integers (for atomicMin/Max)
__device__ __forceinline__ unsigned f_key(float f) {
    unsigned b = __float_as_uint(f);
    return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}
__device__ __forceinline__ float key_f(unsigned k) {
    return __uint_as_float((k & 0x80000000u) ? (k & 0x7fffffffu) : ~k);
}

// one refined offer of the fold (resolve() for a single slot); `tnew` is the
// target atom whose fresh event may now duplicate this pair, or -1
__device__ inline void fold_entry(const DSys &S, Cur &c, const Slots &L, int q, int i, int type, int tnew, Blk &B) {
    int info = L.info[q];
    if (info < 0) return;
    const int j = L.j[q];
    double tdup = L.tdup[q];
    if (j == tnew) {   // CheckDuplication sees the target's new event
        info &= ~F_DUP;
        if (S.ev_partner[j] == i && S.ev_type[j] == type && S.ev_pcounter[j] == S.ev_counter[i]) {
            info |= F_DUP; tdup = S.ev_time[j];
        }
    }
    if ((info & F_DUP) && dup_assign(S, c, j, tdup, type)) return;
    B.warn += (info >> 16) & 0xff;
    if (info & F_FRESH) job_assign(S, c, j, L.t[q], L.pot[q], (info >> 8) & 0xff, type);
}

// Predict's fold for atom a of the pair, in the reference's order (thread 0)
__device__ void fold_atom(const DSys &S, int a, int tnew, ShmS &M, PairScal &PS, Blk &B, DScal &C) {
    const int i = PS.i[a], nb = PS.nb[a], nn = PS.nn[a], rn = PS.rn[a];
    const Slots &L = M.R[a];
    Cur c;
    cur_load(S, i, c);
    int q = 0, bad = 0;
    for (; q < rn && M.rl[a][q] < nb + nn; q++)
        fold_entry(S, c, L, q, i, M.rl[a][q] < nb ? SDMD_EV_BOND : SDMD_EV_COLLISION, tnew, B);
    pcc_time(S, c, M.face + 3 * a);
    thermostat_time(S, c, C, B);
    S.hb_itype[i] = SDMD_HB_NOEVENT;    // HBSkip is one-shot (src/TimePrediction.c:309-327)
    if (PS.mode[a] == 1) {
        const int j = S.hb_bond[i];
        if (!(S.ev_partner[j] == i && S.ev_type[j] == SDMD_EV_HB && S.ev_pcounter[j] == S.ev_counter[i] &&
              dup_assign(S, c, j, S.ev_time[j], SDMD_EV_HB))) {
            const HbbOut &h = PS.hbb[a];
            B.warn += h.warn;
            if (h.bad) bad = 1;
            job_assign(S, c, j, h.t, h.pot, h.sub, SDMD_EV_HB);
        }
    } else if (PS.mode[a] == 2) {
        for (; q < rn; q++) fold_entry(S, c, L, q, i, SDMD_EV_HB, tnew, B);
    }
    hbnb_time(S, i, c, B, &bad);
    if (S.wall) wall_time(S, i, c, B, &bad);
    cur_store(S, i, c);
    B.warn += PS.warn_excl[a];
    if (bad) set_err(B, SDMD_EHBMAP, i);
}

// Predict for the target t and (when p > 0) the partner p, after ResetTarget of
// both: the same results as predict_atom(t) followed by predict_atom(p).
__device__ void predict_two(const DSys &S, int t, int p, ShmS &M, PairScal &PS, Blk &B, DScal &C) {
    const int tid = threadIdx.x, T = blockDim.x, lane = tid & 31, warp = tid >> 5, nw = T >> 5;
    const int na = p ? 2 : 1;
    const double cut = [&] { double c = S.cutoff * 0.90; return c * c; }();
    // 1. per-atom set-up and the two 27-cell gathers (one warp each)
    if (tid < na) {
        const int a = tid, i = a ? p : t;
        PS.i[a] = i;
        PS.nb[a] = S.bond_off[i + 1] - S.bond_off[i];
        int mode;
        if (S.hb_itype[i] == SDMD_HB_SKIP) mode = 0;
        else if (S.hb_bond[i] > 0) mode = 1;
        else { int r = S.hb_role[i]; mode = (r == 'A' || r == 'D' || r == 'S') ? 2 : 0; }
        PS.mode[a] = mode;
        PS.u_key[a] = f_key(INFINITY); PS.dup_key[a] = f_key(-INFINITY);
        PS.warn_excl[a] = 0; PS.rn[a] = 0; PS.over[a] = 0;
        atom_piv(S, i, PS.P[a]);
    }
    for (int a = 0; a < na; a++) {
        if (warp == (a % nw)) {
            int ovf = 0;
            int nn = gather_warp(S, a ? p : t, M.nbj[a], S.nbcap, &ovf);
            if (lane == 0) { PS.nn[a] = nn; if (ovf) set_err(B, SDMD_ECAPACITY, a ? p : t); }
        }
    }
    __syncthreads();
    for (int a = 0; a < na; a++) if (PS.nb[a] > 64 && tid == 0) set_err(B, SDMD_ECAPACITY, PS.i[a]);
    if (tid < na) {
        const int a = tid;
        PS.E[a] = PS.nb[a] + PS.nn[a] + (PS.mode[a] == 2 ? PS.nn[a] : 0);
    }
    const size_t words = (screen_ecap(S.nbcap) + 31) / 32;
    for (size_t w = tid; w < 2 * words; w += T) M.mask[w / words][w % words] = 0;
    __syncthreads();
    if (B.err) return;
    // 2. PCC faces (exact, FP64) and the FP32 screen of every bond / collision / HB candidate
    if (tid < 3 * na) M.face[tid] = pcc_face(S, PS.i[tid / 3], tid % 3);
    const int E0 = PS.E[0], E1 = na > 1 ? PS.E[1] : 0;
    for (int g = tid; g < E0 + E1; g += T) {
        const int a = g < E0 ? 0 : 1, e = a ? g - E0 : g, i = PS.i[a], nb = PS.nb[a], nn = PS.nn[a];
        Verdict v;
        int j;
        if (e < nb) {
            const int qb = S.bond_off[i] + e;
            j = S.bond_j[qb];
            screen_bond(S, i, qb, PS.P[a], v, a == 1 && j == t);
        } else if (e < nb + nn) {
            j = M.nbj[a][e - nb];
            screen_coll(S, i, j, PS.P[a], v, a == 1 && j == t);
        } else {
            j = M.nbj[a][e - nb - nn];
            screen_hbs(S, i, j, PS.P[a], v, a == 1 && j == t);
        }
        M.stat[a][e] = (uint8_t)(v.st | (v.warn << 2));
        M.tlo[a][e] = v.t.lo;
        if (v.st == SC_OFFER && e < nb + nn) atomicMin(&PS.u_key[a], f_key(v.t.hi));
        else if (v.st == SC_NONE && v.warn) atomicAdd(&PS.warn_excl[a], v.warn);
        if (v.dup) {   // CheckDuplication may adopt j's stored time: it bounds what can matter
            double d = S.ev_time[j];
            if (S.lazy) d = d - S.now;
            atomicMax(&PS.dup_key[a], f_key(ivd(d).hi));
        }
    }
    __syncthreads();
    // 3. U: the bond / collision segment of the fold ends at or below U (its smallest
    // certain upper bound).  Bounding only by that segment keeps the whole fold
    // exact, including JobAssign's partnerCounter, which a partner-less winner
    // (PCC, thermostat, wall) leaves at the value of the last bond/collision record.
    // U' adds every duplicate time (and, for the partner, the target's bound).
    if (tid == 0) {
        PS.nowf = S.lazy ? fmaxf(fabsf(ivd(S.now).hi), fabsf(ivd(S.now).lo)) : 0.f;
        float u_t = INFINITY;
        for (int a = 0; a < na; a++) {
            float u = key_f(PS.u_key[a]);
            float up = fmaxf(u, key_f(PS.dup_key[a]));
            if (a == 0) u_t = u;
            else up = fmaxf(up, u_t);      // the target's new event may become a duplicate for the partner
            PS.uprime[a] = up;
        }
    }
    __syncthreads();
    // 4. mark the candidates that need FP64: undecided ones and offers that may reach U'
    for (int g = tid; g < E0 + E1; g += T) {
        const int a = g < E0 ? 0 : 1, e = a ? g - E0 : g;
        const int st = M.stat[a][e] & 3, w = M.stat[a][e] >> 2;
        bool refine = st == SC_REFINE;
        if (st == SC_OFFER) {
            float tl = M.tlo[a][e], up = PS.uprime[a];
            // lazy mode compares now + t: keep a margin of a few FP64 ulps of that sum
            float margin = S.lazy ? __fmul_ru(__fadd_ru(PS.nowf, fabsf(tl)), 0x1p-48f) : 0.f;
            if (__fsub_rd(tl, up) > margin) { if (w) atomicAdd(&PS.warn_excl[a], w); }
            else refine = true;
        }
        if (refine) atomicOr(&M.mask[a][e >> 5], 1u << (e & 31));
    }
    __syncthreads();
    // 5. refined entries of each atom in scan order (one warp per atom)
    for (int a = 0; a < na; a++) {
        if (warp != (a % nw)) continue;
        const int nwords = (PS.E[a] + 31) >> 5;
        int base = 0;
        for (int w0 = 0; w0 < nwords; w0 += 32) {
            const int w = w0 + lane;
            uint32_t bits = w < nwords ? M.mask[a][w] : 0u;
            int cnt = __popc(bits), incl = cnt;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                int y = __shfl_up_sync(0xffffffffu, incl, o);
                if (lane >= o) incl += y;
            }
            int pos = base + incl - cnt;
            while (bits) {
                int b = __ffs(bits) - 1;
                bits &= bits - 1;
                if (pos < RC) M.rl[a][pos] = (w << 5) + b;
                pos++;
            }
            base += __shfl_sync(0xffffffffu, incl, 31);
        }
        if (lane == 0) { PS.rn[a] = base < RC ? base : RC; PS.over[a] = base > RC; }
    }
    __syncthreads();
    // 6. exact FP64 for the refined entries, packed into lanes; one warp per kind
    {
        int bad = 0;
        const int R0 = PS.over[0] ? 0 : PS.rn[0];
        const int R1 = (na > 1 && !PS.over[1]) ? PS.rn[1] : 0;
        for (int q = lane; q < R0 + R1; q += 32) {
            const int a = q < R0 ? 0 : 1, qq = a ? q - R0 : q;
            const int e = M.rl[a][qq], i = PS.i[a], nb = PS.nb[a], nn = PS.nn[a];
            const int kind = e < nb ? 1 : (e < nb + nn ? 0 : 2);
            if (kind % nw != warp) continue;
            if (kind == 1) eval_bond(S, i, S.bond_off[i] + e, M.R[a], qq, &bad);
            else if (kind == 0) eval_collision(S, i, M.nbj[a][e - nb], cut, M.R[a], qq, &bad);
            else eval_hb_scan(S, i, M.nbj[a][e - nb - nn], cut, M.R[a], qq, &bad);
        }
        if (warp == 3 % nw && lane < na && PS.mode[lane] == 1 && !PS.over[lane]) hbb_fresh(S, PS.i[lane], PS.hbb[lane]);
        if (bad) set_err(B, SDMD_EHBMAP, t);
    }
    __syncthreads();
    // 7. the folds: target first, then the partner (which may now see the target's event)
    if (PS.over[0]) predict_atom(S, t, M.F, B, C);
    else {
        if (tid == 0 && !B.err) fold_atom(S, 0, -1, M, PS, B, C);
        __syncthreads();
    }
    if (na > 1 && !B.err) {
        if (PS.over[1]) predict_atom(S, p, M.F, B, C);
        else {
            if (tid == 0) fold_atom(S, 1, t, M, PS, B, C);
            __syncthreads();
        }
    }
}

}  // namespace sdmd
