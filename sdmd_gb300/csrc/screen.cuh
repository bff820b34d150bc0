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
// The helpers below select their operands first and then run one instruction
// sequence for every sign case, so lanes of a warp in different cases do not
// diverge (each case computes the same values as a branch per case would).
__device__ __forceinline__ Iv isqr(Iv a) {
    // the smaller magnitude bound: a.lo when a >= 0, -a.hi when a <= 0, else 0
    const float m = a.lo >= 0.f ? a.lo : (a.hi <= 0.f ? -a.hi : 0.f);
    return {__fmul_rd(m, m), fmaxf(__fmul_ru(a.lo, a.lo), __fmul_ru(a.hi, a.hi))};
}
// sqrt of an interval with a.lo >= 0 (IEEE round-to-nearest, stepped outward)
__device__ __forceinline__ Iv isqrt(Iv a) {
    const float sl = __fsqrt_rn(fmaxf(a.lo, 0.f));
    float lo = a.lo > 0.f ? f_dn(sl) : 0.f;
    return {lo > 0.f ? lo : 0.f, f_up(__fsqrt_rn(a.hi))};
}
// a / b with b.lo > 0 (IEEE round-to-nearest quotients, stepped outward):
// the lower quotient divides by b.hi when a.lo >= 0 (else b.lo), the upper one
// by b.hi when a.hi <= 0 (else b.lo)
__device__ __forceinline__ Iv idiv(Iv a, Iv b) {
    const float ql = __fdiv_rn(a.lo, a.lo >= 0.f ? b.hi : b.lo);
    const float qh = __fdiv_rn(a.hi, a.hi <= 0.f ? b.hi : b.lo);
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

// the FP64 position lzx() would produce, and the velocity, of atom j, from its
// FP64 fields (rounded to float and widened: FP64-pipe conversions)
__device__ __forceinline__ void atom_piv_d(const DSys &S, int j, PIv &P) {
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

// One word of atom k's interval record (w = 0..3).  x and v are doubles, so
// [rd, ru] holds them exactly; tloc - T0 is an FP64 difference, one rounding away
// from the real one, so its bounds step one more float outward.  Then
// (now - T0) - (tloc - T0) in outward-rounded FP32 holds the real now - tloc,
// hence also fl(now - tloc), since rounding to nearest is monotone and the
// bounds are doubles themselves; the same holds for every later step of lzx().
__device__ __forceinline__ void shadow_word(const DSys &S, int k, int w) {
    float4 r;
    switch (w) {
        case 0: r = make_float4(__double2float_rd(S.x[k]), __double2float_ru(S.x[k]),
                                __double2float_rd(S.y[k]), __double2float_ru(S.y[k])); break;
        case 1: r = make_float4(__double2float_rd(S.z[k]), __double2float_ru(S.z[k]),
                                __double2float_rd(S.vx[k]), __double2float_ru(S.vx[k])); break;
        case 2: r = make_float4(__double2float_rd(S.vy[k]), __double2float_ru(S.vy[k]),
                                __double2float_rd(S.vz[k]), __double2float_ru(S.vz[k])); break;
        default: {
            const double d = (S.lazy ? S.tloc[k] : S.now) - S.T0;
            r = make_float4(f_dn(__double2float_rd(d)), f_up(__double2float_ru(d)),
                            __int_as_float(S.cx[k] | S.cy[k] << 10 | S.cz[k] << 20), 0.f);
        }
    }
    S.shr[4 * (size_t)k + w] = r;
}
// [nlo, nhi] around the real now - T0 (the same outward step as tloc - T0)
__device__ __forceinline__ void shadow_now(DSys &S) {
    const double d = S.now - S.T0;
    S.nlo = f_dn(__double2float_rd(d));
    S.nhi = f_up(__double2float_ru(d));
}

// atom_piv_d()'s intervals, from the record when the records are valid
__device__ __forceinline__ void atom_piv(const DSys &S, int j, PIv &P) {
    if (!S.shadow_ok) { atom_piv_d(S, j, P); return; }
    const float4 *r = S.shr + 4 * (size_t)j;
    const float4 a = r[0], b = r[1], c = r[2], e = r[3];
    const Iv dt = isub(ivc(S.nlo, S.nhi), ivc(e.x, e.y));
    P.v[0] = ivc(b.z, b.w); P.v[1] = ivc(c.x, c.y); P.v[2] = ivc(c.z, c.w);
    P.x[0] = iadd(ivc(a.x, a.y), imul(P.v[0], dt));
    P.x[1] = iadd(ivc(a.z, a.w), imul(P.v[1], dt));
    P.x[2] = iadd(ivc(b.x, b.y), imul(P.v[2], dt));
    if (!S.lazy) {   // eager: widen by the rounding of the step-by-step advance since tr
#pragma unroll
        for (int d = 0; d < 3; d++) {
            const float vm = fmaxf(fabsf(P.v[d].lo), fabsf(P.v[d].hi));
            const float mx = __fmaf_ru(S.mxb, vm, S.mxa);
            P.x[d] = ivc(__fsub_rd(P.x[d].lo, mx), __fadd_ru(P.x[d].hi, mx));
        }
    }
    const int cp = __float_as_int(e.z);
    P.c[0] = cp & 1023; P.c[1] = (cp >> 10) & 1023; P.c[2] = cp >> 20;
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
    Iv num = iadd(ineg(k.b), st > 0 ? s : ineg(s));   // a select, not a branch
    Iv t = idiv(num, k.v2);
    ok = t.lo <= t.hi;   // false for NaN
    return t;
}

// the constraint of a1 with partner a2 (index into the constraint arrays), or -1
__device__ __forceinline__ int con_index(const DSys &S, int a1, int a2) {
    if (S.con_ok[a1]) {
        const unsigned idx = (unsigned)(a2 - (a1 - 64));
        if (idx >= 128u) return -1;
        const int r = S.con_win[(size_t)a1 * 128 + idx];
        return r < 0 ? -1 : S.con_off[a1] + r;
    }
    for (int k = S.con_off[a1], e = S.con_off[a1 + 1]; k < e; k++)
        if (S.con_j[k] == a2) return k;
    return -1;
}

// the predicted atom's own fields, loaded once per prediction
struct AtomI {
    int32_t hbb, role, type, prot, aa;
    int32_t nb[4];
    int32_t win[9];               // its conn_win row
    int32_t nbs;                  // nb_status: how many HB-neighbour partners
    int64_t cnt;                  // ev_counter
};
__device__ __forceinline__ void load_atom_i(const DSys &S, int i, const double *xi, AtomI &A) {
    A.hbb = S.hb_bond[i]; A.role = S.hb_role[i]; A.type = S.type[i]; A.prot = S.protein[i]; A.aa = S.aanum[i];
    for (int q = 0; q < 4; q++) A.nb[q] = S.nb_partner[4 * i + q];
    for (int q = 0; q < 9; q++) A.win[q] = S.conn_win[9 * i + q];
    A.nbs = S.nb_status[i];
    A.cnt = S.ev_counter[i];
}

// connection-map bits of (i, j) from the per-atom window (row scan outside it)
__device__ __forceinline__ int conn_bits_w(const DSys &S, int i, int j) {
    const int32_t *w = S.conn_win + 9 * i;
    const int base = w[0];
    if (base < 0) return conn_bits(S, i, j);
    const unsigned idx = (unsigned)(j - base);
    if (idx >= 128u) return 0;
    const unsigned m = 1u << (idx & 31);
    return (((unsigned)w[1 + (idx >> 5)] & m) ? 1 : 0) | (((unsigned)w[5 + (idx >> 5)] & m) ? 2 : 0);
}

// ---- screen outcomes -----------------------------------------------------------
enum : int { SC_NONE = 0, SC_OFFER = 1, SC_REFINE = 2 };
struct Outcome { int st, warn, dup; Iv t; };

__device__ __forceinline__ int bsign3(Iv b) { return b.hi < 0.f ? 1 : (b.lo >= 0.f ? 0 : 2); }   // 1: b < 0

// FindPair as a screen: which step bracket r2 falls in, certain or not.
// t1 / t2 are the atoms' types (K_COLLISION); the first four steps of the entry are
// loaded together before the bracket walk.
struct FPs { int cs, warn; bool lopot0, uppot0, inf; Iv lo, up; };
__device__ bool fp_screen(const DSys &S, int a1, int a2, int kind, int neg, Iv r2, FPs &o, int t1, int t2) {
    const float *thr, *stp;
    const double *se;
    double dmin, dmax;
    int sn;
    if (kind == K_CONSTRAINT) {
        const int k = con_index(S, a1, a2);
        if (k < 0) return false;
        thr = S.con_thr32 + 8 * k; dmin = S.con_dmin[k]; dmax = S.con_dmax[k]; sn = S.con_step_n[k];
        const int so = S.con_step_off[k];
        stp = S.con_step32 + 6 * so; se = S.con_step_e + so;
    } else {
        int e;
        if (kind == K_COLLISION) {
            e = S.rp_idx[t1 * NT + t2];
            if (e < 0) return false;
        } else {   // K_HB
            int bad = 0;
            const int tn = hb_model(S, a1, a2, &bad);
            if (tn < 0 || bad) return false;
            e = tab_idx(tn, 0, 0);
        }
        thr = S.pair_thr32 + 8 * e; dmin = S.pair_dmin[e]; dmax = S.pair_dmax[e]; sn = S.pair_step_n[e];
        const int so = S.pair_step_off[e];
        stp = S.pair_step32 + 6 * so; se = S.pair_step_e + so;
    }
    const int col = neg ? 0 : 2;                    // fl(d + ZERO) when approaching, fl(d - ZERO) otherwise
    float pre[4][4];
    long long pse[4];
#pragma unroll
    for (int q = 0; q < 4; q++) {
        if (q < sn) {
            const float *p = stp + 6 * q;
            pre[q][0] = p[col]; pre[q][1] = p[col + 1]; pre[q][2] = p[4]; pre[q][3] = p[5];
            pse[q] = __double_as_longlong(se[q]);
        }
    }
    if (dbl_is_zero(dmin)) return false;
    const int a1bond = a1 ? S.hb_bond[a1] : 0;
    const bool warnable = !(kind == K_HB && a1bond == 0);
    o.warn = 0; o.inf = false; o.cs = -1;
    if (lt3(r2, thr + 0) != 0) return false;        // inside dmin - ZERO (or undecided): rare, exact path
    o.lo = ivc(thr[4], thr[5]); o.lopot0 = true;
    for (int q = 0; q < sn; q++) {
        float c0, c1, d0, d1;
        long long eb;
        if (q < 4) { c0 = pre[q][0]; c1 = pre[q][1]; d0 = pre[q][2]; d1 = pre[q][3]; eb = pse[q]; }
        else {
            const float *p = stp + 6 * q;
            c0 = p[col]; c1 = p[col + 1]; d0 = p[4]; d1 = p[5]; eb = __double_as_longlong(se[q]);
        }
        if (d0 == 0.f && d1 == 0.f) break;          // d == 0 ends the list
        const float cthr[2] = {c0, c1};
        const int c = lt3(r2, cthr);
        if (c == 2) return false;
        const bool ezero = (eb << 1) == 0;
        if (c == 1) {
            o.up = ivc(d0, d1); o.uppot0 = ezero;
            if (q == 0) { o.cs = 0; return true; }
            if (kind == K_HB && q == sn - 1 && a1bond > 0) { o.cs = 1; return true; }
            return true;
        }
        o.lo = ivc(d0, d1); o.lopot0 = ezero;
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
__device__ void screen_bond(const DSys &S, int i, int q, const PIv &I, Outcome &v, int always_refine) {
    v.warn = 0; v.dup = 0;
    int j = S.bond_j[q];
    if (j < S.dup_limit && S.ev_partner[j] == i && S.ev_type[j] == SDMD_EV_BOND && S.ev_pcounter[j] == S.ev_counter[i]) {
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

// HBTime's scan over one candidate (eval_hb_scan's branches), kinematics given
__device__ void screen_hbs_k(const DSys &S, int i, int j, const KIv &k, Outcome &v) {
    v.st = SC_REFINE;
    if (k.r2.lo > S.cut32[1]) { v.st = SC_NONE; return; }
    if (!(k.r2.hi <= S.cut32[0])) return;
    int bad = 0;
    int pm = pair_match(S, i, j, &bad);
    if (bad) return;
    if (pm < 0) { v.st = SC_NONE; return; }
    int neg = bsign3(k.b);
    if (neg == 2) return;
    FPs o;
    if (!fp_screen(S, i, j, K_HB, neg, k.r2, o, 0, 0)) return;
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

// One 27-cell candidate j of atom i: the collision outcome (CollisionTime) and,
// when the atom scans for hydrogen bonds (hb), the HB-scan outcome, sharing one
// evaluation of the pair's kinematics.  `always` forces "refine" (the partner's
// view of the target, whose event is only known after the target's fold).  Every
// field of j is loaded at once; A holds atom i's own fields.
__device__ void screen_cell(const DSys &S, int i, int j, const PIv &I, const AtomI &A, bool hb, int always,
                            Outcome &vc, Outcome &vh) {
    vc.warn = 0; vc.dup = 0; vc.st = SC_NONE;
    vh.warn = 0; vh.dup = 0; vh.st = SC_NONE;
    if (j == i) return;
    PIv J; atom_piv(S, j, J);                          // loads issued with the rest of j's fields
    const int evp = S.ev_partner[j], evt = S.ev_type[j];
    const int64_t evpc = S.ev_pcounter[j];
    const int rj = S.hb_role[j], tj = S.type[j], hbj = S.hb_bond[j], pj = S.protein[j], aj = S.aanum[j];
    const bool named = j < S.dup_limit && evp == i && evpc == A.cnt;
    bool need_c = true;
    if (named && evt == SDMD_EV_COLLISION) { vc.st = SC_REFINE; vc.dup = 1; need_c = false; }
    else if (always) { vc.st = SC_REFINE; need_c = false; }
    const int ri = A.role;
    const bool pair_ok = (ri == 'A' && rj == 'D') || (ri == 'D' && rj == 'A') || (ri == 'S' && tj == 2) ||
                         (rj == 'S' && A.type == 2) || (ri == 'S' && rj == 'S');   // hb_pair_ok
    bool need_h = hb && pair_ok && hbj == 0 && ((A.prot == pj && abs(A.aa - aj) >= 4) || A.prot != pj);
    if (need_h) {
        if (named && evt == SDMD_EV_HB) { vh.st = SC_REFINE; vh.dup = 1; need_h = false; }
        else if (always) { vh.st = SC_REFINE; need_h = false; }
    }
    int bits = 0;
    if (need_c) {
        if (A.win[0] < 0) bits = conn_bits(S, i, j);
        else {
            const unsigned idx = (unsigned)(j - A.win[0]);
            if (idx < 128u) {
                const unsigned m = 1u << (idx & 31);
                bits = (((unsigned)A.win[1 + (idx >> 5)] & m) ? 1 : 0) | (((unsigned)A.win[5 + (idx >> 5)] & m) ? 2 : 0);
            }
        }
        bool nbh = false;
        for (int q = 0; q < 4; q++) {   // FindElemInList(neighborPartner, j)
            if (A.nb[q] == 0) break;
            if (A.nb[q] == j) { nbh = true; break; }
        }
        if ((bits & 1) || A.hbb == j || nbh) need_c = false;
    }
    if (!need_c && !need_h) return;
    KIv k; kin_iv(S, I, J, k);
    if (need_h) screen_hbs_k(S, i, j, k, vh);
    if (!need_c) return;
    Outcome &v = vc;
    if (k.r2.lo > S.cut32[1]) return;                  // certainly beyond the scan radius
    v.st = SC_REFINE;
    if (!(k.r2.hi <= S.cut32[0])) return;
    int neg = bsign3(k.b);
    if (neg == 2) return;
    const int constrained = bits & 2;
    FPs o;
    if (!fp_screen(S, i, j, constrained ? K_CONSTRAINT : K_COLLISION, neg, k.r2, o, A.type, tj)) return;
    if (!constrained && o.lopot0 && o.uppot0) { v.st = SC_NONE; v.warn = o.warn; return; }
    if (o.inf) return;
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
    else if (t.hi <= 0.f) { v.st = SC_NONE; v.warn = o.warn; }
}

// ---- exact refine: the plain path's FP64 arithmetic, integer-key compares --------
// Each function below performs the same FP64 operations, in the same order, as its
// plain-path counterpart (eval_bond / eval_collision / eval_hb_scan / find_pair),
// so every FP64 value is bit-identical.  Comparisons of FP64 values are made on
// their tkey() images (an order-preserving map, +0 == -0), and thresholds such as
// fl(d + ZERO) come precomputed from the host, which performs the same IEEE
// additions.  The target's own position lzx(i) is computed once per prediction.
constexpr long long KEY_ZERO = 0x3E45798EE2308C3ALL;   // tkey(1e-8)

// x < 0 and x > 0 with IEEE semantics (false for NaN), as integer tests
__device__ __forceinline__ bool dbl_lt0(double x) {
    long long b = __double_as_longlong(x);
    return b < 0 && (b & 0x7fffffffffffffffLL) != 0 && (b & 0x7fffffffffffffffLL) <= 0x7ff0000000000000LL;
}
__device__ __forceinline__ bool dbl_gt0(double x) {
    long long b = __double_as_longlong(x);
    return b > 0 && b <= 0x7ff0000000000000LL;
}

__device__ int find_pair_r(const DSys &S, int a1, int a2, int kind, bool neg, double distance2, Lim &o, int *warn,
                           int *bad) {
    int cs = -1;
    const long long *key, *skey;
    const double *sd, *se;
    double dmin, dmax;
    int sn;
    if (kind == K_CONSTRAINT) {
        const int k = con_index(S, a1, a2);
        if (k < 0) { *bad = 1; return -1; }
        dmin = S.con_dmin[k]; dmax = S.con_dmax[k]; sn = S.con_step_n[k]; key = S.con_key + 2 * k;
        int so = S.con_step_off[k];
        sd = S.con_step_d + so; se = S.con_step_e + so; skey = S.con_stepkey + 2 * so;
    } else {
        int e;
        if (kind == K_COLLISION) {
            e = S.rp_idx[S.type[a1] * NT + S.type[a2]];   // RightPair, resolved on the host
            if (e < 0) { *bad = 1; return -1; }
        } else {   // K_HB
            int tn = hb_model(S, a1, a2, bad);
            if (tn < 0) { *bad = 1; tn = 0; }
            e = tab_idx(tn, 0, 0);
        }
        dmin = S.pair_dmin[e]; dmax = S.pair_dmax[e]; sn = S.pair_step_n[e]; key = S.pair_key + 2 * e;
        int so = S.pair_step_off[e];
        sd = S.pair_step_d + so; se = S.pair_step_e + so; skey = S.pair_stepkey + 2 * so;
    }
    const int flag = (sn == 0);
    if (dbl_is_zero(dmin)) { *bad = 1; return -1; }
    const int a1bond = a1 ? S.hb_bond[a1] : 0;
    const bool warnable = !(kind == K_HB && a1bond == 0);
    const long long kd = tkey(distance2);
    if (kd < key[0]) {
        o.lo = INFINIT; o.up = INFINIT; o.acc = INFINIT; o.lopot = 0; o.uppot = 0;
        if (warnable) ++*warn;
        return cs;
    }
    o.lo = dmin; o.lopot = 0;
    const int col = neg ? 0 : 1;
    // the first four steps are loaded together (a dependent load per step otherwise)
    double pd[4], pe[4];
    long long pk[4];
#pragma unroll
    for (int u = 0; u < 4; u++) {
        pd[u] = u < sn ? sd[u] : 0.0;
        pe[u] = u < sn ? se[u] : 0.0;
        pk[u] = u < sn ? skey[2 * u + col] : 0;
    }
    for (int q = 0; q < sn; q++) {
        double d, e;
        long long kq;
        if (q < 4) {   // static selects keep the prefetched values in registers
            d = q == 0 ? pd[0] : (q == 1 ? pd[1] : (q == 2 ? pd[2] : pd[3]));
            e = q == 0 ? pe[0] : (q == 1 ? pe[1] : (q == 2 ? pe[2] : pe[3]));
            kq = q == 0 ? pk[0] : (q == 1 ? pk[1] : (q == 2 ? pk[2] : pk[3]));
        } else {
            d = sd[q]; e = se[q]; kq = skey[2 * q + col];
        }
        if (dbl_is_zero(d)) break;
        if (kd < kq) {
            o.up = d; o.uppot = -1 * e; o.acc = 0;
            if (q == 0) return 0;
            if (kind == K_HB && q == sn - 1 && a1bond > 0) return 1;
            return cs;
        }
        o.lo = d; o.lopot = e;
    }
    if (kind == K_HB && a1bond > 0) ++*warn;
    if (dbl_pos(dmax)) {
        if (kd < key[1]) {
            o.up = dmax; o.uppot = 0; o.acc = 0;
            cs = 1;
            if (flag == 1 && neg) cs = 0;
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

// pair_kin() with the target's position given (xi = lzx(i) per dimension)
__device__ __forceinline__ void pair_kin_r(const DSys &S, const double *xi, int i, int j, Kin &k) {
    const int ci[3] = {S.cx[i], S.cy[i], S.cz[i]}, cj[3] = {S.cx[j], S.cy[j], S.cz[j]};
    const double *X[3] = {S.x, S.y, S.z}, *V[3] = {S.vx, S.vy, S.vz};
    double r[3], v[3];
#pragma unroll
    for (int d = 0; d < 3; d++) {
        double xj = lzx(S, X[d], V[d], j);
        // xj + 0.0 equals xj except for the sign of a zero, which no later result
        // can observe (squares, and sums with the other terms), so it is skipped
        if (ci[d] != cj[d]) {
            if (ci[d] == 0 && cj[d] == S.cn[d] - 1) xj = xj + -1 * S.box[d];
            else if (ci[d] == S.cn[d] - 1 && cj[d] == 0) xj = xj + S.box[d];
        }
        r[d] = xi[d] - xj;
        v[d] = V[d][i] - V[d][j];
    }
    k.rx = r[0]; k.ry = r[1]; k.rz = r[2];
    k.r2 = r[0] * r[0] + r[1] * r[1] + r[2] * r[2];
    k.b = r[0] * v[0] + r[1] * v[1] + r[2] * v[2];
    k.v2 = v[0] * v[0] + v[1] * v[1] + v[2] * v[2];
}
// CalculateTime with the discriminant given (it is recomputed identically otherwise)
__device__ __forceinline__ double root_d(const Kin &k, int st, double D) {
    double s = sqrt(D);
    return (-k.b + (st > 0 ? s : -s)) / k.v2;
}

__device__ void eval_bond_r(const DSys &S, const double *xi, int i, int q, Slots &L, int k,
                            const Kin *pk = nullptr) {
    int j = S.bond_j[q];
    int info = 0;
    double tdup = 0;
    if (j < S.dup_limit && S.ev_partner[j] == i && S.ev_type[j] == SDMD_EV_BOND && S.ev_pcounter[j] == S.ev_counter[i]) {
        info |= F_DUP; tdup = S.ev_time[j];
    }
    double lng = S.bond_dmax[q], sht = S.bond_dmin[q];
    Kin kk;
    if (pk) kk = *pk; else pair_kin_r(S, xi, i, j, kk);
    const long long kb = tkey(kk.b);
    const bool far = tkey(kk.r2 - lng) > KEY_ZERO;
    int sub; double t;
    if (far && kb >= 0) { sub = SDMD_SUB_WELL_BOUNCE; t = 1e-16 * i * j; }
    else if (!far && tkey(sht - kk.r2) > KEY_ZERO && kb < 0) { sub = SDMD_SUB_CORE; t = 1e-16 * i * j; }
    else {
        double D1 = 0;
        if (kb < 0) D1 = kk.b * kk.b - kk.v2 * (kk.r2 - sht);
        int st;
        double D;
        if (kb < 0 && dbl_gt0(D1)) { sub = SDMD_SUB_CORE; st = -1; D = D1; }
        else { sub = SDMD_SUB_WELL_BOUNCE; st = 1; D = kk.b * kk.b - kk.v2 * (kk.r2 - lng); }
        t = root_d(kk, st, D);   // one call site: lanes in either case share the sqrt and division
        if (dbl_lt0(t)) t = INFINIT;
    }
    put(L, k, j, info | F_FRESH | (sub << 8), t, tdup, 0.0);
}

__device__ void eval_collision_r(const DSys &S, const double *xi, int i, int j, Slots &L, int k, int *bad,
                                 const Kin *pk = nullptr) {
    int info = 0, warn = 0, sub = SDMD_SUB_INVALID;
    double tdup = 0, t = 0, pot = 0;
    if (j == i) { put(L, k, j, -1, 0, 0, 0); return; }
    if (j < S.dup_limit && S.ev_partner[j] == i && S.ev_type[j] == SDMD_EV_COLLISION && S.ev_pcounter[j] == S.ev_counter[i]) {
        info |= F_DUP; tdup = S.ev_time[j];
    }
    int bits = conn_bits_w(S, i, j);
    if (!((bits & 1) || S.hb_bond[i] == j || nb_has(S, i, j))) {
        Kin kk;
        if (pk) kk = *pk; else pair_kin_r(S, xi, i, j, kk);
        if (tkey(kk.r2) <= S.cut_key) {
            const bool neg = tkey(kk.b) < 0;
            Lim o; int cs; bool go = true;
            const int constrained = bits & 2;
            cs = find_pair_r(S, i, j, constrained ? K_CONSTRAINT : K_COLLISION, neg, kk.r2, o, &warn, bad);
            if (!constrained && dbl_is_zero(o.lopot) && dbl_is_zero(o.uppot)) go = false;
            if (go) {
                double D1 = 0;
                if (neg) D1 = kk.b * kk.b - kk.v2 * (kk.r2 - o.lo);
                int st = 0;
                double D = 0;
                if (neg && dbl_gt0(D1)) {
                    pot = o.lopot;
                    sub = (cs == 0) ? SDMD_SUB_CORE : SDMD_SUB_TBD_CAPTURE;
                    st = -1; D = D1;
                } else {
                    pot = o.uppot;
                    if (constrained) sub = (cs == 1) ? SDMD_SUB_WELL_BOUNCE : SDMD_SUB_TBD_ESCAPE;
                    else if (cs == 1) go = false;
                    else sub = SDMD_SUB_TBD_ESCAPE;
                    if (go) { st = 1; D = kk.b * kk.b - kk.v2 * (kk.r2 - o.up); }
                }
                if (st) { t = root_d(kk, st, D); info |= F_FRESH; }   // one call site for both roots
            }
        }
    }
    put(L, k, j, info | (sub << 8) | (warn << 16), t, tdup, pot);
}

__device__ void eval_hb_scan_r(const DSys &S, const double *xi, int i, int j, Slots &L, int k, int *bad,
                               const Kin *pk = nullptr) {
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
    Kin kk;
    if (pk) kk = *pk; else pair_kin_r(S, xi, i, j, kk);
    if (tkey(kk.r2) <= S.cut_key && pair_match(S, i, j, bad) >= 0) {
        Lim o;
        const bool neg = tkey(kk.b) < 0;
        int cs = find_pair_r(S, i, j, K_HB, neg, kk.r2, o, &warn, bad);
        if (neg && cs == 1) {
            double D1 = kk.b * kk.b - kk.v2 * (kk.r2 - o.lo);
            if (dbl_gt0(D1)) {
                pot = o.lopot;
                t = root_d(kk, -1, D1);
                if (dbl_lt0(t)) t = INFINIT;
                info |= F_FRESH;
            }
        }
    }
    put(L, k, j, info | (SDMD_SUB_TBD_HBFORM << 8) | (warn << 16), t, tdup, pot);
}

// ---- HB-bonded partner: the fresh part of hb_bonded(), evaluated by a lane ------
struct HbbOut { double t, pot; int sub, warn, bad, pos; };
__device__ __noinline__ void hbb_fresh(const DSys &S, const double *xi, int i, HbbOut &r) {
    int j = S.hb_bond[i];
    Kin kk; pair_kin_r(S, xi, i, j, kk);
    Lim o; int warn = 0, bad = 0;
    const bool neg = tkey(kk.b) < 0;
    int cs = find_pair_r(S, i, j, K_HB, neg, kk.r2, o, &warn, &bad);
    int sub; double pot, t;
    double D1 = 0;
    if (neg) D1 = kk.b * kk.b - kk.v2 * (kk.r2 - o.lo);
    if (neg && dbl_gt0(D1)) {
        pot = o.lopot; sub = (cs == 0) ? SDMD_SUB_CORE : SDMD_SUB_TBD_CAPTURE;
        t = root_d(kk, -1, D1);
    } else {
        pot = o.uppot; sub = (cs == 1) ? SDMD_SUB_TBD_HBBREAK : SDMD_SUB_TBD_ESCAPE;
        t = root_d(kk, 1, kk.b * kk.b - kk.v2 * (kk.r2 - o.up));
    }
    if (dbl_lt0(t)) t = INFINIT;
    r.pos = tkey(t) > 0;
    if (S.lazy) t = S.now + t;
    r.t = t; r.pot = pot; r.sub = sub; r.warn = warn; r.bad = bad;
}

// RightPair's type-pair index in shared memory for the kernel's lifetime (S: the
// block's shared descriptor)
__device__ __forceinline__ void stage_rp(DSys &S) {
    __shared__ int16_t rp_sh[NT * NT];
    const int16_t *src = S.rp_idx;
    for (int k = threadIdx.x; k < NT * NT; k += blockDim.x) rp_sh[k] = src[k];
    __syncthreads();
    if (threadIdx.x == 0) S.rp_idx = rp_sh;
    __syncthreads();
}

// ---- per-cell atom arrays (screened path) --------------------------------------------
// Cell c holds cell_cnt[c] atoms in cell_arr[c*maxc ...] in insertion order, so the
// reference's list (head = most recently inserted, src/Events.c:158-200) reads
// from the end.  Built from cell_list at kernel start, written back at the end.
__device__ __noinline__ void cells_from_list(const DSys &S, Blk &B) {
    const int N = S.n, M = S.maxc;
    for (int c = 1 + threadIdx.x; c <= S.ncell; c += blockDim.x) {
        int32_t *arr = S.cell_arr + (size_t)c * M;
        int cnt = 0;
        for (int a = S.cell_list[N + c]; a; a = S.cell_list[a]) {
            if (cnt >= M) { set_err(B, SDMD_ECAPACITY, a); break; }
            arr[cnt++] = a;
        }
        for (int k = 0; k < cnt / 2; k++) { int x = arr[k]; arr[k] = arr[cnt - 1 - k]; arr[cnt - 1 - k] = x; }
        S.cell_cnt[c] = cnt;
    }
}
__device__ __noinline__ void cells_to_list(const DSys &S) {
    const int N = S.n, M = S.maxc;
    for (int c = 1 + threadIdx.x; c <= S.ncell; c += blockDim.x) {
        const int32_t *arr = S.cell_arr + (size_t)c * M;
        const int cnt = S.cell_cnt[c];
        S.cell_list[N + c] = cnt ? arr[cnt - 1] : 0;
        for (int k = cnt - 1; k >= 0; k--) S.cell_list[arr[k]] = k ? arr[k - 1] : 0;
    }
}
// LinkList("part") for one atom (remove from oldc, insert as newest of newc), one warp
__device__ __noinline__ void cell_move_warp(const DSys &S, int t, int oldc, int newc, Blk &B) {
    const int lane = threadIdx.x & 31, M = S.maxc;
    int32_t *ao = S.cell_arr + (size_t)oldc * M;
    const int cnt = S.cell_cnt[oldc];
    int pos = -1;
    for (int base = 0; base < cnt; base += 32) {
        const int k = base + lane;
        unsigned m = __ballot_sync(0xffffffffu, k < cnt && ao[k] == t);
        if (m) { pos = base + __ffs(m) - 1; break; }
    }
    if (pos < 0) { if (lane == 0) set_err(B, SDMD_ELINK, t); __syncwarp(); return; }
    for (int base = pos + 1; base < cnt; base += 32) {
        const int k = base + lane;
        const int v = k < cnt ? ao[k] : 0;
        __syncwarp();
        if (k < cnt) ao[k - 1] = v;
        __syncwarp();
    }
    if (lane == 0) {
        if (newc == oldc) ao[cnt - 1] = t;
        else {
            const int c2 = S.cell_cnt[newc];
            S.cell_cnt[oldc] = cnt - 1;
            if (c2 >= M) set_err(B, SDMD_ECAPACITY, t);
            else { S.cell_arr[(size_t)newc * M + c2] = t; S.cell_cnt[newc] = c2 + 1; }
        }
    }
    __syncwarp();
}

// ---- warp helpers ----------------------------------------------------------------
// gather atom i's 27-cell neighbourhood into nbj[] in scan order with one warp
__device__ int gather_warp(const DSys &S, int i, int32_t *nbj, int nbcap, int *overflow) {
    const int lane = threadIdx.x & 31, M = S.maxc;
    int cell = 0, c = 0;
    if (lane < 27) {
        cell = nb_cell(S, i, lane);
        c = S.cell_cnt[cell];
    }
    int incl = c;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += y;
    }
    int tot = __shfl_sync(0xffffffffu, incl, 31);
    if (tot > nbcap) { *overflow = 1; return 0; }
    if (lane < 27) {   // up to eight independent loads in flight per lane
        const int32_t *arr = S.cell_arr + (size_t)cell * M;
        const int off = incl - c;
        for (int m0 = 0; m0 < c; m0 += 8) {
            int32_t v[8];
#pragma unroll
            for (int u = 0; u < 8; u++) if (m0 + u < c) v[u] = arr[c - 1 - m0 - u];
#pragma unroll
            for (int u = 0; u < 8; u++) if (m0 + u < c) nbj[off + m0 + u] = v[u];
        }
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
// With `full`, every node on a's path is set to its winner (no early stop): the
// repair that follows one of another leaf made while a's time was changing.  Since
// each incremental repair leaves every node the winner of its children, both
// orders give the same tree.
__device__ void cbt_update_warp(const DSys &S, int a, bool full = false) {
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
    if (on && (full || lane <= last) && id != old) node[f] = id;
    __syncwarp();
}

// ---- the two-atom screened Predict -------------------------------------------------
constexpr int RC = 64;            // refined candidates per atom before the plain path takes over

struct ShmS {
    Shm F;                        // the plain path's buffers (used when more than RC candidates need FP64)
    int32_t *nbj[2];
    uint8_t *stat[2];             // outcome | warnings << 2, per entry
    float *tlo[2];                // lower time bound of an offer
    int32_t *rl[2];               // refined entries in scan order
    Slots R[2];                   // their exact FP64 results
    // the partner j's stored event fields that the fold's JobAssign and
    // CheckDuplication copy (counter, potential, sub-type), loaded by the refine
    // lanes so that the fold reads shared memory only
    int64_t *jcnt[2];
    double *jpot[2];
    int32_t *jsub[2];
    double *face;                 // PCC face times, 3 per atom
};

struct PairScal {                 // per-atom block scalars of one two-atom prediction
    int i[2], nb[2], nn[2], mode[2], E[2], rn[2], over[2], warn_excl[2];
    unsigned u_key[2], dup_key[2];
    float uprime[2], nowf;
    double xi[2][3];              // lzx(i): the atom's FP64 position now
    AtomI A[2];
    double pcc_abs[2], th_abs[2]; // PCC / thermostat offers as stored (absolute in lazy mode)
    int pcc_pos[2], th_pos[2];    // the offer's time is > 0 (JobAssign's test)
    int64_t smp0;                 // sample index of the target's thermostat draw
    PIv P[2];
    HbbOut hbb[2];
};

__host__ __device__ inline size_t screen_ecap(int nbcap) { return 64 + 2 * (size_t)nbcap; }
__host__ __device__ inline size_t screen_smem_bytes_dev(int nbcap) {
    size_t ecap = screen_ecap(nbcap);
    size_t b = fp64_smem_bytes_dev(nbcap);
    b += al16(2 * (size_t)nbcap * 4) + al16(2 * ecap) + al16(2 * ecap * 4);
    b += al16(2 * RC * 4) + 2 * (2 * al16(RC * 4) + 3 * al16(RC * 8)) + al16(6 * 8);
    b += 2 * (2 * al16(RC * 8) + al16(RC * 4));
    return al16(b);
}
__device__ inline void carve_screen(ShmS &M, int nbcap) {
    extern __shared__ __align__(16) unsigned char smem[];
    carve(M.F, nbcap);
    unsigned char *p = smem + fp64_smem_bytes_dev(nbcap);
    auto take = [&p](size_t bytes) { unsigned char *r = p; p += al16(bytes); return r; };
    size_t ecap = screen_ecap(nbcap);
    int32_t *nbj = (int32_t *)take(2 * (size_t)nbcap * 4);
    uint8_t *st = (uint8_t *)take(2 * ecap);
    float *tl = (float *)take(2 * ecap * 4);
    int32_t *rl = (int32_t *)take(2 * RC * 4);
    for (int a = 0; a < 2; a++) {
        M.nbj[a] = nbj + a * nbcap; M.stat[a] = st + a * ecap; M.tlo[a] = tl + a * ecap;
        M.rl[a] = rl + a * RC;
        M.R[a].j = (int32_t *)take(RC * 4); M.R[a].info = (int32_t *)take(RC * 4);
        M.R[a].t = (double *)take(RC * 8); M.R[a].tdup = (double *)take(RC * 8); M.R[a].pot = (double *)take(RC * 8);
        M.jcnt[a] = (int64_t *)take(RC * 8); M.jpot[a] = (double *)take(RC * 8); M.jsub[a] = (int32_t *)take(RC * 4);
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

// JobAssign (src/TimePrediction.c:1140-1158) for an offer whose stored time (absolute
// in lazy mode) and positivity were computed beforehand by a lane
__device__ __forceinline__ void job_assign_pre(const DSys &S, Cur &c, int j, double ts, int pos, double pot, int sub,
                                               int type) {
    if (!pos) return;
    const long long kt = tkey(ts);
    if (c.key > kt) {
        c.potential = pot; c.sub = sub; c.time = ts; c.key = kt; c.type = type;
        if (j) { c.partner = j; c.pcounter = S.ev_counter[j]; }
        else c.partner = INVALID;
    }
}
constexpr int F_POS = 4;   // slot flag: the fresh time is > 0 (set by the refine lane)

// one refined offer of the fold (resolve() for a single slot); `tnew` is the
// target atom whose fresh event may now duplicate this pair, or -1
__device__ inline void fold_entry(const DSys &S, Cur &c, const ShmS &M, int a, int q, int i, int type, int tnew,
                                  Blk &B) {
    const Slots &L = M.R[a];
    int info = L.info[q];
    if (info < 0) return;
    const int j = L.j[q];
    double tdup = L.tdup[q];
    // j's counter, potential and sub-type as the refine lanes loaded them; only the
    // target's event (seen by the partner's fold) has changed since, so it is read live
    int64_t jc = M.jcnt[a][q];
    double jpo = M.jpot[a][q];
    int js = M.jsub[a][q];
    if (j == tnew) {   // CheckDuplication sees the target's new event
        info &= ~F_DUP;
        if (j < S.dup_limit && S.ev_partner[j] == i && S.ev_type[j] == type && S.ev_pcounter[j] == S.ev_counter[i]) {
            info |= F_DUP; tdup = S.ev_time[j];
        }
        jc = S.ev_counter[j]; jpo = S.ev_potential[j]; js = S.ev_sub[j];
    }
    if (info & F_DUP) {   // dup_assign() with j's fields from above
        const long long kt = tkey(tdup);
        if (c.key > kt) {
            c.partner = j; c.potential = jpo; c.sub = js; c.time = tdup; c.key = kt; c.type = type; c.pcounter = jc;
            return;
        }
    }
    B.warn += (info >> 16) & 0xff;
    if ((info & F_FRESH) && (info & F_POS)) {   // job_assign_pre() with j's counter from above
        const long long kt = tkey(L.t[q]);
        if (c.key > kt) {
            c.potential = L.pot[q]; c.sub = (info >> 8) & 0xff; c.time = L.t[q]; c.key = kt; c.type = type;
            if (j) { c.partner = j; c.pcounter = jc; }
            else c.partner = INVALID;
        }
    }
}

// Predict's fold for atom a of the pair, in the reference's order (thread 0).
// Warnings and errors gather in a register copy of the block scalars and merge
// once at the end: a store to the shared block scalars between two loads of the
// state arrays would serialise the loads.
__device__ void fold_atom(const DSys &S, int a, int tnew, ShmS &M, PairScal &PS, Blk &Bs, DScal &C) {
    const int i = PS.i[a], nb = PS.nb[a], nn = PS.nn[a], rn = PS.rn[a];
    Blk B = Bs;
    B.warn = 0;
    Cur c;
    cur_load(S, i, c);
    int q = 0, bad = 0;
    for (; q < rn && M.rl[a][q] < nb + nn; q++)
        fold_entry(S, c, M, a, q, i, M.rl[a][q] < nb ? SDMD_EV_BOND : SDMD_EV_COLLISION, tnew, B);
    job_assign_pre(S, c, 0, PS.pcc_abs[a], PS.pcc_pos[a], 0, SDMD_SUB_INVALID, SDMD_EV_PCC);
    int smp_take = 0;
    if (S.thermostat) {   // ThermostatTime: the sample was evaluated by a lane
        if (C.smp_used >= C.smp_avail || C.smp_used != PS.smp0 + a) set_err(B, SDMD_ETIMEOUT, 0);
        else {
            smp_take = 1;
            job_assign_pre(S, c, 0, PS.th_abs[a], PS.th_pos[a], 0, SDMD_SUB_INVALID, SDMD_EV_THERMOSTAT);
        }
    }
    if (PS.mode[a] == 1) {
        const int j = S.hb_bond[i];
        if (!(j < S.dup_limit && S.ev_partner[j] == i && S.ev_type[j] == SDMD_EV_HB && S.ev_pcounter[j] == S.ev_counter[i] &&
              dup_assign(S, c, j, S.ev_time[j], SDMD_EV_HB))) {
            const HbbOut &h = PS.hbb[a];
            B.warn += h.warn;
            if (h.bad) bad = 1;
            job_assign_pre(S, c, j, h.t, h.pos, h.pot, h.sub, SDMD_EV_HB);
        }
    } else if (PS.mode[a] == 2) {
        for (; q < rn; q++) fold_entry(S, c, M, a, q, i, SDMD_EV_HB, tnew, B);
    }
    if (PS.A[a].nbs > 0) hbnb_time(S, i, c, B, &bad);   // its loop runs over nb_status[i] partners
    if (S.wall) wall_time(S, i, c, B, &bad);
    if (S.n_obst) obst_time(S, i, c, B, &bad);
    if (S.n_sph) sphobst_time(S, i, c, B);
    S.hb_itype[i] = SDMD_HB_NOEVENT;    // HBSkip is one-shot (src/TimePrediction.c:309-327)
    cur_store(S, i, c);
    B.warn += PS.warn_excl[a];
    if (bad) set_err(B, SDMD_EHBMAP, i);
    Bs.warn += B.warn;
    if (B.err && !Bs.err) { Bs.err = B.err; Bs.err_atom = B.err_atom; }
    C.smp_used += smp_take;
}

// Predict for the target t and (when p > 0) the partner p, after ResetTarget of
// both: the same results as predict_atom(t) followed by predict_atom(p).  Returns
// true when warp 1 already repaired t's tree path, overlapped with the partner's
// fold; p's path then takes the full repair (cbt_update_warp(full)).
__device__ bool predict_two(const DSys &S, int t, int p, ShmS &M, PairScal &PS, Blk &B, DScal &C) {
    const int tid = threadIdx.x, T = blockDim.x, lane = tid & 31, warp = tid >> 5, nw = T >> 5;
    const int na = p ? 2 : 1;
    // 1. per-atom set-up and the two 27-cell gathers (one warp each)
    if (tid < na) {
        const int a = tid, i = a ? p : t;
        // Every load of atom i first, into registers, then the stores to shared
        // memory: the state arrays may themselves live in shared memory (staged
        // state), so a store between two loads would serialise their latencies.
        const int nb = S.bond_off[i + 1] - S.bond_off[i];
        const int hbit = S.hb_itype[i], hbb = S.hb_bond[i], role = S.hb_role[i];
        const double xi[3] = {lzx(S, S.x, S.vx, i), lzx(S, S.y, S.vy, i), lzx(S, S.z, S.vz, i)};
        AtomI A;
        load_atom_i(S, i, xi, A);
        PIv P;
        atom_piv_d(S, i, P);                           // its record is being refreshed below
        int mode;
        if (hbit == SDMD_HB_SKIP) mode = 0;
        else if (hbb > 0) mode = 1;
        else mode = (role == 'A' || role == 'D' || role == 'S') ? 2 : 0;
        PS.i[a] = i;
        PS.nb[a] = nb;
        PS.mode[a] = mode;
        PS.u_key[a] = f_key(INFINITY); PS.dup_key[a] = f_key(-INFINITY);
        PS.warn_excl[a] = 0; PS.rn[a] = 0; PS.over[a] = 0;
        PS.xi[a][0] = xi[0]; PS.xi[a][1] = xi[1]; PS.xi[a][2] = xi[2];
        PS.A[a] = A;
        PS.P[a] = P;
    }
    if (tid == 2)   // |now| bound for step 4's lazy-mode margin (two FP64 conversions, off the chain)
        PS.nowf = S.lazy ? fmaxf(fabsf(ivd(S.now).hi), fabsf(ivd(S.now).lo)) : 0.f;
    if (S.shadow_ok && tid >= T - 32 && tid < T - 32 + 4 * na) {   // t and p moved: refresh their records
        const int l = tid - (T - 32);
        shadow_word(S, l < 4 ? t : p, l & 3);
    }
    for (int a = 0; a < na; a++) {   // on warps 1 and 2 when there are: warp 0 does the set-up above
        if (warp == ((1 + a) % nw)) {
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
    __syncthreads();
    if (B.err) return false;
    // 2. PCC faces (exact, FP64) and the FP32 screen of every bond / collision / HB candidate
    const int E0 = PS.E[0], E1 = na > 1 ? PS.E[1] : 0;
    const int S0 = PS.nb[0] + PS.nn[0], S1 = na > 1 ? PS.nb[1] + PS.nn[1] : 0;
    // When every item fits in one pass, cell candidates take threads from the front
    // and bonds from the back, so that no warp runs the bond screen and the cell
    // screen one after the other (results go to their entry index either way).
    const int NB = PS.nb[0] + (na > 1 ? PS.nb[1] : 0), NC = S0 + S1 - NB;
    const bool split = S0 + S1 <= T;
    for (int g = tid; g < (split ? T : S0 + S1); g += T) {
        int a, e;
        if (split) {
            if (g < NC) { a = g < PS.nn[0] ? 0 : 1; e = PS.nb[a] + (a ? g - PS.nn[0] : g); }
            else if (g >= T - NB) { const int b = T - 1 - g; a = b < PS.nb[0] ? 0 : 1; e = a ? b - PS.nb[0] : b; }
            else continue;
        } else {
            a = g < S0 ? 0 : 1; e = a ? g - S0 : g;
        }
        const int i = PS.i[a], nb = PS.nb[a], nn = PS.nn[a];
        Outcome v[2];
        int j, ne = 1;
        if (e < nb) {
            const int qb = S.bond_off[i] + e;
            j = S.bond_j[qb];
            screen_bond(S, i, qb, PS.P[a], v[0], a == 1 && j == t);
        } else {
            j = M.nbj[a][e - nb];
            const bool hb = PS.mode[a] == 2;
            screen_cell(S, i, j, PS.P[a], PS.A[a], hb, a == 1 && j == t, v[0], v[1]);
            ne = hb ? 2 : 1;
        }
        for (int x = 0; x < ne; x++) {
            const int ee = x ? e + nn : e;
            M.stat[a][ee] = (uint8_t)(v[x].st | (v[x].warn << 2));
            M.tlo[a][ee] = v[x].t.lo;
            if (v[x].st == SC_OFFER && x == 0) atomicMin(&PS.u_key[a], f_key(v[x].t.hi));
            else if (v[x].st == SC_NONE && v[x].warn) atomicAdd(&PS.warn_excl[a], v[x].warn);
            if (v[x].dup) {   // CheckDuplication may adopt j's stored time: it bounds what can matter
                double d = S.ev_time[j];
                if (S.lazy) d = d - S.now;
                atomicMax(&PS.dup_key[a], f_key(ivd(d).hi));
            }
        }
    }
    __syncthreads();
    // 3. U: the bond / collision segment of the fold ends at or below U (its smallest
    // certain upper bound).  Bounding only by that segment keeps the whole fold
    // exact, including JobAssign's partnerCounter, which a partner-less winner
    // (PCC, thermostat, wall) leaves at the value of the last bond/collision record.
    // U' adds every duplicate time (and, for the partner, the target's bound).
    // 4-5. The entries that need FP64 -- undecided ones and offers that may reach
    // U' -- listed in scan order.  One warp per atom does all of it.
    for (int a = 0; a < na; a++) {
        if (warp != (a % nw)) continue;
        float up = fmaxf(key_f(PS.u_key[a]), key_f(PS.dup_key[a]));
        if (a == 1) up = fmaxf(up, key_f(PS.u_key[0]));   // the target's new event may become a duplicate
        const int Ea = PS.E[a];
        int base = 0, wsum = 0;
        for (int e0 = 0; e0 < Ea; e0 += 32) {
            const int e = e0 + lane;
            bool refine = false;
            if (e < Ea) {
                const int st = M.stat[a][e] & 3, w = M.stat[a][e] >> 2;
                refine = st == SC_REFINE;
                if (st == SC_OFFER) {
                    const float tl = M.tlo[a][e];
                    // lazy mode compares now + t: keep a margin of a few FP64 ulps of that sum
                    const float margin = S.lazy ? __fmul_ru(__fadd_ru(PS.nowf, fabsf(tl)), 0x1p-48f) : 0.f;
                    if (__fsub_rd(tl, up) > margin) wsum += w;   // dropped: its warnings still count
                    else refine = true;
                }
            }
            const unsigned m = __ballot_sync(0xffffffffu, refine);
            const int pos = base + __popc(m & ((1u << lane) - 1u));
            if (refine && pos < RC) M.rl[a][pos] = e;
            base += __popc(m);
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) wsum += __shfl_down_sync(0xffffffffu, wsum, o);
        if (lane == 0) {
            PS.uprime[a] = up;
            PS.warn_excl[a] += wsum;
            PS.rn[a] = base < RC ? base : RC;
            PS.over[a] = base > RC;
        }
    }
    // Eager mode with helper blocks: from here on exact positions and event times
    // of other atoms are read (refine, folds, tree repair); the screen above used
    // the records only.
    if (S.adv_on && tid == 0) adv_wait(S, B);
    __syncthreads();
    // 6. exact FP64 for the refined entries, packed into lanes; one warp per kind
    {
        int bad = 0;
        const int R0 = PS.over[0] ? 0 : PS.rn[0];
        const int R1 = (na > 1 && !PS.over[1]) ? PS.rn[1] : 0;
        // one refined entry, evaluated by this lane (pk: its kinematics, when precomputed)
        auto refine_one = [&](int a, int qq, int e, int kind, const Kin *pk) {
            const int i = PS.i[a], nb = PS.nb[a], nn = PS.nn[a];
            {   // the partner's stored event fields, for the fold (loads overlap the FP64 work)
                const int jp = kind == 1 ? S.bond_j[S.bond_off[i] + e] : M.nbj[a][kind == 0 ? e - nb : e - nb - nn];
                const int64_t jc = S.ev_counter[jp];
                const double jpo = S.ev_potential[jp];
                const int js = S.ev_sub[jp];
                M.jcnt[a][qq] = jc; M.jpot[a][qq] = jpo; M.jsub[a][qq] = js;
            }
            if (kind == 1) eval_bond_r(S, PS.xi[a], i, S.bond_off[i] + e, M.R[a], qq, pk);
            else if (kind == 0) eval_collision_r(S, PS.xi[a], i, M.nbj[a][e - nb], M.R[a], qq, &bad, pk);
            else eval_hb_scan_r(S, PS.xi[a], i, M.nbj[a][e - nb - nn], M.R[a], qq, &bad, pk);
            int info = M.R[a].info[qq];
            if (info >= 0 && (info & F_FRESH)) {   // JobAssign's "> 0" test and the stored time
                double tf = M.R[a].t[qq];
                if (tkey(tf) > 0) info |= F_POS;
                if (S.lazy) M.R[a].t[qq] = S.now + tf;
                M.R[a].info[qq] = info;
            }
        };
        const int Rt = R0 + R1;
        int la = 0, lqq = 0, le = 0, lkind = -1;
        if (lane < Rt) {
            la = lane < R0 ? 0 : 1; lqq = la ? lane - R0 : lane; le = M.rl[la][lqq];
            lkind = le < PS.nb[la] ? 1 : (le < PS.nb[la] + PS.nn[la] ? 0 : 2);
        }
        const unsigned mine = __ballot_sync(0xffffffffu, lkind >= 0 && lkind % nw == warp);
        const int nm = __popc(mine);
        if (Rt <= 32 && nm <= 10) {
            // Three lanes per entry (one per axis) compute pair_kin_r()'s per-axis
            // terms; lane 3g adds them in the same order and evaluates entry g.  Same
            // FP64 operations, about a third of the warp-instructions.
            const int g = lane / 3, d = lane - 3 * g;
            unsigned m = mine;
            for (int k = 0; k < g && m; k++) m &= m - 1;
            const int src = (g < nm && m) ? __ffs(m) - 1 : 0;
            const int ga = __shfl_sync(0xffffffffu, la, src), gqq = __shfl_sync(0xffffffffu, lqq, src);
            const int ge = __shfl_sync(0xffffffffu, le, src), gkind = __shfl_sync(0xffffffffu, lkind, src);
            const bool ok = g < nm;
            double r = 0, w = 0;
            if (ok) {
                const int i = PS.i[ga], nb = PS.nb[ga], nn = PS.nn[ga];
                const int j = gkind == 1 ? S.bond_j[S.bond_off[i] + ge] : M.nbj[ga][gkind == 0 ? ge - nb : ge - nb - nn];
                const double *X = d == 0 ? S.x : (d == 1 ? S.y : S.z), *V = d == 0 ? S.vx : (d == 1 ? S.vy : S.vz);
                const int32_t *Cc = d == 0 ? S.cx : (d == 1 ? S.cy : S.cz);
                double xj = lzx(S, X, V, j);
                const int ci = Cc[i], cj = Cc[j];
                if (ci != cj) {
                    if (ci == 0 && cj == S.cn[d] - 1) xj = xj + -1 * S.box[d];
                    else if (ci == S.cn[d] - 1 && cj == 0) xj = xj + S.box[d];
                }
                r = PS.xi[ga][d] - xj;
                w = V[i] - V[j];
            }
            const double rr = r * r, rw = r * w, ww = w * w;
            const double r_1 = __shfl_down_sync(0xffffffffu, r, 1), r_2 = __shfl_down_sync(0xffffffffu, r, 2);
            const double rr1 = __shfl_down_sync(0xffffffffu, rr, 1), rr2 = __shfl_down_sync(0xffffffffu, rr, 2);
            const double rw1 = __shfl_down_sync(0xffffffffu, rw, 1), rw2 = __shfl_down_sync(0xffffffffu, rw, 2);
            const double ww1 = __shfl_down_sync(0xffffffffu, ww, 1), ww2 = __shfl_down_sync(0xffffffffu, ww, 2);
            if (ok && d == 0) {
                Kin kk;
                kk.rx = r; kk.ry = r_1; kk.rz = r_2;
                kk.r2 = rr + rr1 + rr2;
                kk.b = rw + rw1 + rw2;
                kk.v2 = ww + ww1 + ww2;
                refine_one(ga, gqq, ge, gkind, &kk);
            }
        } else {
            for (int q = lane; q < Rt; q += 32) {
                const int a = q < R0 ? 0 : 1, qq = a ? q - R0 : q;
                const int e = M.rl[a][qq], nb = PS.nb[a], nn = PS.nn[a];
                const int kind = e < nb ? 1 : (e < nb + nn ? 0 : 2);
                if (kind % nw != warp) continue;
                refine_one(a, qq, e, kind, nullptr);
            }
        }
        // PCC (PBCandCrossCellTime) and thermostat offers of each atom, by lanes of the last
        // warp: first the face-crossing times (FP64 divisions, three lanes per atom)
        if (warp == nw - 1) {
            if (lane < 3 * na) M.face[lane] = pcc_face(S, PS.i[lane / 3], lane % 3);
            __syncwarp();
        }
        if (warp == nw - 1 && lane < 2 * na) {
            const int a = lane >> 1;
            if ((lane & 1) == 0) {
                double best = INFINIT;
                for (int d = 0; d < 3; d++) {
                    double tf = M.face[3 * a + d];
                    if (tkey(best) > tkey(tf) && tkey(tf) > 0) best = tf;
                }
                PS.pcc_pos[a] = tkey(best) > 0;
                PS.pcc_abs[a] = S.lazy ? S.now + best : best;
            } else if (S.thermostat) {
                const int64_t q = C.smp_used + a;
                double th = 0;
                if (q < C.smp_avail) {
                    double x = S.smp[q] * sqrt(1.0) + 0;
                    th = S.thermo_freq * (x < 0 ? -x : x);
                }
                PS.th_pos[a] = tkey(th) > 0;
                PS.th_abs[a] = S.lazy ? S.now + th : th;
                if (a == 0) PS.smp0 = C.smp_used;
            }
        }
        if (warp == 3 % nw && lane < na && PS.mode[lane] == 1 && !PS.over[lane])
            hbb_fresh(S, PS.xi[lane], PS.i[lane], PS.hbb[lane]);
        if (bad) set_err(B, SDMD_EHBMAP, t);
    }
    __syncthreads();
    // 7. the folds: target first, then the partner (which may now see the target's event)
    if (PS.over[0]) predict_atom(S, t, M.F, B, C);
    else {
        if (tid == 0 && !B.err) fold_atom(S, 0, -1, M, PS, B, C);
        __syncthreads();
    }
    bool t_tree = false;
    if (na > 1 && !B.err) {
        if (PS.over[1]) predict_atom(S, p, M.F, B, C);
        else {
            t_tree = nw > 1;
            if (tid == 0) fold_atom(S, 1, t, M, PS, B, C);
            else if (t_tree && warp == 1) cbt_update_warp(S, t);   // t's event is final
            __syncthreads();
        }
    }
    return t_tree;
}

}  // namespace sdmd
