// sweep_par.cuh -- the full-rebuild sweep (Prepare, src/SGThread.c:47-52) in parallel.
//
// Included by loop_fp64.cu after screen.cuh.  The reference predicts atoms 1..N in
// order after resetting every event; an atom's prediction depends on the earlier
// ones only through CheckDuplication (src/TimePrediction.c:1101-1117): a partner j
// predicted before it whose stored event names it, with the same event type.
// The sweep therefore runs in three phases that give the sequential result:
//   1. every atom is predicted at once, with CheckDuplication disabled
//      (dup_limit = 0);
//   2. each atom checks its partners j < i whose phase-1 event names it.  Adopting
//      j's event is indistinguishable from the fresh offer the atom made for j when
//      both carry the same time, potential and sub-type and the fresh offer added
//      no warning (both then assign under the same condition and write the same
//      fields).  Atoms with any other duplicate are flagged;
//   3. one block re-predicts the flagged atoms in atom order with
//      CheckDuplication limited to j < i, exactly as the reference would; if a
//      result changes, the later atom its new event names is checked the same way
//      and flagged when its own offer differs.
// The thermostat draws its i-th sample for atom i in every phase, as the
// sequential sweep does.  The event tree is then built bottom-up over CreateCBT's
// leaf layout (src/CBT.c:16-30): with every time fixed, CreateCBT's incremental
// repairs leave each node the winner of its two children (ties to the right), the
// one tree the bottom-up construction produces.
#pragma once

namespace sdmd {

__device__ __forceinline__ void latch_err(const DSys &S, int code, int atom) {
    if (atomicCAS(&S.sc->err, 0, code) == 0) S.sc->err_atom = atom;
}

// 0. ResetTarget of every atom, the pre-sweep HB interaction types, per-cell arrays
__global__ void sweep_reset_kernel(const DSys *systems) {
    const DSys &S = systems[blockIdx.y];
    if (S.sc->err) return;
    const int stride = gridDim.x * blockDim.x, t0 = blockIdx.x * blockDim.x + threadIdx.x;
    if (t0 == 0) {
        S.sc->sw_nflag = 0;
        if (S.thermostat && S.sc->smp_avail < S.n) latch_err(S, SDMD_ECAPACITY, 0);   // one sample per atom
    }
    for (int i = 1 + t0; i <= S.n; i += stride) {
        S.ev_type[i] = SDMD_EV_INVALID; S.ev_time[i] = INFINIT; S.ev_partner[i] = INVALID;
        S.sw_hbit[i] = S.hb_itype[i]; S.sw_flag[i] = 0; S.sw_warn[i] = 0;
    }
    const int N = S.n, M = S.maxc;
    for (int c = 1 + t0; c <= S.ncell; c += stride) {
        int32_t *arr = S.cell_arr + (size_t)c * M;
        int cnt = 0;
        for (int a = S.cell_list[N + c]; a; a = S.cell_list[a]) {
            if (cnt >= M) { latch_err(S, SDMD_ECAPACITY, a); break; }
            arr[cnt++] = a;
        }
        for (int k = 0; k < cnt / 2; k++) { int x = arr[k]; arr[k] = arr[cnt - 1 - k]; arr[cnt - 1 - k] = x; }
        S.cell_cnt[c] = cnt;
    }
}

// 1. every atom predicted at once (CheckDuplication off); blocks stride over atoms
__global__ void sweep_predict_kernel(const DSys *systems) {
    __shared__ DSys S;
    __shared__ Blk B;
    __shared__ DScal C;
    __shared__ PairScal PS;
    if (threadIdx.x == 0) {
        S = systems[blockIdx.y];
        S.dup_limit = 0;
        B.err = 0; B.warn = 0;
        C = *S.sc;
        S.now = C.time;
    }
    __syncthreads();
    if (C.err) return;
    stage_rp(S);
    ShmS MS;
    carve_screen(MS, S.nbcap);
    const int64_t base = C.smp_used;
    for (int i = 1 + blockIdx.x; i <= S.n && B.err == 0; i += gridDim.x) {
        __shared__ int64_t warn0;
        if (threadIdx.x == 0) { C.smp_used = base + (i - 1); warn0 = B.warn; }
        __syncthreads();
        predict_two(S, i, 0, MS, PS, B, C);
        if (threadIdx.x == 0) S.sw_warn[i] = (int32_t)(B.warn - warn0);
    }
    if (threadIdx.x == 0) {
        if (B.warn) atomicAdd(reinterpret_cast<unsigned long long *>(&S.sc->c.warnings), (unsigned long long)B.warn);
        if (B.err) latch_err(S, B.err, B.err_atom);
    }
}

// is j's stored event (which names i, with the same type) the same offer as the
// fresh one the prediction of i made for j (slot q)?
__device__ __forceinline__ bool same_offer(const DSys &S, const Slots &L, int q, int j) {
    const int info = L.info[q];
    if (info < 0 || !(info & F_FRESH) || ((info >> 16) & 0xff)) return false;
    const double t = L.t[q];
    if (!(tkey(t) > 0)) return false;
    const double ts = S.lazy ? S.now + t : t;
    return __double_as_longlong(ts) == __double_as_longlong(S.ev_time[j]) &&
           __double_as_longlong(L.pot[q]) == __double_as_longlong(S.ev_potential[j]) &&
           ((info >> 8) & 0xff) == S.ev_sub[j];
}
__device__ __forceinline__ bool names(const DSys &S, int j, int i, int type) {
    return S.ev_partner[j] == i && S.ev_type[j] == type && S.ev_pcounter[j] == S.ev_counter[i];
}

// 2. one warp per atom: does any earlier partner's event differ from the atom's own offer?
__device__ bool duplicate_differs(const DSys &S, int i, int32_t *nbj, Slots &L) {
    const int lane = threadIdx.x & 31;
    int mode;
    if (S.sw_hbit[i] == SDMD_HB_SKIP) mode = 0;
    else if (S.hb_bond[i] > 0) mode = 1;
    else { int r = S.hb_role[i]; mode = (r == 'A' || r == 'D' || r == 'S') ? 2 : 0; }
    bool differs = false;
    if (lane == 0) {   // HB-bonded partner and HB-neighbour partners: any duplicate is re-predicted
        if (mode == 1) { int j = S.hb_bond[i]; if (j < i && names(S, j, i, SDMD_EV_HB)) differs = true; }
        for (int n = 1; n <= S.nb_status[i]; n++) {
            int j = S.nb_partner[4 * i + n - 1];
            if (j < i && names(S, j, i, SDMD_EV_HBNEIGHBOR)) differs = true;
        }
    }
    double xi[3];
    bool have_xi = false;
    auto pos = [&]() {
        if (!have_xi) { xi[0] = lzx(S, S.x, S.vx, i); xi[1] = lzx(S, S.y, S.vy, i); xi[2] = lzx(S, S.z, S.vz, i); }
        have_xi = true;
    };
    int bad = 0;
    const int b0 = S.bond_off[i], nb = S.bond_off[i + 1] - b0;
    for (int k = lane; k < nb; k += 32) {
        const int j = S.bond_j[b0 + k];
        if (j < i && names(S, j, i, SDMD_EV_BOND)) {
            pos();
            eval_bond_r(S, xi, i, b0 + k, L, lane);
            if (!same_offer(S, L, lane, j)) differs = true;
        }
    }
    int ovf = 0;
    const int nn = gather_warp(S, i, nbj, S.nbcap, &ovf);
    if (ovf) differs = true;
    for (int k = lane; k < nn; k += 32) {
        const int j = nbj[k];
        if (j >= i) continue;
        if (names(S, j, i, SDMD_EV_COLLISION)) {
            pos();
            eval_collision_r(S, xi, i, j, L, lane, &bad);
            if (!same_offer(S, L, lane, j)) differs = true;
        }
        if (mode == 2 && names(S, j, i, SDMD_EV_HB)) {
            pos();
            eval_hb_scan_r(S, xi, i, j, L, lane, &bad);
            if (!same_offer(S, L, lane, j)) differs = true;
        }
    }
    if (bad) differs = true;   // the in-order re-prediction reports the error
    return __any_sync(0xffffffffu, differs);
}

__host__ __device__ inline size_t verify_warp_bytes(int nbcap) {
    return al16((size_t)nbcap * 4) + 2 * al16(32 * 4) + 3 * al16(32 * 8);
}
__global__ void sweep_verify_kernel(const DSys *systems) {
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ DSys S;
    if (threadIdx.x == 0) { S = systems[blockIdx.y]; S.now = S.sc->time; }
    __syncthreads();
    if (S.sc->err) return;
    stage_rp(S);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    unsigned char *p = smem + w * verify_warp_bytes(S.nbcap);
    int32_t *nbj = (int32_t *)p; p += al16((size_t)S.nbcap * 4);
    Slots L;
    L.j = (int32_t *)p; p += al16(32 * 4);
    L.info = (int32_t *)p; p += al16(32 * 4);
    L.t = (double *)p; p += al16(32 * 8);
    L.tdup = (double *)p; p += al16(32 * 8);
    L.pot = (double *)p;
    for (int i = 1 + blockIdx.x * nw + w; i <= S.n; i += gridDim.x * nw) {
        if (duplicate_differs(S, i, nbj, L) && lane == 0) {
            S.sw_flag[i] = 1;
            atomicAdd(&S.sc->sw_nflag, 1);
        }
    }
}

// After atom a's re-prediction changed its event: does the new event, which may
// name a later atom k as partner, differ from the fresh offer k's own prediction
// makes for a?  (Only a's new partner can see a new duplicate; an atom that the
// old event named is correct without it, or was flagged already.)  One lane.
__device__ bool new_partner_differs(const DSys &S, int a, int k, Slots &L) {
    const int ty = S.ev_type[a];
    if (!names(S, a, k, ty)) return false;
    double xk[3] = {lzx(S, S.x, S.vx, k), lzx(S, S.y, S.vy, k), lzx(S, S.z, S.vz, k)};
    int bad = 0;
    if (ty == SDMD_EV_BOND) {
        for (int q = S.bond_off[k]; q < S.bond_off[k + 1]; q++) {
            if (S.bond_j[q] == a) { eval_bond_r(S, xk, k, q, L, 0); return !same_offer(S, L, 0, a); }
        }
        return true;
    }
    if (ty == SDMD_EV_COLLISION) {
        eval_collision_r(S, xk, k, a, L, 0, &bad);
        return bad || !same_offer(S, L, 0, a);
    }
    if (ty == SDMD_EV_HB) {
        int mode;
        if (S.sw_hbit[k] == SDMD_HB_SKIP) mode = 0;
        else if (S.hb_bond[k] > 0) mode = 1;
        else { int r = S.hb_role[k]; mode = (r == 'A' || r == 'D' || r == 'S') ? 2 : 0; }
        if (mode == 2) { eval_hb_scan_r(S, xk, k, a, L, 0, &bad); return bad || !same_offer(S, L, 0, a); }
        return mode == 1 && S.hb_bond[k] == a;
    }
    if (ty == SDMD_EV_HBNEIGHBOR) return nb_has(S, k, a) != 0;
    return false;
}

// 3. in-order re-prediction of the flagged atoms, then the event tree (one block per system)
__global__ void sweep_fix_kernel(const DSys *systems, int full) {
    __shared__ DSys S;
    __shared__ Blk B;
    __shared__ DScal C;
    __shared__ PairScal PS;
    __shared__ int32_t chunk[1024];
    __shared__ int32_t changed;
    __shared__ double o_time, o_pot;
    __shared__ int32_t o_partner, o_type, o_sub;
    __shared__ int64_t o_pc, warn0;
    const int tid = threadIdx.x, T = blockDim.x;
    if (tid == 0) {
        S = systems[blockIdx.x];
        B.err = 0; B.warn = 0;
        C = *S.sc;
        S.now = C.time;
    }
    __syncthreads();
    if (C.err) return;
    stage_rp(S);
    ShmS MS;
    carve_screen(MS, S.nbcap);
    const int64_t base = C.smp_used;
    if (full && C.sw_nflag > 0) {
        for (int i0 = 1; i0 <= S.n && B.err == 0; i0 += T) {
            chunk[tid] = (i0 + tid <= S.n) ? S.sw_flag[i0 + tid] : 0;
            if (!__syncthreads_or(chunk[tid])) continue;
            for (int q = 0; q < T && i0 + q <= S.n && B.err == 0; q++) {
                if (!chunk[q]) continue;
                const int a = i0 + q;
                if (tid == 0) {
                    o_time = S.ev_time[a]; o_pot = S.ev_potential[a]; o_partner = S.ev_partner[a];
                    o_type = S.ev_type[a]; o_sub = S.ev_sub[a]; o_pc = S.ev_pcounter[a];
                    S.ev_type[a] = SDMD_EV_INVALID; S.ev_time[a] = INFINIT; S.ev_partner[a] = INVALID;
                    S.hb_itype[a] = S.sw_hbit[a];
                    S.dup_limit = a;
                    C.smp_used = base + (a - 1);
                    warn0 = B.warn;
                }
                __syncthreads();
                predict_two(S, a, 0, MS, PS, B, C);
                if (tid == 0) {
                    B.warn -= S.sw_warn[a];                  // phase 1 already counted its warnings
                    S.sw_warn[a] = (int32_t)(B.warn + S.sw_warn[a] - warn0);
                    changed = __double_as_longlong(o_time) != __double_as_longlong(S.ev_time[a]) ||
                              __double_as_longlong(o_pot) != __double_as_longlong(S.ev_potential[a]) ||
                              o_partner != S.ev_partner[a] || o_type != S.ev_type[a] || o_sub != S.ev_sub[a] ||
                              o_pc != S.ev_pcounter[a];
                }
                __syncthreads();
                if (changed && tid == 0) {   // the later atom a's new event names may now see a duplicate
                    const int k = S.ev_partner[a];
                    if (k > a && new_partner_differs(S, a, k, MS.R[0])) {
                        S.sw_flag[k] = 1;
                        if (k < i0 + T) chunk[k - i0] = 1;
                    }
                }
                __syncthreads();
            }
        }
    }
    // CreateCBT: leaves at their layout positions, internal nodes bottom-up
    const int N = S.n;
    int32_t *node = S.cbt_node;
    const double *tm = S.ev_time;
    if (B.err == 0) {
        if (N == 1) {
            if (tid == 0) { node[1] = 1; S.cbt_leaf[1] = S.cbt_leaf0[1]; }
        } else {
            for (int a = 1 + tid; a <= N; a += T) { const int lf = S.cbt_leaf0[a]; S.cbt_leaf[a] = lf; node[lf] = a; }
            __syncthreads();
            for (int k = 31 - __clz(N - 1); k >= 0; k--) {
                const int lo = 1 << k, hi = min(1 << (k + 1), N);
                for (int f = lo + tid; f < hi; f += T) {
                    const int l = node[2 * f], r = node[2 * f + 1];
                    node[f] = tkey(tm[l]) < tkey(tm[r]) ? l : r;
                }
                __syncthreads();
            }
        }
    }
    if (tid == 0) {
        if (full && S.thermostat) C.smp_used = base + N;
        C.c.warnings += B.warn;
        C.cbt_built = 1;
        if (B.err) { C.err = B.err; C.err_atom = B.err_atom; C.err_event = C.c.frame; }
        *S.sc = C;
    }
}

}  // namespace sdmd
