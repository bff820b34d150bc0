// remd.cu -- system energies and the replica exchange, on the device.
//
// energy_kernel restates CalKinetE / CalPotenE (src/ToolFunctions.c:626-752): the
// kinetic energy sums 0.5 m v^2 over atoms 1..N; the potential energy visits each
// pair once (partner index above the atom's) within the cutoff, in the reference's
// order -- atoms ascending, the 27 cells in scan order, each cell list head first --
// adding the accumulated step energy of the pair's shell (and subtracting the HB
// barrier for HB-bonded pairs).  The FP64 sum keeps that order, so the result is
// bit-identical to the reference's.  One warp per system: the lanes evaluate the
// pair terms of one atom, lane 0 accumulates them in order.
//
// remd_exchange_kernel restates the exchange server's rearrange()
// (src/Server.c:145-192): one pass over replica pairs with neighbouring ladder
// indices, Metropolis test exp(-(b_i - b_j)(E_j - E_i)) against the server's own
// rand() stream, swap of the (index, temperature) records.  The new temperatures
// become each replica's thermostat target (REMDRun, src/REMD.c:97-101).
#include "dev.cuh"
#include "engine.h"

namespace sdmd {

__global__ void energy_kernel(const DSys *systems, double *pot, double *kin, int64_t *warn) {
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ DSys S;
    if (threadIdx.x == 0) { S = systems[blockIdx.x]; S.now = S.sc->time; }
    __syncthreads();
    const int lane = threadIdx.x & 31, N = S.n;
    int32_t *nbj = reinterpret_cast<int32_t *>(smem);          // candidates of one atom, scan order
    int8_t *kcell = reinterpret_cast<int8_t *>(nbj + S.nbcap);  // the scan cell each came from
    __shared__ double term[32], bar[32];
    __shared__ int8_t has[32];
    double tpe = 0, tke = 0;
    int64_t warns = 0;
    int bad = 0, over = 0;
    const double cut2 = S.cutoff * S.cutoff;
    for (int i = 1; i <= N; i++) {
        // the 27-cell candidates of atom i, each list head first (lanes 0..26 walk one cell each)
        int cell = 0, c = 0, head = 0;
        if (lane < 27) {
            cell = nb_cell(S, i, lane);
            head = S.cell_list[N + cell];
            for (int a = head; a && c <= N; a = S.cell_list[a]) c++;
        }
        int incl = c;
        for (int o = 1; o < 32; o <<= 1) {
            int y = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += y;
        }
        const int nn = __shfl_sync(0xffffffffu, incl, 31);
        if (nn > S.nbcap) { over = 1; break; }
        if (lane < 27) {
            int m = incl - c;
            for (int a = head; a && m < incl; a = S.cell_list[a]) { nbj[m] = a; kcell[m] = (int8_t)lane; m++; }
        }
        __syncwarp();
        const double xi = lzx(S, S.x, S.vx, i), yi = lzx(S, S.y, S.vy, i), zi = lzx(S, S.z, S.vz, i);
        for (int k0 = 0; k0 < nn; k0 += 32) {
            const int k = k0 + lane;
            int h = 0;
            double tv = 0, bv = 0;
            if (k < nn) {
                const int pj = nbj[k], kc = kcell[k];
                if (pj > i) {
                    const int cc[3] = {S.cx[i] + c_nbx[kc], S.cy[i] + c_nby[kc], S.cz[i] + c_nbz[kc]};
                    double sh[3];
                    for (int d = 0; d < 3; d++) {
                        sh[d] = 0;
                        if (cc[d] < 0) sh[d] = -1 * S.box[d];
                        else if (cc[d] >= S.cn[d]) sh[d] = S.box[d];
                    }
                    const double rx = xi - (lzx(S, S.x, S.vx, pj) + sh[0]);
                    const double ry = yi - (lzx(S, S.y, S.vy, pj) + sh[1]);
                    const double rz = zi - (lzx(S, S.z, S.vz, pj) + sh[2]);
                    const double d2 = rx * rx + ry * ry + rz * rz;
                    const int bits = conn_bits(S, i, pj);
                    if (d2 <= cut2 && !(bits & 1)) {
                        int ai = i, aj = pj, kind, hbp = 0;
                        h = 1;
                        if (S.hb_bond[ai] == aj) { kind = K_HB; bv = hb_barrier(S, ai, aj); h = 2; }
                        else if (bits & 2) kind = K_CONSTRAINT;
                        else if (nb_has(S, ai, aj)) {
                            if (S.hb_neighbor[S.hb_bond[ai]] == aj) { int q = ai; ai = aj; aj = q; }
                            hbp = S.hb_bond[aj];
                            kind = K_NEIGHBOR;
                        } else kind = K_COLLISION;
                        const double wx = S.vx[ai] - S.vx[aj], wy = S.vy[ai] - S.vy[aj], wz = S.vz[ai] - S.vz[aj];
                        const double dirn = rx * wx + ry * wy + rz * wz;
                        Lim o;
                        o.acc = 0;
                        int w = 0;
                        find_pair(S, ai, aj, kind, dirn, d2, o, hbp, 0, 0, &w, &bad);
                        warns += w;
                        tv = o.acc;
                    }
                }
            }
            term[lane] = tv; bar[lane] = bv; has[lane] = (int8_t)h;
            __syncwarp();
            if (lane == 0) {
                const int kmax = nn - k0 < 32 ? nn - k0 : 32;
                for (int q = 0; q < kmax; q++) {
                    if (!has[q]) continue;
                    if (has[q] == 2) tpe -= bar[q];
                    if (term[q] < INFINIT / 2) tpe += term[q];
                }
            }
            __syncwarp();
        }
    }
    // CalKinetE: 0.5 m |v - 0|^2 summed over atoms in order (lanes compute, lane 0 adds)
    for (int i0 = 1; i0 <= N; i0 += 32) {
        const int i = i0 + lane;
        double e = 0;
        if (i <= N) {
            const double tx = S.vx[i] - 0, ty = S.vy[i] - 0, tz = S.vz[i] - 0;
            const double t0 = tx * tx + ty * ty + tz * tz;
            e = 0.5 * S.mass[i] * t0;
        }
        term[lane] = e;
        __syncwarp();
        if (lane == 0) for (int q = 0; q < 32 && i0 + q <= N; q++) tke += term[q];
        __syncwarp();
    }
    for (int o = 16; o > 0; o >>= 1) warns += __shfl_down_sync(0xffffffffu, warns, o);
    bad = __any_sync(0xffffffffu, bad);
    over = __any_sync(0xffffffffu, over);
    if (lane == 0) {
        pot[blockIdx.x] = tpe;
        kin[blockIdx.x] = tke;
        warn[blockIdx.x] = warns;
        if ((bad || over) && S.sc->err == 0) { S.sc->err = over ? SDMD_ECAPACITY : SDMD_EHBMAP; S.sc->err_atom = 0; }
    }
}

size_t energy_smem_bytes(int nbcap) { return (size_t)nbcap * 5 + 16; }

// every system's exchange trigger for the next round
__global__ void remd_round_kernel(const DSys *systems, int n, int64_t every_events, const double *stop_time) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    DScal *C = systems[k].sc;
    C->target_frame = every_events > 0 ? C->c.frame + every_events : 0x7fffffffffffffffLL;
    C->stop_time = stop_time ? stop_time[k] : 0;
    C->at_stop = 0;
    C->paused = 0;
}

// per-system stop points: an event limit (0: the system does not run) and an
// exchange / dump time (<= 0: none)
__global__ void stops_round_kernel(const DSys *systems, int n, const int64_t *limit, const double *stop_time) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    DScal *C = systems[k].sc;
    const int64_t room = 0x7fffffffffffffffLL - C->c.frame;
    C->target_frame = limit[k] < room ? C->c.frame + limit[k] : 0x7fffffffffffffffLL;
    C->stop_time = stop_time[k] > 0 ? stop_time[k] : 0;
    C->at_stop = 0;
    C->paused = 0;
}

// rearrange() of the exchange server, then the replicas' new thermostat targets
__global__ void remd_exchange_kernel(DSys *systems, int n, int32_t *num, double *T, const double *E,
                                     const int64_t *warn, sdmd_rng *rng, int64_t *stats) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    sdmd_rng r = *rng;
    int64_t att = 0, acc = 0;
    for (int i = 0; i < n; i++) {
        if (!(T[i] != 0)) continue;
        for (int j = 0; j < n; j++) {
            if (!(T[j] != 0)) continue;
            if (num[i] == num[j] + 1 || (num[i] == 1 && num[j] == 2)) {
                const double b1 = 1 / T[i], b2 = 1 / T[j];
                const double dE = (b1 - b2) * (E[j] - E[i]);
                att++;
                if (dE <= 0.0 || rv01(r) < cr_exp(-1 * dE)) {
                    int tn = num[i]; num[i] = num[j]; num[j] = tn;
                    double tt = T[i]; T[i] = T[j]; T[j] = tt;
                    acc++;
                }
                break;
            }
        }
    }
    *rng = r;
    stats[0] += att;
    stats[1] += acc;
    for (int k = 0; k < n; k++) {
        if (!(T[k] != 0)) continue;             // a replica that has left the exchange (its run ended)
        systems[k].temperature = T[k];
        systems[k].sc->c.warnings += warn[k];   // CalPotenE's FindPair calls count warnings too
    }
}

}  // namespace sdmd
