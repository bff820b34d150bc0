// api.cu -- the C ABI of include/sdmd_gpu.h.
//
// A handle owns one device arena holding every system's SoA arrays, the event
// trees, per-system scalars (clock, RNG, counters, error word) and the optional
// pop trace.  Launches go to the handle's own stream and are timed with CUDA
// events on that stream.  Nothing here falls back to the CPU: without a usable
// device every entry point returns SDMD_ENODEV / SDMD_ECUDA.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <algorithm>
#include <mutex>
#include <thread>
#include <vector>

#include "dev.cuh"
#include "engine.h"
#include "sdmd_gpu.h"

using namespace sdmd;

struct SysMeta {
    int32_t n, ncell, n_bonds, n_cons, n_con_steps, n_conn, n_pair_steps, nbcap, n_sph, n_obst;
};

struct sdmd_gpu {
    int32_t n_systems = 0;
    sdmd_opts opts{};
    cudaStream_t stream = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    std::vector<DSys> hs;
    std::vector<SysMeta> meta;
    DSys *ds = nullptr;
    unsigned char *arena = nullptr;
    size_t arena_bytes = 0;
    int threads = 128;
    int sms = 0;                                   // the device's SM count
    size_t smem = 0, smem_loop = 0, vsmem = 0;
    int staged = 0;
    std::vector<int32_t> smp_cap_of;
    void (*sweep_k)(const DSys *, int) = nullptr;            // plain FP64 or FP32-screened kernels
    void (*loop_k)(const DSys *, double, int) = nullptr;
    int helpers = 0;                               // helper blocks of the eager advance (0: none)
    const void *coop_k = nullptr;                  // the cooperative loop build for this block size
    int sweep_threads = 128;                       // block size of the per-system sweep kernels (<= 256)
    std::vector<int> pair_src;                     // system whose (identical) pair tables system k shares
    size_t dyn_begin = 0, dyn_end = 0;             // the dynamic arrays' block in the arena
    DScal *sc_all = nullptr;                       // the systems' scalar blocks, contiguous
    Adv *adv = nullptr;                            // their per-system protocol words (in the arena)
    double prep_ms = 0, run_ms = 0;
    // energies / replica exchange scratch (one block: num, T, E, kin, warn, stop, lim, rng, stats)
    unsigned char *aux = nullptr;
    int32_t *x_num = nullptr;
    double *x_T = nullptr, *x_E = nullptr, *x_kin = nullptr, *x_stop = nullptr;
    int64_t *x_warn = nullptr, *x_stats = nullptr, *x_lim = nullptr;
    sdmd_rng *x_rng = nullptr;
    size_t esmem = 0;
    cudaEvent_t l0 = nullptr, l1 = nullptr;        // around each loop-kernel launch
    double loop_ms = 0;                            // loop-kernel time of the last run
    int64_t launches = 0, loop_launches = 0;       // kernels launched by the last run
    sdmd_error_info err{};
};

static int cuda_fail(cudaError_t e) {
    if (e == cudaSuccess) return SDMD_OK;
    fprintf(stderr, "sdmd_gpu: CUDA error %s\n", cudaGetErrorString(e));
    return e == cudaErrorMemoryAllocation ? SDMD_ENOMEM : SDMD_ECUDA;
}
#define CK(x) do { int _r = cuda_fail(x); if (_r) return _r; } while (0)

extern "C" int sdmd_gpu_abi_version(void) { return SDMD_ABI_VERSION; }

extern "C" int sdmd_gpu_device_count(int32_t *count) {
    int c = 0;
    cudaError_t e = cudaGetDeviceCount(&c);
    if (count) *count = (e == cudaSuccess) ? c : 0;
    if (e != cudaSuccess || c == 0) return SDMD_ENODEV;
    return SDMD_OK;
}

extern "C" const char *sdmd_gpu_strerror(int code) {
    switch (code) {
        case SDMD_OK: return "ok";
        case SDMD_EINVAL: return "invalid argument";
        case SDMD_ENOMEM: return "out of memory";
        case SDMD_ECUDA: return "CUDA runtime error";
        case SDMD_ENODEV: return "no CUDA device";
        case SDMD_ENEGTIME: return "predicted event time is negative";
        case SDMD_ENAN: return "phi is NaN in a velocity update";
        case SDMD_EWALL: return "an atom is outside of the wall";
        case SDMD_ELINK: return "the cell list has errors";
        case SDMD_EHBMAP: return "HB bookkeeping or pair table is inconsistent";
        case SDMD_ECAPACITY: return "a fixed device capacity was exceeded";
        case SDMD_ETIMEOUT: return "a bounded device-side loop ran out (degenerate RNG state or stuck event loop)";
        case SDMD_EUNSUPPORTED: return "configuration outside the engine's scope";
        case SDMD_EEVENTTYPE: return "invalid event type popped";
        default: return "unknown error";
    }
}

// ---- validation ---------------------------------------------------------------
static int validate(const sdmd_system &s) {
    if (s.n_atoms <= 0 || s.cellnum[0] < 1 || s.cellnum[1] < 1 || s.cellnum[2] < 1) return SDMD_EINVAL;
    const void *ptrs[] = {s.mass, s.protein, s.aanum, s.aatype, s.hb_neighbor, s.hb_role, s.name_code,
                          s.bond_off, s.con_off, s.conn_off, s.pair_dmin, s.pair_dmax, s.pair_step_off,
                          s.pair_step_n, s.x, s.y, s.z, s.vx, s.vy, s.vz, s.cx, s.cy, s.cz, s.type, s.hb_bond,
                          s.hb_itype, s.nb_partner, s.nb_status, s.nb_pnum, s.ev_time, s.ev_partner,
                          s.ev_counter, s.ev_pcounter, s.ev_potential, s.ev_type, s.ev_sub, s.cell_list};
    for (const void *p : ptrs) if (!p) return SDMD_EINVAL;
    int N = s.n_atoms;
    if (s.bond_off[N + 1] != s.n_bonds || s.con_off[N + 1] != s.n_cons || s.conn_off[N + 1] != s.n_conn)
        return SDMD_EINVAL;
    if ((s.n_bonds && (!s.bond_j || !s.bond_dmin || !s.bond_dmax)) ||
        (s.n_cons && (!s.con_j || !s.con_dmin || !s.con_dmax || !s.con_step_off || !s.con_step_n)) ||
        (s.n_conn && (!s.conn_j || !s.conn_bits)))
        return SDMD_EINVAL;
    if (s.wall < 0 || s.wall > SDMD_WALL_SPHERE || s.thermostat < 0 || s.thermostat > 1) return SDMD_EUNSUPPORTED;
    if (s.wall_dyn != 0) return SDMD_EUNSUPPORTED;   // dynamic walls: the oracle only
    if (s.n_sphobst < 0 || s.n_sphobst > SDMD_MAX_SPHOBST || (s.n_sphobst && !s.sphobst)) return SDMD_EINVAL;
    for (int k = 0; k < s.n_sphobst; k++)
        if (!(s.sphobst[4 * k + 3] > 0) || !std::isfinite(s.sphobst[4 * k]) || !std::isfinite(s.sphobst[4 * k + 1]) ||
            !std::isfinite(s.sphobst[4 * k + 2]))
            return SDMD_EINVAL;
    if (s.n_obst < 0 || s.n_obst > SDMD_MAX_OBST || (s.n_obst && !s.obst)) return SDMD_EINVAL;
    for (int k = 0; k < 3 * s.n_obst; k++) if (!std::isfinite(s.obst[k])) return SDMD_EINVAL;
    // the RNG must be a reachable glibc state: never all zero
    bool nz = false;
    for (int k = 0; k < 31; k++) nz |= s.rng.tab[k] != 0;
    if (!nz || s.rng.front < 0 || s.rng.front > 30 || s.rng.rear < 0 || s.rng.rear > 30) return SDMD_EINVAL;
    // every index the kernels dereference must be in range
    auto atom_ok = [N](int a) { return a >= 0 && a <= N; };
    for (int k = 0; k < s.n_bonds; k++) if (s.bond_j[k] < 1 || s.bond_j[k] > N) return SDMD_EINVAL;
    for (int k = 0; k < s.n_cons; k++) {
        if (s.con_j[k] < 1 || s.con_j[k] > N || s.con_step_n[k] < 0 || s.con_step_off[k] < 0 ||
            s.con_step_off[k] + s.con_step_n[k] > s.n_con_steps)
            return SDMD_EINVAL;
        if (s.con_step_n[k] && (!s.con_step_d || !s.con_step_e || !s.con_step_acc)) return SDMD_EINVAL;
    }
    for (int k = 0; k < s.n_conn; k++) if (!atom_ok(s.conn_j[k])) return SDMD_EINVAL;
    const int NT3 = SDMD_NTABLES * SDMD_NTYPES * SDMD_NTYPES;
    for (int k = 0; k < NT3; k++) {
        if (s.pair_step_n[k] < 0 || s.pair_step_off[k] < 0 || s.pair_step_off[k] + s.pair_step_n[k] > s.n_pair_steps)
            return SDMD_EINVAL;
    }
    if (s.n_pair_steps && (!s.pair_step_d || !s.pair_step_e || !s.pair_step_acc)) return SDMD_EINVAL;
    if (s.bond_off[0] < 0 || s.con_off[0] < 0 || s.conn_off[0] < 0) return SDMD_EINVAL;
    for (int k = 1; k <= N + 1; k++) {
        if (s.bond_off[k] < s.bond_off[k - 1] || s.con_off[k] < s.con_off[k - 1] || s.conn_off[k] < s.conn_off[k - 1])
            return SDMD_EINVAL;
    }
    if ((s.wall || s.n_obst) && (s.wall_type < 0 || s.wall_type >= SDMD_NTYPES)) return SDMD_EINVAL;
    long ncell = (long)s.cellnum[0] * s.cellnum[1] * s.cellnum[2];
    for (long k = 0; k <= N + ncell; k++) if (!atom_ok(s.cell_list[k])) return SDMD_EINVAL;
    // every atom must sit in a valid cell, with in-range ids and types
    for (int i = 1; i <= N; i++) {
        if (!atom_ok(s.hb_neighbor[i]) || !atom_ok(s.hb_bond[i]) || s.type[i] < 0 || s.type[i] >= SDMD_NTYPES)
            return SDMD_EINVAL;
        if (!(s.ev_partner[i] <= 0 || s.ev_partner[i] <= N)) return SDMD_EINVAL;
        for (int q = 0; q < 4; q++) if (!atom_ok(s.nb_partner[4 * i + q])) return SDMD_EINVAL;
        if (!(s.mass[i] > 0)) return SDMD_EINVAL;
        if (s.cx[i] < 0 || s.cx[i] >= s.cellnum[0] || s.cy[i] < 0 || s.cy[i] >= s.cellnum[1] || s.cz[i] < 0 ||
            s.cz[i] >= s.cellnum[2])
            return SDMD_EINVAL;
        if (s.nb_status[i] < 0 || s.nb_status[i] > 4) return SDMD_EINVAL;
    }
    return SDMD_OK;
}

// largest 27-cell neighbourhood population at upload time
// ---- host staging for the one-copy upload and download ---------------------------
// A pinned host buffer, kept for the process and grown on demand: handles are
// created and destroyed repeatedly by drivers that hand a batch back and forth
// (and by the benchmark's end-to-end loop), and a pinned source lets the copy
// run at the link's rate.  One user at a time (the lock is held from filling the
// buffer until its copy has completed).
struct PinnedStage {
    std::mutex mu;
    unsigned char *p = nullptr;
    size_t bytes = 0;
    unsigned char *get(size_t need) {   // with mu held
        if (need <= bytes) return p;
        if (p) cudaFreeHost(p);
        p = nullptr; bytes = 0;
        const size_t want = need + need / 8;
        if (cudaHostAlloc((void **)&p, want, cudaHostAllocPortable) != cudaSuccess) { cudaGetLastError(); p = nullptr; return nullptr; }
        bytes = want;
        return p;
    }
};
static PinnedStage g_up, g_down;

// fn(k) for k = 0..n-1 on up to 8 host threads, in contiguous ranges (per-system
// host work of large batches; each k writes only its own outputs)
template <class F> static void parallel_for(int n, F fn) {
    const int nt = n < 16 ? 1 : (int)std::min<unsigned>({8u, (unsigned)n / 8, std::max(1u, std::thread::hardware_concurrency())});
    if (nt <= 1) {
        for (int k = 0; k < n; k++) fn(k);
        return;
    }
    std::vector<std::thread> th;
    for (int t = 0; t < nt; t++)
        th.emplace_back([&fn, a = (int)((long)n * t / nt), b = (int)((long)n * (t + 1) / nt)] {
            for (int k = a; k < b; k++) fn(k);
        });
    for (auto &x : th) x.join();
}

// memcpy of many (dst, src, bytes) pieces on up to 8 host threads (large batches)
struct Piece { void *dst; const void *src; size_t bytes; };
static void copy_pieces(const std::vector<Piece> &v) {
    size_t total = 0;
    for (auto &c : v) total += c.bytes;
    const int nt = total < (32u << 20) ? 1 : (int)std::min<unsigned>(8u, std::max(1u, std::thread::hardware_concurrency()));
    if (nt == 1) {
        for (auto &c : v) memcpy(c.dst, c.src, c.bytes);
        return;
    }
    // contiguous runs of pieces with about equal bytes per thread
    std::vector<size_t> cut{0};
    size_t acc = 0, per = total / nt + 1;
    for (size_t i = 0; i < v.size(); i++) {
        acc += v[i].bytes;
        if (acc >= per * cut.size() && cut.size() < (size_t)nt) cut.push_back(i + 1);
    }
    cut.push_back(v.size());
    std::vector<std::thread> th;
    for (size_t t = 0; t + 1 < cut.size(); t++)
        th.emplace_back([&v, a = cut[t], b = cut[t + 1]] { for (size_t i = a; i < b; i++) memcpy(v[i].dst, v[i].src, v[i].bytes); });
    for (auto &x : th) x.join();
}

static int max_neighbourhood(const sdmd_system &s) {
    int N = s.n_atoms, cn0 = s.cellnum[0], cn1 = s.cellnum[1], cn2 = s.cellnum[2];
    long ncell = (long)cn0 * cn1 * cn2;
    std::vector<int> occ(ncell + 1, 0);
    for (long c = 1; c <= ncell; c++) {
        int k = 0;
        for (int a = s.cell_list[N + c]; a && k <= N; a = s.cell_list[a]) k++;
        occ[c] = k;
    }
    int best = 0;
    for (int z = 0; z < cn2; z++)
        for (int y = 0; y < cn1; y++)
            for (int x = 0; x < cn0; x++) {
                int tot = 0;
                for (int dz = -1; dz <= 1; dz++)
                    for (int dy = -1; dy <= 1; dy++)
                        for (int dx = -1; dx <= 1; dx++) {
                            int a = (x + dx + cn0) % cn0, b = (y + dy + cn1) % cn1, c = (z + dz + cn2) % cn2;
                            tot += occ[(long)c * cn0 * cn1 + (long)b * cn0 + a + 1];
                        }
                if (tot > best) best = tot;
            }
    return best;
}

// ---- FP32 brackets for the screen ------------------------------------------------
// [lo, hi]: the nearest floats below and above the double v (equal when v is a float)
static void f32_bracket(double v, float *out) {
    float f = (float)v;
    out[0] = ((double)f > v) ? nextafterf(f, -INFINITY) : f;
    out[1] = ((double)f < v) ? nextafterf(f, INFINITY) : f;
}

struct Screen32 {
    std::vector<float> pair_thr, pair_step, con_thr, con_step, bond;
    std::vector<long long> pair_key, pair_stepkey, con_key, con_stepkey;
    std::vector<int32_t> conn_win;
    std::vector<int32_t> leaf0;   // CreateCBT's leaf of every atom (src/CBT.c:16-30)
    std::vector<int16_t> rp_idx;
    std::vector<int8_t> con_win, con_ok;
};

// The leaf each atom gets from CreateCBT: atoms are inserted in order 1..N and
// each insertion splits the leaf at position `count` into (old atom, new atom).
// The layout depends on N alone; atom 1 of a one-atom tree keeps leaf 0.
static void cbt_leaf_layout(int N, std::vector<int32_t> &leaf) {
    leaf.assign((size_t)N + 2, 0);
    std::vector<int32_t> node((size_t)2 * N + 2, 0);
    int count = 0;
    for (int a = 1; a <= N; a++) {
        if (count == 0) { node[1] = a; count = 1; continue; }
        int i = node[count];
        node[2 * count] = i; node[2 * count + 1] = a;
        leaf[i] = 2 * count; leaf[a] = 2 * count + 1;
        count++;
    }
}

// the device's tkey(): an order-preserving map of non-NaN doubles onto int64
static long long host_tkey(double d) {
    long long b;
    memcpy(&b, &d, 8);
    return b >= 0 ? b : -(b & 0x7fffffffffffffffLL);
}
constexpr int kConnWin = 9;   // ints per atom in conn_win
constexpr int kMaxPerCell = 64; // screened path: atoms per cell array
constexpr int kSweepBlocksPerSM = 8;   // parallel sweep: blocks in flight per SM

// brackets of every FP64 threshold the prediction compares against, computed with
// the same FP64 operations as the device (d + ZERO, d - ZERO, dmin - ZERO, dmax + ZERO)
static void build_screen32(const sdmd_system &s, Screen32 &o, bool with_pairs) {
    const size_t NT3 = (size_t)SDMD_NTABLES * SDMD_NTYPES * SDMD_NTYPES;
    auto entry = [](double dmin, double dmax, float *e) {
        f32_bracket(dmin - SDMD_ZERO, e + 0);
        f32_bracket(dmax + SDMD_ZERO, e + 2);
        f32_bracket(dmin, e + 4);
        f32_bracket(dmax, e + 6);
    };
    auto step = [](double d, float *e) {
        f32_bracket(d + SDMD_ZERO, e + 0);
        f32_bracket(d - SDMD_ZERO, e + 2);
        f32_bracket(d, e + 4);
    };
    if (with_pairs) {
        o.pair_thr.assign(NT3 * 8, 0.f);
        for (size_t k = 0; k < NT3; k++) entry(s.pair_dmin[k], s.pair_dmax[k], &o.pair_thr[8 * k]);
        o.pair_step.assign(((size_t)s.n_pair_steps + 1) * 6, 0.f);
        for (int k = 0; k < s.n_pair_steps; k++) step(s.pair_step_d[k], &o.pair_step[6 * (size_t)k]);
    }
    o.con_thr.assign(((size_t)s.n_cons + 1) * 8, 0.f);
    for (int k = 0; k < s.n_cons; k++) entry(s.con_dmin[k], s.con_dmax[k], &o.con_thr[8 * (size_t)k]);
    o.con_step.assign(((size_t)s.n_con_steps + 1) * 6, 0.f);
    for (int k = 0; k < s.n_con_steps; k++) step(s.con_step_d[k], &o.con_step[6 * (size_t)k]);
    o.bond.assign(((size_t)s.n_bonds + 1) * 4, 0.f);
    for (int k = 0; k < s.n_bonds; k++) {
        f32_bracket(s.bond_dmin[k], &o.bond[4 * (size_t)k]);
        f32_bracket(s.bond_dmax[k], &o.bond[4 * (size_t)k + 2]);
    }
    if (with_pairs) {
        o.pair_key.assign(NT3 * 2, 0);
        for (size_t k = 0; k < NT3; k++) {
            o.pair_key[2 * k] = host_tkey(s.pair_dmin[k] - SDMD_ZERO);
            o.pair_key[2 * k + 1] = host_tkey(s.pair_dmax[k] + SDMD_ZERO);
        }
        o.pair_stepkey.assign(((size_t)s.n_pair_steps + 1) * 2, 0);
        for (int k = 0; k < s.n_pair_steps; k++) {
            o.pair_stepkey[2 * (size_t)k] = host_tkey(s.pair_step_d[k] + SDMD_ZERO);
            o.pair_stepkey[2 * (size_t)k + 1] = host_tkey(s.pair_step_d[k] - SDMD_ZERO);
        }
    }
    o.con_key.assign(((size_t)s.n_cons + 1) * 2, 0);
    for (int k = 0; k < s.n_cons; k++) {
        o.con_key[2 * (size_t)k] = host_tkey(s.con_dmin[k] - SDMD_ZERO);
        o.con_key[2 * (size_t)k + 1] = host_tkey(s.con_dmax[k] + SDMD_ZERO);
    }
    o.con_stepkey.assign(((size_t)s.n_con_steps + 1) * 2, 0);
    for (int k = 0; k < s.n_con_steps; k++) {
        o.con_stepkey[2 * (size_t)k] = host_tkey(s.con_step_d[k] + SDMD_ZERO);
        o.con_stepkey[2 * (size_t)k + 1] = host_tkey(s.con_step_d[k] - SDMD_ZERO);
    }
    const int N = s.n_atoms;
    cbt_leaf_layout(N, o.leaf0);
    // RightPair: the first of (t1,t2), (t1',t2), (t1,t2'), (t1',t2') with dmin > 0, ' = AtomTypeChange(., 0)
    auto unhb = [](int t) { return t == 3 ? 1 : t == 4 ? 2 : t == 27 ? 26 : t; };
    auto idx0 = [](int a, int b) { return a * SDMD_NTYPES + b; };
    if (with_pairs) o.rp_idx.assign((size_t)SDMD_NTYPES * SDMD_NTYPES, -1);
    for (int t1 = 0; with_pairs && t1 < SDMD_NTYPES; t1++)
        for (int t2 = 0; t2 < SDMD_NTYPES; t2++) {
            const int a = unhb(t1), b = unhb(t2);
            const int cand[4] = {idx0(t1, t2), idx0(a, t2), idx0(t1, b), idx0(a, b)};
            for (int c : cand)
                if (s.pair_dmin[c] > 0) { o.rp_idx[(size_t)idx0(t1, t2)] = (int16_t)c; break; }
        }
    o.con_win.assign((size_t)(N + 1) * 128, -1);
    o.con_ok.assign((size_t)N + 1, 0);
    for (int i = 1; i <= N; i++) {
        int8_t *w = &o.con_win[(size_t)i * 128];
        bool ok = s.con_off[i + 1] - s.con_off[i] <= 127;
        for (int k = s.con_off[i]; ok && k < s.con_off[i + 1]; k++) {
            const int idx = s.con_j[k] - (i - 64);
            if (idx < 0 || idx >= 128) { ok = false; break; }
            if (w[idx] < 0) w[idx] = (int8_t)(k - s.con_off[i]);
        }
        o.con_ok[i] = ok ? 1 : 0;
    }
    o.conn_win.assign((size_t)(N + 1) * kConnWin, 0);
    for (int i = 1; i <= N; i++) {
        int32_t *w = &o.conn_win[(size_t)i * kConnWin];
        w[0] = i - 64;
        for (int k = s.conn_off[i]; k < s.conn_off[i + 1]; k++) {
            int idx = s.conn_j[k] - (i - 64), bits = s.conn_bits[k];
            if (idx < 0 || idx >= 128) { w[0] = -1; break; }
            if (bits & 1) w[1 + (idx >> 5)] |= (int32_t)(1u << (idx & 31));
            if (bits & 2) w[5 + (idx >> 5)] |= (int32_t)(1u << (idx & 31));
        }
        if (w[0] < 0) for (int q = 1; q < kConnWin; q++) w[q] = 0;
    }
}

// ---- arena carving --------------------------------------------------------------
struct Carver {
    unsigned char *base;
    size_t off;
    template <class T> T *take(size_t count) {
        off = (off + 255) & ~size_t(255);
        T *p = reinterpret_cast<T *>(base + off);
        off += count * sizeof(T);
        return p;
    }
};

template <class T> static void put(std::vector<std::pair<void *, std::pair<const void *, size_t>>> &cp, T *dst,
                                   const T *src, size_t count) {
    if (count && src) cp.push_back({(void *)dst, {(const void *)src, count * sizeof(T)}});
}

// The arena holds, in this order: every system's static arrays (topology, tables
// and the host-derived screen tables; identical pair tables are stored once and
// shared), every system's dynamic arrays (the state sdmd_gpu_create uploads and
// sdmd_gpu_download returns), then the per-system scalar blocks and the
// device-only scratch.  Upload and download are then one copy each.
static size_t layout(sdmd_gpu *h, const sdmd_system *sys, unsigned char *base,
                     std::vector<std::pair<void *, std::pair<const void *, size_t>>> *copies,
                     const std::vector<Screen32> *s32 = nullptr) {
    Carver cv{base, 0};
    const int trace_cap = h->opts.trace_capacity > 0 ? h->opts.trace_capacity : 0;
    const size_t NT3 = (size_t)SDMD_NTABLES * SDMD_NTYPES * SDMD_NTYPES;
    // ---- static arrays ----
    for (int k = 0; k < h->n_systems; k++) {
        const sdmd_system &s = sys[k];
        const SysMeta &m = h->meta[k];
        DSys &d = h->hs[k];
        const size_t N1 = (size_t)m.n + 1;
        d.mass = cv.take<double>(N1);
        d.protein = cv.take<int32_t>(N1); d.aanum = cv.take<int32_t>(N1); d.aatype = cv.take<int32_t>(N1);
        d.hb_neighbor = cv.take<int32_t>(N1); d.hb_role = cv.take<int32_t>(N1); d.name_code = cv.take<int32_t>(N1);
        d.bond_off = cv.take<int32_t>(N1 + 1); d.bond_j = cv.take<int32_t>(m.n_bonds + 1);
        d.bond_dmin = cv.take<double>(m.n_bonds + 1); d.bond_dmax = cv.take<double>(m.n_bonds + 1);
        d.con_off = cv.take<int32_t>(N1 + 1); d.con_j = cv.take<int32_t>(m.n_cons + 1);
        d.con_step_off = cv.take<int32_t>(m.n_cons + 1); d.con_step_n = cv.take<int32_t>(m.n_cons + 1);
        d.con_dmin = cv.take<double>(m.n_cons + 1); d.con_dmax = cv.take<double>(m.n_cons + 1);
        d.con_step_d = cv.take<double>(m.n_con_steps + 1); d.con_step_e = cv.take<double>(m.n_con_steps + 1);
        d.con_step_acc = cv.take<double>(m.n_con_steps + 1);
        d.conn_off = cv.take<int32_t>(N1 + 1); d.conn_j = cv.take<int32_t>(m.n_conn + 1);
        d.conn_bits = cv.take<int32_t>(m.n_conn + 1);
        const int src = h->pair_src[k];
        const bool own_pairs = src == k;
        if (own_pairs) {
            d.pair_dmin = cv.take<double>(NT3); d.pair_dmax = cv.take<double>(NT3);
            d.pair_step_off = cv.take<int32_t>(NT3); d.pair_step_n = cv.take<int32_t>(NT3);
            d.pair_step_d = cv.take<double>(m.n_pair_steps + 1); d.pair_step_e = cv.take<double>(m.n_pair_steps + 1);
            d.pair_step_acc = cv.take<double>(m.n_pair_steps + 1);
            d.pair_thr32 = cv.take<float>(NT3 * 8);
            d.pair_step32 = cv.take<float>(((size_t)m.n_pair_steps + 1) * 6);
            d.pair_key = cv.take<long long>(NT3 * 2);
            d.pair_stepkey = cv.take<long long>(((size_t)m.n_pair_steps + 1) * 2);
            d.rp_idx = cv.take<int16_t>((size_t)SDMD_NTYPES * SDMD_NTYPES);
        } else {   // the same tables as system src: share its device copies
            const DSys &o = h->hs[src];
            d.pair_dmin = o.pair_dmin; d.pair_dmax = o.pair_dmax;
            d.pair_step_off = o.pair_step_off; d.pair_step_n = o.pair_step_n;
            d.pair_step_d = o.pair_step_d; d.pair_step_e = o.pair_step_e; d.pair_step_acc = o.pair_step_acc;
            d.pair_thr32 = o.pair_thr32; d.pair_step32 = o.pair_step32;
            d.pair_key = o.pair_key; d.pair_stepkey = o.pair_stepkey; d.rp_idx = o.rp_idx;
        }
        d.sph = m.n_sph ? cv.take<double>(4 * (size_t)m.n_sph) : nullptr;
        d.obst = m.n_obst ? cv.take<double>(3 * (size_t)m.n_obst) : nullptr;
        d.con_thr32 = cv.take<float>(((size_t)m.n_cons + 1) * 8);
        d.con_step32 = cv.take<float>(((size_t)m.n_con_steps + 1) * 6);
        d.bond32 = cv.take<float>(((size_t)m.n_bonds + 1) * 4);
        d.con_key = cv.take<long long>(((size_t)m.n_cons + 1) * 2);
        d.con_stepkey = cv.take<long long>(((size_t)m.n_con_steps + 1) * 2);
        d.conn_win = cv.take<int32_t>(N1 * kConnWin);
        d.cbt_leaf0 = cv.take<int32_t>(N1 + 1);
        d.con_win = cv.take<int8_t>(N1 * 128);
        d.con_ok = cv.take<int8_t>(N1);
        if (copies && s32) {
            const Screen32 &q = (*s32)[k];
            if (own_pairs) {
                put(*copies, (float *)d.pair_thr32, q.pair_thr.data(), q.pair_thr.size());
                put(*copies, (float *)d.pair_step32, q.pair_step.data(), q.pair_step.size());
                put(*copies, (long long *)d.pair_key, q.pair_key.data(), q.pair_key.size());
                put(*copies, (long long *)d.pair_stepkey, q.pair_stepkey.data(), q.pair_stepkey.size());
                put(*copies, (int16_t *)d.rp_idx, q.rp_idx.data(), q.rp_idx.size());
            }
            put(*copies, (float *)d.con_thr32, q.con_thr.data(), q.con_thr.size());
            put(*copies, (float *)d.con_step32, q.con_step.data(), q.con_step.size());
            put(*copies, (float *)d.bond32, q.bond.data(), q.bond.size());
            put(*copies, (long long *)d.con_key, q.con_key.data(), q.con_key.size());
            put(*copies, (long long *)d.con_stepkey, q.con_stepkey.data(), q.con_stepkey.size());
            put(*copies, (int32_t *)d.conn_win, q.conn_win.data(), q.conn_win.size());
            put(*copies, (int32_t *)d.cbt_leaf0, q.leaf0.data(), q.leaf0.size());
            put(*copies, (int8_t *)d.con_win, q.con_win.data(), q.con_win.size());
            put(*copies, (int8_t *)d.con_ok, q.con_ok.data(), q.con_ok.size());
        }
        if (copies) {
            auto &c = *copies;
            put(c, (double *)d.mass, s.mass, N1);
            if (m.n_sph) put(c, (double *)d.sph, s.sphobst, 4 * (size_t)m.n_sph);
            if (m.n_obst) put(c, (double *)d.obst, s.obst, 3 * (size_t)m.n_obst);
            put(c, (int32_t *)d.protein, s.protein, N1); put(c, (int32_t *)d.aanum, s.aanum, N1);
            put(c, (int32_t *)d.aatype, s.aatype, N1); put(c, (int32_t *)d.hb_neighbor, s.hb_neighbor, N1);
            put(c, (int32_t *)d.hb_role, s.hb_role, N1); put(c, (int32_t *)d.name_code, s.name_code, N1);
            put(c, (int32_t *)d.bond_off, s.bond_off, N1 + 1); put(c, (int32_t *)d.bond_j, s.bond_j, (size_t)m.n_bonds);
            put(c, (double *)d.bond_dmin, s.bond_dmin, (size_t)m.n_bonds);
            put(c, (double *)d.bond_dmax, s.bond_dmax, (size_t)m.n_bonds);
            put(c, (int32_t *)d.con_off, s.con_off, N1 + 1); put(c, (int32_t *)d.con_j, s.con_j, (size_t)m.n_cons);
            put(c, (int32_t *)d.con_step_off, s.con_step_off, (size_t)m.n_cons);
            put(c, (int32_t *)d.con_step_n, s.con_step_n, (size_t)m.n_cons);
            put(c, (double *)d.con_dmin, s.con_dmin, (size_t)m.n_cons);
            put(c, (double *)d.con_dmax, s.con_dmax, (size_t)m.n_cons);
            put(c, (double *)d.con_step_d, s.con_step_d, (size_t)m.n_con_steps);
            put(c, (double *)d.con_step_e, s.con_step_e, (size_t)m.n_con_steps);
            put(c, (double *)d.con_step_acc, s.con_step_acc, (size_t)m.n_con_steps);
            put(c, (int32_t *)d.conn_off, s.conn_off, N1 + 1); put(c, (int32_t *)d.conn_j, s.conn_j, (size_t)m.n_conn);
            put(c, (int32_t *)d.conn_bits, s.conn_bits, (size_t)m.n_conn);
            if (own_pairs) {
                put(c, (double *)d.pair_dmin, s.pair_dmin, NT3); put(c, (double *)d.pair_dmax, s.pair_dmax, NT3);
                put(c, (int32_t *)d.pair_step_off, s.pair_step_off, NT3);
                put(c, (int32_t *)d.pair_step_n, s.pair_step_n, NT3);
                put(c, (double *)d.pair_step_d, s.pair_step_d, (size_t)m.n_pair_steps);
                put(c, (double *)d.pair_step_e, s.pair_step_e, (size_t)m.n_pair_steps);
                put(c, (double *)d.pair_step_acc, s.pair_step_acc, (size_t)m.n_pair_steps);
            }
        }
    }
    // ---- dynamic arrays: one contiguous block for all systems ----
    cv.off = (cv.off + 255) & ~size_t(255);
    h->dyn_begin = cv.off;
    for (int k = 0; k < h->n_systems; k++) {
        const SysMeta &m = h->meta[k];
        DSys &d = h->hs[k];
        const size_t N1 = (size_t)m.n + 1;
        d.x = cv.take<double>(N1); d.y = cv.take<double>(N1); d.z = cv.take<double>(N1);
        d.vx = cv.take<double>(N1); d.vy = cv.take<double>(N1); d.vz = cv.take<double>(N1);
        d.cx = cv.take<int32_t>(N1); d.cy = cv.take<int32_t>(N1); d.cz = cv.take<int32_t>(N1);
        d.type = cv.take<int32_t>(N1); d.hb_bond = cv.take<int32_t>(N1); d.hb_itype = cv.take<int32_t>(N1);
        d.nb_partner = cv.take<int32_t>(4 * N1); d.nb_status = cv.take<int32_t>(N1); d.nb_pnum = cv.take<int32_t>(N1);
        d.ev_time = cv.take<double>(N1); d.ev_partner = cv.take<int32_t>(N1);
        d.ev_counter = cv.take<int64_t>(N1); d.ev_pcounter = cv.take<int64_t>(N1);
        d.ev_potential = cv.take<double>(N1); d.ev_type = cv.take<int32_t>(N1); d.ev_sub = cv.take<int32_t>(N1);
        d.cell_list = cv.take<int32_t>(N1 + m.ncell);
    }
    h->dyn_end = cv.off;
    // ---- scalar blocks of all systems (one copy each way), then device-only scratch ----
    DScal *scs = cv.take<DScal>((size_t)h->n_systems);
    h->sc_all = scs;
    for (int k = 0; k < h->n_systems; k++) h->hs[k].sc = scs + k;
    for (int k = 0; k < h->n_systems; k++) {
        const sdmd_system &s = sys[k];
        const SysMeta &m = h->meta[k];
        DSys &d = h->hs[k];
        const size_t N1 = (size_t)m.n + 1;
        d.cbt_node = cv.take<int32_t>(2 * N1 + 2); d.cbt_leaf = cv.take<int32_t>(N1 + 1);
        d.trace = cv.take<sdmd_trace_rec>(trace_cap > 0 ? trace_cap : 1);
        d.trace_cap = trace_cap;
        d.smp_cap = s.thermostat ? h->smp_cap_of[k] : 0;
        size_t sc_ = d.smp_cap > 0 ? (size_t)d.smp_cap : 1;
        d.smp = cv.take<double>(sc_);
        d.smp_raw = cv.take<int32_t>(3 * sc_);
        d.smp_cum = cv.take<int64_t>(sc_);
        d.tloc = cv.take<double>(N1);
        d.lazy = h->opts.advance == SDMD_ADVANCE_LAZY ? 1 : 0;
        if (h->opts.screen == SDMD_SCREEN_FP32) {
            d.sw_hbit = cv.take<int32_t>(N1);
            d.sw_flag = cv.take<int32_t>(N1);
            d.sw_warn = cv.take<int32_t>(N1);
            // the records pack a cell index in 10 bits per axis
            d.shr = s.cellnum[0] <= 1024 && s.cellnum[1] <= 1024 && s.cellnum[2] <= 1024 ? cv.take<float4>(N1 * 4)
                                                                                        : nullptr;
            d.maxc = std::min<int32_t>(kMaxPerCell, m.n);
            d.cell_cnt = cv.take<int32_t>((size_t)m.ncell + 1);
            d.cell_arr = cv.take<int32_t>(((size_t)m.ncell + 1) * d.maxc);
        }
    }
    // the helper protocol words of every system, contiguous (cleared before each launch)
    h->adv = cv.take<Adv>((size_t)h->n_systems);
    for (int k = 0; k < h->n_systems; k++) h->hs[k].adv = h->adv + k;
    return cv.off;
}

// dynamic arrays of system k: (device pointer, host pointer, bytes) triples
template <class F> static void for_dynamic(sdmd_gpu *h, int k, const sdmd_system &s, F f) {
    const DSys &d = h->hs[k];
    size_t N1 = (size_t)h->meta[k].n + 1;
    f((void *)d.x, (void *)s.x, N1 * 8); f((void *)d.y, (void *)s.y, N1 * 8); f((void *)d.z, (void *)s.z, N1 * 8);
    f((void *)d.vx, (void *)s.vx, N1 * 8); f((void *)d.vy, (void *)s.vy, N1 * 8); f((void *)d.vz, (void *)s.vz, N1 * 8);
    f((void *)d.cx, (void *)s.cx, N1 * 4); f((void *)d.cy, (void *)s.cy, N1 * 4); f((void *)d.cz, (void *)s.cz, N1 * 4);
    f((void *)d.type, (void *)s.type, N1 * 4); f((void *)d.hb_bond, (void *)s.hb_bond, N1 * 4);
    f((void *)d.hb_itype, (void *)s.hb_itype, N1 * 4); f((void *)d.nb_partner, (void *)s.nb_partner, 4 * N1 * 4);
    f((void *)d.nb_status, (void *)s.nb_status, N1 * 4); f((void *)d.nb_pnum, (void *)s.nb_pnum, N1 * 4);
    f((void *)d.ev_time, (void *)s.ev_time, N1 * 8); f((void *)d.ev_partner, (void *)s.ev_partner, N1 * 4);
    f((void *)d.ev_counter, (void *)s.ev_counter, N1 * 8); f((void *)d.ev_pcounter, (void *)s.ev_pcounter, N1 * 8);
    f((void *)d.ev_potential, (void *)s.ev_potential, N1 * 8); f((void *)d.ev_type, (void *)s.ev_type, N1 * 4);
    f((void *)d.ev_sub, (void *)s.ev_sub, N1 * 4);
    f((void *)d.cell_list, (void *)s.cell_list, (N1 + h->meta[k].ncell) * 4);
}

extern "C" void sdmd_gpu_destroy(sdmd_gpu *h) {
    if (!h) return;
    if (h->stream) cudaStreamSynchronize(h->stream);
    if (h->arena) cudaFree(h->arena);
    if (h->aux) cudaFree(h->aux);
    if (h->ds) cudaFree(h->ds);
    if (h->e0) cudaEventDestroy(h->e0);
    if (h->e1) cudaEventDestroy(h->e1);
    if (h->l0) cudaEventDestroy(h->l0);
    if (h->l1) cudaEventDestroy(h->l1);
    if (h->stream) cudaStreamDestroy(h->stream);
    delete h;
}

extern "C" int sdmd_gpu_create(const sdmd_system *systems, int32_t n_systems, const sdmd_opts *opts, sdmd_gpu **out) {
    if (!systems || n_systems <= 0 || !out) return SDMD_EINVAL;
    *out = nullptr;
    {
        std::vector<int> bad(n_systems);
        parallel_for(n_systems, [&](int k) { bad[k] = validate(systems[k]); });
        for (int k = 0; k < n_systems; k++)
            if (bad[k]) return bad[k];
    }
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return SDMD_ENODEV;
    sdmd_gpu *h = new sdmd_gpu();
    if (opts) h->opts = *opts;
    if (h->opts.device < 0 || h->opts.device >= ndev) { delete h; return SDMD_EINVAL; }
    if ((h->opts.advance != SDMD_ADVANCE_EAGER && h->opts.advance != SDMD_ADVANCE_LAZY) ||
        (h->opts.screen != SDMD_SCREEN_FP64 && h->opts.screen != SDMD_SCREEN_FP32)) {
        delete h;
        return SDMD_EUNSUPPORTED;
    }
    int r = cuda_fail(cudaSetDevice(h->opts.device));
    if (r) { delete h; return r; }
    h->n_systems = n_systems;
    h->hs.resize(n_systems);
    h->meta.resize(n_systems);
    int nbcap_max = 0;
    h->smp_cap_of.resize(n_systems);
    // Neighbour capacity of a system: 4x its fullest 27-cell neighbourhood at upload
    // (room for density fluctuations during a run), less for dense systems whose
    // buffers would not fit one CTA's shared memory: 3x, 2x, then 1.5x.  A gather
    // that overflows at run time stops the run with SDMD_ECAPACITY.
    const bool scr0 = h->opts.screen == SDMD_SCREEN_FP32;
    std::vector<int> occ_of(n_systems);
    parallel_for(n_systems, [&](int k) { occ_of[k] = max_neighbourhood(systems[k]); });
    auto cap_of = [&](int k, int num, int den) {
        const sdmd_system &s = systems[k];
        return s.n_atoms <= 2048 ? s.n_atoms : std::min(s.n_atoms, std::max(512, num * occ_of[k] / den + 64));
    };
    int head_num = 4, head_den = 1;
    static const int heads[4][2] = {{4, 1}, {3, 1}, {2, 1}, {3, 2}};
    for (const auto &f : heads) {
        head_num = f[0]; head_den = f[1];
        int mx = 0;
        for (int k = 0; k < n_systems; k++) mx = std::max(mx, cap_of(k, head_num, head_den));
        if ((scr0 ? screen_smem_bytes(mx) : fp64_smem_bytes(mx)) <= 227 * 1024) break;
    }
    for (int k = 0; k < n_systems; k++) {
        long per = (1L << 23) / n_systems;
        per = per < 4096 ? 4096 : per > 65536 ? 65536 : per;
        h->smp_cap_of[k] = (int32_t)std::max<long>(per, (long)systems[k].n_atoms + 64);
        const sdmd_system &s = systems[k];
        SysMeta &m = h->meta[k];
        m.n = s.n_atoms;
        m.ncell = s.cellnum[0] * s.cellnum[1] * s.cellnum[2];
        m.n_bonds = s.n_bonds; m.n_cons = s.n_cons; m.n_con_steps = s.n_con_steps; m.n_conn = s.n_conn;
        m.n_pair_steps = s.n_pair_steps;
        m.n_sph = s.n_sphobst;
        m.n_obst = s.n_obst;
        m.nbcap = cap_of(k, head_num, head_den);
        nbcap_max = std::max(nbcap_max, m.nbcap);
        DSys &d = h->hs[k];
        memset(&d, 0, sizeof(d));
        d.n = s.n_atoms; d.ncell = m.ncell;
        for (int q = 0; q < 3; q++) {
            d.cn[q] = s.cellnum[q]; d.box[q] = s.box[q]; d.cs[q] = s.cellsize[q];
            d.wall_pos[q] = s.wall_pos[q]; d.wall_vel[q] = s.wall_vel[q]; d.hb_barrier[q] = s.hb_barrier[q];
        }
        d.thermostat = s.thermostat; d.wall = s.wall; d.wall_type = s.wall_type;
        d.n_sph = s.n_sphobst;
        d.n_obst = s.n_obst;
        d.cutoff = s.cutoff; d.temperature = s.temperature; d.thermo_freq = s.thermo_freq; d.t_end = s.t_end;
        d.nbcap = m.nbcap;
        d.n_bonds = s.n_bonds; d.n_cons = s.n_cons; d.n_con_steps = s.n_con_steps; d.n_conn = s.n_conn;
        d.screen = h->opts.screen;
        d.dup_limit = 0x7fffffff;
        double cut = s.cutoff * 0.90;   // the prediction's scan radius, as the device computes it
        cut *= cut;
        f32_bracket(cut, d.cut32);
        d.cut_key = host_tkey(cut);
        f32_bracket(SDMD_ZERO, d.zero32);
        for (int q = 0; q < 3; q++) f32_bracket(s.box[q], d.box32 + 2 * q);
        {   // |x| bound for the eager records' rounding margin: 4 times the largest box edge
            float b[2];
            f32_bracket(4.0 * std::max(s.box[0], std::max(s.box[1], s.box[2])), b);
            d.xmax32 = b[1];
        }
    }
    const bool scr = h->opts.screen == SDMD_SCREEN_FP32;
    h->smem = scr ? screen_smem_bytes(nbcap_max) : fp64_smem_bytes(nbcap_max);
    h->sweep_k = scr ? sweep_kernel_screen : sweep_kernel_fp64;
    h->vsmem = verify_smem_bytes(nbcap_max, 4);
    h->loop_k = scr ? loop_kernel_screen : loop_kernel_fp64;
    // stage whole systems in shared memory when they fit (small systems, batches)
    size_t st_max = 0;
    for (int k = 0; k < n_systems; k++) {
        const sdmd_system &s = systems[k];
        st_max = std::max(st_max, staged_state_bytes(s.n_atoms, h->meta[k].ncell, s.n_bonds, s.n_cons,
                                                     s.n_con_steps, s.n_conn));
    }
    h->staged = (h->smem + st_max <= 192 * 1024) ? 1 : 0;
    // helper blocks read and write the state in global memory: asking for them
    // explicitly keeps the systems unstaged
    if (scr && h->opts.advance == SDMD_ADVANCE_EAGER && h->opts.helper_blocks > 0) h->staged = 0;
    h->smem_loop = h->staged ? h->smem + st_max : h->smem;
    h->threads = h->opts.threads_per_system > 0 ? h->opts.threads_per_system : 128;
    if (h->threads < 32 || h->threads > 1024 || (h->threads & 31)) { delete h; return SDMD_EINVAL; }
    if (h->threads > 512) { delete h; return SDMD_EUNSUPPORTED; }
    h->sweep_threads = std::min(h->threads, 256);
    if (h->smem > 227 * 1024) { delete h; return SDMD_ECAPACITY; }
    // systems whose pair tables are identical (the same force field) share one device copy
    h->pair_src.assign(n_systems, 0);
    {
        std::vector<int> distinct;
        auto same = [](const sdmd_system &a, const sdmd_system &b) {
            const size_t NT3 = (size_t)SDMD_NTABLES * SDMD_NTYPES * SDMD_NTYPES, ns = (size_t)a.n_pair_steps;
            if (a.n_pair_steps != b.n_pair_steps) return false;
            auto eq = [](const void *x, const void *y, size_t bytes) { return x == y || !memcmp(x, y, bytes); };
            return eq(a.pair_dmin, b.pair_dmin, NT3 * 8) && eq(a.pair_dmax, b.pair_dmax, NT3 * 8) &&
                   eq(a.pair_step_off, b.pair_step_off, NT3 * 4) && eq(a.pair_step_n, b.pair_step_n, NT3 * 4) &&
                   eq(a.pair_step_d, b.pair_step_d, ns * 8) && eq(a.pair_step_e, b.pair_step_e, ns * 8) &&
                   eq(a.pair_step_acc, b.pair_step_acc, ns * 8);
        };
        // the comparison with system 0 (the common case: one force field) on all
        // host threads, the rest in order
        std::vector<char> like0(n_systems, 0);
        parallel_for(n_systems - 1, [&](int k) { like0[k + 1] = same(systems[0], systems[k + 1]); });
        for (int k = 0; k < n_systems; k++) {
            h->pair_src[k] = k;
            if (like0[k]) { h->pair_src[k] = 0; continue; }
            for (int j : distinct)
                if (same(systems[j], systems[k])) { h->pair_src[k] = j; break; }
            if (h->pair_src[k] == k && distinct.size() < 16) distinct.push_back(k);
        }
    }
    h->arena_bytes = layout(h, systems, nullptr, nullptr) + 256;
    if ((r = cuda_fail(cudaDeviceGetAttribute(&h->sms, cudaDevAttrMultiProcessorCount, h->opts.device))) ||
        (r = cuda_fail(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking))) ||
        (r = cuda_fail(cudaEventCreate(&h->e0))) || (r = cuda_fail(cudaEventCreate(&h->e1))) ||
        (r = cuda_fail(cudaEventCreate(&h->l0))) || (r = cuda_fail(cudaEventCreate(&h->l1))) ||
        (r = cuda_fail(cudaMalloc(&h->arena, h->arena_bytes))) ||
        (r = cuda_fail(cudaMalloc(&h->aux, 256 * 10 + (size_t)n_systems * 56))) ||
        (r = cuda_fail(cudaMalloc(&h->ds, sizeof(DSys) * n_systems)))) {
        sdmd_gpu_destroy(h);
        return r;
    }
    cudaMemsetAsync(h->arena, 0, h->arena_bytes, h->stream);
    {
        Carver ax{h->aux, 0};
        h->x_num = ax.take<int32_t>(n_systems); h->x_T = ax.take<double>(n_systems);
        h->x_E = ax.take<double>(n_systems); h->x_kin = ax.take<double>(n_systems);
        h->x_warn = ax.take<int64_t>(n_systems); h->x_stop = ax.take<double>(n_systems);
        h->x_lim = ax.take<int64_t>(n_systems);
        h->x_rng = ax.take<sdmd_rng>(1); h->x_stats = ax.take<int64_t>(2);
    }
    h->esmem = energy_smem_bytes(nbcap_max);
    std::vector<std::pair<void *, std::pair<const void *, size_t>>> copies;
    std::vector<Screen32> s32(n_systems);
    parallel_for(n_systems, [&](int k) { build_screen32(systems[k], s32[k], h->pair_src[k] == k); });
    layout(h, systems, h->arena, &copies, &s32);
    // one staging image of the static and dynamic blocks, one copy to the device;
    // the bytes no piece covers (alignment gaps) are zero, as the arena's memset left them
    std::vector<Piece> pieces;
    pieces.reserve(copies.size() + 64 * (size_t)n_systems);
    for (auto &c : copies) pieces.push_back({(void *)((unsigned char *)c.first - h->arena), c.second.first, c.second.second});
    std::vector<DScal> sc(n_systems);
    for (int k = 0; k < n_systems; k++) {
        const sdmd_system &s = systems[k];
        for_dynamic(h, k, s, [&](void *dv, void *hp, size_t bytes) {
            pieces.push_back({(void *)((unsigned char *)dv - h->arena), hp, bytes});
        });
        memset(&sc[k], 0, sizeof(DScal));
        sc[k].time = s.time; sc[k].rng = s.rng; sc[k].c = s.counters;
    }
    std::sort(pieces.begin(), pieces.end(), [](const Piece &a, const Piece &b) { return a.dst < b.dst; });
    std::unique_lock<std::mutex> up_lock(g_up.mu);
    std::vector<unsigned char> pageable;
    unsigned char *stage = g_up.get(h->dyn_end);
    if (!stage) { pageable.resize(h->dyn_end); stage = pageable.data(); }   // pinned memory unavailable
    {
        size_t at = 0;   // zero the gaps, then fill the pieces
        for (auto &c : pieces) {
            const size_t off = (size_t)c.dst;
            if (off > at) memset(stage + at, 0, off - at);
            at = std::max(at, off + c.bytes);
            c.dst = stage + off;
        }
        if (h->dyn_end > at) memset(stage + at, 0, h->dyn_end - at);
    }
    copy_pieces(pieces);
    cudaMemcpyAsync(h->arena, stage, h->dyn_end, cudaMemcpyHostToDevice, h->stream);
    if ((r = cuda_fail(cudaStreamSynchronize(h->stream)))) { up_lock.unlock(); sdmd_gpu_destroy(h); return r; }
    up_lock.unlock();
    cudaMemcpyAsync(h->sc_all, sc.data(), sizeof(DScal) * n_systems, cudaMemcpyHostToDevice, h->stream);
    cudaMemcpyAsync(h->ds, h->hs.data(), sizeof(DSys) * n_systems, cudaMemcpyHostToDevice, h->stream);
    // the dynamic shared-memory limit must cover dynamic + static usage: always set it
    if ((r = cuda_fail(cudaFuncSetAttribute(h->sweep_k, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                            (int)h->smem))) ||
        (r = cuda_fail(cudaFuncSetAttribute(h->loop_k, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                            (int)h->smem_loop))) ||
        (scr && ((r = cuda_fail(cudaFuncSetAttribute(sweep_predict_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                     (int)h->smem))) ||
                 (r = cuda_fail(cudaFuncSetAttribute(sweep_fix_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                     (int)h->smem))) ||
                 (r = cuda_fail(cudaFuncSetAttribute(sweep_verify_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                     (int)h->vsmem)))))) {
        sdmd_gpu_destroy(h);
        return r;
    }
    // A batch with more systems than the full build keeps resident at once runs in
    // waves; the 128-register build fits more CTAs per SM when registers are the
    // limit (the occupancy calculator decides, for this launch shape).
    if (scr && n_systems > 1 && h->threads <= 256) {
        int sms = 0, full = 0, capped = 0;
        if ((r = cuda_fail(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, h->opts.device))) ||
            (r = cuda_fail(cudaFuncSetAttribute(loop_kernel_screen_r128, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                (int)h->smem_loop))) ||
            (r = cuda_fail(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&full, loop_kernel_screen, h->threads,
                                                                         h->smem_loop))) ||
            (r = cuda_fail(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&capped, loop_kernel_screen_r128, h->threads,
                                                                         h->smem_loop)))) {
            sdmd_gpu_destroy(h);
            return r;
        }
        if ((long)full * sms < n_systems && capped > full) h->loop_k = loop_kernel_screen_r128;
    }
    // Eager advance on the screened path: for a few large systems, helper blocks on
    // the SMs the systems leave free advance every atom the pop does not involve
    // (one cooperative launch; the blocks must all be resident at once).
    if (scr && h->opts.advance == SDMD_ADVANCE_EAGER && !h->staged && h->opts.helper_blocks >= 0) {
        int32_t nmax = 0;
        for (auto &m : h->meta) nmax = std::max(nmax, m.n);
        int coop = 0, per_sm = 0;
        // blocks of more than 256 threads: the 128-register build of the same launch
        h->coop_k = h->threads > 256 ? (const void *)loop_kernel_screen_coop512 : (const void *)loop_kernel_screen_coop;
        if ((r = cuda_fail(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, h->opts.device))) ||
            (r = cuda_fail(cudaFuncSetAttribute(h->coop_k, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                (int)h->smem_loop))) ||
            (r = cuda_fail(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, h->coop_k, h->threads,
                                                                         h->smem_loop)))) {
            sdmd_gpu_destroy(h);
            return r;
        }
        const int room = per_sm * h->sms - n_systems;
        int want = h->opts.helper_blocks;
        if (want == 0) want = (n_systems * 2 <= h->sms && nmax >= 2048) ? room : 0;
        if (coop && want > 0 && room > 0) h->helpers = std::min(want, room);
    }
    // blocks of more than 256 threads exist only as the cooperative loop with helpers
    if (h->threads > 256 && h->helpers == 0) { sdmd_gpu_destroy(h); return SDMD_EUNSUPPORTED; }
    if (h->opts.advance == SDMD_ADVANCE_LAZY) lazy_enter_kernel<<<n_systems, 128, 0, h->stream>>>(h->ds);
    if ((r = cuda_fail(cudaStreamSynchronize(h->stream)))) { sdmd_gpu_destroy(h); return r; }
    *out = h;
    return SDMD_OK;
}

// copy every system's scalar block back and report the first device error
static int collect_errors(sdmd_gpu *h) {
    std::vector<DScal> sc(h->n_systems);
    CK(cudaMemcpyAsync(sc.data(), h->sc_all, sizeof(DScal) * h->n_systems, cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    for (int k = 0; k < h->n_systems; k++) {
        if (sc[k].err) {
            h->err.code = sc[k].err; h->err.system = k; h->err.atom = sc[k].err_atom; h->err.event = sc[k].err_event;
            return sc[k].err;
        }
    }
    return SDMD_OK;
}

static int n_blocks(int n, int t) { return (n + t - 1) / t; }

// draw a fresh batch of normal samples for every system that still runs
static void launch_samples(sdmd_gpu *h, int64_t want) {
    samples_walk_kernel<<<n_blocks(h->n_systems, 64), 64, 0, h->stream>>>(h->ds, h->n_systems, want);
    int64_t cap = 0;
    for (auto &m : h->hs) cap = std::max<int64_t>(cap, m.smp_cap);
    if (cap > 0) {
        int64_t w = std::min<int64_t>(want, cap);
        dim3 grid((unsigned)std::max<int64_t>(1, std::min<int64_t>((w + 255) / 256, 1024)), (unsigned)h->n_systems);
        samples_values_kernel<<<grid, 256, 0, h->stream>>>(h->ds, w);
    }
}

extern "C" int sdmd_gpu_prepare(sdmd_gpu *h, int32_t full_predict) {
    if (!h) return SDMD_EINVAL;
    CK(cudaSetDevice(h->opts.device));
    int32_t nmax = 0;
    for (auto &m : h->meta) nmax = std::max(nmax, m.n);
    CK(cudaEventRecord(h->e0, h->stream));
    if (full_predict) launch_samples(h, (int64_t)nmax + 8);
    if (h->opts.screen == SDMD_SCREEN_FP32) {
        // parallel sweep: reset + cell arrays, every atom at once, duplicate check,
        // in-order fix-up and the event tree
        const unsigned ns = (unsigned)h->n_systems;
        if (full_predict) {
            const int per_sys = std::max(1, kSweepBlocksPerSM * h->sms / h->n_systems);
            const unsigned rx = (unsigned)std::max(1, std::min(per_sys, (nmax + 255) / 256));
            const unsigned px = (unsigned)std::max(1, std::min(per_sys, nmax));
            const unsigned vx = (unsigned)std::max(1, std::min(per_sys, (nmax + 3) / 4));
            sweep_reset_kernel<<<dim3(rx, ns), 256, 0, h->stream>>>(h->ds);
            // latency-bound single-atom predictions: small blocks keep 4 of them per SM
            sweep_predict_kernel<<<dim3(px, ns), 64, h->smem, h->stream>>>(h->ds);
            sweep_verify_kernel<<<dim3(vx, ns), 128, h->vsmem, h->stream>>>(h->ds);
        }
        sweep_fix_kernel<<<ns, h->sweep_threads, h->smem, h->stream>>>(h->ds, full_predict ? 1 : 0);
    } else {
        h->sweep_k<<<h->n_systems, h->sweep_threads, h->smem, h->stream>>>(h->ds, full_predict ? 1 : 0);
    }
    if (full_predict) samples_commit_kernel<<<n_blocks(h->n_systems, 64), 64, 0, h->stream>>>(h->ds, h->n_systems);
    CK(cudaGetLastError());
    CK(cudaEventRecord(h->e1, h->stream));
    CK(cudaEventSynchronize(h->e1));
    float ms = 0;
    cudaEventElapsedTime(&ms, h->e0, h->e1);
    h->prep_ms = ms;
    return collect_errors(h);
}

static int run_rounds(sdmd_gpu *h, int64_t want, double t_end);

extern "C" int sdmd_gpu_run_to_dump(sdmd_gpu *h, double dump_time, int64_t max_events, double t_end,
                                    int32_t *at_dump) {
    if (!h || max_events < 0 || !(dump_time > 0)) return SDMD_EINVAL;
    if (at_dump)
        for (int k = 0; k < h->n_systems; k++) at_dump[k] = 0;
    if (max_events == 0) return SDMD_OK;
    CK(cudaSetDevice(h->opts.device));
    CK(cudaEventRecord(h->e0, h->stream));
    // every system stops after its first executed event at a time >= dump_time (the
    // loop's stop point of the replica exchange), or at the event limit
    const int n = h->n_systems;
    std::vector<double> stop(n, dump_time);
    CK(cudaMemcpyAsync(h->x_stop, stop.data(), sizeof(double) * n, cudaMemcpyHostToDevice, h->stream));
    remd_round_kernel<<<n_blocks(n, 64), 64, 0, h->stream>>>(h->ds, n, max_events, h->x_stop);
    h->launches = 1; h->loop_launches = 0; h->loop_ms = 0;
    int r = run_rounds(h, std::min<int64_t>(4 * max_events + 64, 1 << 16), t_end);
    if (r) return r;
    std::vector<DScal> sc(n);
    CK(cudaMemcpyAsync(sc.data(), h->sc_all, sizeof(DScal) * n, cudaMemcpyDeviceToHost, h->stream));
    // the stop point off again for later runs
    remd_round_kernel<<<n_blocks(n, 64), 64, 0, h->stream>>>(h->ds, n, 0, nullptr);
    CK(cudaGetLastError());
    CK(cudaEventRecord(h->e1, h->stream));
    CK(cudaEventSynchronize(h->e1));
    float ms = 0;
    cudaEventElapsedTime(&ms, h->e0, h->e1);
    h->run_ms = ms;
    if (at_dump)
        for (int k = 0; k < n; k++) at_dump[k] = sc[k].at_stop ? 1 : 0;
    return collect_errors(h);
}

extern "C" int sdmd_gpu_run_to_stops(sdmd_gpu *h, const double *stop_time, const int64_t *max_events, double t_end,
                                     int32_t *at_stop) {
    if (!h || !stop_time || !max_events) return SDMD_EINVAL;
    const int n = h->n_systems;
    int64_t most = 0;
    for (int k = 0; k < n; k++) {
        if (max_events[k] < 0 || !(stop_time[k] == stop_time[k])) return SDMD_EINVAL;
        most = std::max(most, max_events[k]);
    }
    if (at_stop)
        for (int k = 0; k < n; k++) at_stop[k] = 0;
    if (most == 0) {   // nothing runs
        h->launches = 0; h->loop_launches = 0; h->loop_ms = 0; h->run_ms = 0;
        return SDMD_OK;
    }
    CK(cudaSetDevice(h->opts.device));
    CK(cudaEventRecord(h->e0, h->stream));
    CK(cudaMemcpyAsync(h->x_stop, stop_time, sizeof(double) * n, cudaMemcpyHostToDevice, h->stream));
    CK(cudaMemcpyAsync(h->x_lim, max_events, sizeof(int64_t) * n, cudaMemcpyHostToDevice, h->stream));
    stops_round_kernel<<<n_blocks(n, 64), 64, 0, h->stream>>>(h->ds, n, h->x_lim, h->x_stop);
    h->launches = 1; h->loop_launches = 0; h->loop_ms = 0;
    int r = run_rounds(h, std::min<int64_t>(4 * most + 64, 1 << 16), t_end);
    if (r) return r;
    std::vector<DScal> sc(n);
    CK(cudaMemcpyAsync(sc.data(), h->sc_all, sizeof(DScal) * n, cudaMemcpyDeviceToHost, h->stream));
    remd_round_kernel<<<n_blocks(n, 64), 64, 0, h->stream>>>(h->ds, n, 0, nullptr);   // the stop points off again
    CK(cudaGetLastError());
    CK(cudaEventRecord(h->e1, h->stream));
    CK(cudaEventSynchronize(h->e1));
    float ms = 0;
    cudaEventElapsedTime(&ms, h->e0, h->e1);
    h->run_ms = ms;
    if (at_stop)
        for (int k = 0; k < n; k++)
            at_stop[k] = max_events[k] > 0 && (sc[k].at_stop || sc[k].c.frame >= sc[k].target_frame) ? 1 : 0;
    return collect_errors(h);
}

extern "C" int sdmd_gpu_exchange(sdmd_gpu *h, sdmd_remd *x) {
    if (!h || !x || !x->num || !x->T) return SDMD_EINVAL;
    CK(cudaSetDevice(h->opts.device));
    const int n = h->n_systems;
    int64_t stats[2] = {x->attempted, x->accepted};
    CK(cudaMemcpyAsync(h->x_num, x->num, sizeof(int32_t) * n, cudaMemcpyHostToDevice, h->stream));
    CK(cudaMemcpyAsync(h->x_T, x->T, sizeof(double) * n, cudaMemcpyHostToDevice, h->stream));
    CK(cudaMemcpyAsync(h->x_rng, &x->rng, sizeof(sdmd_rng), cudaMemcpyHostToDevice, h->stream));
    CK(cudaMemcpyAsync(h->x_stats, stats, sizeof(stats), cudaMemcpyHostToDevice, h->stream));
    energy_kernel<<<n, 32, h->esmem, h->stream>>>(h->ds, h->x_E, h->x_kin, h->x_warn);
    remd_exchange_kernel<<<1, 1, 0, h->stream>>>(h->ds, n, h->x_num, h->x_T, h->x_E, h->x_warn, h->x_rng, h->x_stats);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(x->num, h->x_num, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, h->stream));
    CK(cudaMemcpyAsync(x->T, h->x_T, sizeof(double) * n, cudaMemcpyDeviceToHost, h->stream));
    if (x->E) CK(cudaMemcpyAsync(x->E, h->x_E, sizeof(double) * n, cudaMemcpyDeviceToHost, h->stream));
    CK(cudaMemcpyAsync(&x->rng, h->x_rng, sizeof(sdmd_rng), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaMemcpyAsync(stats, h->x_stats, sizeof(stats), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    x->attempted = stats[0];
    x->accepted = stats[1];
    x->exchanges_done = 1;
    return collect_errors(h);
}

extern "C" int sdmd_gpu_run(sdmd_gpu *h, int64_t max_events, double t_end) {
    if (!h || max_events < 0) return SDMD_EINVAL;
    CK(cudaSetDevice(h->opts.device));
    CK(cudaEventRecord(h->e0, h->stream));
    begin_run_kernel<<<n_blocks(h->n_systems, 64), 64, 0, h->stream>>>(h->ds, h->n_systems, max_events);
    // each round: a sample batch, the loop until it runs low, then the rand() state
    // is moved past the consumed draws; systems without a thermostat need one round
    h->launches = 1; h->loop_launches = 0; h->loop_ms = 0;
    int r = run_rounds(h, std::min<int64_t>(4 * max_events + 64, 1 << 16), t_end);
    if (r) return r;
    CK(cudaEventRecord(h->e1, h->stream));
    CK(cudaEventSynchronize(h->e1));
    float ms = 0;
    cudaEventElapsedTime(&ms, h->e0, h->e1);
    h->run_ms = ms;
    return collect_errors(h);
}

// sample batch, event loop, RNG commit -- repeated while any system paused because
// its batch of thermostat samples ran low
static int run_rounds(sdmd_gpu *h, int64_t want, double t_end) {
    std::vector<DScal> sc(h->n_systems);
    for (int round = 0; round < 1 << 20; round++) {
        launch_samples(h, want);
        CK(cudaEventRecord(h->l0, h->stream));
        if (h->helpers > 0) {   // the systems' blocks and their helper blocks, all resident at once
            CK(cudaMemsetAsync(h->adv, 0, sizeof(Adv) * (size_t)h->n_systems, h->stream));
            const DSys *ds = h->ds;
            double te = t_end;
            int nc = h->n_systems;
            void *args[] = {(void *)&ds, (void *)&te, (void *)&nc};
            CK(cudaLaunchCooperativeKernel(h->coop_k, dim3(nc + h->helpers),
                                           dim3(h->threads), args, h->smem_loop, h->stream));
        } else {
            h->loop_k<<<h->n_systems, h->threads, h->smem_loop, h->stream>>>(h->ds, t_end, h->staged);
        }
        CK(cudaEventRecord(h->l1, h->stream));
        samples_commit_kernel<<<n_blocks(h->n_systems, 64), 64, 0, h->stream>>>(h->ds, h->n_systems);
        CK(cudaGetLastError());
        h->launches += 4;
        h->loop_launches += 1;
        CK(cudaMemcpyAsync(sc.data(), h->sc_all, sizeof(DScal) * h->n_systems, cudaMemcpyDeviceToHost, h->stream));
        CK(cudaStreamSynchronize(h->stream));
        float lms = 0;
        cudaEventElapsedTime(&lms, h->l0, h->l1);
        h->loop_ms += lms;
        bool again = false;
        for (auto &c : sc) if (c.paused && !c.err) again = true;
        if (!again) break;
    }
    return SDMD_OK;
}

extern "C" int sdmd_gpu_download(sdmd_gpu *h, sdmd_system *systems, int32_t n_systems) {
    if (!h || !systems || n_systems != h->n_systems) return SDMD_EINVAL;
    CK(cudaSetDevice(h->opts.device));
    std::vector<DScal> sc(n_systems);
    for (int k = 0; k < n_systems; k++)
        if (systems[k].n_atoms != h->meta[k].n) return SDMD_EINVAL;
    // the dynamic block of every system in one copy, then scattered into the caller's arrays
    std::unique_lock<std::mutex> down_lock(g_down.mu);
    const size_t dyn_bytes = h->dyn_end - h->dyn_begin;
    std::vector<unsigned char> pageable;
    unsigned char *dyn = g_down.get(dyn_bytes);
    if (!dyn) { pageable.resize(dyn_bytes); dyn = pageable.data(); }   // pinned memory unavailable
    CK(cudaMemcpyAsync(dyn, h->arena + h->dyn_begin, dyn_bytes, cudaMemcpyDeviceToHost, h->stream));
    CK(cudaMemcpyAsync(sc.data(), h->sc_all, sizeof(DScal) * n_systems, cudaMemcpyDeviceToHost, h->stream));
    std::vector<std::vector<double>> tl(n_systems);
    if (h->opts.advance == SDMD_ADVANCE_LAZY)
        for (int k = 0; k < n_systems; k++) {
            tl[k].resize((size_t)h->meta[k].n + 1);
            cudaMemcpyAsync(tl[k].data(), h->hs[k].tloc, tl[k].size() * 8, cudaMemcpyDeviceToHost, h->stream);
        }
    CK(cudaStreamSynchronize(h->stream));
    {
        std::vector<Piece> pieces;
        for (int k = 0; k < n_systems; k++)
            for_dynamic(h, k, systems[k], [&](void *dv, void *hp, size_t bytes) {
                pieces.push_back({hp, dyn + ((unsigned char *)dv - (h->arena + h->dyn_begin)), bytes});
            });
        copy_pieces(pieces);
    }
    down_lock.unlock();
    for (int k = 0; k < n_systems; k++) {
        sdmd_system &s = systems[k];
        s.time = sc[k].time;
        s.rng = sc[k].rng;
        s.counters = sc[k].c;
        if (h->opts.advance == SDMD_ADVANCE_LAZY) {
            // back to the reference's representation: positions at the current
            // time (same expression as the device's extrapolation), relative times
            const double T = s.time;
            for (int i = 1; i <= s.n_atoms; i++) {
                double dt = T - tl[k][i];
                s.x[i] = s.x[i] + s.vx[i] * dt;
                s.y[i] = s.y[i] + s.vy[i] * dt;
                s.z[i] = s.z[i] + s.vz[i] * dt;
                s.ev_time[i] = s.ev_time[i] - T;
            }
        }
    }
    return SDMD_OK;
}

extern "C" int sdmd_gpu_trace(sdmd_gpu *h, int32_t s, sdmd_trace_rec *out, int32_t cap, int32_t *n_out) {
    if (!h || s < 0 || s >= h->n_systems || !out || cap < 0) return SDMD_EINVAL;
    CK(cudaSetDevice(h->opts.device));
    DScal sc;
    CK(cudaMemcpy(&sc, h->hs[s].sc, sizeof(DScal), cudaMemcpyDeviceToHost));
    int tc = h->hs[s].trace_cap;
    int64_t have = sc.pops < tc ? sc.pops : tc;
    int64_t n = have < cap ? have : cap;
    // the last n records, oldest first
    for (int64_t q = 0; q < n; q++) {
        int64_t pop = sc.pops - n + q;
        CK(cudaMemcpy(&out[q], &h->hs[s].trace[pop % tc], sizeof(sdmd_trace_rec), cudaMemcpyDeviceToHost));
    }
    if (n_out) *n_out = (int32_t)n;
    return SDMD_OK;
}

extern "C" int sdmd_gpu_last_ms(sdmd_gpu *h, double *prepare_ms, double *run_ms) {
    if (!h) return SDMD_EINVAL;
    if (prepare_ms) *prepare_ms = h->prep_ms;
    if (run_ms) *run_ms = h->run_ms;
    return SDMD_OK;
}

extern "C" int sdmd_gpu_energies(sdmd_gpu *h, double *pot, double *kin) {
    if (!h) return SDMD_EINVAL;
    CK(cudaSetDevice(h->opts.device));
    energy_kernel<<<h->n_systems, 32, h->esmem, h->stream>>>(h->ds, h->x_E, h->x_kin, h->x_warn);
    CK(cudaGetLastError());
    if (pot) CK(cudaMemcpyAsync(pot, h->x_E, sizeof(double) * h->n_systems, cudaMemcpyDeviceToHost, h->stream));
    if (kin) CK(cudaMemcpyAsync(kin, h->x_kin, sizeof(double) * h->n_systems, cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    return collect_errors(h);
}

extern "C" int sdmd_gpu_run_remd(sdmd_gpu *h, int64_t n_exchanges, double t_end, sdmd_remd *x) {
    if (!h || !x || !x->num || !x->T || n_exchanges < 0) return SDMD_EINVAL;
    if (!(x->every_events > 0) && !(x->every_time > 0)) return SDMD_EINVAL;
    CK(cudaSetDevice(h->opts.device));
    const int n = h->n_systems;
    std::vector<double> rate(n, 0);
    std::vector<DScal> scs(n);
    if (!(x->every_events > 0)) {   // REMDRun: rate = ((int)(currenttime / outputRate) + 1) * outputRate
        CK(cudaMemcpyAsync(scs.data(), h->sc_all, sizeof(DScal) * n, cudaMemcpyDeviceToHost, h->stream));
        CK(cudaStreamSynchronize(h->stream));
        for (int k = 0; k < n; k++)
            rate[k] = (double)((long long)(scs[k].time / x->every_time) + 1) * x->every_time;
    }
    int64_t stats[2] = {x->attempted, x->accepted};
    CK(cudaMemcpyAsync(h->x_num, x->num, sizeof(int32_t) * n, cudaMemcpyHostToDevice, h->stream));
    CK(cudaMemcpyAsync(h->x_T, x->T, sizeof(double) * n, cudaMemcpyHostToDevice, h->stream));
    CK(cudaMemcpyAsync(h->x_rng, &x->rng, sizeof(sdmd_rng), cudaMemcpyHostToDevice, h->stream));
    CK(cudaMemcpyAsync(h->x_stats, stats, sizeof(stats), cudaMemcpyHostToDevice, h->stream));
    CK(cudaEventRecord(h->e0, h->stream));
    h->launches = 0; h->loop_launches = 0; h->loop_ms = 0;
    int64_t done = 0;
    for (; done < n_exchanges; done++) {
        if (!(x->every_events > 0))
            CK(cudaMemcpyAsync(h->x_stop, rate.data(), sizeof(double) * n, cudaMemcpyHostToDevice, h->stream));
        remd_round_kernel<<<n_blocks(n, 64), 64, 0, h->stream>>>(h->ds, n, x->every_events > 0 ? x->every_events : 0,
                                                                 x->every_events > 0 ? nullptr : h->x_stop);
        h->launches += 1;
        int r = run_rounds(h, std::min<int64_t>(4 * (x->every_events > 0 ? x->every_events : 16384) + 64, 1 << 16),
                           t_end);
        if (r) return r;
        if ((r = collect_errors(h))) return r;
        // every replica must have reached its exchange point (not the end of the run)
        bool reached = true;
        CK(cudaMemcpyAsync(scs.data(), h->sc_all, sizeof(DScal) * n, cudaMemcpyDeviceToHost, h->stream));
        CK(cudaStreamSynchronize(h->stream));
        for (const DScal &c : scs)
            if (x->every_events > 0 ? c.c.frame < c.target_frame : !c.at_stop) reached = false;
        if (!reached) break;
        energy_kernel<<<n, 32, h->esmem, h->stream>>>(h->ds, h->x_E, h->x_kin, h->x_warn);
        remd_exchange_kernel<<<1, 1, 0, h->stream>>>(h->ds, n, h->x_num, h->x_T, h->x_E, h->x_warn, h->x_rng,
                                                     h->x_stats);
        CK(cudaGetLastError());
        h->launches += 2;
        for (int k = 0; k < n; k++) rate[k] += x->every_time;
    }
    CK(cudaEventRecord(h->e1, h->stream));
    CK(cudaEventSynchronize(h->e1));
    float ms = 0;
    cudaEventElapsedTime(&ms, h->e0, h->e1);
    h->run_ms = ms;
    CK(cudaMemcpy(x->num, h->x_num, sizeof(int32_t) * n, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(x->T, h->x_T, sizeof(double) * n, cudaMemcpyDeviceToHost));
    if (x->E) CK(cudaMemcpy(x->E, h->x_E, sizeof(double) * n, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(&x->rng, h->x_rng, sizeof(sdmd_rng), cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(stats, h->x_stats, sizeof(stats), cudaMemcpyDeviceToHost));
    x->attempted = stats[0];
    x->accepted = stats[1];
    x->exchanges_done = done;
    return collect_errors(h);
}

extern "C" int sdmd_gpu_last_run_stats(sdmd_gpu *h, int64_t *launches, int64_t *loop_launches, double *loop_ms) {
    if (!h) return SDMD_EINVAL;
    if (launches) *launches = h->launches;
    if (loop_launches) *loop_launches = h->loop_launches;
    if (loop_ms) *loop_ms = h->loop_ms;
    return SDMD_OK;
}

extern "C" int sdmd_gpu_last_error(sdmd_gpu *h, sdmd_error_info *info) {
    if (!h || !info) return SDMD_EINVAL;
    *info = h->err;
    return SDMD_OK;
}

// ---- host-side RNG helpers: glibc srand()/rand() stream -------------------------
extern "C" void sdmd_rng_seed(sdmd_rng *r, uint32_t seed) {
    int32_t *t = r->tab;
    t[0] = seed ? (int32_t)seed : 1;
    for (int i = 1; i < 31; i++) {   // Lehmer 16807 seeding, Schrage's decomposition
        long hi = t[i - 1] / 127773, lo = t[i - 1] % 127773;
        long w = 16807 * lo - 2836 * hi;
        if (w < 0) w += 2147483647;
        t[i] = (int32_t)w;
    }
    r->front = 3; r->rear = 0;
    sdmd_rng_skip(r, 310);
}

extern "C" int32_t sdmd_rng_next(sdmd_rng *r) {
    uint32_t v = (uint32_t)r->tab[r->front] + (uint32_t)r->tab[r->rear];
    r->tab[r->front] = (int32_t)v;
    int32_t out = (int32_t)((v >> 1) & 0x7fffffffu);
    if (++r->front >= 31) { r->front = 0; ++r->rear; }
    else if (++r->rear >= 31) r->rear = 0;
    return out;
}

extern "C" void sdmd_rng_skip(sdmd_rng *r, int64_t n) {
    for (int64_t k = 0; k < n; k++) sdmd_rng_next(r);
}

// ---- allocation-free full-rebuild sweep -------------------------------------------
// sdmd_gpu_prepare_noalloc gives the results of sdmd_gpu_prepare, but the scratch
// it needs -- the descriptor table the launches read and each system's thermostat
// sample buffers -- lives in one file-scope device array instead of the handle's
// arena, and the host side uses no heap.  On both prediction paths it runs the
// sequential sweep kernel (one block per system, atoms in order): on the FP32
// screened path that is sweep_kernel_screen, whose results equal the parallel
// sweep's bit for bit but which takes longer on large systems (about 0.7 s
// against 18 ms for 42k atoms).  Layout of the array:
//   [descriptor table: n_systems DSys, 256-aligned]
//   [first-error record, 256-aligned]
//   per system with a thermostat: [smp: cap doubles][smp_raw: 3 cap int32][smp_cum: cap int64],
//   each 256-aligned, cap = atoms + 8 (one sample per predicted atom plus slack).
// Every element a call reads is written earlier in the same call, so nothing in
// the array needs to start at zero and stale contents of an earlier call are harmless.
static __device__ __align__(256) unsigned char g_noalloc_scratch[SDMD_NOALLOC_SCRATCH_BYTES];

namespace {
constexpr int kNoallocMaxDevices = 64;
// The array's device address, resolved once per device by the first call there.
// The cache assumes the device's primary context lives as long as the process:
// after a cudaDeviceReset the next call would use a stale address.
unsigned char *g_noalloc_addr[kNoallocMaxDevices];

__host__ __device__ inline size_t al256(size_t b) { return (b + 255) & ~size_t(255); }
__host__ __device__ inline int64_t noalloc_cap(int32_t n, int32_t thermostat) { return thermostat ? (int64_t)n + 8 : 0; }
__host__ __device__ inline size_t noalloc_sys_bytes(int64_t cap) {
    return cap ? al256((size_t)cap * 8) + al256((size_t)cap * 12) + al256((size_t)cap * 8) : 0;
}
__host__ __device__ inline size_t noalloc_head_bytes(int n_systems) {
    return al256(sizeof(DSys) * (size_t)n_systems) + al256(sizeof(sdmd_error_info));
}

// copy the handle's descriptors into the table; with full_predict the sample
// buffers point into the array (continue mode draws no sample and keeps the
// handle's buffers, which the host-side size check did not count)
__global__ void noalloc_table_kernel(const DSys *src, int n_systems, unsigned char *base, int full_predict) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    DSys *table = reinterpret_cast<DSys *>(base);
    size_t off = noalloc_head_bytes(n_systems);
    for (int k = 0; k < n_systems; k++) {
        DSys s = src[k];
        const int64_t cap = full_predict ? noalloc_cap(s.n, s.thermostat) : 0;
        if (cap) {
            s.smp_cap = (int32_t)cap;
            s.smp = reinterpret_cast<double *>(base + off);
            s.smp_raw = reinterpret_cast<int32_t *>(base + off + al256((size_t)cap * 8));
            s.smp_cum = reinterpret_cast<int64_t *>(base + off + al256((size_t)cap * 8) + al256((size_t)cap * 12));
        }
        off += noalloc_sys_bytes(cap);
        table[k] = s;
    }
}

// the first system with a latched error, or code 0
__global__ void noalloc_first_error_kernel(const DSys *table, int n_systems, sdmd_error_info *out) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    sdmd_error_info e{0, 0, 0, 0};
    for (int k = 0; k < n_systems; k++) {
        const DScal &c = *table[k].sc;
        if (c.err) { e.code = c.err; e.system = k; e.atom = c.err_atom; e.event = c.err_event; break; }
    }
    *out = e;
}
}  // namespace

extern "C" int sdmd_gpu_prepare_noalloc(sdmd_gpu *h, int32_t full_predict) {
    if (!h) return SDMD_EINVAL;
    const int dev = h->opts.device;
    if (dev < 0 || dev >= kNoallocMaxDevices) return SDMD_EINVAL;
    CK(cudaSetDevice(dev));
    size_t need = noalloc_head_bytes(h->n_systems);
    int32_t nmax = 0;
    for (int k = 0; k < h->n_systems; k++) {
        nmax = std::max(nmax, h->meta[k].n);
        if (full_predict) need += noalloc_sys_bytes(noalloc_cap(h->meta[k].n, h->hs[k].thermostat));
    }
    if (need > (size_t)SDMD_NOALLOC_SCRATCH_BYTES) {
        fprintf(stderr,
                "sdmd_gpu_prepare_noalloc: this batch needs %zu bytes of static scratch, the limit is %zu "
                "(SDMD_NOALLOC_SCRATCH_BYTES); use sdmd_gpu_prepare\n",
                need, (size_t)SDMD_NOALLOC_SCRATCH_BYTES);
        return SDMD_ECAPACITY;
    }
    if (!g_noalloc_addr[dev]) {   // first call on this device
        void *p = nullptr;
        CK(cudaGetSymbolAddress(&p, g_noalloc_scratch));
        g_noalloc_addr[dev] = static_cast<unsigned char *>(p);
    }
    unsigned char *base = g_noalloc_addr[dev];
    DSys *table = reinterpret_cast<DSys *>(base);
    sdmd_error_info *first = reinterpret_cast<sdmd_error_info *>(base + al256(sizeof(DSys) * (size_t)h->n_systems));

    CK(cudaEventRecord(h->e0, h->stream));
    noalloc_table_kernel<<<1, 1, 0, h->stream>>>(h->ds, h->n_systems, base, full_predict ? 1 : 0);
    if (full_predict) {
        const int64_t want = (int64_t)nmax + 8;
        samples_walk_kernel<<<n_blocks(h->n_systems, 64), 64, 0, h->stream>>>(table, h->n_systems, want);
        dim3 grid((unsigned)std::max<int64_t>(1, std::min<int64_t>((want + 255) / 256, 1024)), (unsigned)h->n_systems);
        samples_values_kernel<<<grid, 256, 0, h->stream>>>(table, want);
    }
    h->sweep_k<<<h->n_systems, h->sweep_threads, h->smem, h->stream>>>(table, full_predict ? 1 : 0);
    if (full_predict) samples_commit_kernel<<<n_blocks(h->n_systems, 64), 64, 0, h->stream>>>(table, h->n_systems);
    noalloc_first_error_kernel<<<1, 1, 0, h->stream>>>(table, h->n_systems, first);
    CK(cudaGetLastError());
    sdmd_error_info e;
    CK(cudaMemcpyAsync(&e, first, sizeof(e), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaEventRecord(h->e1, h->stream));
    CK(cudaEventSynchronize(h->e1));
    float ms = 0;
    cudaEventElapsedTime(&ms, h->e0, h->e1);
    h->prep_ms = ms;
    if (e.code) {
        h->err = e;
        return e.code;
    }
    return SDMD_OK;
}

extern "C" int sdmd_gpu_launch_info(sdmd_gpu *h, int32_t *threads, int32_t *helper_blocks, int32_t *staged,
                                    int32_t *loop_kernel) {
    if (!h) return SDMD_EINVAL;
    if (threads) *threads = h->threads;
    if (helper_blocks) *helper_blocks = h->helpers;
    if (staged) *staged = h->staged;
    if (loop_kernel) {
        if (h->helpers > 0) *loop_kernel = h->threads > 256 ? SDMD_LOOP_SCREEN_HELPERS_512 : SDMD_LOOP_SCREEN_HELPERS;
        else if (h->loop_k == loop_kernel_screen_r128) *loop_kernel = SDMD_LOOP_SCREEN_R128;
        else if (h->loop_k == loop_kernel_screen) *loop_kernel = SDMD_LOOP_SCREEN;
        else *loop_kernel = SDMD_LOOP_FP64;
    }
    return SDMD_OK;
}
