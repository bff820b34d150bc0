// samples.cu -- the thermostat's normal-sample stream, precomputed in parallel.
//
// The reference draws every Maxwell-Boltzmann value with the polar Box-Muller
// method on glibc's rand() (Maxwell_Boltzmann_Distribution, src/ToolFunctions.c
// 544-569): pairs (a, b) = 2u - 1 are drawn until a^2 + b^2 < 1, then a third
// draw picks a * f or b * f with f = sqrt(-2 log(s) / s).  Every call site then
// scales the same standard-normal value (ThermostatTime: x1, src/TimePrediction.c
// 582-595; ThermostatEvent via RandomVelocity: x sqrt(T/m), src/Events.c:396-420),
// so the stream of standard-normal values is independent of where it is used.
//
// Three kernels replace the sequential draws:
//   walk   (one thread per system) decides which rand() outputs form each sample.
//          Only integer work and an FP32 estimate of a^2 + b^2 are needed; the
//          exact FP64 test runs when the estimate is within 1e-5 of 1.
//   values (one thread per sample) computes a, b, s, the correctly rounded log,
//          sqrt and division exactly as the reference does.
//   commit (one thread per system) advances the rand() state past the draws of
//          the samples the event loop actually consumed.
#include "dev.cuh"
#include "engine.h"

namespace sdmd {

constexpr int32_t RAND_MAX_I = 2147483647;

// exact acceptance test of one polar attempt (r1, r2)
__device__ inline bool polar_accept(int32_t r1, int32_t r2) {
    int32_t ia = (int32_t)(2u * (uint32_t)r1 - (uint32_t)RAND_MAX_I);   // 2 r1 - RAND_MAX, fits in int32
    int32_t ib = (int32_t)(2u * (uint32_t)r2 - (uint32_t)RAND_MAX_I);
    float fa = (float)ia / 2147483647.0f, fb = (float)ib / 2147483647.0f;
    float s32 = __fmaf_rn(fa, fa, fb * fb);
    if (s32 < 1.0f - 1e-5f) return true;
    if (s32 > 1.0f + 1e-5f) return false;
    double a = 2 * (0 + (double)r1 / ((double)RAND_MAX_I / (1 - 0))) - 1;
    double b = 2 * (0 + (double)r2 / ((double)RAND_MAX_I / (1 - 0))) - 1;
    double s = a * a + b * b;
    return s < 1;
}

// glibc's TYPE_3 state keeps front == rear + 3 (mod 31).  With the table rotated
// so that rear is at index 0 (R[k] = tab[(rear + k) % 31]), draw s of a block
// writes R[(3 + s) % 31] += R[s % 31]; after 31 draws the pattern repeats.  A
// fully unrolled block therefore indexes the table statically and keeps it in
// registers.  The commit uses it to skip the consumed draws; the walk keeps the
// plain generator (its sample logic would be unrolled 31 times).
__device__ inline bool ring_ok(const sdmd_rng &r) {
    return r.rear >= 0 && r.rear < 31 && r.front == (r.rear + 3) % 31;
}
__device__ inline void ring_load(const sdmd_rng &r, int32_t (&R)[31]) {
#pragma unroll
    for (int k = 0; k < 31; k++) {
        int q = r.rear + k;
        R[k] = r.tab[q >= 31 ? q - 31 : q];
    }
}
// the state after `m` draws from the one ring_load() read (rear advanced by m)
__device__ inline void ring_store(sdmd_rng &r, const int32_t (&R)[31], int64_t m) {
    const int rear0 = r.rear;
#pragma unroll
    for (int k = 0; k < 31; k++) {
        int q = rear0 + k;
        r.tab[q >= 31 ? q - 31 : q] = R[k];
    }
    r.rear = (int)((rear0 + m) % 31);
    r.front = (r.rear + 3) % 31;
}
#define RING_DRAW(R, k, out)                                                        \
    do {                                                                            \
        const uint32_t v_ = (uint32_t)R[(3 + (k)) % 31] + (uint32_t)R[(k)];         \
        R[(3 + (k)) % 31] = (int32_t)v_;                                            \
        (out) = (int32_t)((v_ >> 1) & 0x7fffffffu);                                 \
    } while (0)

__global__ void samples_walk_kernel(const DSys *systems, int n_systems, int64_t want) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n_systems) return;
    const DSys &S = systems[k];
    DScal *C = S.sc;
    C->rng0 = C->rng;
    C->smp_used = 0;
    C->smp_avail = 0;
    C->paused = 0;
    if (!S.thermostat || C->err) return;
    sdmd_rng r = C->rng;
    int64_t n = want < S.smp_cap ? want : S.smp_cap, cum = 0;
    for (int64_t q = 0; q < n; q++) {
        int32_t r1, r2;
        int tries = 0;
        for (;;) {
            r1 = rng_next(r);
            r2 = rng_next(r);
            cum += 2;
            if (polar_accept(r1, r2)) break;
            if (++tries >= 4096) {   // only a degenerate state rejects this often
                C->err = SDMD_ETIMEOUT; C->err_atom = 0; C->err_event = C->c.frame;
                return;
            }
        }
        int32_t r3 = rng_next(r);
        cum += 1;
        S.smp_raw[3 * q] = r1; S.smp_raw[3 * q + 1] = r2; S.smp_raw[3 * q + 2] = r3;
        S.smp_cum[q] = cum;
    }
    C->smp_avail = n;
}

__global__ void samples_values_kernel(const DSys *systems, int64_t want) {
    const DSys &S = systems[blockIdx.y];
    int64_t n = S.sc->smp_avail;
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x) {
        int32_t r1 = S.smp_raw[3 * q], r2 = S.smp_raw[3 * q + 1], r3 = S.smp_raw[3 * q + 2];
        double a = 2 * (0 + (double)r1 / ((double)RAND_MAX_I / (1 - 0))) - 1;
        double b = 2 * (0 + (double)r2 / ((double)RAND_MAX_I / (1 - 0))) - 1;
        double s = a * a + b * b;
        s = sqrt(-2 * cr_log(s) / s);
        double choose = 0 + (double)r3 / ((double)RAND_MAX_I / (1 - 0));
        S.smp[q] = (choose >= 0.5) ? a * s : b * s;
    }
}

__global__ void samples_commit_kernel(const DSys *systems, int n_systems) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n_systems) return;
    const DSys &S = systems[k];
    DScal *C = S.sc;
    if (C->smp_used <= 0) { C->rng = C->rng0; return; }
    sdmd_rng r = C->rng0;
    const int64_t n = S.smp_cum[C->smp_used - 1];
    if (ring_ok(r)) {   // whole blocks of 31 draws with the table in registers, then the rest
        int32_t R[31];
        ring_load(r, R);
        for (int64_t b = 0; b < n / 31; b++) {
#pragma unroll
            for (int s = 0; s < 31; s++) {
                int32_t out;
                RING_DRAW(R, s, out);
                (void)out;
            }
        }
        const int rem = (int)(n % 31);
#pragma unroll
        for (int s = 0; s < 31; s++) {
            if (s < rem) {
                int32_t out;
                RING_DRAW(R, s, out);
                (void)out;
            }
        }
        ring_store(r, R, n);
    } else {
        for (int64_t q = 0; q < n; q++) rng_next(r);
    }
    C->rng = r;
    C->smp_avail = 0;
    C->smp_used = 0;
}

__global__ void begin_run_kernel(const DSys *systems, int n_systems, int64_t max_events) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n_systems) return;
    DScal *C = systems[k].sc;
    C->target_frame = C->c.frame + max_events;
    C->paused = 0;
}

}  // namespace sdmd
