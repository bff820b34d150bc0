// engine.h -- internal interface between the C ABI (api.cu) and the kernels.
#pragma once
#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

namespace sdmd {
struct DSys;
struct DScal;
struct Adv;

// exact FP64 path (loop_fp64.cu)
size_t fp64_smem_bytes(int nbcap);
__global__ void sweep_kernel_fp64(const DSys *systems, int full);
__global__ void loop_kernel_fp64(const DSys *systems, double t_end_override, int staged);
size_t staged_state_bytes(int n, int ncell, int nb, int nc, int ncs, int nconn);
__global__ void lazy_enter_kernel(const DSys *systems);

// FP32-screened prediction, identical results (loop_fp64.cu + screen.cuh)
size_t screen_smem_bytes(int nbcap);
__global__ void sweep_kernel_screen(const DSys *systems, int full);
__global__ void loop_kernel_screen(const DSys *systems, double t_end_override, int staged);
__global__ void loop_kernel_screen_r128(const DSys *systems, double t_end_override, int staged);
// the screened loop with helper blocks for the eager advance (cooperative launch:
// blocks 0 .. n_chain-1 run the systems, the rest advance their atoms)
__global__ void loop_kernel_screen_coop(const DSys *systems, double t_end_override, int n_chain);
__global__ void loop_kernel_screen_coop512(const DSys *systems, double t_end_override, int n_chain);

// parallel full-rebuild sweep of the screened path (sweep_par.cuh)
size_t verify_smem_bytes(int nbcap, int warps);
__global__ void sweep_reset_kernel(const DSys *systems);
__global__ void sweep_predict_kernel(const DSys *systems);
__global__ void sweep_verify_kernel(const DSys *systems);
__global__ void sweep_fix_kernel(const DSys *systems, int full);

// energies and the replica exchange (remd.cu)
size_t energy_smem_bytes(int nbcap);
__global__ void energy_kernel(const DSys *systems, double *pot, double *kin, int64_t *warn);
__global__ void remd_round_kernel(const DSys *systems, int n, int64_t every_events, const double *stop_time);
__global__ void stops_round_kernel(const DSys *systems, int n, const int64_t *limit, const double *stop_time);
__global__ void remd_exchange_kernel(DSys *systems, int n, int32_t *num, double *T, const double *E,
                                     const int64_t *warn, sdmd_rng *rng, int64_t *stats);

// thermostat sample stream (samples.cu)
__global__ void samples_walk_kernel(const DSys *systems, int n_systems, int64_t want);
__global__ void samples_values_kernel(const DSys *systems, int64_t want);
__global__ void samples_commit_kernel(const DSys *systems, int n_systems);
__global__ void begin_run_kernel(const DSys *systems, int n_systems, int64_t max_events);
}  // namespace sdmd
