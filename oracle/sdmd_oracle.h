/*
 * sdmd_oracle.h -- CPU restatement of the reference sDMD event loop.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the checker the CUDA engine is compared
 * against (tests/, __graft_entry__.smoke() and bench.py's cpu_baseline leg); the
 * product never links it.  It is pinned against the reference itself through the
 * golden fixtures in tests/golden/ (generated from the reference's own sources by
 * tests/golden/make_golden.py), compared event for event.
 *
 * It works on the engine's plain sdmd_system struct (include/sdmd_gpu.h) and
 * follows the reference's operation order exactly (FP64, no contraction), so it
 * reproduces the reference bit for bit on the same input state.
 */
#ifndef SDMD_ORACLE_H
#define SDMD_ORACLE_H
#include "sdmd_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct oracle_loop oracle_loop;

/* Predict() over atoms 1..N (src/SGThread.c:47-52). Returns 0 or SDMD_E*. */
int oracle_predict_all(sdmd_system *s);

/* Create the loop context and the event tree (CreateCBT, src/CBT.c:16-30). */
oracle_loop *oracle_loop_create(sdmd_system *s);
void oracle_loop_destroy(oracle_loop *L);

/* Event loop of src/SGThread.c:75-151: runs until `max_events` more events were
 * executed or the time exceeds t_end.  Pops are recorded into `trace` (up to
 * trace_cap records, the first ones kept); *n_pops receives the pop count. */
int oracle_run(oracle_loop *L, int64_t max_events, double t_end,
               sdmd_trace_rec *trace, int64_t trace_cap, int64_t *n_pops);
/* run until the first executed event at time >= stop_time (or t_end) */
int oracle_run_until(oracle_loop *L, double t_end, double stop_time, int64_t *n_pops);
/* CalPotenE with FindPair's warnings counted in s->counters (as REMDRun calls it) */
double oracle_potential_energy_counted(sdmd_system *s);

/* The tree's node[] (2N entries) and leaf[] (N+1 entries), for checks. */
int oracle_cbt(oracle_loop *L, int32_t *node, int32_t *leaf);

/* Potential energy CalPotenE (src/ToolFunctions.c:659-752) and kinetic energy
 * CalKinetE (src/ToolFunctions.c:626-656). */
double oracle_potential_energy(const sdmd_system *s);
double oracle_kinetic_energy(const sdmd_system *s);

/* glibc rand() restatement and the Box-Muller draw (src/ToolFunctions.c:544-569). */
int32_t oracle_rand(sdmd_rng *r);
double  oracle_mb(sdmd_rng *r, double mean, double variance);
double  oracle_log(double x);

/* REMD server sweep (src/Server.c:145-192) on n slots; rng drives the draws. */
void oracle_remd_rearrange(int32_t n, int32_t *num, double *T, const double *E, sdmd_rng *rng);

#ifdef __cplusplus
}
#endif
#endif
