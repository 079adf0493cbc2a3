/* mqi_oracle.h - CPU restatement of moqui's proton transport (TEST INFRASTRUCTURE ONLY).
 *
 * This oracle restates, in plain C, the reference algorithm of the path the GPU engine replaces:
 * the history loop with its LIFO track stack (moqui/kernel_functions/mqi_transport.hpp:113-250),
 * fippel_physics::stepping (moqui/base/mqi_fippel_physics.hpp:67-216), the four processes, the
 * grid3d voxel traversal and the dose scorers.  It is the checker for the CUDA path: only tests,
 * the smoke check and the bench's CPU-baseline leg call it; the product never links it.
 *
 * Random numbers: the reference draws from cuRAND XORWOW (GPU) or std::default_random_engine
 * (CPU), which no re-implementation can reproduce stream for stream.  The oracle instead draws from
 * the same counter-based Philox4x32-10 streams as the GPU engine (keyed by seed, history and track
 * uid, one fresh block per physics step), so the oracle and the GPU can be compared history by
 * history, while the oracle itself is pinned to the reference's own CPU build through golden
 * vectors (deterministic functions, voxel walks) and dose statistics (tests/golden/).
 */
#ifndef MQI_ORACLE_H
#define MQI_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
    int          nx, ny, nz;
    const float* xe; /* nx+1 edges */
    const float* ye;
    const float* ze;
    const float* rho; /* g/mm^3, x fastest */
} mqo_grid;

/* A tabulated SPR(rho, E) / X0(rho) calibration on uniform grids (mqi_set_calibration's
 * MQI_CALIB_TABLE): spr[i_rho * n_e + i_e], x0[i_rho]; bilinear / linear, clamped to the grid. */
typedef struct {
    uint32_t     n_rho, n_e;
    float        rho0, drho, e0, de;
    const float* spr;
    const float* x0;
} mqo_calib;

typedef struct {
    int              physics_debug; /* 1: moqui built with __PHYSICS_DEBUG__ */
    int              scorer;        /* 1 EDEP, 2 DOSE_W, 3 DOSE_W2 (mqi_gpu.h numbering) */
    const mqo_calib* calib;         /* NULL: spr_default / radiation_length_default */
} mqo_config;

typedef struct {
    uint64_t histories, tracks, steps, pushed, dropped;
} mqo_stats;

/* Transport histories [h0, h1) of `vertices` (7 floats each: ke, pos[3], dir[3]) through one
 * child grid, adding the scorer's per-voxel values into `tally` (nx*ny*nz doubles).  If
 * `per_history_edep` is non-NULL it receives, per history, the summed energy scored (MeV). */
int mqo_transport(const mqo_grid* g, const mqo_config* cfg, const float* vertices, uint64_t h0, uint64_t h1,
                  uint64_t seed, double* tally, double* per_history_edep, mqo_stats* stats);

/* Deterministic probes: for each energy, {cs_ion, cs_pp, cs_poe, cs_poi (per g/mm^3), dEdx, beta^2,
 * Te_max, momentum}; SPR(rho, E); X0(rho); HU -> density. */
void  mqo_eval_physics(const float* energies, uint64_t n, float* out8);
float mqo_spr(float rho, float ke, int physics_debug);
float mqo_x0(float rho, int physics_debug);
float mqo_hu_to_density(int hu);

/* One Philox4x32-10 block of counter[4] under key[2] (the generator every stream is drawn from). */
void mqo_philox(const uint32_t* counter, const uint32_t* key, uint32_t* out);

/* Sampling probes of the transport's processes at fixed energy and density (the restatement's
 * twin of the reference driver's `sample` mode): process 0 along_step over 1 mm, 1 delta ray,
 * 2 p-p elastic, 3 p-O elastic, 4 p-O inelastic; out holds 2, 1, 3, 2, 3 blocks of n floats. */
int mqo_sample(int process, float ke, float rho, uint64_t n, uint64_t seed, int physics_debug, float* out);

/* Voxel walk of one ray (the transport's entry + voxel loop with boundary-only steps).
 * Returns the number of entries written (<= max_steps). */
int mqo_trace_ray(const mqo_grid* g, const float ray[6], int max_steps, uint64_t* cnb, float* dist, int32_t* cells);

#ifdef __cplusplus
}
#endif

#endif
