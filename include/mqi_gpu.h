/* mqi_gpu.h - C ABI of the GB300 proton transport engine (libmqigpu.so).
 *
 * This is the drop-in boundary for moqui's device path.  In moqui the device boundary is a pair of
 * templated kernels plus the upload/download helpers that x_environment<R> calls:
 *
 *   upload_node / upload_materials / upload_vertices  (moqui/kernel_functions/mqi_upload_data.hpp:144-420)
 *   transport_particles_patient[_stat]                 (moqui/kernel_functions/mqi_transport.hpp:113-389)
 *   download_node                                      (moqui/kernel_functions/mqi_download_data.hpp:35-121)
 *   calculate_standard_deviation / calculate_average   (moqui/kernel_functions/mqi_variables.hpp:19-66)
 *
 * Each entry point below names the reference interface it replaces.  Conventions:
 *   - every function returns an int status: MQI_OK (0) or a negative MQI_ERR_* code; none exits;
 *   - the caller owns every host array and the library copies what it keeps;
 *   - the context owns its device buffers; outputs go to caller-allocated buffers;
 *   - one context per host thread; a context is bound to one CUDA device;
 *   - pointers are host pointers unless a function's `on_device` flag says otherwise.
 * Device function pointers cannot cross a C ABI, so moqui's scorer and calibration plug-ins
 * (fp_compute_hit, fp_compute_rsp/rl) are selected by enum here.
 */
#ifndef MQI_GPU_H
#define MQI_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---------------------------------------------------------------------- */
#define MQI_OK               0
#define MQI_ERR_INVALID     -1 /* bad argument or size */
#define MQI_ERR_CUDA        -2 /* a CUDA runtime call failed (see mqi_last_error) */
#define MQI_ERR_NOMEM       -3 /* device allocation failed */
#define MQI_ERR_STATE       -4 /* call order: e.g. transport before a grid was set */
#define MQI_ERR_UNSUPPORTED -5 /* a plug-in that has no enum counterpart */
#define MQI_ERR_OVERFLOW    -6 /* a device queue or buffer ran out of capacity */
#define MQI_ERR_DEVICE      -7 /* a kernel reported a device-side error (bounded loop expired) */

/* ---- scorer plug-ins: moqui's fp_compute_hit callbacks
 *      (moqui/base/scorers/mqi_scorer_energy_deposit.hpp:12-177) ------------------------- */
typedef enum {
    MQI_SCORER_EDEP           = 1,  /* energy_deposit: dE + local_dE                           */
    MQI_SCORER_DOSE_W         = 2,  /* dose_to_water (Dw_pointer)                              */
    MQI_SCORER_DOSE_W2        = 3,  /* dose_to_water_square (Dw_square_pointer)                */
    MQI_SCORER_DOSE_M         = 4,  /* dose_to_medium (Dm_pointer)                             */
    MQI_SCORER_LETD_NUM       = 5,  /* LETd_weight1                                            */
    MQI_SCORER_LETD_DEN       = 6,  /* LETd_weight2                                            */
    MQI_SCORER_LETT_NUM       = 7,  /* LETt_weight1                                            */
    MQI_SCORER_LETT_DEN       = 8,  /* LETt_weight2                                            */
    MQI_SCORER_EDEP_PRIMARY   = 9,  /* energy_deposit_primary                                  */
    MQI_SCORER_EDEP_SECONDARY = 10, /* energy_deposit_secondary                                */
    MQI_SCORER_DIJ            = 11  /* dose_to_water keyed by (voxel, spot): the Dij scorer    */
} mqi_scorer_type;

/* ---- ROI mapping (moqui/base/mqi_roi.hpp:13-17) ------------------------------------------ */
typedef enum {
    MQI_ROI_DIRECT   = 0,
    MQI_ROI_INDIRECT = 1,
    MQI_ROI_CONTOUR  = 2
} mqi_roi_method;

/* ---- a source vertex, layout-identical to mqi::vertex_t<float> (moqui/base/mqi_vertex.hpp:16-29) */
typedef struct {
    float ke;     /* kinetic energy, MeV */
    float pos[3]; /* mm, world frame */
    float dir[3]; /* unit vector */
} mqi_vertex;

/* ---- a pencil-beam spot of a plan: moqui's beamlet = energy pdf x 6-D phase-space pdf x coordinate
 *      transform (moqui/base/mqi_beamlet.hpp:40-90) with the Gaussian phsp_6d
 *      (moqui/base/distributions/mqi_phsp6d.hpp) and norm_1d/const_1d energy ------------------- */
typedef struct {
    float    energy;        /* mean kinetic energy, MeV */
    float    energy_sigma;  /* Gaussian energy spread, MeV (0: mono-energetic, const_1d) */
    float    mean[5];       /* beam frame: x, y, z (mm) and x', y' (direction cosines) */
    float    sigma[5];      /* Gaussian sigmas of the five variables above */
    float    corr[2];       /* x-x' and y-y' correlation */
    float    rot[9];        /* beam frame -> world rotation, row-major (coordinate_transform) */
    float    trans[3];      /* beam frame -> world translation, mm */
    uint64_t histories;     /* histories of this spot */
} mqi_spot;

/* ---- run counters ------------------------------------------------------------------------- */
typedef struct {
    uint64_t histories;        /* primaries transported (moqui's tracked_particles)           */
    uint64_t tracks;           /* tracks popped from the queue, primaries included             */
    uint64_t steps;            /* voxel steps taken                                            */
    uint64_t secondaries;      /* daughters pushed to the queue                                */
    uint64_t local_daughters;  /* deposit-only daughters scored at creation (debug physics)    */
    uint64_t dropped;          /* daughters dropped by the emulated stack limit                */
    uint64_t waves;            /* queue generations processed                                  */
    uint64_t device_errors;    /* bounded device loops that gave up                            */
    uint64_t kernel_launches;  /* engine kernels launched by mqi_transport                     */
    uint64_t wave_launches;    /* launches of the transport wave kernel                        */
    double   wave_ms;          /* summed CUDA-event time of the wave kernel launches           */
} mqi_stats;

typedef struct mqi_ctx mqi_ctx;

/* ---- context ------------------------------------------------------------------------------ */

/* Create a context on CUDA device `device`.  Replaces cudaSetDevice(gpu_id) in
 * phantom_env/tps_env (moqui/base/environments/mqi_phantom_env.hpp:44-46). */
int mqi_create(int device, mqi_ctx** out);
int mqi_destroy(mqi_ctx* ctx);

/* Last error message of this context (or of the calling thread when ctx is NULL). */
const char* mqi_last_error(const mqi_ctx* ctx);

/* Run all subsequent work of this context on `cuda_stream` (a cudaStream_t; NULL = a new stream
 * of the context's own, which does not synchronise with the legacy default stream: pass
 * cudaStreamLegacy, (void*) 1, to order the work with that stream). */
int mqi_set_stream(mqi_ctx* ctx, void* cuda_stream);

/* Physics options.  physics_debug = 1 reproduces moqui built with -D__PHYSICS_DEBUG__ (the
 * phantom example, tests/mc/phantom/CMakeLists.txt:10): delta cut 0.08511 MeV, 200-deep track
 * stack, water shortcuts in the calibration, zero-energy local-deposit daughters.  0 is the
 * release build (delta cut 0.0815 MeV, 10-deep stack).  score_local_deposit mirrors the
 * kernel argument of the same name (mqi_transport.hpp:123). */
int mqi_set_physics(mqi_ctx* ctx, int physics_debug, int score_local_deposit);

/* ---- calibration plug-in: material_t::compute_rsp_ / compute_rl_
 *      (moqui/base/materials/mqi_material.hpp:10-25) ------------------------------------------ */
#define MQI_CALIB_DEFAULT 0 /* spr_default / radiation_length_default (mqi_patient_materials.hpp:414-473) */
#define MQI_CALIB_TABLE   1 /* SPR(rho, E) and X0(rho) tabulated on uniform grids */

/* Select the stopping-power-ratio and radiation-length curves.  moqui's patient material installs
 * spr_default and radiation_length_default as its compute_rsp_ / compute_rl_ function pointers
 * (mqi_patient_materials.hpp:474-497); a user material installs its own.  Device function pointers
 * cannot cross a C ABI, so a custom curve is given as tables on uniform grids:
 *   spr[i_rho * n_e + i_e] at rho = rho0 + i_rho * drho (g/mm^3) and E = e0 + i_e * de (MeV);
 *   x0[i_rho] (radiation length, mm) at the same densities.
 * SPR is interpolated bilinearly and X0 linearly, with the fractional index (x - x0) / dx clamped
 * to the grid (n_rho, n_e >= 2; drho, de > 0; every entry finite, X0 > 0).  Voxels below 1e-7 g/mm^3
 * stay vacuum and above 99.9 stay stops, as with the default curves; the default curves' water
 * shortcut of debug physics does not apply to tables.  calib = MQI_CALIB_DEFAULT restores the
 * default curves (the other arguments are then ignored).  Applies to transports started after it. */
int mqi_set_calibration(mqi_ctx* ctx, int calib, uint32_t n_rho, float rho0, float drho, uint32_t n_e, float e0,
                        float de, const float* spr, const float* x0);

/* Add a child geometry to the world: a rectilinear voxel grid with nx+1/ny+1/nz+1 edges (mm),
 * an optional rotation (row-major 3x3, fwd = child->world; NULL = identity) and translation
 * (NULL = 0).  Replaces the grid3d construction + upload_node/add_node_geometry
 * (moqui/base/mqi_grid3d.hpp grid3d(...) ctors; mqi_upload_data.hpp:69-103, 144-398).
 * Children are visited in the order they were added, as world->children[] is. */
int mqi_add_child(mqi_ctx* ctx, int nx, int ny, int nz, const float* xe, const float* ye,
                  const float* ze, const float* rot_fwd, const float* translation, int* child_id);

/* Mass density per voxel in g/mm^3, x fastest ([nz][ny][nx]), as grid3d::set_data. */
int mqi_set_density(mqi_ctx* ctx, int child_id, const float* rho, int on_device);

/* HU per voxel converted on the device with patient_material_t::hu_to_density
 * (moqui/base/materials/mqi_patient_materials.hpp:514-542), then multiplied by density_scale
 * (tps_env's DensityScaling, moqui/base/environments/mqi_tps_env.hpp:766-769). */
int mqi_set_hu(mqi_ctx* ctx, int child_id, const int16_t* hu, float density_scale, int on_device);

/* Add a scorer to a child: scorer<R>(name, capacity, fp_compute_hit) + roi_t
 * (moqui/base/mqi_scorer.hpp:39-79, moqui/base/mqi_roi.hpp:18-194).  For MQI_ROI_DIRECT the
 * three arrays may be NULL.  The tally is a dense FP64 array over the child's voxels, keyed by
 * voxel as the reference's tables are (entries outside the ROI stay zero). */
int mqi_add_scorer(mqi_ctx* ctx, int child_id, int type, int roi_method, uint32_t roi_length,
                   const uint32_t* roi_start, const uint32_t* roi_stride, const uint32_t* roi_acc,
                   int* scorer_id);

/* Source vertices for histories [0, n) and, optionally, their spot index (Dij column;
 * scorer_offset_vector in mqi_transport.hpp:150-154).  Replaces upload_vertices
 * (mqi_upload_data.hpp:413-420) and upload_scorer_offset_vector. */
int mqi_set_vertices(mqi_ctx* ctx, const mqi_vertex* v, const uint32_t* spot_ids, uint64_t n,
                     int on_device);

/* Transport histories [h0, h1) of the current vertices with run seed `seed`, adding into the
 * tallies.  Replaces transport_particles_patient<float><<<...>>> (mqi_transport.hpp:113-250).
 * Blocks until the work is done. */
int mqi_transport(mqi_ctx* ctx, uint64_t h0, uint64_t h1, uint64_t seed);

/* A plan of spots whose histories are sampled on the device: history h belongs to spot s when
 * sum(histories of spots < s) <= h < sum(histories of spots <= s), and spot s is its Dij column.
 * Replaces beamsource::append_beamlet + the host vertex loop + upload_vertices
 * (moqui/base/mqi_beamsource.hpp:48-112, moqui/base/environments/mqi_tps_env.hpp:1182-1236).
 * `total_histories` receives the plan's history count. */
int mqi_set_spot_plan(mqi_ctx* ctx, const mqi_spot* spots, uint32_t n_spots, uint64_t* total_histories);

/* Transport histories [h0, h1) of the spot plan with run seed `seed`: one queue drain for any
 * number of spots (one spot per call gives moqui's per-spot runs, tps_env::run_by_spot,
 * mqi_tps_env.hpp:1477-1603). */
int mqi_transport_plan(mqi_ctx* ctx, uint64_t h0, uint64_t h1, uint64_t seed);

/* ---- robust scenarios ----------------------------------------------------------------------- */

/* Robust scenarios: n instances of child `child_id` that differ in their voxel edges and density
 * scale, transported together.  tps_env runs one scenario per job: XShift/YShift/ZShift move the
 * CT origin before its edges are formed (mqi_tps_env.hpp:475-477, 507-514) and DensityScaling
 * multiplies every voxel density (mqi_tps_env.hpp:766-769).  Here every transport call runs each
 * history once per scenario in one queue drain (the scenarios of a history share its random
 * numbers), and every scorer holds one tally per scenario, scenario-major (mqi_get_tally returns
 * n * tally length; the statistics calls return the worst scenario).  xe/ye/ze hold n x (nx+1),
 * n x (ny+1), n x (nz+1) edges; density_scale n factors (NULL: 1); the child's density must be
 * the unscaled one.  At most 64 scenarios; spot indices stay below 2^24 - 1.  n <= 1 removes the
 * scenarios.  Existing tallies are reallocated and zeroed.  Not with a Dij scorer. */
int mqi_set_scenarios(mqi_ctx* ctx, int child_id, uint32_t n, const float* xe, const float* ye,
                      const float* ze, const float* density_scale);

/* Statistical stopping over whole passes of the spot plan: transport the plan with a fresh seed
 * per pass until the reference estimate (mqi_stat_uncertainty, worst scenario) is <= criteria
 * or max_passes ran, then scale the child's other scorers to one pass (tps_env::run with
 * record_statistics + calculate_average_results, mqi_tps_env.hpp:1238-1300, 1428-1476). */
int mqi_run_plan_until_stat(mqi_ctx* ctx, int dose_id, int dose2_id, float criteria, float threshold,
                            uint64_t max_passes, uint64_t seed, uint64_t* passes_done, double* achieved);

/* Write the source vertices (and spot ids, when spot_out is not NULL) that mqi_transport_plan
 * with run seed `seed` starts for histories [h0, h1) of the plan: the sampled beamlet vertices
 * beamsource produces (mqi_beamlet.hpp:80-90).  Host buffers of h1-h0 entries. */
int mqi_sample_plan(mqi_ctx* ctx, uint64_t h0, uint64_t h1, uint64_t seed, mqi_vertex* out, uint32_t* spot_out);

/* ---- Dij ------------------------------------------------------------------------------------ */

/* Add a Dij scorer to a child: moqui's DOSE_Dij scorer (scorer<R>(name, 512*512*300*5, fp_dose)
 * over a key_value table, mqi_tps_env.hpp:920-931): dose_to_water per step keyed by (voxel cnb,
 * spot index of the history), gated by the ROI like the dense scorers, inserted into an
 * open-addressing table (insert_hashtable, mqi_transport.hpp:68-111).  `capacity` = table slots,
 * rounded up to a power of two, 16 bytes each (0: 2^26); a full table makes the transport call
 * return MQI_ERR_OVERFLOW. */
int mqi_add_dij_scorer(mqi_ctx* ctx, int child_id, int roi_method, uint32_t roi_length,
                       const uint32_t* roi_start, const uint32_t* roi_stride, const uint32_t* roi_acc,
                       uint64_t capacity, int* scorer_id);

/* Build the Dij matrix from the table: n_spots columns (0: the spot plan's count), values = FP64
 * tally * scale rounded once to FP32 (save_sparse_file's scale: particles per history * RBE *
 * fractions, mqi_tps_env.hpp:1905-1930).  Builds the spot-row CSR and the voxel-row layout the
 * products read.  `nnz` receives the entry count.  Transporting again invalidates the matrix. */
int mqi_dij_build(mqi_ctx* ctx, int scorer_id, uint32_t n_spots, double scale, uint64_t* nnz);

/* The spot-row CSR, the layout of save_to_npz (moqui/base/mqi_io.hpp:251-320): shape
 * [n_spots, n_voxels], indptr (n_spots + 1), voxel indices ascending within a row, FP32 values. */
int mqi_dij_get_csr(mqi_ctx* ctx, int scorer_id, uint64_t* indptr, uint32_t* indices, float* data,
                    int on_device);

/* Table slots, occupied slots (counted by one pass over the table on the context's stream; the
 * call waits for it), and (after a build) entries and voxel rows of the matrix. */
int mqi_dij_info(mqi_ctx* ctx, int scorer_id, uint64_t* table_slots, uint64_t* occupied,
                 uint64_t* nnz, uint64_t* n_voxel_rows);

/* Record every insertion into Dij scorer `scorer_id`'s table by later transports: the voxel (cnb),
 * the spot column and the FP64 value that moqui's insert_hashtable(table, cnb, spot, value, ...)
 * receives for the same step (mqi_transport.hpp:68-111, called at :204-225), in the order the
 * GPU issued them.  A log of `capacity` entries (16 bytes each) is allocated; 0 stops recording
 * and frees it.  For checking a table against a replay through the reference's insertion. */
int mqi_dij_record_hits(mqi_ctx* ctx, int scorer_id, uint64_t capacity);

/* Copy the recorded insertions (host buffers of *n_out entries; all three may be NULL to query
 * the count).  Returns MQI_ERR_OVERFLOW, with *n_out = capacity, when more were made than the log
 * holds. */
int mqi_dij_get_hits(mqi_ctx* ctx, int scorer_id, uint32_t* voxel, uint32_t* spot, double* value,
                     uint64_t* n_out);

/* dose = D.w (n_voxels outputs from n_spots weights) and grad = D^T.g (n_spots outputs from
 * n_voxels inputs); fp64 selects double buffers (the matrix stays FP32).  With on_device = 1 the
 * buffers are device pointers and the work is queued on the context's stream without a sync.
 * Both use fixed reduction orders: repeated calls give identical bits.  Calls on one matrix share
 * its work buffers and must not overlap on the GPU (the context's stream orders them).
 * No reference counterpart: moqui stops at writing the matrix. */
int mqi_dij_matvec(mqi_ctx* ctx, int scorer_id, const void* w, void* dose, int fp64, int on_device);
int mqi_dij_rmatvec(mqi_ctx* ctx, int scorer_id, const void* g, void* grad, int fp64, int on_device);

/* Copy scorer `scorer_id`'s tally (FP64, roi mask size) to `out`.  Replaces download_node
 * (mqi_download_data.hpp:35-121) followed by x_environment::reshape_data
 * (moqui/base/environments/mqi_xenvironment.hpp:150-167).  `n_out` receives the element count;
 * `out` may be NULL to query it. */
int mqi_get_tally(mqi_ctx* ctx, int scorer_id, double* out, uint64_t* n_out, int on_device);

/* Zero every tally and the run counters. */
int mqi_reset_tallies(mqi_ctx* ctx);

int mqi_get_stats(mqi_ctx* ctx, mqi_stats* out);

/* Convert HU to density for n voxels (patient_material_t::hu_to_density, then * scale). */
int mqi_hu_to_density(mqi_ctx* ctx, const int16_t* hu, float* rho, uint64_t n, float scale,
                      int on_device);

/* Walk rays through a child grid exactly as the transport's voxel loop does
 * (mqi_transport.hpp:161-239) with the physics replaced by a boundary-only step.  rays: 6 floats
 * each (pos, dir; world frame).  For ray r, entries [offsets[r], offsets[r+1]) of cnb/dist/cell
 * hold the visited voxel, the exit distance grid3d::intersect returned there, and the cell.
 * At most max_steps entries per ray; `capacity` bounds the total.  n_out receives the total. */
int mqi_trace_rays(mqi_ctx* ctx, int child_id, const float* rays, uint64_t n_rays,
                   uint32_t max_steps, int64_t* offsets, uint64_t* cnb, float* dist,
                   int32_t* cells, uint64_t capacity, uint64_t* n_out);

/* Evaluate the transport's tabulated physics functions on the device, for parity tests.
 * For each energy E[i]: out[i*8 + {0..7}] = {cs_ion, cs_pp, cs_poe, cs_poi (per g/mm^3),
 * dEdx (negative, MeV/mm in water), beta^2, Te_max, momentum}. */
int mqi_eval_physics(mqi_ctx* ctx, const float* energies, uint64_t n, float* out);

/* Evaluate a scorer's callback on the device for given step states, for parity tests: the values
 * the transport's scoring forms for fp_compute_hit (moqui/base/scorers/mqi_scorer_energy_deposit.hpp:
 * 12-177) in voxel cnb[i] of child `child_id` (its densities and edges, the context's calibration
 * and physics setting).  steps: 9 floats per step -- vtx0.ke, dE, local_dE, vtx0.pos[3],
 * vtx1.pos[3]; primary: nonzero for a primary.  out: n doubles.  Before the ROI gate and the
 * "value > 0" filter of insert_hashtable. */
int mqi_eval_hits(mqi_ctx* ctx, int child_id, int scorer_type, const float* steps, const uint32_t* cnb,
                  const int32_t* primary, uint64_t n, double* out);

/* Evaluate scorer `scorer_id`'s ROI mapping on the device, for parity tests: roi_t::idx (the
 * scoring gate) and roi_t::get_mask_idx (the statistics key) of each voxel (moqui/base/mqi_roi.hpp:
 * 47-71, 87-160).  Where moqui's CONTOUR idx reads before its start array (a voxel below the first
 * run), the transport returns -1 (not scored). */
int mqi_eval_roi(mqi_ctx* ctx, int scorer_id, const uint32_t* voxels, uint64_t n, int32_t* idx,
                 int32_t* mask_idx);

/* ---- statistics --------------------------------------------------------------------------- */

/* Add tps_env's statistics pair to a child (Dose_stat and DoseSquare_stat,
 * moqui/base/environments/mqi_tps_env.hpp:936-960): per-step dose_to_water and its square, keyed by
 * the stat ROI's mask index (roi_t::get_mask_idx, moqui/base/mqi_roi.hpp:58-69) as the _stat
 * kernel's last two scorers are (mqi_transport.hpp:353-364).  DIRECT: every voxel (voxel 0
 * included); INDIRECT: roi_start holds one mask index per voxel (0xFFFFFFFF = outside) and
 * roi_length is the mask size; CONTOUR: start/stride/acc as roi_t.  A child carrying the pair is
 * scored like the _stat kernel: its other scorers are inserted once per step. */
int mqi_add_stat_scorers(mqi_ctx* ctx, int child_id, int roi_method, uint32_t roi_length,
                         const uint32_t* roi_start, const uint32_t* roi_stride,
                         const uint32_t* roi_acc, int* dose_id, int* dose2_id);

/* The reference's uncertainty estimate (calculate_standard_deviation,
 * moqui/kernel_functions/mqi_variables.hpp:19-48, and tps_env::calculate_stat,
 * moqui/base/environments/mqi_tps_env.hpp:1338-1426): with n histories, sigma_i =
 * sqrt((S2_i/n - (S1_i/n)^2)/(n-1)) and mean_i = S1_i/n per scored voxel; returns the average of
 * sigma_i/mean_i over voxels with mean_i > threshold * max_i mean_i, as a fraction (the reference
 * prints it x100), and the number of such voxels. */
int mqi_stat_uncertainty(mqi_ctx* ctx, int dose_id, int dose2_id, uint64_t n_histories,
                         float threshold, double* mean_rel_sigma, uint64_t* n_voxels);

/* Batch estimator (no counterpart in moqui, whose estimator squares per-step deposits): fold the
 * scorer's tally -- one batch of histories -- into running per-voxel sums of batch tallies and of
 * their squares, and zero the tally. */
int mqi_batch_accumulate(mqi_ctx* ctx, int scorer_id);

/* Relative standard error of the batch mean, averaged over voxels whose batch mean exceeds
 * threshold * max (>= 2 batches). */
int mqi_batch_uncertainty(mqi_ctx* ctx, int scorer_id, float threshold, double* mean_rel_sigma,
                          uint64_t* n_voxels, uint64_t* n_batches);

/* The batch-mean tally (sum of batches / number of batches). */
int mqi_get_batch_mean(mqi_ctx* ctx, int scorer_id, double* out, uint64_t* n_out, int on_device);

/* calculate_average (moqui/kernel_functions/mqi_variables.hpp:50-66): multiply a tally by weight. */
int mqi_scale_tally(mqi_ctx* ctx, int scorer_id, double weight);

/* tps_env::run_by_beam_stat (moqui/base/environments/mqi_tps_env.hpp:1241-1336): transport
 * histories [0, histories_per_run) again with a new seed until the reference estimate over the
 * stat pair is <= criteria (a fraction, e.g. 0.01) or max_runs runs are done, then scale the
 * child's other scorers by histories_per_run / histories_done (calculate_average_results,
 * :1428-1476).  The vertices are re-used each run (moqui re-samples them). */
int mqi_run_until_stat(mqi_ctx* ctx, int dose_id, int dose2_id, uint64_t histories_per_run,
                       float criteria, float threshold, uint64_t max_runs, uint64_t seed,
                       uint64_t* histories_done, double* achieved);

/* Launch shape of the transport (no counterpart in moqui, whose launch is fixed at 512 threads per
 * block).  block: threads per block (multiple of 32, <= 256); blocks_per_sm: resident blocks per
 * SM the wave kernel is launched with; slice_steps: voxel steps a track takes before it is
 * re-queued (0 = run each track to completion); primary_chunk: primaries loaded per queue
 * generation.  block, blocks_per_sm and primary_chunk keep their values when <= 0, slice_steps
 * when < 0.  Results do not depend on any of these. */
int mqi_set_tuning(mqi_ctx* ctx, int block, int blocks_per_sm, int slice_steps, int primary_chunk);

/* How the queue is driven (no counterpart in moqui, which runs one kernel over all histories).
 * streamed = 1 (default): before every wave the queue is topped up on the device with the next
 * histories, and graph_waves waves are captured once into a CUDA graph, so the host synchronises
 * once per graph_waves waves; streamed = 0: queue generations -- load primary_chunk histories,
 * run waves until a generation is empty, one host synchronisation per wave.  graph_waves must be
 * even (default 8); values <= 0 / < 0 keep the current setting.  Results do not depend on it. */
int mqi_set_launch_mode(mqi_ctx* ctx, int streamed, int graph_waves);

/* Where the post-step of a nuclear interaction (p-p elastic, p-O elastic, p-O inelastic; ~0.2% of
 * the steps) runs (no counterpart in moqui, which runs it inside the step, mqi_fippel_physics.hpp:
 * 178-196): 0 inside the wave kernel's step loop; 1 in a post-step kernel after each wave, which
 * takes that rarely used code out of the step loop (faster per step, one extra wave per
 * interaction); -1 (default) chooses 1 for runs of at least 2^19 queue entries (histories x
 * scenarios) and 0 below.  Results do not depend on it. */
int mqi_set_post_step_mode(mqi_ctx* ctx, int mode);

/* Sort the particle queue by energy before each wave that holds at least min_entries entries
 * (0: never; default 262144): a counting sort on 1 MeV kinetic-energy bins, highest first, so the
 * lanes of a warp step tracks of similar energy; primaries that have not taken a step yet follow,
 * in the order they were loaded (no counterpart in moqui, whose threads each pop their own
 * stack).  Protons are the only transported particle, so there is no type key.  Results do not
 * depend on it. */
int mqi_set_queue_sort(mqi_ctx* ctx, uint32_t min_entries);

/* One candidate of mqi_autotune and its measured rate. */
typedef struct {
    int      block;            /* threads per block of the wave kernel */
    int      blocks_per_sm;    /* resident blocks per SM it is launched with */
    int      streamed;         /* launch mode (mqi_set_launch_mode) */
    int      graph_waves;
    uint32_t primary_chunk;    /* queue entries a wave starts with / histories per generation */
    double   histories_per_s;  /* measured on the sample */
} mqi_tune_result;

/* Tuner (no counterpart in moqui): transport the sample [h0, h1) of the current source (vertices,
 * or the spot plan when source_plan = 1) once per candidate launch shape, queue size and launch
 * mode, into scratch tallies (the caller's tallies and counters are kept), and keep the fastest
 * candidate as the context's setting.  A sample of several queue loads (several times the queue
 * size, 2^21 entries by default, counting each history once per scenario) lets the launch modes'
 * behaviour at load boundaries show; on a single load they time alike.  Up to max_results
 * measurements go to `results`;
 * n_results receives the number of candidates run.  Results of later runs do not depend on the
 * choice.  Not with a Dij scorer present (add it after tuning). */
int mqi_autotune(mqi_ctx* ctx, int source_plan, uint64_t h0, uint64_t h1, uint64_t seed,
                 mqi_tune_result* results, uint32_t max_results, uint32_t* n_results);

/* Transport without any device allocation, for callers that cannot call cudaMalloc once running
 * (device memory owned by a pre-sized pool or another framework's allocator, plug-in hosts that
 * forbid allocation after start-up, loops that cannot afford cudaMalloc's device synchronisation).
 * No counterpart in the reference, whose upload/run path allocates on every call.
 *
 * The caller supplies every buffer as device memory on the current device: the grid edges
 * (nx+1, ny+1, nz+1 floats), the density (g/mm^3, x fastest), `n_histories` vertices, and the FP64
 * tally (nx*ny*nz doubles, DIRECT ROI, accumulated into, not cleared).  scorer_type is one of
 * EDEP, DOSE_W, DOSE_W2, DOSE_M.  Work is issued on `cuda_stream` (NULL = the legacy default
 * stream) and the call returns when it is done.
 *
 * The transport's own scratch (its particle queues) is a 24 MiB static device array in the
 * library, held by every GPU that loads it until the process exits.  At most 16777216 histories
 * per call (larger requests return MQI_ERR_INVALID); a queue generation that outgrows the
 * scratch returns MQI_ERR_OVERFLOW.  All calls share the array: calls whose GPU work overlaps
 * race and must be serialised.  Every call resolves the array's address on the current device
 * (cudaGetSymbolAddress); the physics tables are initialised in the library's device image, so
 * nothing is uploaded.  The first call on a device may load the library's device code there:
 * make it before any stream capture begins.  After a non-zero return the tally holds the partial sum of the histories
 * transported before the error: clear it before a retry.
 * Messages: mqi_last_error(NULL). */
int mqi_transport_noalloc(int nx, int ny, int nz, const float* d_xe, const float* d_ye,
                          const float* d_ze, const float* d_rho, const mqi_vertex* d_vertices,
                          uint64_t n_histories, int scorer_type, int physics_debug, uint64_t seed,
                          double* d_tally, void* cuda_stream);

/* One block of the engine's random-number generator, computed on the host: Philox4x32-10
 * (Salmon et al., SC'11) of counter[4] under key[2], written to out[4].  Every random number of a
 * transport is such a block, keyed by the run seed and countered by (block index, history, track
 * uid), so a caller can reproduce any track's stream.  No counterpart in moqui, which draws from
 * cuRAND's XORWOW state per history (mqi_transport.hpp:148). */
int mqi_philox4x32_10(const uint32_t* counter, const uint32_t* key, uint32_t* out);

/* Library version string. */
const char* mqi_version(void);

#ifdef __cplusplus
}
#endif

#endif /* MQI_GPU_H */
