// Internal interface between the C ABI (mqi_capi.cu) and the kernels (mqi_kernels.cu).
#pragma once

#include <cstdint>
#include <string>
#include <cuda_runtime.h>

#include "mqi_gpu.h"

namespace mqi_gpu
{

constexpr int kMaxChildren  = 4;
constexpr int kMaxScorers   = 8;
constexpr int kMaxScenarios = 64;

/// The queue's spot word: spot index (Dij column) in the low 24 bits, robust scenario in the high
/// 8 bits.  kNoSpot marks a history without a spot index.
constexpr uint32_t kSpotMask  = 0x00FFFFFFu;
constexpr uint32_t kNoSpot    = 0x00FFFFFFu;
constexpr int      kScenShift = 24;

/// One slot of a Dij table: key = ((spot << 32) | voxel) + 1, 0 = empty; value = FP64 dose.
/// The reference's key_value holds two 32-bit keys claimed by two separate CAS operations
/// (insert_hashtable, mqi_transport.hpp:68-111); one 64-bit CAS claims a slot atomically here.
struct alignas(16) DijSlot {
    unsigned long long key;
    double             value;
};

constexpr uint32_t kDijMaxProbes = 4096;   // linear-probe bound before the table counts as full

/// One recorded Dij insertion (mqi_dij_record_hits): the arguments insert_hashtable receives.
struct DijHit {
    uint32_t voxel;
    uint32_t spot;
    double   value;
};

/// Wave-kernel instance modes: the scoring code an instance carries.
constexpr int kModeDij  = 1;   // a Dij scorer
constexpr int kModeFull = 2;   // dose_to_medium or LET scorers
constexpr int kModeRoi  = 4;   // INDIRECT or CONTOUR ROI mappings
constexpr int kModeAll  = kModeDij | kModeFull | kModeRoi;
constexpr int kModeSingle = 8; // exactly one energy-deposit or dose-to-water scorer, DIRECT ROI,
                               // one child, no statistics pair, no scenarios (the phantom example)
constexpr int kModeStat = 16;  // one dose-to-water scorer and the statistics pair, DIRECT ROIs, on one
                               // child (any number of children and scenarios): tps_env's Dose with
                               // StoppingStatistics

/// Flat device description of one scorer (scorer<R> + roi_t, mqi_scorer.hpp:39-79,
/// mqi_roi.hpp:18-194).
struct ScorerDev {
    int             type;          // mqi_scorer_type
    int             roi_method;    // mqi_roi_method
    int             stat_mode;     // 1: gate/key by roi get_mask_idx (the _stat kernel's last scorers)
    int             double_score;  // 1: scored twice per step (non-stat kernel quirk, mqi_transport.hpp:204-225)
    uint32_t        roi_len;
    const uint32_t* start;
    const uint32_t* stride;
    const uint32_t* acc;
    double*         tally;         // dense: value of key k in scenario c at tally[(c * tally_len + k) * tstride]
    uint64_t        tally_len;
    uint32_t        tstride;       // 1, or 2 for the interleaved statistics pair (dose, dose^2)
    DijSlot*        dij;           // MQI_SCORER_DIJ: open-addressing table of dij_mask + 1 slots
    uint64_t        dij_mask;
    DijHit*         hit_log;       // optional: every insertion, appended (null: not recorded)
    unsigned long long* hit_count; // device: insertions recorded (counts on past hit_cap)
    uint64_t        hit_cap;
};

/// One child geometry: grid + the contiguous range of its scorers.
struct ChildDev {
    int          nx, ny, nz;
    const float* xe;
    const float* ye;
    const float* ze;
    const float* rho;
    float        rf[9], ri[9], tr[3];
    int          identity;
    int          scorer_begin, n_scorers;
};

/// Structure-of-arrays particle queue (replaces track_stack_t, mqi_track_stack.hpp:11-67).
struct Queue {
    float*    ke;      // vtx0.ke
    float*    px;      // position (world frame for phase ENTER, child frame for phase STEP)
    float*    py;
    float*    pz;
    float*    dx;
    float*    dy;
    float*    dz;
    float*    dE0;     // deposit carried from creation (debug-physics daughters)
    uint32_t* hist;    // history index
    uint32_t* uid_lo;  // track uid within the history (0 = primary)
    uint32_t* uid_hi;
    uint32_t* ctr;     // next Philox block of this track
    uint32_t* meta;    // below:16 | primary:1 | ke1_zero:1 | phase:1 | child:3 | npush:10 (bit layout in kernels)
    uint32_t* cell;    // voxel index (cnb) of a track re-queued mid-grid (phase STEP); the
                       // library keeps nx * ny * nz below 2^32, so any grid size round-trips
    uint32_t* spot;    // spot word of the history: spot | scenario << 24 (kNoSpot: no spot)
    uint32_t  capacity;
};

/// A track stopped by the wave kernel at a nuclear interaction (p-p elastic, p-O elastic or p-O
/// inelastic), after its along-step and the draw that chose the process: the post-step kernel runs
/// the process, scores the step, moves the track and queues it (and its daughters) for the next
/// wave.  These processes end ~0.2% of the steps, but their code is most of the step loop's
/// instructions and registers; taking it out of the loop shrinks what every step carries.
struct Deferred {
    float    ke0, ke1;
    float    p0[3], d0[3], p1[3];
    float    dE;
    float    spr0;     // SPR the step computed
    uint32_t cnb;      // voxel of the step
    uint32_t uid_lo, uid_hi, hist, spot;
    uint32_t meta;     // below | primary | child | npush, as the queue's meta word
    uint32_t ctr;      // Philox counter after the step's process draw
    uint32_t proc;     // 1 p-p elastic, 2 p-O elastic, 3 p-O inelastic
};

/// A tabulated calibration (mqi_set_calibration); mode 0 = the default curves.
struct CalibDev {
    int          mode;
    uint32_t     n_rho, n_e;
    float        rho0, drho, e0, de;
    const float* spr;   // device: n_rho x n_e, E fastest
    const float* x0;    // device: n_rho
};

/// Kernel parameters for one transport wave.
struct WaveParams {
    int       n_children;
    ChildDev  child[kMaxChildren];
    ScorerDev scorer[kMaxScorers];
    int       physics_debug;
    int       score_local;
    int       stack_limit;
    float     t_cut;
    uint32_t  k0, k1;           // Philox key (run seed)
    uint32_t  max_slice_steps;  // 0 = run each track to completion
    int       inline_local;     // score deposit-only daughters at creation (single-child worlds)
    int       kernel_mode;      // kModeDij | kModeFull | kModeRoi: the scoring code the run needs
    int       n_scen;           // robust scenarios (0 or 1: none)
    int       scen_child;       // the child the scenarios vary
    int       scen_stride;      // floats per scenario in scen_edges: nx+1 + ny+1 + nz+1
    const float* scen_edges;    // device: per-scenario x, y, z edges of scen_child
    float     scen_scale[kMaxScenarios];   // per-scenario density scale
    Queue     in;
    Queue     out;
    const uint32_t* n_in;       // device: number of entries in `in`
    uint32_t*       n_out;      // device: append cursor of `out`
    uint32_t*       head;       // device: fetch cursor of `in`
    unsigned long long* stats;  // device: mqi_stats fields (8 x u64)
    const uint32_t* spot_ids;   // per history (may be null)
    uint32_t*       error_flag; // device: 1 a bounded loop gave up, 2 queue overflow, 4 Dij table full
    int             split;      // 1: nuclear post-steps in the post-step kernel; 0: inside the wave
    Queue           sort_tmp;   // queue-sized scratch of the energy-bin sort (sort_bins null: no sort)
    uint32_t*       sort_bins;  // device: kSortBins counts (zero between sorts) then kSortBins cursors
    uint32_t        sort_min;   // sort a wave's input only when it holds at least this many entries
    Deferred*       def;        // device: tracks stopped at a nuclear interaction (capacity in.capacity)
    uint32_t*       n_def;      // device: entries in def (zeroed before each wave)
    int             smem_edge_floats; // shared-memory floats for staged child edges
    const float*    tables;     // device: the six physics tables, 6 x 600 floats in Tables order
                                // (followed by the 3996 HU density-correction factors)
    CalibDev        calib;      // SPR / X0 curves
};

std::string& thread_error_slot();

/// Device state of a streamed transport: before every wave the queue is topped up to `target`
/// entries with the next histories, so the GPU stays full until the last histories drain.
struct TopUp {
    unsigned long long next;   // next history to load
    unsigned long long end;    // one past the last history
    unsigned long long base;   // first history of the current top-up
    uint32_t target;           // queue entries a wave should start with
    uint32_t n_scen;           // queue entries per history (robust scenarios)
    uint32_t count;            // entries appended by the current top-up
    uint32_t dst;              // first appended entry
};

/// Classes of the queue sort: 1 MeV energy bins, the last one open (tracks above 319 MeV), and
/// one more class for primaries that have not taken a step yet.
constexpr int kSortBins = 321;

/// Record the calling thread's last error message (returned by mqi_last_error(NULL)).
void set_thread_error(const char* msg);

// ---- Dij (mqi_dij.cu) ----
cudaError_t dij_clear(DijSlot* tab, uint64_t cap, int sms, cudaStream_t s);
// Occupied slots of a Dij table into *out (cleared first).
cudaError_t dij_count(const DijSlot* tab, uint64_t cap, unsigned long long* out, int sms, cudaStream_t s);
cudaError_t dij_compact(const DijSlot* tab, uint64_t cap, uint64_t n_voxels, unsigned long long* keys, uint32_t* idx,
                        uint64_t n_max, unsigned long long* cursor, int sms, cudaStream_t s);
uint64_t    scan_scratch_words(uint64_t n);
cudaError_t scan_exclusive_u32(const uint32_t* in, uint32_t* out, uint64_t n, uint32_t* scratch, cudaStream_t s);
uint64_t    radix_hist_words(uint64_t n);
cudaError_t radix_sort_pairs(unsigned long long*& keys, uint32_t*& vals, unsigned long long*& keys_alt,
                             uint32_t*& vals_alt, uint64_t n, int bits, uint32_t* hist, uint32_t* offs,
                             uint32_t* scan_scratch, cudaStream_t s);
cudaError_t dij_row_bounds(const unsigned long long* keys, uint64_t n, uint64_t row_span, uint64_t n_rows,
                           uint64_t* indptr, cudaStream_t s);
cudaError_t dij_spot_rows(const unsigned long long* keys, const uint32_t* slot, uint64_t n, uint64_t n_voxels,
                          const DijSlot* tab, double scale, uint32_t* vox, float* val, unsigned long long* vkeys,
                          uint32_t* vpos, cudaStream_t s);
cudaError_t dij_row_flags(const unsigned long long* vkeys, uint64_t n, uint32_t* flags, cudaStream_t s);
cudaError_t dij_voxel_rows(const unsigned long long* vkeys, const uint32_t* vpos, uint64_t n,
                           const unsigned long long* skeys, uint64_t n_voxels, const float* sval, const uint32_t* flags,
                           const uint32_t* rowid, uint32_t* row_voxel, uint64_t* indptr, uint32_t* spot, float* val,
                           cudaStream_t s);
constexpr uint64_t kFwdEntries = 4096;    // entries whose rows one forward block owns
constexpr uint64_t kFwdStage   = 8192;    // staged products per forward block (rows up to 4096 entries)
cudaError_t dij_forward_blocks(const uint64_t* indptr, uint64_t n_rows, uint64_t nnz, uint32_t* row_first,
                               uint64_t* run_k, uint64_t* n_blocks, cudaStream_t s);
constexpr uint64_t kFwdPipeStageEntries = 6144;   // entries one stage of the persistent forward holds
constexpr int      kFwdStages           = 2;      // its ring of stages (one run in flight while one is summed)
constexpr int      kFwdPipeThreads      = 512;    // persistent forward block
constexpr int      kFwdPipeBlocksPerSm  = 2;      // two 96 KB blocks per SM
constexpr uint32_t kBulkSpinLimit = 1u << 20;   // bounded polls of a bulk-copy mbarrier
cudaError_t dij_forward(const uint32_t* row_voxel, const uint64_t* indptr, const uint32_t* row_first,
                        const uint64_t* run_k, uint64_t n_blocks, const uint32_t* spot, const float* val, const void* w,
                        void* dose, int fp64, uint32_t* err, int sms, cudaStream_t s);
constexpr uint64_t kDijSegment = 16384;   // entries per backward segment (segments never cross a row)
cudaError_t dij_seg_order_keys(const uint64_t* seg_start, uint32_t n_seg, const unsigned long long* keys,
                               uint64_t n_voxels, unsigned long long* okeys, uint32_t* oval, cudaStream_t s);
cudaError_t dij_backward(const uint32_t* order, const uint64_t* seg_start, uint32_t n_seg, const uint32_t* row_seg,
                         uint32_t n_rows, const uint32_t* vox, const float* val, double* partial, uint32_t* cursor,
                         const void* g, void* grad, int fp64, int sms, cudaStream_t s);

// ---- launchers (mqi_kernels.cu) ----
// Loaders: n histories from h0, each once per scenario (n_scen >= 1), scenario-interleaved:
// queue entry i holds history h0 + i / n_scen in scenario i % n_scen.
cudaError_t launch_load_primaries(const Queue& q, const mqi_vertex* v, const uint32_t* spot_ids, uint64_t h0, uint32_t n,
                                  uint32_t n_scen, cudaStream_t s);
cudaError_t launch_sample_primaries(const Queue& q, const mqi_spot* spots, const uint64_t* cum, uint32_t n_spots,
                                    uint64_t h0, uint32_t n, uint32_t n_scen, uint32_t k0, uint32_t k1, cudaStream_t s);
cudaError_t launch_sample_vertices(mqi_vertex* out, uint32_t* spot_out, const mqi_spot* spots, const uint64_t* cum,
                                   uint32_t n_spots, uint64_t h0, uint32_t n, uint32_t k0, uint32_t k1, cudaStream_t s);
// Streamed loaders: k_topup sizes the top-up of the queue whose count is *n_in (one thread), the
// loaders then append tu->count entries at tu->dst.
cudaError_t launch_topup(TopUp* tu, uint32_t* n_in, const uint32_t* error_flag, cudaStream_t s);
cudaError_t launch_load_topup(const Queue& q, const TopUp* tu, const mqi_vertex* v, const uint32_t* spot_ids, int sms,
                              cudaStream_t s);
cudaError_t launch_sample_topup(const Queue& q, const TopUp* tu, const mqi_spot* spots, const uint64_t* cum,
                                uint32_t n_spots, uint32_t k0, uint32_t k1, int sms, cudaStream_t s);
cudaError_t launch_wave(const WaveParams& p, int grid, int block, int blocks_per_sm, cudaStream_t s);
int         wave_smem_bytes(const WaveParams& p);
int         wave_edge_floats(const ChildDev* c, int n);
cudaError_t launch_hu_to_density(const float* corr, const int16_t* hu, float* rho, uint64_t n, float scale,
                                 cudaStream_t s);
cudaError_t launch_trace_rays(const ChildDev& c, const float* rays, uint64_t n_rays, uint32_t max_steps,
                              uint64_t* cnb, float* dist, int32_t* cells, uint32_t* counts, cudaStream_t s);
cudaError_t launch_stat(const double* s1, const double* s2, uint64_t n, uint32_t stride, double nh, int mode,
                        float threshold, int sms,
                        unsigned long long* scratch, cudaStream_t s);
cudaError_t launch_batch_fold(double* tally, uint32_t stride, double* s1, double* s2, uint64_t n, int sms, cudaStream_t s);
cudaError_t launch_scale(double* a, uint32_t stride, uint64_t n, double w, int sms, cudaStream_t s);
cudaError_t launch_copy_strided(const double* a, uint32_t stride, double* out, uint64_t n, int sms, cudaStream_t s);
cudaError_t launch_copy_scaled(const double* a, double* out, uint64_t n, double w, int sms, cudaStream_t s);
cudaError_t launch_eval_physics(const float* tables, const float* e, uint64_t n, float* out, cudaStream_t s);
cudaError_t launch_eval_hits(const ChildDev& c, const CalibDev& cal, int dbg, int type, const float* steps,
                             const uint32_t* cnb, const int32_t* prim, uint64_t n, double* out, cudaStream_t s);
cudaError_t launch_eval_roi(const ScorerDev& sc, const uint32_t* vox, uint64_t n, int32_t* idx, int32_t* mask,
                            cudaStream_t s);

}   // namespace mqi_gpu
