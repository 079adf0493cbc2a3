// Host-side state of a context (struct mqi_ctx of the C ABI) and the helpers every entry-point
// file uses.
//
// The reference keeps its device state in globals (mc::mc_world, mc_materials, mc_vertices,
// moqui/kernel_functions/mqi_variables.hpp:8-17) built by <<<1,1>>> kernels that call device-side
// `new` (mqi_upload_data.hpp:69-142).  Here a context owns flat device buffers, and every kernel
// receives what it reads by value.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "mqi_gpu.h"
#include "mqi_internal.h"

namespace mqi_gpu
{

struct ChildHost {
    int    nx = 0, ny = 0, nz = 0;
    float* xe = nullptr;
    float* ye = nullptr;
    float* ze = nullptr;
    float* rho = nullptr;
    bool   has_rho = false;
    float  rf[9], ri[9], tr[3];
    int    identity = 1;
};

/// A Dij scorer's built matrix: spot rows (the transposed operator, the reference's npz layout)
/// and voxel rows (only voxels with an entry).
struct DijCsr {
    bool      built = false;
    uint32_t  n_spots = 0;
    uint64_t  n_voxels = 0;
    uint64_t  nnz = 0;
    uint64_t  n_vrows = 0;
    uint64_t* s_indptr = nullptr;   // n_spots + 1
    uint32_t* s_voxel = nullptr;    // nnz
    float*    s_value = nullptr;    // nnz
    uint32_t* v_row = nullptr;      // n_vrows: voxel of each voxel row
    uint64_t* v_indptr = nullptr;   // n_vrows + 1
    uint32_t* v_spot = nullptr;     // nnz
    float*    v_value = nullptr;    // nnz
    uint64_t  n_seg = 0;            // backward segments: contiguous runs of one row's entries
    uint64_t* seg_start = nullptr;  // n_seg + 1
    uint32_t* row_seg = nullptr;    // n_spots + 1: first segment of each row
    uint32_t* seg_order = nullptr;  // n_seg: segments by first voxel (the backward's work order)
    uint32_t* bwd_cursor = nullptr; // the backward's work cursor (zero between calls)
    double*   partial = nullptr;    // n_seg
    uint64_t  n_fwd_blocks = 0;     // forward blocks: kFwdEntries entries' worth of voxel rows each
    uint32_t* fwd_row_first = nullptr;   // n_fwd_blocks + 1: first voxel row of each forward block
    uint64_t* fwd_run_k = nullptr;       // n_fwd_blocks + 1: first entry of each forward block's rows
};

struct ScorerHost {
    int       child = 0;
    int       type = 0;
    int       roi_method = 0;
    int       stat_mode = 0;
    uint32_t  roi_len = 0;
    uint32_t* start = nullptr;
    uint32_t* stride = nullptr;
    uint32_t* acc = nullptr;
    double*   tally = nullptr;
    uint64_t  tally_len = 0;       // per scenario; the tally holds copies * tally_len values
    uint32_t  copies = 1;          // robust scenarios: one tally per scenario, scenario-major
    uint32_t  tstride = 1;         // doubles between consecutive values (2: the interleaved stat pair)
    int       partner = -1;        // the stat pair's other scorer (shares the buffer)
    bool      owns = true;         // this scorer allocated `tally` (the dose half of the stat pair does)
    double*   batch_s1 = nullptr;   // batch estimator: running sums of batch tallies and squares
    double*   batch_s2 = nullptr;
    uint64_t  n_batches = 0;
    DijSlot*  dij = nullptr;        // MQI_SCORER_DIJ: hash table of dij_cap slots (power of two)
    uint64_t  dij_cap = 0;
    unsigned long long* dij_count = nullptr;   // device: occupied slots, counted on demand (dij_count())
    DijHit*   hit_log = nullptr;    // mqi_dij_record_hits: recorded insertions
    unsigned long long* hit_count = nullptr;
    uint64_t  hit_cap = 0;
    DijCsr    csr;

    uint64_t total() const { return tally_len * copies; }   // values (not doubles: see tstride)
};

struct QueueBuf {
    Queue    q{};
    void*    base = nullptr;
};

/// The calling thread's last error message.
std::string& thread_error_slot();

/// Free a Dij scorer's table and matrix (mqi_capi_dij.cu).
void dij_release(ScorerHost& s);
/// Empty a Dij scorer's table and drop its matrix.
cudaError_t dij_reset(ScorerHost& s, int sms, cudaStream_t st);

struct DeviceGuard {
    int prev = -1;
    explicit DeviceGuard(int dev) {
        cudaGetDevice(&prev);
        if (prev != dev) cudaSetDevice(dev);
    }
    ~DeviceGuard() {
        int cur = -1;
        cudaGetDevice(&cur);
        if (prev >= 0 && cur != prev) cudaSetDevice(prev);
    }
};

}   // namespace mqi_gpu

struct mqi_ctx {
    int                     device = 0;
    cudaStream_t            stream = nullptr;
    bool                    own_stream = false;
    std::string             err;
    int                     physics_debug = 0;
    int                     score_local = 1;
    std::vector<mqi_gpu::ChildHost>  children;
    std::vector<mqi_gpu::ScorerHost> scorers;
    mqi_vertex*             vertices = nullptr;
    uint64_t                n_vertices = 0;
    uint64_t                vertex_cap = 0;
    uint32_t*               spot_ids = nullptr;
    uint64_t                spot_cap = 0;
    bool                    has_spots = false;
    mqi_gpu::QueueBuf       qa, qb;
    uint32_t                queue_cap = 0;
    mqi_gpu::Deferred*      def = nullptr;          // tracks a wave stopped at nuclear interactions (queue_cap)
    mqi_gpu::QueueBuf       qsort;                  // scratch of the energy-bin queue sort (queue_cap)
    uint32_t*               sort_bins = nullptr;    // 2 x kSortBins counters of the sort
    uint32_t                sort_min = 1u << 18;    // sort waves of at least this many entries (0: never)
    uint32_t*               counters = nullptr;     // [0,1] queue sizes, [2] head, [3] error flag, [4] deferred
    unsigned long long*     stats = nullptr;        // 8 x u64
    uint32_t*               host_counts = nullptr;  // pinned: 4 x u32
    float*                  tables = nullptr;       // 6*600 physics + 3996 HU correction
    mqi_gpu::CalibDev       calib{};                // SPR / X0 curves (mode 0: the defaults)
    float*                  calib_buf = nullptr;    // device: the tables of calib (SPR then X0)
    int                     num_sms = 0;
    int                     wave_block = 128;
    int                     wave_grid = 0;
    uint32_t                max_slice_steps = 0;
    uint32_t                primary_chunk = 1u << 21;
    uint64_t                waves = 0;
    uint64_t                kernel_launches = 0;
    uint64_t                wave_launches = 0;
    double                  wave_ms = 0.0;
    cudaEvent_t             ev0 = nullptr, ev1 = nullptr;
    unsigned long long*     stat_scratch = nullptr;   // 3 x u64 for the statistics reductions
    mqi_spot*               plan_spots = nullptr;     // spot plan (device)
    uint64_t*               plan_cum = nullptr;       // cumulative histories, n_plan_spots + 1 (device)
    uint32_t                n_plan_spots = 0;
    uint64_t                plan_histories = 0;
    std::vector<uint64_t>   plan_cum_host;
    int                     streamed = 1;             // 1: device top-up + graph-captured waves; 0: generations
    int                     post_step_mode = -1;      // nuclear post-steps: -1 by run size, 0 in the wave, 1 post-step kernel
    int                     graph_waves = 8;          // waves per captured graph (even)
    mqi_gpu::TopUp*         topup = nullptr;          // device: streamed-transport state
    unsigned long long*     host_next = nullptr;      // pinned: TopUp::next after a graph launch
    cudaStream_t            cap_stream = nullptr;     // stream the graphs are captured on
    uint32_t                n_scen = 1;               // robust scenarios (1: none)
    int                     scen_child = -1;
    int                     scen_stride = 0;
    float*                  scen_edges = nullptr;     // device: n_scen x scen_stride
    std::vector<float>      scen_scale;
};

namespace mqi_gpu
{

inline int
fail(mqi_ctx* c, int code, const std::string& msg) {
    if (c) c->err = msg;
    thread_error_slot() = msg;
    return code;
}

/// Report a failed CUDA call.  The runtime keeps a non-sticky error as its "last error" until it
/// is read; it is read here, so that the next launch's cudaGetLastError reports that launch.
inline int
cuda_fail(mqi_ctx* c, cudaError_t e, const char* what) {
    (void) cudaGetLastError();
    return fail(c, e == cudaErrorMemoryAllocation ? MQI_ERR_NOMEM : MQI_ERR_CUDA,
                std::string(what) + ": " + cudaGetErrorString(e));
}

inline bool
valid_ctx(const mqi_ctx* c) {
    return c != nullptr;
}

}   // namespace mqi_gpu

#define MQI_CUDA(c, expr, what)                                        \
    do {                                                               \
        cudaError_t _e = (expr);                                       \
        if (_e != cudaSuccess) return mqi_gpu::cuda_fail(c, _e, what); \
    } while (0)
