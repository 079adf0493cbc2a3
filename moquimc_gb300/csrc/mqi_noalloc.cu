// mqi_transport_noalloc: the transport for callers that cannot allocate device memory.
//
// Some callers of this library may not call cudaMalloc once they are running: a treatment-planning
// or serving process whose device memory is owned by a pre-sized pool or by another framework's
// allocator, a plug-in host that forbids allocation after start-up, or a latency-bound loop that
// cannot afford cudaMalloc's implicit device synchronisation.  For them this entry point
// transports histories with every buffer supplied by the caller except the transport's own
// scratch -- the two particle queues and their counters -- which lives in a file-scope static
// device array that each GPU loading the library holds until the process exits.
//
// Limits and sharing, stated once for users:
//   * the scratch is kNoallocScratchBytes (24 MiB): queues of kNoallocQueueCap entries, i.e. at
//     most kNoallocChunk primaries per queue generation; a call processes its histories in such
//     chunks and accepts at most kNoallocMaxHistories histories;
//   * every call shares the one array and leaves its contents behind; the counters a call needs
//     at zero are cleared by the call itself, on the caller's stream;
//   * two calls whose GPU work overlaps (different streams or host threads) race on the array:
//     serialise them;
//   * every call resolves the array's device address (cudaGetSymbolAddress) with the caller's
//     device current; the physics tables sit in a second static array initialised in the module
//     image, so nothing is copied, and a context that is torn down and created again
//     (cudaDeviceReset) finds them again.  The first call on a device may load the library's
//     device code there: make that first call before any stream capture begins;
//   * each call returns after its work on the stream has completed; on an error return the
//     tally holds a partial sum of the histories transported so far and must be cleared by the
//     caller before a retry.
// Errors are reported as status codes; mqi_last_error(NULL) returns the message.
#include <string>

#include <cuda_runtime.h>

#include "mqi_device.cuh"
#include "mqi_gpu.h"
#include "mqi_internal.h"

using namespace mqi_gpu;

namespace
{

constexpr uint32_t kNoallocChunk        = 1u << 16;            // primaries per queue generation
constexpr uint32_t kNoallocQueueCap     = 3u * kNoallocChunk;  // entries per queue
constexpr size_t   kNoallocCol          = (size_t) kNoallocQueueCap * 4;   // bytes per queue column
constexpr int      kNoallocCols         = 15;
constexpr size_t   kNoallocQueueBytes   = kNoallocCol * kNoallocCols;
constexpr size_t   kNoallocCounterBytes = 256;                 // 8 x u32 counters, 8 x u64 stats
constexpr size_t   kNoallocScratchBytes = 24u << 20;
constexpr uint64_t kNoallocMaxHistories = 1ull << 24;
constexpr int      kNoallocTableFloats  = 6 * MQI_TABLE_N + MQI_DENSITY_CORRECTION_N;

static_assert(2 * kNoallocQueueBytes + kNoallocCounterBytes <= kNoallocScratchBytes, "scratch too small");
static_assert(kNoallocCol % 256 == 0, "queue columns must stay 256-byte aligned");

// The scratch: two SoA particle queues followed by the wave counters and run statistics.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoallocScratchBytes];
// The physics tables the wave kernel stages into shared memory, in its order (the six 600-node
// tables, then the HU density-correction factors), initialised at compile time.
struct NoallocTables {
    float v[kNoallocTableFloats];
};

constexpr NoallocTables
noalloc_tables_init() {
    NoallocTables t{};
    for (int i = 0; i < MQI_TABLE_N; ++i) {
        t.v[0 * MQI_TABLE_N + i] = mqi_tab_cs_p_ion[i];
        t.v[1 * MQI_TABLE_N + i] = mqi_tab_dedx[i];
        t.v[2 * MQI_TABLE_N + i] = mqi_tab_range[i];
        t.v[3 * MQI_TABLE_N + i] = mqi_tab_cs_pp_e[i];
        t.v[4 * MQI_TABLE_N + i] = mqi_tab_cs_po_e[i];
        t.v[5 * MQI_TABLE_N + i] = mqi_tab_cs_po_i[i];
    }
    for (int i = 0; i < MQI_DENSITY_CORRECTION_N; ++i) t.v[6 * MQI_TABLE_N + i] = mqi_tab_density_correction[i];
    return t;
}

static __device__ __align__(256) NoallocTables g_noalloc_tables = noalloc_tables_init();

int
noalloc_fail(int code, const std::string& msg) {
    if (code == MQI_ERR_CUDA) (void) cudaGetLastError();   // read a failed call's error so the next launch reports its own
    set_thread_error(msg.c_str());
    return code;
}

/// The static arrays' device addresses on the current device.  The symbol names are host-side
/// stand-ins; only the addresses returned here may be handed to a kernel.
int
resolve_scratch(void** scratch, float** tables) {
    void*       t = nullptr;
    cudaError_t e = cudaGetSymbolAddress(scratch, g_noalloc_scratch);
    if (e != cudaSuccess)
        return noalloc_fail(MQI_ERR_CUDA, std::string("mqi_transport_noalloc: cudaGetSymbolAddress(scratch): ") + cudaGetErrorString(e));
    e = cudaGetSymbolAddress(&t, g_noalloc_tables);
    if (e != cudaSuccess)
        return noalloc_fail(MQI_ERR_CUDA, std::string("mqi_transport_noalloc: cudaGetSymbolAddress(tables): ") + cudaGetErrorString(e));
    *tables = static_cast<float*>(t);
    return MQI_OK;
}

Queue
carve_queue(unsigned char* base) {
    Queue q{};
    auto  f = [&](int k) { return reinterpret_cast<float*>(base + kNoallocCol * k); };
    auto  u = [&](int k) { return reinterpret_cast<uint32_t*>(base + kNoallocCol * k); };
    q.ke = f(0); q.px = f(1); q.py = f(2); q.pz = f(3);
    q.dx = f(4); q.dy = f(5); q.dz = f(6); q.dE0 = f(7);
    q.hist = u(8); q.uid_lo = u(9); q.uid_hi = u(10); q.ctr = u(11); q.meta = u(12);
    q.cell = reinterpret_cast<uint32_t*>(base + kNoallocCol * 13);
    q.spot = u(14);
    q.capacity = kNoallocQueueCap;
    return q;
}

}   // namespace

extern "C" {

int
mqi_transport_noalloc(int nx, int ny, int nz, const float* d_xe, const float* d_ye, const float* d_ze,
                      const float* d_rho, const mqi_vertex* d_vertices, uint64_t n_histories, int scorer_type,
                      int physics_debug, uint64_t seed, double* d_tally, void* cuda_stream) {
    if (nx <= 0 || ny <= 0 || nz <= 0 || nx > 2047 || ny > 2047 || nz > 2047)
        return noalloc_fail(MQI_ERR_INVALID, "mqi_transport_noalloc: grid dimensions must be 1..2047");
    if (!d_xe || !d_ye || !d_ze || !d_rho || !d_tally || (!d_vertices && n_histories))
        return noalloc_fail(MQI_ERR_INVALID, "mqi_transport_noalloc: a required device pointer is NULL");
    if (n_histories > kNoallocMaxHistories)
        return noalloc_fail(MQI_ERR_INVALID, "mqi_transport_noalloc: at most 16777216 histories per call "
                                             "(the static scratch holds 65536-primary queue generations)");
    if (scorer_type != MQI_SCORER_EDEP && scorer_type != MQI_SCORER_DOSE_W && scorer_type != MQI_SCORER_DOSE_W2 &&
        scorer_type != MQI_SCORER_DOSE_M)
        return noalloc_fail(MQI_ERR_UNSUPPORTED, "mqi_transport_noalloc: scorer must be EDEP, DOSE_W, DOSE_W2 or DOSE_M");
    if (n_histories == 0) return MQI_OK;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return noalloc_fail(MQI_ERR_CUDA, std::string("mqi_transport_noalloc: cudaGetDevice: ") + cudaGetErrorString(e));
    void*  scratch = nullptr;
    float* tables  = nullptr;
    const int rc = resolve_scratch(&scratch, &tables);
    if (rc != MQI_OK) return rc;
    int sms = 0;
    e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return noalloc_fail(MQI_ERR_CUDA, std::string("mqi_transport_noalloc: device query: ") + cudaGetErrorString(e));
    cudaStream_t   stream   = static_cast<cudaStream_t>(cuda_stream);
    unsigned char* base     = static_cast<unsigned char*>(scratch);
    uint32_t*      counters = reinterpret_cast<uint32_t*>(base + 2 * kNoallocQueueBytes);
    auto*          stats    = reinterpret_cast<unsigned long long*>(base + 2 * kNoallocQueueBytes + 64);
    Queue          qa       = carve_queue(base);
    Queue          qb       = carve_queue(base + kNoallocQueueBytes);

    WaveParams P{};
    P.n_children = 1;
    ChildDev& ch = P.child[0];
    ch.nx = nx; ch.ny = ny; ch.nz = nz;
    ch.xe = d_xe; ch.ye = d_ye; ch.ze = d_ze; ch.rho = d_rho;
    for (int i = 0; i < 9; ++i) ch.rf[i] = ch.ri[i] = (i % 4 == 0) ? 1.0f : 0.0f;
    ch.tr[0] = ch.tr[1] = ch.tr[2] = 0.0f;
    ch.identity     = 1;
    ch.scorer_begin = 0;
    ch.n_scorers    = 1;
    ScorerDev& sc = P.scorer[0];
    sc.type       = scorer_type;
    sc.roi_method = MQI_ROI_DIRECT;
    sc.tally      = d_tally;
    sc.tally_len  = (uint64_t) nx * ny * nz;
    sc.tstride    = 1;
    if (scorer_type == MQI_SCORER_DOSE_M || (scorer_type >= MQI_SCORER_LETD_NUM && scorer_type <= MQI_SCORER_LETT_DEN))
        P.kernel_mode = kModeFull;
    else if (scorer_type == MQI_SCORER_EDEP || scorer_type == MQI_SCORER_DOSE_W)
        P.kernel_mode = kModeSingle;
    P.physics_debug    = physics_debug ? 1 : 0;
    P.score_local      = 1;
    P.stack_limit      = physics_debug ? 200 : 10;
    P.t_cut            = physics_debug ? kTcutDebug : kTcutRelease;
    P.k0               = (uint32_t) seed;
    P.k1               = (uint32_t) (seed >> 32);
    P.max_slice_steps  = 0;
    P.inline_local     = 1;
    P.head             = counters + 2;
    P.error_flag       = counters + 3;
    P.split            = 0;   // nuclear post-steps inside the wave: no post-step records to hold
    P.stats            = stats;
    P.spot_ids         = nullptr;
    P.tables           = tables;
    P.smem_edge_floats = wave_edge_floats(P.child, 1);

    // counters and statistics start at zero for every call (the array keeps the last call's)
    e = cudaMemsetAsync(counters, 0, kNoallocCounterBytes, stream);
    if (e != cudaSuccess) return noalloc_fail(MQI_ERR_CUDA, std::string("mqi_transport_noalloc: ") + cudaGetErrorString(e));
    const int block = 128, grid = sms * 5;
    Queue*    A = &qa;
    Queue*    B = &qb;
    for (uint64_t h = 0; h < n_histories; h += kNoallocChunk) {
        const uint32_t n = (uint32_t) ((n_histories - h) < kNoallocChunk ? (n_histories - h) : kNoallocChunk);
        e = launch_load_primaries(*A, d_vertices, nullptr, h, n, 1, stream);
        // a copy from pageable host memory returns once its source has been staged, so `n` may
        // change before the copy reaches the device
        if (e == cudaSuccess) e = cudaMemcpyAsync(counters, &n, sizeof(uint32_t), cudaMemcpyHostToDevice, stream);
        if (e != cudaSuccess) return noalloc_fail(MQI_ERR_CUDA, std::string("mqi_transport_noalloc: ") + cudaGetErrorString(e));
        int cur = 0;
        for (int wave = 0;; ++wave) {
            if (wave > 100000) return noalloc_fail(MQI_ERR_DEVICE, "mqi_transport_noalloc: wave limit reached");
            P.in    = *A;
            P.out   = *B;
            P.n_in  = counters + cur;
            P.n_out = counters + (1 - cur);
            uint32_t host_counts[4] = { 0, 0, 0, 0 };
            e = cudaMemsetAsync(counters + (1 - cur), 0, sizeof(uint32_t), stream);
            if (e == cudaSuccess) e = cudaMemsetAsync(counters + 2, 0, sizeof(uint32_t), stream);
            if (e == cudaSuccess) e = launch_wave(P, grid, block, grid / sms, stream);
            if (e == cudaSuccess) e = cudaMemcpyAsync(host_counts, counters, sizeof(host_counts), cudaMemcpyDeviceToHost, stream);
            if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
            if (e != cudaSuccess) return noalloc_fail(MQI_ERR_CUDA, std::string("mqi_transport_noalloc: ") + cudaGetErrorString(e));
            if (host_counts[3] & 2u) return noalloc_fail(MQI_ERR_OVERFLOW, "mqi_transport_noalloc: particle queue overflow (static scratch)");
            if (host_counts[3] & 1u) return noalloc_fail(MQI_ERR_DEVICE, "mqi_transport_noalloc: a bounded device loop gave up");
            if (host_counts[1 - cur] == 0) break;
            Queue* t = A;
            A        = B;
            B        = t;
            cur      = 1 - cur;
        }
    }
    return MQI_OK;
}

}   // extern "C"
