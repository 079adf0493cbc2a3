// Reference GPU driver: test infrastructure only.
//
// Compiled with nvcc for sm_103a against the staged, patched copy of the reference headers
// (oracle/stage_ref.py), with the reference phantom example's own flags (-D__PHYSICS_DEBUG__
// --use_fast_math, tests/mc/phantom/CMakeLists.txt), so that the reference's own CUDA kernel
// mc::transport_particles_patient<float> (moqui/kernel_functions/mqi_transport.hpp:113-250) can be
// timed and its dose compared on the same GB300 as the product library.  Nothing in the product
// links it.
//
// Usage: ref_gpu_dbg <phantom_env CLI> [--beam uniform|gaussian] [--json <file>]
//
// The stock class mqi::phantom_env<float> (moqui/base/environments/mqi_phantom_env.hpp) does
// everything: CLI parsing, world/material/beam set-up, the device upload in
// x_environment::initialize, the download in finalize and the .raw/.mhd writer.  run() is
// overridden to follow the GPU branch of phantom_env::run (mqi_phantom_env.hpp:294-415) with three
// differences, none of which touches the kernel:
//   * CUDA events around the transport launch (the stock code times the whole of run() on the host
//     and prints it scaled by 1e-4);
//   * the per-history seed buffer is allocated for h1 entries (the stock sizeof(int32_t) * (h0-h1)
//     wraps to about 17 GB in unsigned arithmetic) and the tracked-particle counter for 4 bytes;
//   * the kernel's module is loaded (cudaFuncGetAttributes) before the start event, so lazy module
//     loading is not timed.
// The launch shape is the stock one (threads[0] x threads[1] from the constructor: 512 threads,
// ceil(N/512) blocks, capped at 65535), and the RNG set-up is the stock one: initialize_threads
// with master seed 0, then curand_init(transport_seed[i], 0, 0) per history inside the kernel with
// seeds drawn from std::default_random_engine seeded by --random_seed.
//
// Safety review before the first run on a GPU: the range-table loop whose uint16 index wraps
// (moqui/base/mqi_p_ionization.hpp:318-320) is guarded in the staged copy; the scorer table is
// addressed directly by voxel index for this single-scorer, no-spot configuration, so the
// open-addressing loop of insert_hashtable (mqi_transport.hpp:70-111) never probes; the
// secondary stack is bounded (track_stack_t::push_secondary).  The CPU build of the same headers
// ran clean under AddressSanitizer on these workloads.
#include <moqui/base/environments/mqi_phantom_env.hpp>
#include <moqui/kernel_functions/mqi_transport.hpp>

#include "ref_beams.hpp"

#include <chrono>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <string>
#include <vector>

namespace
{

#define REF_CHECK(call)                                                                            \
    do {                                                                                           \
        cudaError_t e_ = (call);                                                                   \
        if (e_ != cudaSuccess) {                                                                   \
            std::fprintf(stderr, "ref_gpu_driver: %s failed: %s\n", #call, cudaGetErrorString(e_)); \
            std::exit(3);                                                                          \
        }                                                                                          \
    } while (0)

class gpu_phantom_env : public mqi::phantom_env<float>
{
public:
    bool     gaussian    = false;
    float    kernel_ms   = 0.0f;
    double   run_ms      = 0.0;
    uint32_t tracked     = 0;
    int      regs        = 0;
    size_t   local_bytes = 0;

    gpu_phantom_env(mqi::cli& c, bool g) : mqi::phantom_env<float>(c), gaussian(g) {}

    void
    setup_beamsource() override {
        if (gaussian)
            gaussian_phantom_beamsource(*this);
        else
            mqi::phantom_env<float>::setup_beamsource();
    }

    void
    run() override {
        auto           t0 = std::chrono::steady_clock::now();
        const uint32_t h1 = this->beamsource.total_histories();
        this->num_spots   = this->beamsource.total_beamlets();
        std::vector<int32_t>       transport_seed(h1);
        std::default_random_engine tmp_rng;
        tmp_rng.seed(this->random_seed);
        for (uint32_t i = 0; i < h1; ++i)
            transport_seed[i] = tmp_rng();

        mc::upload_vertices(this->vertices, mc::mc_vertices, 0, h1);
        const uint32_t n_threads = this->threads[0] * this->threads[1];
        mqi::thrd_t*   worker_threads;
        REF_CHECK(cudaMalloc(&worker_threads, size_t(n_threads) * sizeof(mqi::thrd_t)));
        mqi::initialize_threads<<<this->threads[1], this->threads[0]>>>(worker_threads, n_threads, 0);
        REF_CHECK(cudaGetLastError());
        int32_t* d_seed;
        REF_CHECK(cudaMalloc(&d_seed, sizeof(int32_t) * size_t(h1)));
        REF_CHECK(cudaMemcpy(d_seed, transport_seed.data(), sizeof(int32_t) * size_t(h1), cudaMemcpyHostToDevice));
        uint32_t* d_tracked;
        REF_CHECK(cudaMalloc(&d_tracked, sizeof(uint32_t)));
        REF_CHECK(cudaMemset(d_tracked, 0, sizeof(uint32_t)));

        cudaFuncAttributes attr;
        REF_CHECK(cudaFuncGetAttributes(&attr, mc::transport_particles_patient<float>));
        regs        = attr.numRegs;
        local_bytes = attr.localSizeBytes;
        REF_CHECK(cudaDeviceSynchronize());

        cudaEvent_t e0, e1;
        REF_CHECK(cudaEventCreate(&e0));
        REF_CHECK(cudaEventCreate(&e1));
        REF_CHECK(cudaEventRecord(e0));
        mc::transport_particles_patient<float><<<this->threads[1], this->threads[0]>>>(
          worker_threads, mc::mc_world, mc::mc_vertices, mc::mc_materials, h1, d_tracked, d_seed);
        REF_CHECK(cudaGetLastError());
        REF_CHECK(cudaEventRecord(e1));
        REF_CHECK(cudaEventSynchronize(e1));
        REF_CHECK(cudaEventElapsedTime(&kernel_ms, e0, e1));
        REF_CHECK(cudaMemcpy(&tracked, d_tracked, sizeof(uint32_t), cudaMemcpyDeviceToHost));
        REF_CHECK(cudaEventDestroy(e0));
        REF_CHECK(cudaEventDestroy(e1));
        REF_CHECK(cudaFree(d_tracked));
        REF_CHECK(cudaFree(d_seed));
        REF_CHECK(cudaFree(worker_threads));
        REF_CHECK(cudaFree(mc::mc_vertices));
        run_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    }
};

}   // namespace

int
main(int argc, char** argv) {
    bool               gaussian = false;
    std::string        json;
    std::vector<char*> rest;
    rest.push_back(argv[0]);
    for (int i = 1; i < argc; ++i) {
        if (!std::strcmp(argv[i], "--beam") && i + 1 < argc) {
            gaussian = !std::strcmp(argv[++i], "gaussian");
        } else if (!std::strcmp(argv[i], "--json") && i + 1 < argc) {
            json = argv[++i];
        } else {
            rest.push_back(argv[i]);
        }
    }
    mqi::cli cl;
    cl.read(static_cast<int>(rest.size()), rest.data());
    gpu_phantom_env env(cl, gaussian);
    env.initialize();
    env.run();
    env.finalize();
    env.save_reshaped_files();
    if (!json.empty()) {
        std::ofstream f(json);
        f << "{\"kernel_ms\": " << env.kernel_ms << ", \"run_ms\": " << env.run_ms
          << ", \"histories\": " << env.beamsource.total_histories() << ", \"tracked\": " << env.tracked
          << ", \"blocks\": " << env.threads[1] << ", \"threads\": " << env.threads[0]
          << ", \"registers\": " << env.regs << ", \"local_bytes\": " << env.local_bytes
#ifdef __PHYSICS_DEBUG__
          << ", \"physics_debug\": 1"
#else
          << ", \"physics_debug\": 0"
#endif
          << "}\n";
    }
    return 0;
}
