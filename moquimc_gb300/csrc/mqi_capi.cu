// C ABI of the GB300 proton transport engine: context, buffers and the wave loop.
//
// The reference keeps its device state in globals (mc::mc_world, mc_materials, mc_vertices,
// moqui/kernel_functions/mqi_variables.hpp:8-17) built by <<<1,1>>> kernels that call device-side
// `new` (mqi_upload_data.hpp:69-142).  Here a context owns flat device buffers, and every kernel
// receives what it reads by value.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "mqi_device.cuh"
#include "mqi_gpu.h"
#include "mqi_ctx.h"
#include "mqi_internal.h"

using namespace mqi_gpu;

namespace
{

void
free_queue(QueueBuf& b) {
    if (b.base) cudaFree(b.base);
    b.base = nullptr;
    b.q    = Queue{};
}

/// One allocation per queue, carved into the SoA columns (each 256-byte aligned).
cudaError_t
alloc_queue(QueueBuf& b, uint32_t cap) {
    free_queue(b);
    const size_t col   = ((size_t) cap * 4 + 255) & ~(size_t) 255;
    const int    ncols = 15;
    cudaError_t  e     = cudaMalloc(&b.base, col * ncols);
    if (e != cudaSuccess) return e;
    char* p = static_cast<char*>(b.base);
    auto  f = [&](int k) { return reinterpret_cast<float*>(p + col * k); };
    auto  u = [&](int k) { return reinterpret_cast<uint32_t*>(p + col * k); };
    b.q.ke = f(0); b.q.px = f(1); b.q.py = f(2); b.q.pz = f(3);
    b.q.dx = f(4); b.q.dy = f(5); b.q.dz = f(6); b.q.dE0 = f(7);
    b.q.hist = u(8); b.q.uid_lo = u(9); b.q.uid_hi = u(10); b.q.ctr = u(11); b.q.meta = u(12);
    b.q.cell = reinterpret_cast<uint32_t*>(p + col * 13);
    b.q.spot = u(14);
    b.q.capacity = cap;
    return cudaSuccess;
}

void
identity3(float* m) {
    for (int i = 0; i < 9; ++i) m[i] = (i % 4 == 0) ? 1.0f : 0.0f;
}

}   // namespace

std::string&
mqi_gpu::thread_error_slot() {
    thread_local std::string msg;
    return msg;
}

void
mqi_gpu::set_thread_error(const char* msg) {
    thread_error_slot() = msg ? msg : "";
}

extern "C" {

const char*
mqi_version(void) {
    return "mqi-gb300 0.1 (sm_103a)";
}

int
mqi_set_post_step_mode(mqi_ctx* c, int mode) {
    if (!valid_ctx(c)) return fail(c, MQI_ERR_INVALID, "mqi_set_post_step_mode: ctx is NULL");
    if (mode < -1 || mode > 1) return fail(c, MQI_ERR_INVALID, "mqi_set_post_step_mode: mode must be -1, 0 or 1");
    c->post_step_mode = mode;
    return MQI_OK;
}

int
mqi_set_queue_sort(mqi_ctx* c, uint32_t min_entries) {
    if (!valid_ctx(c)) return fail(c, MQI_ERR_INVALID, "mqi_set_queue_sort: ctx is NULL");
    c->sort_min = min_entries;
    return MQI_OK;
}

int
mqi_philox4x32_10(const uint32_t* counter, const uint32_t* key, uint32_t* out) {
    if (!counter || !key || !out) {
        set_thread_error("mqi_philox4x32_10: a pointer is NULL");
        return MQI_ERR_INVALID;
    }
    const u32x4 r = philox4x32_10(u32x4{ counter[0], counter[1], counter[2], counter[3] }, key[0], key[1]);
    out[0] = r.x;
    out[1] = r.y;
    out[2] = r.z;
    out[3] = r.w;
    return MQI_OK;
}

const char*
mqi_last_error(const mqi_ctx* ctx) {
    return ctx ? ctx->err.c_str() : thread_error_slot().c_str();
}

int
mqi_create(int device, mqi_ctx** out) {
    if (!out) return fail(nullptr, MQI_ERR_INVALID, "mqi_create: out is NULL");
    *out = nullptr;
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess) return cuda_fail(nullptr, e, "mqi_create: cudaGetDeviceCount");
    if (device < 0 || device >= n) return fail(nullptr, MQI_ERR_INVALID, "mqi_create: no such device");
    auto* c   = new mqi_ctx();
    c->device = device;
    DeviceGuard g(device);
    cudaDeviceProp prop{};
    if ((e = cudaGetDeviceProperties(&prop, device)) != cudaSuccess) {
        delete c;
        return cuda_fail(nullptr, e, "mqi_create: cudaGetDeviceProperties");
    }
    c->num_sms = prop.multiProcessorCount;
    if ((e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking)) != cudaSuccess) {
        delete c;
        return cuda_fail(nullptr, e, "mqi_create: cudaStreamCreate");
    }
    c->own_stream = true;
    const size_t tbytes = (6 * MQI_TABLE_N + MQI_DENSITY_CORRECTION_N) * sizeof(float);
    std::vector<float> host(6 * MQI_TABLE_N + MQI_DENSITY_CORRECTION_N);
    std::memcpy(&host[0 * MQI_TABLE_N], mqi_tab_cs_p_ion, sizeof(mqi_tab_cs_p_ion));
    std::memcpy(&host[1 * MQI_TABLE_N], mqi_tab_dedx, sizeof(mqi_tab_dedx));
    std::memcpy(&host[2 * MQI_TABLE_N], mqi_tab_range, sizeof(mqi_tab_range));
    std::memcpy(&host[3 * MQI_TABLE_N], mqi_tab_cs_pp_e, sizeof(mqi_tab_cs_pp_e));
    std::memcpy(&host[4 * MQI_TABLE_N], mqi_tab_cs_po_e, sizeof(mqi_tab_cs_po_e));
    std::memcpy(&host[5 * MQI_TABLE_N], mqi_tab_cs_po_i, sizeof(mqi_tab_cs_po_i));
    std::memcpy(&host[6 * MQI_TABLE_N], mqi_tab_density_correction, sizeof(mqi_tab_density_correction));
    if ((e = cudaMalloc(&c->tables, tbytes)) != cudaSuccess ||
        (e = cudaMemcpy(c->tables, host.data(), tbytes, cudaMemcpyHostToDevice)) != cudaSuccess ||
        (e = cudaMalloc(&c->counters, 8 * sizeof(uint32_t))) != cudaSuccess ||
        (e = cudaMemset(c->counters, 0, 8 * sizeof(uint32_t))) != cudaSuccess ||
        (e = cudaMalloc(&c->stats, 8 * sizeof(unsigned long long))) != cudaSuccess ||
        (e = cudaMemset(c->stats, 0, 8 * sizeof(unsigned long long))) != cudaSuccess ||
        (e = cudaMallocHost(&c->host_counts, 8 * sizeof(uint32_t))) != cudaSuccess ||
        (e = cudaMallocHost(&c->host_next, sizeof(unsigned long long))) != cudaSuccess ||
        (e = cudaMalloc(&c->topup, sizeof(TopUp))) != cudaSuccess ||
        (e = cudaStreamCreateWithFlags(&c->cap_stream, cudaStreamNonBlocking)) != cudaSuccess ||
        (e = cudaEventCreate(&c->ev0)) != cudaSuccess || (e = cudaEventCreate(&c->ev1)) != cudaSuccess) {
        mqi_destroy(c);
        return cuda_fail(nullptr, e, "mqi_create: allocation");
    }
    c->wave_grid = c->num_sms * 5;   // 128-thread blocks, 5 per SM (96 registers): fastest measured shape
    *out = c;
    return MQI_OK;
}

int
mqi_destroy(mqi_ctx* c) {
    if (!c) return MQI_OK;
    DeviceGuard g(c->device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    for (auto& ch : c->children) {
        cudaFree(ch.xe); cudaFree(ch.ye); cudaFree(ch.ze); cudaFree(ch.rho);
    }
    for (auto& s : c->scorers) {
        cudaFree(s.start); cudaFree(s.stride); cudaFree(s.acc);
        if (s.owns) cudaFree(s.tally);
        cudaFree(s.batch_s1); cudaFree(s.batch_s2);
        dij_release(s);
    }
    cudaFree(c->stat_scratch);
    cudaFree(c->plan_spots);
    cudaFree(c->plan_cum);
    cudaFree(c->scen_edges);
    cudaFree(c->vertices);
    cudaFree(c->spot_ids);
    free_queue(c->qa);
    free_queue(c->qb);
    free_queue(c->qsort);
    cudaFree(c->sort_bins);
    cudaFree(c->def);
    cudaFree(c->counters);
    cudaFree(c->stats);
    cudaFree(c->tables);
    cudaFree(c->calib_buf);
    if (c->host_counts) cudaFreeHost(c->host_counts);
    if (c->host_next) cudaFreeHost(c->host_next);
    cudaFree(c->topup);
    if (c->cap_stream) cudaStreamDestroy(c->cap_stream);
    if (c->ev0) cudaEventDestroy(c->ev0);
    if (c->ev1) cudaEventDestroy(c->ev1);
    if (c->own_stream && c->stream) cudaStreamDestroy(c->stream);
    delete c;
    return MQI_OK;
}

int
mqi_set_stream(mqi_ctx* c, void* s) {
    if (!valid_ctx(c)) return fail(c, MQI_ERR_INVALID, "mqi_set_stream: ctx is NULL");
    if (s && !c->own_stream && c->stream == static_cast<cudaStream_t>(s)) return MQI_OK;
    DeviceGuard g(c->device);
    if (c->own_stream && c->stream) {
        cudaStreamSynchronize(c->stream);
        cudaStreamDestroy(c->stream);
    }
    if (s) {
        c->stream     = static_cast<cudaStream_t>(s);
        c->own_stream = false;
    } else {
        MQI_CUDA(c, cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking), "mqi_set_stream");
        c->own_stream = true;
    }
    return MQI_OK;
}

int
mqi_set_tuning(mqi_ctx* c, int block, int blocks_per_sm, int slice_steps, int primary_chunk) {
    if (!valid_ctx(c)) return fail(c, MQI_ERR_INVALID, "mqi_set_tuning: ctx is NULL");
    if (block > 0) {
        if (block % 32 != 0 || block > 256) return fail(c, MQI_ERR_INVALID, "mqi_set_tuning: block must be a multiple of 32, <= 256");
        c->wave_block = block;
    }
    if (blocks_per_sm > 0) {
        if (blocks_per_sm > 64) return fail(c, MQI_ERR_INVALID, "mqi_set_tuning: blocks_per_sm must be <= 64");
        c->wave_grid = c->num_sms * blocks_per_sm;
    }
    if (slice_steps >= 0) c->max_slice_steps = (uint32_t) slice_steps;
    if (primary_chunk > 0) {
        if (primary_chunk > (1 << 24)) return fail(c, MQI_ERR_INVALID, "mqi_set_tuning: primary_chunk must be <= 2^24");
        c->primary_chunk = (uint32_t) primary_chunk;
    }
    return MQI_OK;
}

int
mqi_set_launch_mode(mqi_ctx* c, int streamed, int graph_waves) {
    if (!valid_ctx(c)) return fail(c, MQI_ERR_INVALID, "mqi_set_launch_mode: ctx is NULL");
    if (graph_waves > 0) {
        if (graph_waves % 2 != 0 || graph_waves > 64)
            return fail(c, MQI_ERR_INVALID, "mqi_set_launch_mode: graph_waves must be even and <= 64");
        c->graph_waves = graph_waves;
    }
    if (streamed >= 0) c->streamed = streamed ? 1 : 0;
    return MQI_OK;
}

int
mqi_set_physics(mqi_ctx* c, int physics_debug, int score_local_deposit) {
    if (!valid_ctx(c)) return fail(c, MQI_ERR_INVALID, "mqi_set_physics: ctx is NULL");
    c->physics_debug = physics_debug ? 1 : 0;
    c->score_local   = score_local_deposit ? 1 : 0;
    return MQI_OK;
}

int
mqi_set_calibration(mqi_ctx* c, int calib, uint32_t n_rho, float rho0, float drho, uint32_t n_e, float e0, float de,
                    const float* spr, const float* x0) {
    if (!valid_ctx(c)) return fail(c, MQI_ERR_INVALID, "mqi_set_calibration: ctx is NULL");
    if (calib == MQI_CALIB_DEFAULT) {
        c->calib = CalibDev{};
        return MQI_OK;
    }
    if (calib != MQI_CALIB_TABLE) return fail(c, MQI_ERR_INVALID, "mqi_set_calibration: unknown calibration");
    if (n_rho < 2 || n_e < 2 || !(drho > 0.0f) || !(de > 0.0f) || !std::isfinite(rho0) || !std::isfinite(e0) ||
        !std::isfinite(drho) || !std::isfinite(de) || !spr || !x0 || n_rho > (1u << 20) || n_e > (1u << 20) ||
        (uint64_t) n_rho * n_e > (1ull << 26))
        return fail(c, MQI_ERR_INVALID, "mqi_set_calibration: tables need n >= 2, positive finite pitches, data");
    const size_t n_spr = (size_t) n_rho * n_e;
    for (size_t i = 0; i < n_spr; ++i)
        if (!std::isfinite(spr[i])) return fail(c, MQI_ERR_INVALID, "mqi_set_calibration: SPR table is not finite");
    for (uint32_t i = 0; i < n_rho; ++i)
        if (!std::isfinite(x0[i]) || !(x0[i] > 0.0f))
            return fail(c, MQI_ERR_INVALID, "mqi_set_calibration: X0 table must be finite and positive");
    DeviceGuard g(c->device);
    cudaStreamSynchronize(c->stream);   // a running transport may still read the previous tables
    cudaFree(c->calib_buf);
    c->calib_buf = nullptr;
    c->calib     = CalibDev{};
    MQI_CUDA(c, cudaMalloc(&c->calib_buf, (n_spr + n_rho) * sizeof(float)), "mqi_set_calibration");
    MQI_CUDA(c, cudaMemcpy(c->calib_buf, spr, n_spr * sizeof(float), cudaMemcpyHostToDevice), "mqi_set_calibration");
    MQI_CUDA(c, cudaMemcpy(c->calib_buf + n_spr, x0, n_rho * sizeof(float), cudaMemcpyHostToDevice),
             "mqi_set_calibration");
    c->calib.mode  = MQI_CALIB_TABLE;
    c->calib.n_rho = n_rho;
    c->calib.n_e   = n_e;
    c->calib.rho0  = rho0;
    c->calib.drho  = drho;
    c->calib.e0    = e0;
    c->calib.de    = de;
    c->calib.spr   = c->calib_buf;
    c->calib.x0    = c->calib_buf + n_spr;
    return MQI_OK;
}

int
mqi_add_child(mqi_ctx* c, int nx, int ny, int nz, const float* xe, const float* ye, const float* ze,
              const float* rot_fwd, const float* translation, int* child_id) {
    if (!valid_ctx(c)) return fail(c, MQI_ERR_INVALID, "mqi_add_child: ctx is NULL");
    if (nx <= 0 || ny <= 0 || nz <= 0 || nx > 2047 || ny > 2047 || nz > 2047 || !xe || !ye || !ze)
        return fail(c, MQI_ERR_INVALID, "mqi_add_child: grid dimensions must be 1..2047 with edge arrays");
    if ((int) c->children.size() >= kMaxChildren)
        return fail(c, MQI_ERR_INVALID, "mqi_add_child: too many children");
    if ((uint64_t) nx * ny * nz > 0xFFFFFFFEull)
        return fail(c, MQI_ERR_INVALID, "mqi_add_child: more voxels than a 32-bit key can index");
    for (int i = 0; i < nx; ++i) if (!(xe[i] < xe[i + 1])) return fail(c, MQI_ERR_INVALID, "mqi_add_child: x edges not increasing");
    for (int i = 0; i < ny; ++i) if (!(ye[i] < ye[i + 1])) return fail(c, MQI_ERR_INVALID, "mqi_add_child: y edges not increasing");
    for (int i = 0; i < nz; ++i) if (!(ze[i] < ze[i + 1])) return fail(c, MQI_ERR_INVALID, "mqi_add_child: z edges not increasing");
    DeviceGuard g(c->device);
    ChildHost ch;
    ch.nx = nx; ch.ny = ny; ch.nz = nz;
    MQI_CUDA(c, cudaMalloc(&ch.xe, (nx + 1) * sizeof(float)), "mqi_add_child");
    MQI_CUDA(c, cudaMalloc(&ch.ye, (ny + 1) * sizeof(float)), "mqi_add_child");
    MQI_CUDA(c, cudaMalloc(&ch.ze, (nz + 1) * sizeof(float)), "mqi_add_child");
    MQI_CUDA(c, cudaMemcpy(ch.xe, xe, (nx + 1) * sizeof(float), cudaMemcpyHostToDevice), "mqi_add_child");
    MQI_CUDA(c, cudaMemcpy(ch.ye, ye, (ny + 1) * sizeof(float), cudaMemcpyHostToDevice), "mqi_add_child");
    MQI_CUDA(c, cudaMemcpy(ch.ze, ze, (nz + 1) * sizeof(float), cudaMemcpyHostToDevice), "mqi_add_child");
    MQI_CUDA(c, cudaMalloc(&ch.rho, (size_t) nx * ny * nz * sizeof(float)), "mqi_add_child");
    identity3(ch.rf);
    ch.tr[0] = ch.tr[1] = ch.tr[2] = 0.0f;
    if (rot_fwd) std::memcpy(ch.rf, rot_fwd, sizeof(ch.rf));
    if (translation) std::memcpy(ch.tr, translation, sizeof(ch.tr));
    // inverse = transpose (mat3x3::inverse, mqi_matrix.hpp)
    const float* m = ch.rf;
    float inv[9] = { m[0], m[3], m[6], m[1], m[4], m[7], m[2], m[5], m[8] };
    std::memcpy(ch.ri, inv, sizeof(inv));
    float id[9];
    identity3(id);
    ch.identity = (std::memcmp(ch.rf, id, sizeof(id)) == 0 && ch.tr[0] == 0.0f && ch.tr[1] == 0.0f && ch.tr[2] == 0.0f) ? 1 : 0;
    c->children.push_back(ch);
    if (child_id) *child_id = (int) c->children.size() - 1;
    return MQI_OK;
}

int
mqi_set_density(mqi_ctx* c, int id, const float* rho, int on_device) {
    if (!valid_ctx(c) || !rho) return fail(c, MQI_ERR_INVALID, "mqi_set_density: bad argument");
    if (id < 0 || id >= (int) c->children.size()) return fail(c, MQI_ERR_INVALID, "mqi_set_density: no such child");
    DeviceGuard g(c->device);
    ChildHost& ch = c->children[id];
    const size_t bytes = (size_t) ch.nx * ch.ny * ch.nz * sizeof(float);
    MQI_CUDA(c, cudaMemcpyAsync(ch.rho, rho, bytes, on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, c->stream),
             "mqi_set_density");
    MQI_CUDA(c, cudaStreamSynchronize(c->stream), "mqi_set_density");
    ch.has_rho = true;
    return MQI_OK;
}

int
mqi_hu_to_density(mqi_ctx* c, const int16_t* hu, float* rho, uint64_t n, float scale, int on_device) {
    if (!valid_ctx(c) || (!hu && n) || (!rho && n)) return fail(c, MQI_ERR_INVALID, "mqi_hu_to_density: bad argument");
    DeviceGuard g(c->device);
    if (on_device) {
        MQI_CUDA(c, launch_hu_to_density(c->tables + 6 * MQI_TABLE_N, hu, rho, n, scale, c->stream), "mqi_hu_to_density");
        MQI_CUDA(c, cudaStreamSynchronize(c->stream), "mqi_hu_to_density");
        return MQI_OK;
    }
    int16_t* dh = nullptr;
    float*   dr = nullptr;
    MQI_CUDA(c, cudaMalloc(&dh, n * sizeof(int16_t) + 16), "mqi_hu_to_density");
    cudaError_t e = cudaMalloc(&dr, n * sizeof(float) + 16);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dh, hu, n * sizeof(int16_t), cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess) e = launch_hu_to_density(c->tables + 6 * MQI_TABLE_N, dh, dr, n, scale, c->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(rho, dr, n * sizeof(float), cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    cudaFree(dh);
    cudaFree(dr);
    if (e != cudaSuccess) return cuda_fail(c, e, "mqi_hu_to_density");
    return MQI_OK;
}

int
mqi_set_hu(mqi_ctx* c, int id, const int16_t* hu, float scale, int on_device) {
    if (!valid_ctx(c) || !hu) return fail(c, MQI_ERR_INVALID, "mqi_set_hu: bad argument");
    if (id < 0 || id >= (int) c->children.size()) return fail(c, MQI_ERR_INVALID, "mqi_set_hu: no such child");
    DeviceGuard g(c->device);
    ChildHost&     ch = c->children[id];
    const uint64_t n  = (uint64_t) ch.nx * ch.ny * ch.nz;
    const int16_t* src = hu;
    int16_t*       tmp = nullptr;
    if (!on_device) {
        MQI_CUDA(c, cudaMalloc(&tmp, n * sizeof(int16_t)), "mqi_set_hu");
        cudaError_t e = cudaMemcpyAsync(tmp, hu, n * sizeof(int16_t), cudaMemcpyHostToDevice, c->stream);
        if (e != cudaSuccess) { cudaFree(tmp); return cuda_fail(c, e, "mqi_set_hu"); }
        src = tmp;
    }
    cudaError_t e = launch_hu_to_density(c->tables + 6 * MQI_TABLE_N, src, ch.rho, n, scale, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (tmp) cudaFree(tmp);
    if (e != cudaSuccess) return cuda_fail(c, e, "mqi_set_hu");
    ch.has_rho = true;
    return MQI_OK;
}

int
mqi_add_scorer(mqi_ctx* c, int child_id, int type, int roi_method, uint32_t roi_length, const uint32_t* roi_start,
               const uint32_t* roi_stride, const uint32_t* roi_acc, int* scorer_id) {
    if (!valid_ctx(c)) return fail(c, MQI_ERR_INVALID, "mqi_add_scorer: ctx is NULL");
    if (child_id < 0 || child_id >= (int) c->children.size())
        return fail(c, MQI_ERR_INVALID, "mqi_add_scorer: no such child");
    if (type < MQI_SCORER_EDEP || type > MQI_SCORER_DIJ)
        return fail(c, MQI_ERR_UNSUPPORTED, "mqi_add_scorer: unknown scorer type (custom fp_compute_hit callbacks have no C-ABI form)");
    if (type == MQI_SCORER_DIJ)
        return fail(c, MQI_ERR_UNSUPPORTED, "mqi_add_scorer: use the Dij entry points for MQI_SCORER_DIJ");
    if ((int) c->scorers.size() >= kMaxScorers) return fail(c, MQI_ERR_INVALID, "mqi_add_scorer: too many scorers");
    // scorers of one child are contiguous
    if (!c->scorers.empty() && c->scorers.back().child != child_id) {
        for (auto& s : c->scorers)
            if (s.child == child_id) return fail(c, MQI_ERR_INVALID, "mqi_add_scorer: add a child's scorers together");
    }
    const ChildHost& ch = c->children[child_id];
    const uint64_t nvox = (uint64_t) ch.nx * ch.ny * ch.nz;
    DeviceGuard g(c->device);
    ScorerHost s;
    s.child      = child_id;
    s.type       = type;
    s.roi_method = roi_method;
    s.stat_mode  = 0;
    s.roi_len    = roi_length;
    if (roi_method == MQI_ROI_DIRECT) {
        s.tally_len = nvox;
    } else if (roi_method == MQI_ROI_INDIRECT) {
        if (!roi_start) return fail(c, MQI_ERR_INVALID, "mqi_add_scorer: INDIRECT needs roi_start (one entry per voxel)");
        MQI_CUDA(c, cudaMalloc(&s.start, nvox * sizeof(uint32_t)), "mqi_add_scorer");
        MQI_CUDA(c, cudaMemcpy(s.start, roi_start, nvox * sizeof(uint32_t), cudaMemcpyHostToDevice), "mqi_add_scorer");
        s.tally_len = nvox;
    } else if (roi_method == MQI_ROI_CONTOUR) {
        if (!roi_start || !roi_stride || !roi_acc || roi_length == 0)
            return fail(c, MQI_ERR_INVALID, "mqi_add_scorer: CONTOUR needs start/stride/acc arrays");
        MQI_CUDA(c, cudaMalloc(&s.start, roi_length * sizeof(uint32_t)), "mqi_add_scorer");
        MQI_CUDA(c, cudaMalloc(&s.stride, roi_length * sizeof(uint32_t)), "mqi_add_scorer");
        MQI_CUDA(c, cudaMalloc(&s.acc, roi_length * sizeof(uint32_t)), "mqi_add_scorer");
        MQI_CUDA(c, cudaMemcpy(s.start, roi_start, roi_length * sizeof(uint32_t), cudaMemcpyHostToDevice), "mqi_add_scorer");
        MQI_CUDA(c, cudaMemcpy(s.stride, roi_stride, roi_length * sizeof(uint32_t), cudaMemcpyHostToDevice), "mqi_add_scorer");
        MQI_CUDA(c, cudaMemcpy(s.acc, roi_acc, roi_length * sizeof(uint32_t), cudaMemcpyHostToDevice), "mqi_add_scorer");
        s.tally_len = nvox;
    } else {
        return fail(c, MQI_ERR_INVALID, "mqi_add_scorer: unknown roi method");
    }
    s.copies = c->n_scen;
    MQI_CUDA(c, cudaMalloc(&s.tally, s.total() * sizeof(double)), "mqi_add_scorer");
    MQI_CUDA(c, cudaMemset(s.tally, 0, s.total() * sizeof(double)), "mqi_add_scorer");
    c->scorers.push_back(s);
    if (scorer_id) *scorer_id = (int) c->scorers.size() - 1;
    return MQI_OK;
}

int
mqi_set_vertices(mqi_ctx* c, const mqi_vertex* v, const uint32_t* spot_ids, uint64_t n, int on_device) {
    if (!valid_ctx(c) || (!v && n)) return fail(c, MQI_ERR_INVALID, "mqi_set_vertices: bad argument");
    if (n > 0xFFFFFFFFull) return fail(c, MQI_ERR_INVALID, "mqi_set_vertices: at most 2^32-1 histories per call");
    DeviceGuard g(c->device);
    if (n > c->vertex_cap) {
        cudaFree(c->vertices);
        c->vertices = nullptr;
        MQI_CUDA(c, cudaMalloc(&c->vertices, n * sizeof(mqi_vertex)), "mqi_set_vertices");
        c->vertex_cap = n;
    }
    if (spot_ids && !on_device)
        for (uint64_t i = 0; i < n; ++i)
            if (spot_ids[i] >= kNoSpot) return fail(c, MQI_ERR_INVALID, "mqi_set_vertices: spot indices must be < 2^24 - 1");
    const cudaMemcpyKind k = on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
    if (n) MQI_CUDA(c, cudaMemcpyAsync(c->vertices, v, n * sizeof(mqi_vertex), k, c->stream), "mqi_set_vertices");
    c->has_spots = spot_ids != nullptr;
    if (spot_ids && n) {
        if (n > c->spot_cap) {
            cudaFree(c->spot_ids);
            c->spot_ids = nullptr;
            MQI_CUDA(c, cudaMalloc(&c->spot_ids, n * sizeof(uint32_t)), "mqi_set_vertices");
            c->spot_cap = n;
        }
        MQI_CUDA(c, cudaMemcpyAsync(c->spot_ids, spot_ids, n * sizeof(uint32_t), k, c->stream), "mqi_set_vertices");
    }
    c->n_vertices = n;
    return MQI_OK;
}

}   // extern "C"

namespace
{

/// Runs with at least this many queue entries (histories x scenarios) hand nuclear post-steps to
/// the post-step kernel when the post-step mode is automatic.
constexpr uint64_t kSplitMinEntries = 1ull << 19;

/// The source stream of a plan history is keyed apart from its transport streams.
constexpr uint32_t kSourceKeyXor = 0xA5A5A5A5u;

/// Kernel parameters of a transport run: children, scorers (with the double-scoring quirk),
/// physics options, seed, scenarios.
void
make_wave_params(mqi_ctx* c, uint64_t seed, WaveParams& P) {
    P = WaveParams{};
    P.calib      = c->calib;
    P.n_children = (int) c->children.size();
    for (int i = 0; i < P.n_children; ++i) {
        const ChildHost& h = c->children[i];
        ChildDev&        d = P.child[i];
        d.nx = h.nx; d.ny = h.ny; d.nz = h.nz;
        d.xe = h.xe; d.ye = h.ye; d.ze = h.ze; d.rho = h.rho;
        std::memcpy(d.rf, h.rf, sizeof(d.rf));
        std::memcpy(d.ri, h.ri, sizeof(d.ri));
        std::memcpy(d.tr, h.tr, sizeof(d.tr));
        d.identity = h.identity;
        d.scorer_begin = 0;
        d.n_scorers = 0;
    }
    for (int i = 0; i < (int) c->scorers.size(); ++i) {
        const ScorerHost& s = c->scorers[i];
        ScorerDev&        d = P.scorer[i];
        d.type = s.type; d.roi_method = s.roi_method; d.stat_mode = s.stat_mode;
        d.roi_len = s.roi_len; d.start = s.start; d.stride = s.stride; d.acc = s.acc;
        d.tally = s.tally; d.tally_len = s.tally_len; d.tstride = s.tstride;
        d.dij = s.dij; d.dij_mask = s.dij_cap ? s.dij_cap - 1 : 0;
        d.hit_log = s.hit_log; d.hit_count = s.hit_count; d.hit_cap = s.hit_cap;
        if (s.dij) {
            c->scorers[i].csr.built = false;   // new entries invalidate a built matrix
            P.kernel_mode |= kModeDij;
        }
        if (s.type == MQI_SCORER_DOSE_M || (s.type >= MQI_SCORER_LETD_NUM && s.type <= MQI_SCORER_LETT_DEN))
            P.kernel_mode |= kModeFull;
        if (s.roi_method != MQI_ROI_DIRECT) P.kernel_mode |= kModeRoi;
        ChildDev& ch = P.child[s.child];
        if (ch.n_scorers == 0) ch.scorer_begin = i;
        ++ch.n_scorers;
    }
    // Non-stat kernel quirk (mqi_transport.hpp:204-225): with n >= 3 scorers on a node, scorers
    // 0..n-3 are inserted twice per step.  A node that carries the statistics pair runs the _stat
    // kernel instead (mqi_transport.hpp:342-364), which scores each scorer once.
    for (int i = 0; i < P.n_children; ++i) {
        const ChildDev& ch = P.child[i];
        bool has_stat = false;
        for (int k = 0; k < ch.n_scorers; ++k) has_stat = has_stat || P.scorer[ch.scorer_begin + k].stat_mode;
        if (ch.n_scorers >= 3 && !has_stat)
            for (int k = 0; k < ch.n_scorers - 2; ++k) P.scorer[ch.scorer_begin + k].double_score = 1;
    }
    if (P.kernel_mode == 0 && P.n_children == 1 && c->scorers.size() == 1 && c->n_scen == 1) {
        const ScorerHost& s0 = c->scorers[0];
        if (!s0.stat_mode && s0.tstride == 1 && (s0.type == MQI_SCORER_EDEP || s0.type == MQI_SCORER_DOSE_W))
            P.kernel_mode = kModeSingle;
    }
    if (P.kernel_mode == 0 && c->scorers.size() == 3) {
        // a dose scorer followed by the statistics pair, all DIRECT, on one child
        const ScorerHost& a = c->scorers[0];
        const ScorerHost& b = c->scorers[1];
        const ScorerHost& d = c->scorers[2];
        if (a.type == MQI_SCORER_DOSE_W && !a.stat_mode && a.tstride == 1 && a.roi_method == MQI_ROI_DIRECT &&
            b.type == MQI_SCORER_DOSE_W && b.stat_mode && b.tstride == 2 && b.roi_method == MQI_ROI_DIRECT &&
            d.type == MQI_SCORER_DOSE_W2 && d.stat_mode && d.tally == b.tally + 1 && a.child == b.child &&
            b.child == d.child && a.tally_len == b.tally_len)
            P.kernel_mode = kModeStat;
    }
    P.physics_debug   = c->physics_debug;
    P.score_local     = c->score_local;
    P.stack_limit     = c->physics_debug ? 200 : 10;
    P.t_cut           = c->physics_debug ? kTcutDebug : kTcutRelease;
    P.k0              = (uint32_t) seed;
    P.k1              = (uint32_t) (seed >> 32);
    P.max_slice_steps = c->max_slice_steps;
    P.inline_local    = (P.n_children == 1) ? 1 : 0;
    P.head            = c->counters + 2;
    P.error_flag      = c->counters + 3;
    P.def             = c->def;
    P.n_def           = c->counters + 4;
    P.stats           = c->stats;
    P.spot_ids        = c->has_spots ? c->spot_ids : nullptr;
    P.tables          = c->tables;
    P.smem_edge_floats = wave_edge_floats(P.child, P.n_children);
    if (c->n_scen > 1) {
        P.n_scen      = (int) c->n_scen;
        P.scen_child  = c->scen_child;
        P.scen_stride = c->scen_stride;
        P.scen_edges  = c->scen_edges;
        for (uint32_t k = 0; k < c->n_scen; ++k) P.scen_scale[k] = c->scen_scale[k];
    }
}

/// Queue generations (moqui's order of work, one host synchronisation per wave): load (or sample) a
/// chunk of primaries, run waves until a generation is empty, repeat.
int
run_generations(mqi_ctx* c, WaveParams P, uint64_t h0, uint64_t h1, bool plan) {
    const uint32_t chunk = c->primary_chunk;
    QueueBuf* A = &c->qa;
    QueueBuf* B = &c->qb;
    const uint32_t S       = c->n_scen;
    const uint32_t per_ld  = std::max<uint32_t>(chunk / S, 1u);   // histories per load; S queue entries each
    for (uint64_t h = h0; h < h1; h += per_ld) {
        const uint32_t n = (uint32_t) std::min<uint64_t>(per_ld, h1 - h);
        if (plan)
            MQI_CUDA(c, launch_sample_primaries(A->q, c->plan_spots, c->plan_cum, c->n_plan_spots, h, n, S, P.k0,
                                                P.k1 ^ kSourceKeyXor, c->stream), "mqi_transport: sample primaries");
        else
            MQI_CUDA(c, launch_load_primaries(A->q, c->vertices, c->has_spots ? c->spot_ids : nullptr, h, n, S, c->stream),
                     "mqi_transport: load primaries");
        ++c->kernel_launches;
        c->host_counts[0] = n * S;
        MQI_CUDA(c, cudaMemcpyAsync(c->counters + 0, c->host_counts, sizeof(uint32_t), cudaMemcpyHostToDevice, c->stream),
                 "mqi_transport");
        int cur = 0;
        for (int wave = 0;; ++wave) {
            if (wave > 100000) return fail(c, MQI_ERR_DEVICE, "mqi_transport: wave limit reached");
            P.in    = A->q;
            P.out   = B->q;
            P.n_in  = c->counters + cur;
            P.n_out = c->counters + (1 - cur);
            MQI_CUDA(c, cudaMemsetAsync(c->counters + (1 - cur), 0, sizeof(uint32_t), c->stream), "mqi_transport");
            MQI_CUDA(c, cudaMemsetAsync(c->counters + 2, 0, sizeof(uint32_t), c->stream), "mqi_transport");
            MQI_CUDA(c, cudaEventRecord(c->ev0, c->stream), "mqi_transport");
            MQI_CUDA(c, launch_wave(P, c->wave_grid, c->wave_block, c->wave_grid / c->num_sms, c->stream), "mqi_transport: wave");
            MQI_CUDA(c, cudaEventRecord(c->ev1, c->stream), "mqi_transport");
            MQI_CUDA(c, cudaMemcpyAsync(c->host_counts, c->counters, 4 * sizeof(uint32_t), cudaMemcpyDeviceToHost, c->stream),
                     "mqi_transport");
            MQI_CUDA(c, cudaStreamSynchronize(c->stream), "mqi_transport: wave");
            ++c->waves;
            // the wave, its post-step kernel when split, the four sort kernels when sorting is on
            c->kernel_launches += (P.split ? 2 : 1) + (P.sort_bins ? 4 : 0);
            ++c->wave_launches;
            float ms = 0.0f;
            if (cudaEventElapsedTime(&ms, c->ev0, c->ev1) == cudaSuccess) c->wave_ms += ms;
            if (c->host_counts[3] & 2u) return fail(c, MQI_ERR_OVERFLOW, "mqi_transport: particle queue overflow");
            const uint32_t n_next = c->host_counts[1 - cur];
            if (n_next == 0) break;
            std::swap(A, B);
            cur = 1 - cur;
        }
    }
    return MQI_OK;
}

/// Streamed transport: before every wave the queue is topped up on the device with the next
/// histories, so waves never run with the GPU half empty while the long tracks of a generation
/// finish; `graph_waves` waves (top-up, load, wave) are captured once into a CUDA graph, and the
/// host synchronises once per graph launch.  The work done does not depend on how it is split
/// into waves (every random number is keyed by history and track).
int
run_streamed(mqi_ctx* c, WaveParams P, uint64_t h0, uint64_t h1, bool plan) {
    const int      K = c->graph_waves;
    const uint32_t S = c->n_scen;
    TopUp tu{};
    tu.next   = h0;
    tu.end    = h1;
    tu.target = std::max<uint32_t>(c->primary_chunk / S, 1u) * S;
    tu.n_scen = S;
    MQI_CUDA(c, cudaMemcpyAsync(c->topup, &tu, sizeof(tu), cudaMemcpyHostToDevice, c->stream), "mqi_transport");
    MQI_CUDA(c, cudaMemsetAsync(c->counters, 0, 2 * sizeof(uint32_t), c->stream), "mqi_transport");
    MQI_CUDA(c, cudaStreamSynchronize(c->stream), "mqi_transport");

    cudaStream_t cs = c->cap_stream;
    cudaGraph_t  graph = nullptr;
    cudaError_t  e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeRelaxed);
    for (int i = 0; e == cudaSuccess && i < K; ++i) {
        const int in  = i & 1;
        QueueBuf& Qin = in ? c->qb : c->qa;
        QueueBuf& Qo  = in ? c->qa : c->qb;
        e = launch_topup(c->topup, c->counters + in, c->counters + 3, cs);
        if (e == cudaSuccess)
            e = plan ? launch_sample_topup(Qin.q, c->topup, c->plan_spots, c->plan_cum, c->n_plan_spots, P.k0,
                                           P.k1 ^ kSourceKeyXor, c->num_sms, cs)
                     : launch_load_topup(Qin.q, c->topup, c->vertices, c->has_spots ? c->spot_ids : nullptr, c->num_sms,
                                         cs);
        if (e == cudaSuccess) e = cudaMemsetAsync(c->counters + (1 - in), 0, sizeof(uint32_t), cs);
        if (e == cudaSuccess) e = cudaMemsetAsync(c->counters + 2, 0, sizeof(uint32_t), cs);
        P.in    = Qin.q;
        P.out   = Qo.q;
        P.n_in  = c->counters + in;
        P.n_out = c->counters + (1 - in);
        if (e == cudaSuccess) e = launch_wave(P, c->wave_grid, c->wave_block, c->wave_grid / c->num_sms, cs);
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(c->host_counts, c->counters, 4 * sizeof(uint32_t), cudaMemcpyDeviceToHost, cs);
    if (e == cudaSuccess) e = cudaMemcpyAsync(c->host_next, &c->topup->next, sizeof(unsigned long long),
                                              cudaMemcpyDeviceToHost, cs);
    const cudaError_t e_end = cudaStreamEndCapture(cs, &graph);
    if (e == cudaSuccess) e = e_end;
    cudaGraphExec_t exec = nullptr;
    if (e == cudaSuccess) e = cudaGraphInstantiate(&exec, graph, 0);
    if (graph) cudaGraphDestroy(graph);
    if (e != cudaSuccess) {
        if (exec) cudaGraphExecDestroy(exec);
        return cuda_fail(c, e, "mqi_transport: graph capture");
    }
    int rc = MQI_OK;
    for (uint64_t launch = 0;; ++launch) {
        if (launch * (uint64_t) K > 200000) {
            rc = fail(c, MQI_ERR_DEVICE, "mqi_transport: wave limit reached");
            break;
        }
        e = cudaEventRecord(c->ev0, c->stream);
        if (e == cudaSuccess) e = cudaGraphLaunch(exec, c->stream);
        if (e == cudaSuccess) e = cudaEventRecord(c->ev1, c->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
        if (e != cudaSuccess) {
            rc = cuda_fail(c, e, "mqi_transport: graph launch");
            break;
        }
        c->waves += K;
        c->wave_launches += K;
        // per wave: top-up, load, wave (+ post-step when split, + 4 sort kernels when sorting is on)
        c->kernel_launches += (3 + (P.split ? 1 : 0) + (P.sort_bins ? 4 : 0)) * (uint64_t) K;
        float ms = 0.0f;
        if (cudaEventElapsedTime(&ms, c->ev0, c->ev1) == cudaSuccess) c->wave_ms += ms;
        if (c->host_counts[3] & 2u) {
            rc = fail(c, MQI_ERR_OVERFLOW, "mqi_transport: particle queue overflow");
            break;
        }
        if (*c->host_next >= h1 && c->host_counts[0] == 0) break;
    }
    cudaGraphExecDestroy(exec);
    return rc;
}

/// Transport histories [h0, h1) from the vertices or the spot plan.
int
run_transport(mqi_ctx* c, uint64_t h0, uint64_t h1, uint64_t seed, bool plan) {
    DeviceGuard g(c->device);
    const uint32_t need = c->primary_chunk * 3u;
    if (c->queue_cap < need) {
        cudaFree(c->def);
        c->def        = nullptr;
        cudaError_t e = alloc_queue(c->qa, need);
        if (e == cudaSuccess) e = alloc_queue(c->qb, need);
        if (e == cudaSuccess) e = cudaMalloc(&c->def, (size_t) need * sizeof(Deferred));
        if (e == cudaSuccess) e = alloc_queue(c->qsort, need);
        if (e == cudaSuccess && !c->sort_bins) e = cudaMalloc(&c->sort_bins, 2 * kSortBins * sizeof(uint32_t));
        if (e == cudaSuccess) e = cudaMemsetAsync(c->sort_bins, 0, 2 * kSortBins * sizeof(uint32_t), c->stream);
        if (e != cudaSuccess) {
            c->queue_cap = 0;
            return cuda_fail(c, e, "mqi_transport: queue allocation");
        }
        c->queue_cap = need;
    }
    WaveParams P;
    make_wave_params(c, seed, P);
    // Nuclear post-steps in the post-step kernel pay off when a wave holds many tracks: the step
    // loop then carries less code (+30% on the 1e6-history slab phantom), while each interaction
    // ends its track's wave, which lengthens the drain of small runs (-12% on the 1e5-history
    // phantom example); runs below kSplitMinEntries queue entries keep them inside the wave.
    P.split = c->post_step_mode >= 0 ? c->post_step_mode
                                     : ((h1 - h0) * (uint64_t) c->n_scen >= kSplitMinEntries ? 1 : 0);
    if (c->sort_min > 0) {
        P.sort_tmp  = c->qsort.q;
        P.sort_bins = c->sort_bins;
        P.sort_min  = c->sort_min;
    }
    MQI_CUDA(c, cudaMemsetAsync(c->counters + 3, 0, sizeof(uint32_t), c->stream), "mqi_transport");
    const int rc = c->streamed ? run_streamed(c, P, h0, h1, plan) : run_generations(c, P, h0, h1, plan);
    if (rc != MQI_OK) return rc;
    if (c->host_counts[3] & 4u)
        return fail(c, MQI_ERR_OVERFLOW, "mqi_transport: a Dij table is full (raise its capacity)");
    if (c->host_counts[3] & 1u) return fail(c, MQI_ERR_DEVICE, "mqi_transport: a bounded device loop gave up");
    return MQI_OK;
}

int
check_ready(mqi_ctx* c, const char* who) {
    if (!valid_ctx(c)) return fail(c, MQI_ERR_INVALID, std::string(who) + ": ctx is NULL");
    if (c->children.empty()) return fail(c, MQI_ERR_STATE, std::string(who) + ": no child geometry");
    for (auto& ch : c->children)
        if (!ch.has_rho) return fail(c, MQI_ERR_STATE, std::string(who) + ": a child has no density");
    return MQI_OK;
}

}   // namespace

extern "C" {

int
mqi_transport(mqi_ctx* c, uint64_t h0, uint64_t h1, uint64_t seed) {
    const int rc = check_ready(c, "mqi_transport");
    if (rc != MQI_OK) return rc;
    if (h1 < h0 || h1 > c->n_vertices) return fail(c, MQI_ERR_INVALID, "mqi_transport: history range outside the vertices");
    if (h0 == h1) return MQI_OK;
    return run_transport(c, h0, h1, seed, false);
}

int
mqi_set_spot_plan(mqi_ctx* c, const mqi_spot* spots, uint32_t n_spots, uint64_t* total_histories) {
    if (!valid_ctx(c) || (!spots && n_spots)) return fail(c, MQI_ERR_INVALID, "mqi_set_spot_plan: bad argument");
    if (n_spots >= kNoSpot) return fail(c, MQI_ERR_INVALID, "mqi_set_spot_plan: at most 2^24 - 2 spots");
    std::vector<uint64_t> cum(n_spots + 1, 0);
    for (uint32_t i = 0; i < n_spots; ++i) cum[i + 1] = cum[i] + spots[i].histories;
    if (cum[n_spots] > 0xFFFFFFFFull) return fail(c, MQI_ERR_INVALID, "mqi_set_spot_plan: at most 2^32-1 histories per plan");
    DeviceGuard g(c->device);
    cudaFree(c->plan_spots);
    cudaFree(c->plan_cum);
    c->plan_spots = nullptr;
    c->plan_cum   = nullptr;
    MQI_CUDA(c, cudaMalloc(&c->plan_spots, std::max<size_t>(n_spots, 1) * sizeof(mqi_spot)), "mqi_set_spot_plan");
    MQI_CUDA(c, cudaMalloc(&c->plan_cum, (n_spots + 1) * sizeof(uint64_t)), "mqi_set_spot_plan");
    if (n_spots) MQI_CUDA(c, cudaMemcpy(c->plan_spots, spots, n_spots * sizeof(mqi_spot), cudaMemcpyHostToDevice), "mqi_set_spot_plan");
    MQI_CUDA(c, cudaMemcpy(c->plan_cum, cum.data(), (n_spots + 1) * sizeof(uint64_t), cudaMemcpyHostToDevice), "mqi_set_spot_plan");
    c->n_plan_spots    = n_spots;
    c->plan_histories  = cum[n_spots];
    c->plan_cum_host   = cum;
    if (total_histories) *total_histories = cum[n_spots];
    return MQI_OK;
}

int
mqi_set_scenarios(mqi_ctx* c, int child_id, uint32_t n, const float* xe, const float* ye, const float* ze,
                  const float* density_scale) {
    if (!valid_ctx(c)) return fail(c, MQI_ERR_INVALID, "mqi_set_scenarios: ctx is NULL");
    if (n > (uint32_t) kMaxScenarios) return fail(c, MQI_ERR_INVALID, "mqi_set_scenarios: at most 64 scenarios");
    if (n > 1) {
        if (child_id < 0 || child_id >= (int) c->children.size())
            return fail(c, MQI_ERR_INVALID, "mqi_set_scenarios: no such child");
        if (!xe || !ye || !ze) return fail(c, MQI_ERR_INVALID, "mqi_set_scenarios: edge arrays are required");
    }
    for (auto& s : c->scorers)
        if (s.type == MQI_SCORER_DIJ && n > 1)
            return fail(c, MQI_ERR_UNSUPPORTED, "mqi_set_scenarios: a Dij scorer cannot run with robust scenarios");
    const uint32_t copies = n > 1 ? n : 1;
    DeviceGuard g(c->device);
    float* edges = nullptr;
    int    stride = 0;
    if (n > 1) {
        const ChildHost& ch = c->children[child_id];
        stride = ch.nx + ch.ny + ch.nz + 3;
        std::vector<float> host((size_t) n * stride);
        for (uint32_t k = 0; k < n; ++k) {
            float* e = host.data() + (size_t) k * stride;
            std::memcpy(e, xe + (size_t) k * (ch.nx + 1), (ch.nx + 1) * sizeof(float));
            std::memcpy(e + ch.nx + 1, ye + (size_t) k * (ch.ny + 1), (ch.ny + 1) * sizeof(float));
            std::memcpy(e + ch.nx + ch.ny + 2, ze + (size_t) k * (ch.nz + 1), (ch.nz + 1) * sizeof(float));
        }
        MQI_CUDA(c, cudaMalloc(&edges, host.size() * sizeof(float)), "mqi_set_scenarios");
        cudaError_t e = cudaMemcpy(edges, host.data(), host.size() * sizeof(float), cudaMemcpyHostToDevice);
        if (e != cudaSuccess) {
            cudaFree(edges);
            return cuda_fail(c, e, "mqi_set_scenarios");
        }
    }
    // one tally per scenario for every scorer; accumulated results are dropped
    for (auto& s : c->scorers) {
        cudaFree(s.batch_s1);
        cudaFree(s.batch_s2);
        s.batch_s1 = s.batch_s2 = nullptr;
        s.n_batches = 0;
        if (s.type == MQI_SCORER_DIJ || !s.owns) continue;
        cudaFree(s.tally);
        s.tally  = nullptr;
        s.copies = copies;
        MQI_CUDA(c, cudaMalloc(&s.tally, s.tstride * s.total() * sizeof(double)), "mqi_set_scenarios");
        MQI_CUDA(c, cudaMemset(s.tally, 0, s.tstride * s.total() * sizeof(double)), "mqi_set_scenarios");
        if (s.partner >= 0) {   // the stat pair's dose^2 half lives in the same buffer
            c->scorers[s.partner].tally  = s.tally + 1;
            c->scorers[s.partner].copies = copies;
        }
    }
    cudaFree(c->scen_edges);
    c->scen_edges  = edges;
    c->scen_stride = stride;
    c->scen_child  = n > 1 ? child_id : -1;
    c->n_scen      = copies;
    c->scen_scale.assign(copies, 1.0f);
    if (density_scale && n > 1)
        for (uint32_t k = 0; k < n; ++k) c->scen_scale[k] = density_scale[k];
    return MQI_OK;
}

int
mqi_run_plan_until_stat(mqi_ctx* c, int dose_id, int dose2_id, float criteria, float threshold, uint64_t max_passes,
                        uint64_t seed, uint64_t* passes_done, double* achieved) {
    if (!valid_ctx(c)) return fail(c, MQI_ERR_INVALID, "mqi_run_plan_until_stat: ctx is NULL");
    if (!c->plan_spots || c->plan_histories == 0) return fail(c, MQI_ERR_STATE, "mqi_run_plan_until_stat: no spot plan");
    if (dose_id < 0 || dose_id >= (int) c->scorers.size() || !c->scorers[dose_id].stat_mode)
        return fail(c, MQI_ERR_INVALID, "mqi_run_plan_until_stat: dose_id must be a stat scorer");
    const uint64_t N = c->plan_histories;
    uint64_t passes = 0;
    double   stat   = 1.0;   // current_stat = 100% before the first run (mqi_tps_env.hpp:1244)
    for (; passes < max_passes && stat > (double) criteria; ++passes) {
        const int rc = mqi_transport_plan(c, 0, N, seed + 0x9E3779B97F4A7C15ull * passes);
        if (rc != MQI_OK) return rc;
        const int rs = mqi_stat_uncertainty(c, dose_id, dose2_id, N * (passes + 1), threshold, &stat, nullptr);
        if (rs != MQI_OK) return rs;
    }
    // calculate_average_results (mqi_tps_env.hpp:1428-1476): the child's other scorers are scaled
    // to one pass of the plan
    const int child = c->scorers[dose_id].child;
    for (int i = 0; i < (int) c->scorers.size(); ++i) {
        const ScorerHost& s = c->scorers[i];
        if (s.child == child && !s.stat_mode && s.type != MQI_SCORER_DIJ && passes > 0) {
            const int rc = mqi_scale_tally(c, i, 1.0 / (double) passes);
            if (rc != MQI_OK) return rc;
        }
    }
    if (passes_done) *passes_done = passes;
    if (achieved) *achieved = stat;
    return MQI_OK;
}

int
mqi_transport_plan(mqi_ctx* c, uint64_t h0, uint64_t h1, uint64_t seed) {
    const int rc = check_ready(c, "mqi_transport_plan");
    if (rc != MQI_OK) return rc;
    if (!c->plan_spots) return fail(c, MQI_ERR_STATE, "mqi_transport_plan: no spot plan");
    if (h1 < h0 || h1 > c->plan_histories) return fail(c, MQI_ERR_INVALID, "mqi_transport_plan: history range outside the plan");
    if (h0 == h1) return MQI_OK;
    return run_transport(c, h0, h1, seed, true);
}

int
mqi_autotune(mqi_ctx* c, int source_plan, uint64_t h0, uint64_t h1, uint64_t seed, mqi_tune_result* results,
             uint32_t max_results, uint32_t* n_results) {
    const int rc0 = check_ready(c, "mqi_autotune");
    if (rc0 != MQI_OK) return rc0;
    if (source_plan ? (!c->plan_spots || h1 > c->plan_histories) : (h1 > c->n_vertices))
        return fail(c, MQI_ERR_INVALID, "mqi_autotune: sample range outside the source");
    if (h1 <= h0) return fail(c, MQI_ERR_INVALID, "mqi_autotune: empty sample");
    for (auto& s : c->scorers)
        if (s.type == MQI_SCORER_DIJ) return fail(c, MQI_ERR_STATE, "mqi_autotune: tune before adding a Dij scorer");
    DeviceGuard g(c->device);
    // The sample is transported into scratch tallies: the caller's tallies and counters are kept.
    std::vector<double*> saved(c->scorers.size(), nullptr);
    std::vector<double*> scratch(c->scorers.size(), nullptr);
    unsigned long long   stats_saved[8];
    MQI_CUDA(c, cudaMemcpy(stats_saved, c->stats, sizeof(stats_saved), cudaMemcpyDeviceToHost), "mqi_autotune");
    const uint64_t waves0 = c->waves, kl0 = c->kernel_launches, wl0 = c->wave_launches;
    const double   wms0   = c->wave_ms;
    const int blk0 = c->wave_block, grid0 = c->wave_grid, str0 = c->streamed, gw0 = c->graph_waves;
    const uint32_t chunk0 = c->primary_chunk;
    int rc = MQI_OK;
    for (size_t i = 0; i < c->scorers.size() && rc == MQI_OK; ++i) {
        ScorerHost& s = c->scorers[i];
        if (!s.owns) continue;
        const size_t bytes = s.tstride * s.total() * sizeof(double);
        cudaError_t e = cudaMalloc(&scratch[i], bytes);
        if (e == cudaSuccess) e = cudaMemset(scratch[i], 0, bytes);
        if (e != cudaSuccess) rc = cuda_fail(c, e, "mqi_autotune: scratch tallies");
    }
    auto swap_tallies = [&]() {
        for (size_t i = 0; i < c->scorers.size(); ++i) {
            ScorerHost& s = c->scorers[i];
            if (!s.owns) continue;
            std::swap(s.tally, scratch[i]);
            if (s.partner >= 0) c->scorers[s.partner].tally = s.tally + 1;
        }
    };
    struct Cand { int block, bps, streamed, graph_waves; uint32_t chunk; };
    // queue sizes above the sample behave alike (one load holds the whole sample): only the
    // largest of them is tried
    const uint64_t n_sample = (h1 - h0) * c->n_scen;
    std::vector<uint32_t> chunks;
    bool                  above = false;   // a queue size >= the sample is in the list
    for (uint32_t chunk : { 1u << 19, 1u << 20, 1u << 21 }) {
        if (chunk < n_sample) {
            chunks.push_back(chunk);
        } else if (!above) {
            chunks.push_back(chunk);
            above = true;
        } else {
            chunks.back() = chunk;
        }
    }
    std::vector<Cand> cands;
    for (int streamed : { 1, 0 })
        for (uint32_t chunk : chunks)
            for (auto shape : { std::make_pair(128, 5), std::make_pair(128, 4), std::make_pair(128, 6), std::make_pair(256, 2) })
                cands.push_back({ shape.first, shape.second, streamed, 8, chunk });
    uint32_t n = 0;
    int best = -1;
    double best_rate = 0.0;
    if (rc == MQI_OK) {
        swap_tallies();
        for (size_t k = 0; k < cands.size() && rc == MQI_OK; ++k) {
            const Cand& q = cands[k];
            c->wave_block = q.block;
            c->wave_grid = c->num_sms * q.bps;
            c->streamed = q.streamed;
            c->graph_waves = q.graph_waves;
            c->primary_chunk = q.chunk;
            MQI_CUDA(c, cudaStreamSynchronize(c->stream), "mqi_autotune");
            const auto t0 = std::chrono::steady_clock::now();
            rc = run_transport(c, h0, h1, seed, source_plan != 0);
            MQI_CUDA(c, cudaStreamSynchronize(c->stream), "mqi_autotune");
            const double sec = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
            if (rc != MQI_OK) break;
            const double rate = (double) (h1 - h0) / sec;
            if (results && n < max_results) {
                results[n].block = q.block;
                results[n].blocks_per_sm = q.bps;
                results[n].streamed = q.streamed;
                results[n].graph_waves = q.graph_waves;
                results[n].primary_chunk = q.chunk;
                results[n].histories_per_s = rate;
            }
            ++n;
            if (rate > best_rate) {
                best_rate = rate;
                best = (int) k;
            }
        }
        swap_tallies();
    }
    for (double* p : scratch) cudaFree(p);
    cudaMemcpy(c->stats, stats_saved, sizeof(stats_saved), cudaMemcpyHostToDevice);
    c->waves = waves0; c->kernel_launches = kl0; c->wave_launches = wl0; c->wave_ms = wms0;
    if (rc != MQI_OK || best < 0) {
        c->wave_block = blk0; c->wave_grid = grid0; c->streamed = str0; c->graph_waves = gw0; c->primary_chunk = chunk0;
        return rc != MQI_OK ? rc : fail(c, MQI_ERR_DEVICE, "mqi_autotune: no candidate ran");
    }
    const Cand& q = cands[best];
    c->wave_block = q.block;
    c->wave_grid = c->num_sms * q.bps;
    c->streamed = q.streamed;
    c->graph_waves = q.graph_waves;
    c->primary_chunk = q.chunk;
    if (n_results) *n_results = n;
    return MQI_OK;
}

int
mqi_sample_plan(mqi_ctx* c, uint64_t h0, uint64_t h1, uint64_t seed, mqi_vertex* out, uint32_t* spot_out) {
    if (!valid_ctx(c)) return fail(c, MQI_ERR_INVALID, "mqi_sample_plan: ctx is NULL");
    if (!c->plan_spots) return fail(c, MQI_ERR_STATE, "mqi_sample_plan: no spot plan");
    if (h1 < h0 || h1 > c->plan_histories) return fail(c, MQI_ERR_INVALID, "mqi_sample_plan: history range outside the plan");
    if (h0 == h1) return MQI_OK;
    if (!out) return fail(c, MQI_ERR_INVALID, "mqi_sample_plan: out is NULL");
    DeviceGuard g(c->device);
    const uint64_t n = h1 - h0;
    mqi_vertex* dv = nullptr;
    uint32_t*   ds = nullptr;
    cudaError_t e  = cudaMalloc(&dv, n * sizeof(mqi_vertex));
    if (e == cudaSuccess && spot_out) e = cudaMalloc(&ds, n * sizeof(uint32_t));
    for (uint64_t off = 0; e == cudaSuccess && off < n; off += 0x40000000ull) {
        const uint32_t m = (uint32_t) std::min<uint64_t>(0x40000000ull, n - off);
        e = launch_sample_vertices(dv + off, ds ? ds + off : nullptr, c->plan_spots, c->plan_cum, c->n_plan_spots,
                                   h0 + off, m, (uint32_t) seed, (uint32_t) (seed >> 32) ^ kSourceKeyXor, c->stream);
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(out, dv, n * sizeof(mqi_vertex), cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess && ds) e = cudaMemcpyAsync(spot_out, ds, n * sizeof(uint32_t), cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    cudaFree(dv);
    cudaFree(ds);
    if (e != cudaSuccess) return cuda_fail(c, e, "mqi_sample_plan");
    return MQI_OK;
}

int
mqi_get_tally(mqi_ctx* c, int id, double* out, uint64_t* n_out, int on_device) {
    if (!valid_ctx(c)) return fail(c, MQI_ERR_INVALID, "mqi_get_tally: ctx is NULL");
    if (id < 0 || id >= (int) c->scorers.size()) return fail(c, MQI_ERR_INVALID, "mqi_get_tally: no such scorer");
    const ScorerHost& s = c->scorers[id];
    if (n_out) *n_out = s.total();
    if (!out) return MQI_OK;
    DeviceGuard g(c->device);
    const size_t bytes = s.total() * sizeof(double);
    if (s.tstride == 1) {
        MQI_CUDA(c, cudaMemcpyAsync(out, s.tally, bytes, on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost,
                                    c->stream), "mqi_get_tally");
    } else if (on_device) {
        MQI_CUDA(c, launch_copy_strided(s.tally, s.tstride, out, s.total(), c->num_sms, c->stream), "mqi_get_tally");
    } else {
        double* tmp = nullptr;
        MQI_CUDA(c, cudaMalloc(&tmp, bytes), "mqi_get_tally");
        cudaError_t e = launch_copy_strided(s.tally, s.tstride, tmp, s.total(), c->num_sms, c->stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(out, tmp, bytes, cudaMemcpyDeviceToHost, c->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
        cudaFree(tmp);
        if (e != cudaSuccess) return cuda_fail(c, e, "mqi_get_tally");
    }
    MQI_CUDA(c, cudaStreamSynchronize(c->stream), "mqi_get_tally");
    return MQI_OK;
}

int
mqi_reset_tallies(mqi_ctx* c) {
    if (!valid_ctx(c)) return fail(c, MQI_ERR_INVALID, "mqi_reset_tallies: ctx is NULL");
    DeviceGuard g(c->device);
    for (auto& s : c->scorers) {
        if (s.type == MQI_SCORER_DIJ) MQI_CUDA(c, dij_reset(s, c->num_sms, c->stream), "mqi_reset_tallies");
        else if (s.owns)
            MQI_CUDA(c, cudaMemsetAsync(s.tally, 0, s.tstride * s.total() * sizeof(double), c->stream), "mqi_reset_tallies");
    }
    MQI_CUDA(c, cudaMemsetAsync(c->stats, 0, 8 * sizeof(unsigned long long), c->stream), "mqi_reset_tallies");
    MQI_CUDA(c, cudaMemsetAsync(c->counters + 3, 0, sizeof(uint32_t), c->stream), "mqi_reset_tallies");
    MQI_CUDA(c, cudaStreamSynchronize(c->stream), "mqi_reset_tallies");
    c->waves = 0;
    c->kernel_launches = 0;
    c->wave_launches = 0;
    c->wave_ms = 0.0;
    return MQI_OK;
}

int
mqi_get_stats(mqi_ctx* c, mqi_stats* out) {
    if (!valid_ctx(c) || !out) return fail(c, MQI_ERR_INVALID, "mqi_get_stats: bad argument");
    DeviceGuard g(c->device);
    unsigned long long v[8];
    MQI_CUDA(c, cudaMemcpyAsync(v, c->stats, sizeof(v), cudaMemcpyDeviceToHost, c->stream), "mqi_get_stats");
    MQI_CUDA(c, cudaStreamSynchronize(c->stream), "mqi_get_stats");
    out->histories       = v[0];
    out->tracks          = v[1];
    out->steps           = v[2];
    out->secondaries     = v[3];
    out->local_daughters = v[4];
    out->dropped         = v[5];
    out->waves           = c->waves;
    out->device_errors   = v[7];
    out->kernel_launches = c->kernel_launches;
    out->wave_launches   = c->wave_launches;
    out->wave_ms         = c->wave_ms;
    return MQI_OK;
}

int
mqi_trace_rays(mqi_ctx* c, int id, const float* rays, uint64_t n_rays, uint32_t max_steps, int64_t* offsets,
               uint64_t* cnb, float* dist, int32_t* cells, uint64_t capacity, uint64_t* n_out) {
    if (!valid_ctx(c) || (!rays && n_rays) || !offsets || max_steps == 0)
        return fail(c, MQI_ERR_INVALID, "mqi_trace_rays: bad argument");
    if (id < 0 || id >= (int) c->children.size()) return fail(c, MQI_ERR_INVALID, "mqi_trace_rays: no such child");
    if (n_rays * (uint64_t) max_steps > (1ull << 31)) return fail(c, MQI_ERR_INVALID, "mqi_trace_rays: n_rays * max_steps too large");
    DeviceGuard g(c->device);
    const ChildHost& h = c->children[id];
    ChildDev d{};
    d.nx = h.nx; d.ny = h.ny; d.nz = h.nz; d.xe = h.xe; d.ye = h.ye; d.ze = h.ze; d.rho = h.rho;
    std::memcpy(d.rf, h.rf, sizeof(d.rf));
    std::memcpy(d.ri, h.ri, sizeof(d.ri));
    std::memcpy(d.tr, h.tr, sizeof(d.tr));
    d.identity = h.identity;
    const uint64_t slots = n_rays * (uint64_t) max_steps;
    float*    d_rays = nullptr;
    uint64_t* d_cnb = nullptr;
    float*    d_dist = nullptr;
    int32_t*  d_cells = nullptr;
    uint32_t* d_counts = nullptr;
    cudaError_t e = cudaMalloc(&d_rays, n_rays * 6 * sizeof(float) + 16);
    if (e == cudaSuccess) e = cudaMalloc(&d_cnb, slots * sizeof(uint64_t) + 16);
    if (e == cudaSuccess) e = cudaMalloc(&d_dist, slots * sizeof(float) + 16);
    if (e == cudaSuccess) e = cudaMalloc(&d_cells, slots * 3 * sizeof(int32_t) + 16);
    if (e == cudaSuccess) e = cudaMalloc(&d_counts, n_rays * sizeof(uint32_t) + 16);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_rays, rays, n_rays * 6 * sizeof(float), cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess) e = launch_trace_rays(d, d_rays, n_rays, max_steps, d_cnb, d_dist, d_cells, d_counts, c->stream);
    std::vector<uint32_t> counts(n_rays);
    std::vector<uint64_t> hc(slots);
    std::vector<float>    hd(slots);
    std::vector<int32_t>  hcell(slots * 3);
    if (e == cudaSuccess && n_rays) e = cudaMemcpyAsync(counts.data(), d_counts, n_rays * sizeof(uint32_t), cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess && slots) e = cudaMemcpyAsync(hc.data(), d_cnb, slots * sizeof(uint64_t), cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess && slots) e = cudaMemcpyAsync(hd.data(), d_dist, slots * sizeof(float), cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess && slots) e = cudaMemcpyAsync(hcell.data(), d_cells, slots * 3 * sizeof(int32_t), cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    cudaFree(d_rays); cudaFree(d_cnb); cudaFree(d_dist); cudaFree(d_cells); cudaFree(d_counts);
    if (e != cudaSuccess) return cuda_fail(c, e, "mqi_trace_rays");
    uint64_t total = 0;
    offsets[0] = 0;
    for (uint64_t r = 0; r < n_rays; ++r) {
        for (uint32_t k = 0; k < counts[r]; ++k) {
            if (total < capacity) {
                const uint64_t src = r * max_steps + k;
                if (cnb) cnb[total] = hc[src];
                if (dist) dist[total] = hd[src];
                if (cells) { cells[3 * total] = hcell[3 * src]; cells[3 * total + 1] = hcell[3 * src + 1]; cells[3 * total + 2] = hcell[3 * src + 2]; }
            }
            ++total;
        }
        offsets[r + 1] = (int64_t) total;
    }
    if (n_out) *n_out = total;
    if (total > capacity) return fail(c, MQI_ERR_OVERFLOW, "mqi_trace_rays: output capacity too small");
    return MQI_OK;
}

int
mqi_eval_physics(mqi_ctx* c, const float* energies, uint64_t n, float* out) {
    if (!valid_ctx(c) || (!energies && n) || (!out && n)) return fail(c, MQI_ERR_INVALID, "mqi_eval_physics: bad argument");
    DeviceGuard g(c->device);
    float* de = nullptr;
    float* dout = nullptr;
    cudaError_t e = cudaMalloc(&de, n * sizeof(float) + 16);
    if (e == cudaSuccess) e = cudaMalloc(&dout, n * 8 * sizeof(float) + 16);
    if (e == cudaSuccess) e = cudaMemcpyAsync(de, energies, n * sizeof(float), cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess) e = launch_eval_physics(c->tables, de, n, dout, c->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(out, dout, n * 8 * sizeof(float), cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    cudaFree(de);
    cudaFree(dout);
    if (e != cudaSuccess) return cuda_fail(c, e, "mqi_eval_physics");
    return MQI_OK;
}

int
mqi_eval_hits(mqi_ctx* c, int child_id, int scorer_type, const float* steps, const uint32_t* cnb,
              const int32_t* primary, uint64_t n, double* out) {
    if (!valid_ctx(c) || (n && (!steps || !cnb || !primary || !out)))
        return fail(c, MQI_ERR_INVALID, "mqi_eval_hits: bad argument");
    if (child_id < 0 || child_id >= (int) c->children.size() || !c->children[child_id].has_rho)
        return fail(c, MQI_ERR_INVALID, "mqi_eval_hits: no such child with a density");
    if (scorer_type < MQI_SCORER_EDEP || scorer_type > MQI_SCORER_DIJ)
        return fail(c, MQI_ERR_UNSUPPORTED, "mqi_eval_hits: unknown scorer type");
    const ChildHost& h = c->children[child_id];
    const uint64_t   nvox = (uint64_t) h.nx * h.ny * h.nz;
    for (uint64_t i = 0; i < n; ++i)
        if (cnb[i] >= nvox) return fail(c, MQI_ERR_INVALID, "mqi_eval_hits: a voxel index is outside the grid");
    ChildDev d{};
    d.nx = h.nx; d.ny = h.ny; d.nz = h.nz;
    d.xe = h.xe; d.ye = h.ye; d.ze = h.ze; d.rho = h.rho;
    std::memcpy(d.rf, h.rf, sizeof(d.rf));
    std::memcpy(d.ri, h.ri, sizeof(d.ri));
    std::memcpy(d.tr, h.tr, sizeof(d.tr));
    d.identity = h.identity;
    DeviceGuard g(c->device);
    float*    ds = nullptr;
    uint32_t* dc = nullptr;
    int32_t*  dp = nullptr;
    double*   dout = nullptr;
    cudaError_t e = cudaMalloc(&ds, n * 9 * sizeof(float) + 16);
    if (e == cudaSuccess) e = cudaMalloc(&dc, n * sizeof(uint32_t) + 16);
    if (e == cudaSuccess) e = cudaMalloc(&dp, n * sizeof(int32_t) + 16);
    if (e == cudaSuccess) e = cudaMalloc(&dout, n * sizeof(double) + 16);
    if (e == cudaSuccess) e = cudaMemcpyAsync(ds, steps, n * 9 * sizeof(float), cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dc, cnb, n * sizeof(uint32_t), cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dp, primary, n * sizeof(int32_t), cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess) e = launch_eval_hits(d, c->calib, c->physics_debug, scorer_type, ds, dc, dp, n, dout, c->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(out, dout, n * sizeof(double), cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    cudaFree(ds);
    cudaFree(dc);
    cudaFree(dp);
    cudaFree(dout);
    if (e != cudaSuccess) return cuda_fail(c, e, "mqi_eval_hits");
    return MQI_OK;
}

int
mqi_eval_roi(mqi_ctx* c, int scorer_id, const uint32_t* voxels, uint64_t n, int32_t* idx, int32_t* mask_idx) {
    if (!valid_ctx(c) || (n && (!voxels || !idx || !mask_idx))) return fail(c, MQI_ERR_INVALID, "mqi_eval_roi: bad argument");
    if (scorer_id < 0 || scorer_id >= (int) c->scorers.size()) return fail(c, MQI_ERR_INVALID, "mqi_eval_roi: no such scorer");
    const ScorerHost& s = c->scorers[scorer_id];
    const ChildHost&  h = c->children[s.child];
    const uint64_t    nvox = (uint64_t) h.nx * h.ny * h.nz;
    for (uint64_t i = 0; i < n; ++i)
        if (voxels[i] >= nvox) return fail(c, MQI_ERR_INVALID, "mqi_eval_roi: a voxel index is outside the grid");
    ScorerDev d{};
    d.type = s.type; d.roi_method = s.roi_method; d.stat_mode = s.stat_mode;
    d.roi_len = s.roi_len; d.start = s.start; d.stride = s.stride; d.acc = s.acc;
    DeviceGuard g(c->device);
    uint32_t* dv = nullptr;
    int32_t*  di = nullptr;
    int32_t*  dm = nullptr;
    cudaError_t e = cudaMalloc(&dv, n * sizeof(uint32_t) + 16);
    if (e == cudaSuccess) e = cudaMalloc(&di, n * sizeof(int32_t) + 16);
    if (e == cudaSuccess) e = cudaMalloc(&dm, n * sizeof(int32_t) + 16);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dv, voxels, n * sizeof(uint32_t), cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess) e = launch_eval_roi(d, dv, n, di, dm, c->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(idx, di, n * sizeof(int32_t), cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(mask_idx, dm, n * sizeof(int32_t), cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    cudaFree(dv);
    cudaFree(di);
    cudaFree(dm);
    if (e != cudaSuccess) return cuda_fail(c, e, "mqi_eval_roi");
    return MQI_OK;
}

}   // extern "C"

// ------------------------------------------------------------------------------------------
// Statistics: the stat scorer pair, the reference estimator, the batch estimator, averaging
// ------------------------------------------------------------------------------------------
namespace
{

int
ensure_stat_scratch(mqi_ctx* c) {
    if (!c->stat_scratch) MQI_CUDA(c, cudaMalloc(&c->stat_scratch, 4 * sizeof(unsigned long long)), "statistics scratch");
    return MQI_OK;
}

int
read_stat(mqi_ctx* c, double* mean_rel, uint64_t* n_vox) {
    unsigned long long h[3] = { 0, 0, 0 };
    MQI_CUDA(c, cudaMemcpyAsync(h, c->stat_scratch, sizeof(h), cudaMemcpyDeviceToHost, c->stream), "statistics");
    MQI_CUDA(c, cudaStreamSynchronize(c->stream), "statistics");
    double sum = 0.0;
    std::memcpy(&sum, &h[2], sizeof(sum));
    if (n_vox) *n_vox = h[1];
    if (mean_rel) *mean_rel = h[1] ? sum / (double) h[1] : 0.0;
    return MQI_OK;
}

}   // namespace

extern "C" {

int
mqi_add_stat_scorers(mqi_ctx* c, int child_id, int roi_method, uint32_t roi_length, const uint32_t* roi_start,
                     const uint32_t* roi_stride, const uint32_t* roi_acc, int* dose_id, int* dose2_id) {
    if (!valid_ctx(c)) return fail(c, MQI_ERR_INVALID, "mqi_add_stat_scorers: ctx is NULL");
    if (child_id < 0 || child_id >= (int) c->children.size())
        return fail(c, MQI_ERR_INVALID, "mqi_add_stat_scorers: no such child");
    if ((int) c->scorers.size() + 2 > kMaxScorers) return fail(c, MQI_ERR_INVALID, "mqi_add_stat_scorers: too many scorers");
    if (!c->scorers.empty() && c->scorers.back().child != child_id)
        for (auto& s : c->scorers)
            if (s.child == child_id) return fail(c, MQI_ERR_INVALID, "mqi_add_stat_scorers: add a child's scorers together");
    const ChildHost& ch   = c->children[child_id];
    const uint64_t   nvox = (uint64_t) ch.nx * ch.ny * ch.nz;
    DeviceGuard g(c->device);
    ScorerHost proto;
    proto.child      = child_id;
    proto.roi_method = roi_method;
    proto.stat_mode  = 1;
    proto.roi_len    = roi_length;
    if (roi_method == MQI_ROI_DIRECT) {
        proto.tally_len = nvox;
    } else if (roi_method == MQI_ROI_INDIRECT) {
        if (!roi_start || roi_length == 0)
            return fail(c, MQI_ERR_INVALID, "mqi_add_stat_scorers: INDIRECT needs roi_start (mask index per voxel) and the mask size");
        proto.tally_len = roi_length;
    } else if (roi_method == MQI_ROI_CONTOUR) {
        if (!roi_start || !roi_stride || !roi_acc || roi_length == 0)
            return fail(c, MQI_ERR_INVALID, "mqi_add_stat_scorers: CONTOUR needs start/stride/acc arrays");
        proto.tally_len = roi_acc[roi_length - 1];
    } else {
        return fail(c, MQI_ERR_INVALID, "mqi_add_stat_scorers: unknown roi method");
    }
    int ids[2];
    const int types[2] = { MQI_SCORER_DOSE_W, MQI_SCORER_DOSE_W2 };
    for (int k = 0; k < 2; ++k) {
        ScorerHost s = proto;
        s.type       = types[k];
        const uint64_t n_start = (roi_method == MQI_ROI_INDIRECT) ? nvox : roi_length;
        if (roi_method != MQI_ROI_DIRECT) {
            MQI_CUDA(c, cudaMalloc(&s.start, n_start * sizeof(uint32_t)), "mqi_add_stat_scorers");
            MQI_CUDA(c, cudaMemcpy(s.start, roi_start, n_start * sizeof(uint32_t), cudaMemcpyHostToDevice), "mqi_add_stat_scorers");
        }
        if (roi_method == MQI_ROI_CONTOUR) {
            MQI_CUDA(c, cudaMalloc(&s.stride, roi_length * sizeof(uint32_t)), "mqi_add_stat_scorers");
            MQI_CUDA(c, cudaMalloc(&s.acc, roi_length * sizeof(uint32_t)), "mqi_add_stat_scorers");
            MQI_CUDA(c, cudaMemcpy(s.stride, roi_stride, roi_length * sizeof(uint32_t), cudaMemcpyHostToDevice), "mqi_add_stat_scorers");
            MQI_CUDA(c, cudaMemcpy(s.acc, roi_acc, roi_length * sizeof(uint32_t), cudaMemcpyHostToDevice), "mqi_add_stat_scorers");
        }
        s.copies = c->n_scen;
        s.tstride = 2;
        if (k == 0) {
            // dose and dose^2 of a voxel side by side: the two per-step updates hit one 16-byte slot
            MQI_CUDA(c, cudaMalloc(&s.tally, 2 * s.total() * sizeof(double)), "mqi_add_stat_scorers");
            MQI_CUDA(c, cudaMemset(s.tally, 0, 2 * s.total() * sizeof(double)), "mqi_add_stat_scorers");
        } else {
            s.tally = c->scorers[ids[0]].tally + 1;
            s.owns  = false;
        }
        c->scorers.push_back(s);
        ids[k] = (int) c->scorers.size() - 1;
    }
    c->scorers[ids[0]].partner = ids[1];
    c->scorers[ids[1]].partner = ids[0];
    if (dose_id) *dose_id = ids[0];
    if (dose2_id) *dose2_id = ids[1];
    return MQI_OK;
}

int
mqi_stat_uncertainty(mqi_ctx* c, int dose_id, int dose2_id, uint64_t n_histories, float threshold, double* mean_rel_sigma,
                     uint64_t* n_voxels) {
    if (!valid_ctx(c)) return fail(c, MQI_ERR_INVALID, "mqi_stat_uncertainty: ctx is NULL");
    if (dose_id < 0 || dose_id >= (int) c->scorers.size() || dose2_id < 0 || dose2_id >= (int) c->scorers.size())
        return fail(c, MQI_ERR_INVALID, "mqi_stat_uncertainty: no such scorer");
    const ScorerHost& a = c->scorers[dose_id];
    const ScorerHost& b = c->scorers[dose2_id];
    if (a.tally_len != b.tally_len || a.tstride != b.tstride)
        return fail(c, MQI_ERR_INVALID, "mqi_stat_uncertainty: tallies differ in layout");
    if (n_histories < 2) return fail(c, MQI_ERR_INVALID, "mqi_stat_uncertainty: needs at least 2 histories");
    DeviceGuard g(c->device);
    if (ensure_stat_scratch(c) != MQI_OK) return MQI_ERR_NOMEM;
    // robust scenarios: each scenario's estimate; the worst one is returned
    double   worst = -1.0;
    uint64_t worst_n = 0;
    for (uint32_t k = 0; k < a.copies; ++k) {
        MQI_CUDA(c, launch_stat(a.tally + k * a.tally_len * a.tstride, b.tally + k * b.tally_len * b.tstride, a.tally_len,
                                a.tstride, (double) n_histories, 0, threshold, c->num_sms, c->stat_scratch, c->stream),
                 "mqi_stat_uncertainty");
        double   v = 0.0;
        uint64_t nv = 0;
        const int rc = read_stat(c, &v, &nv);
        if (rc != MQI_OK) return rc;
        if (v > worst) { worst = v; worst_n = nv; }
    }
    if (mean_rel_sigma) *mean_rel_sigma = worst;
    if (n_voxels) *n_voxels = worst_n;
    return MQI_OK;
}

int
mqi_batch_accumulate(mqi_ctx* c, int scorer_id) {
    if (!valid_ctx(c)) return fail(c, MQI_ERR_INVALID, "mqi_batch_accumulate: ctx is NULL");
    if (scorer_id < 0 || scorer_id >= (int) c->scorers.size()) return fail(c, MQI_ERR_INVALID, "mqi_batch_accumulate: no such scorer");
    ScorerHost& s = c->scorers[scorer_id];
    DeviceGuard g(c->device);
    if (!s.batch_s1) {
        MQI_CUDA(c, cudaMalloc(&s.batch_s1, s.total() * sizeof(double)), "mqi_batch_accumulate");
        MQI_CUDA(c, cudaMalloc(&s.batch_s2, s.total() * sizeof(double)), "mqi_batch_accumulate");
        MQI_CUDA(c, cudaMemsetAsync(s.batch_s1, 0, s.total() * sizeof(double), c->stream), "mqi_batch_accumulate");
        MQI_CUDA(c, cudaMemsetAsync(s.batch_s2, 0, s.total() * sizeof(double), c->stream), "mqi_batch_accumulate");
        s.n_batches = 0;
    }
    MQI_CUDA(c, launch_batch_fold(s.tally, s.tstride, s.batch_s1, s.batch_s2, s.total(), c->num_sms, c->stream),
             "mqi_batch_accumulate");
    MQI_CUDA(c, cudaStreamSynchronize(c->stream), "mqi_batch_accumulate");
    ++s.n_batches;
    return MQI_OK;
}

int
mqi_batch_uncertainty(mqi_ctx* c, int scorer_id, float threshold, double* mean_rel_sigma, uint64_t* n_voxels,
                      uint64_t* n_batches) {
    if (!valid_ctx(c)) return fail(c, MQI_ERR_INVALID, "mqi_batch_uncertainty: ctx is NULL");
    if (scorer_id < 0 || scorer_id >= (int) c->scorers.size()) return fail(c, MQI_ERR_INVALID, "mqi_batch_uncertainty: no such scorer");
    const ScorerHost& s = c->scorers[scorer_id];
    if (n_batches) *n_batches = s.n_batches;
    if (s.n_batches < 2) return fail(c, MQI_ERR_STATE, "mqi_batch_uncertainty: needs at least 2 accumulated batches");
    DeviceGuard g(c->device);
    if (ensure_stat_scratch(c) != MQI_OK) return MQI_ERR_NOMEM;
    double   worst = -1.0;
    uint64_t worst_n = 0;
    for (uint32_t k = 0; k < s.copies; ++k) {
        MQI_CUDA(c, launch_stat(s.batch_s1 + k * s.tally_len, s.batch_s2 + k * s.tally_len, s.tally_len, 1,
                                (double) s.n_batches, 1, threshold, c->num_sms, c->stat_scratch, c->stream),
                 "mqi_batch_uncertainty");
        double   v = 0.0;
        uint64_t nv = 0;
        const int rc = read_stat(c, &v, &nv);
        if (rc != MQI_OK) return rc;
        if (v > worst) { worst = v; worst_n = nv; }
    }
    if (mean_rel_sigma) *mean_rel_sigma = worst;
    if (n_voxels) *n_voxels = worst_n;
    return MQI_OK;
}

int
mqi_get_batch_mean(mqi_ctx* c, int scorer_id, double* out, uint64_t* n_out, int on_device) {
    if (!valid_ctx(c)) return fail(c, MQI_ERR_INVALID, "mqi_get_batch_mean: ctx is NULL");
    if (scorer_id < 0 || scorer_id >= (int) c->scorers.size()) return fail(c, MQI_ERR_INVALID, "mqi_get_batch_mean: no such scorer");
    const ScorerHost& s = c->scorers[scorer_id];
    if (n_out) *n_out = s.total();
    if (!out) return MQI_OK;
    if (s.n_batches == 0) return fail(c, MQI_ERR_STATE, "mqi_get_batch_mean: no accumulated batch");
    DeviceGuard g(c->device);
    double* dst = out;
    if (!on_device) MQI_CUDA(c, cudaMalloc(&dst, s.total() * sizeof(double)), "mqi_get_batch_mean");
    cudaError_t e = launch_copy_scaled(s.batch_s1, dst, s.total(), 1.0 / (double) s.n_batches, c->num_sms, c->stream);
    if (e == cudaSuccess && !on_device)
        e = cudaMemcpyAsync(out, dst, s.total() * sizeof(double), cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (!on_device) cudaFree(dst);
    if (e != cudaSuccess) return cuda_fail(c, e, "mqi_get_batch_mean");
    return MQI_OK;
}

int
mqi_scale_tally(mqi_ctx* c, int scorer_id, double weight) {
    if (!valid_ctx(c)) return fail(c, MQI_ERR_INVALID, "mqi_scale_tally: ctx is NULL");
    if (scorer_id < 0 || scorer_id >= (int) c->scorers.size()) return fail(c, MQI_ERR_INVALID, "mqi_scale_tally: no such scorer");
    const ScorerHost& s = c->scorers[scorer_id];
    DeviceGuard g(c->device);
    MQI_CUDA(c, launch_scale(s.tally, s.tstride, s.total(), weight, c->num_sms, c->stream), "mqi_scale_tally");
    MQI_CUDA(c, cudaStreamSynchronize(c->stream), "mqi_scale_tally");
    return MQI_OK;
}

int
mqi_run_until_stat(mqi_ctx* c, int dose_id, int dose2_id, uint64_t histories_per_run, float criteria, float threshold,
                   uint64_t max_runs, uint64_t seed, uint64_t* histories_done, double* achieved) {
    if (!valid_ctx(c)) return fail(c, MQI_ERR_INVALID, "mqi_run_until_stat: ctx is NULL");
    if (histories_per_run == 0 || histories_per_run > c->n_vertices)
        return fail(c, MQI_ERR_INVALID, "mqi_run_until_stat: histories_per_run must be 1..number of vertices");
    if (dose_id < 0 || dose_id >= (int) c->scorers.size() || !c->scorers[dose_id].stat_mode)
        return fail(c, MQI_ERR_INVALID, "mqi_run_until_stat: dose_id must be a stat scorer");
    uint64_t done = 0;
    double   stat = 1.0;   // current_stat = 100% before the first run (mqi_tps_env.hpp:1244)
    for (uint64_t run = 0; run < max_runs && stat > (double) criteria; ++run) {
        const int rc = mqi_transport(c, 0, histories_per_run, seed + 0x9E3779B97F4A7C15ull * run);
        if (rc != MQI_OK) return rc;
        done += histories_per_run;
        const int rs = mqi_stat_uncertainty(c, dose_id, dose2_id, done, threshold, &stat, nullptr);
        if (rs != MQI_OK) return rs;
    }
    // calculate_average_results (mqi_tps_env.hpp:1428-1476): the child's other scorers are scaled
    // to the planned number of histories
    const int child = c->scorers[dose_id].child;
    const double w  = (double) histories_per_run / (double) done;
    for (int i = 0; i < (int) c->scorers.size(); ++i) {
        const ScorerHost& s = c->scorers[i];
        if (s.child == child && !s.stat_mode) {
            const int rc = mqi_scale_tally(c, i, w);
            if (rc != MQI_OK) return rc;
        }
    }
    if (histories_done) *histories_done = done;
    if (achieved) *achieved = stat;
    return MQI_OK;
}

}   // extern "C"
