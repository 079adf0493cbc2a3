// Statistics kernels: the reference's uncertainty estimator, a batch estimator, and tally scaling.
//
// The reference computes, per stat-ROI voxel, sigma_i = sqrt((S2_i/n - (S1_i/n)^2) / (n - 1)) and
// mean_i = S1_i/n from per-step dose and dose^2 tallies (calculate_standard_deviation,
// moqui/kernel_functions/mqi_variables.hpp:19-48), then averages sigma_i/mean_i over the voxels
// whose mean exceeds threshold * max on the host (tps_env::calculate_stat,
// moqui/base/environments/mqi_tps_env.hpp:1338-1426).  Here both passes are device reductions
// over the dense tallies (one max pass, one sum pass), so only two numbers cross to the host.
#include <cstdint>
#include <cuda_runtime.h>

#include "mqi_internal.h"

namespace mqi_gpu
{

namespace
{

/// Positive doubles order like their bit patterns: atomicMax on the 64-bit image.
__device__ inline void
atomic_max_pos(unsigned long long* addr, double v) {
    if (v > 0.0) atomicMax(addr, (unsigned long long) __double_as_longlong(v));
}

__device__ inline double
warp_sum(double v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xFFFFFFFFu, v, o);
    return v;
}

__device__ inline double
warp_max(double v) {
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_down_sync(0xFFFFFFFFu, v, o));
    return v;
}

/// Per-voxel mean and relative sigma of the reference estimator (mqi_variables.hpp:38-45):
/// sigma is evaluated in double and rounded to float before the square root, as the reference
/// stores it in a float array; a negative variance from rounding gives 0 (the reference's sqrtf
/// of it would be NaN).
__device__ inline void
ref_mean_sigma(double s1, double s2, double n, float& mean, float& sigma) {
    const double m = s1 / n;
    float        v = (float) ((s2 / n - m * m) / (n - 1.0));
    if (!(v > 0.0f)) v = 0.0f;
    sigma = sqrtf(v);
    mean  = (float) m;
}

/// Batch estimator: relative standard error of the mean over B batches.
__device__ inline void
batch_mean_rel(double s1, double s2, double B, double& mean, double& rel) {
    mean = s1 / B;
    double var = (s2 / B - mean * mean) / (B - 1.0);   // variance of one batch
    if (!(var > 0.0)) var = 0.0;
    rel = (mean > 0.0) ? sqrt(var / B) / mean : 0.0;
}

__global__ void
k_stat_max(const double* __restrict__ s1, const double* __restrict__ s2, uint64_t n, uint32_t stride, double nh,
           int mode, unsigned long long* out_max) {
    double m = 0.0;
    for (uint64_t i = blockIdx.x * (uint64_t) blockDim.x + threadIdx.x; i < n; i += (uint64_t) gridDim.x * blockDim.x) {
        const double a = s1[i * stride];
        if (a > 0.0) {
            if (mode == 0) {
                float mean, sigma;
                ref_mean_sigma(a, s2[i * stride], nh, mean, sigma);
                m = fmax(m, (double) mean);
            } else {
                m = fmax(m, a / nh);
            }
        }
    }
    m = warp_max(m);
    if ((threadIdx.x & 31) == 0) atomic_max_pos(out_max, m);
}

__global__ void
k_stat_sum(const double* __restrict__ s1, const double* __restrict__ s2, uint64_t n, uint32_t stride, double nh,
           int mode, const unsigned long long* max_bits, float threshold, double* out_sum,
           unsigned long long* out_count) {
    const double cut = __longlong_as_double((long long) *max_bits) * (double) threshold;
    double       acc = 0.0;
    unsigned long long cnt = 0;
    for (uint64_t i = blockIdx.x * (uint64_t) blockDim.x + threadIdx.x; i < n; i += (uint64_t) gridDim.x * blockDim.x) {
        const double a = s1[i * stride];
        if (!(a > 0.0)) continue;
        if (mode == 0) {
            float mean, sigma;
            ref_mean_sigma(a, s2[i * stride], nh, mean, sigma);
            if ((double) mean > cut) {   // dose_mean[i] > dose_max * stat_threshold (mqi_tps_env.hpp:1418)
                acc += (double) (sigma / mean);
                ++cnt;
            }
        } else {
            double mean, rel;
            batch_mean_rel(a, s2[i * stride], nh, mean, rel);
            if (mean > cut) {
                acc += rel;
                ++cnt;
            }
        }
    }
    acc = warp_sum(acc);
    for (int o = 16; o > 0; o >>= 1) cnt += __shfl_down_sync(0xFFFFFFFFu, cnt, o);
    if ((threadIdx.x & 31) == 0 && cnt) {
        atomicAdd(out_sum, acc);
        atomicAdd(out_count, cnt);
    }
}

__global__ void
k_batch_fold(double* __restrict__ tally, uint32_t stride, double* __restrict__ s1, double* __restrict__ s2, uint64_t n) {
    for (uint64_t i = blockIdx.x * (uint64_t) blockDim.x + threadIdx.x; i < n; i += (uint64_t) gridDim.x * blockDim.x) {
        const double t = tally[i * stride];
        if (t != 0.0) {
            s1[i] += t;
            s2[i] += t * t;
            tally[i * stride] = 0.0;
        }
    }
}

__global__ void
k_scale(double* __restrict__ a, uint32_t stride, uint64_t n, double w) {
    for (uint64_t i = blockIdx.x * (uint64_t) blockDim.x + threadIdx.x; i < n; i += (uint64_t) gridDim.x * blockDim.x)
        a[i * stride] *= w;
}

__global__ void
k_copy_strided(const double* __restrict__ a, uint32_t stride, double* __restrict__ out, uint64_t n) {
    for (uint64_t i = blockIdx.x * (uint64_t) blockDim.x + threadIdx.x; i < n; i += (uint64_t) gridDim.x * blockDim.x)
        out[i] = a[i * stride];
}

__global__ void
k_copy_scaled(const double* __restrict__ a, double* __restrict__ out, uint64_t n, double w) {
    for (uint64_t i = blockIdx.x * (uint64_t) blockDim.x + threadIdx.x; i < n; i += (uint64_t) gridDim.x * blockDim.x)
        out[i] = a[i] * w;
}

unsigned
grid_for(uint64_t n, int sms) {
    const uint64_t b = (n + 255) / 256;
    const uint64_t cap = (uint64_t) sms * 16;
    return (unsigned) (b < cap ? (b ? b : 1) : cap);
}

}   // namespace

cudaError_t
launch_stat(const double* s1, const double* s2, uint64_t n, uint32_t stride, double nh, int mode, float threshold,
            int sms, unsigned long long* scratch, cudaStream_t s) {
    // scratch: [0] max bits, [1] count, [2] sum (as double bits)
    cudaError_t e = cudaMemsetAsync(scratch, 0, 3 * sizeof(unsigned long long), s);
    if (e != cudaSuccess) return e;
    const unsigned g = grid_for(n, sms);
    k_stat_max<<<g, 256, 0, s>>>(s1, s2, n, stride, nh, mode, scratch);
    k_stat_sum<<<g, 256, 0, s>>>(s1, s2, n, stride, nh, mode, scratch, threshold, reinterpret_cast<double*>(scratch + 2),
                                 scratch + 1);
    return cudaGetLastError();
}

cudaError_t
launch_batch_fold(double* tally, uint32_t stride, double* s1, double* s2, uint64_t n, int sms, cudaStream_t s) {
    k_batch_fold<<<grid_for(n, sms), 256, 0, s>>>(tally, stride, s1, s2, n);
    return cudaGetLastError();
}

cudaError_t
launch_scale(double* a, uint32_t stride, uint64_t n, double w, int sms, cudaStream_t s) {
    k_scale<<<grid_for(n, sms), 256, 0, s>>>(a, stride, n, w);
    return cudaGetLastError();
}

cudaError_t
launch_copy_strided(const double* a, uint32_t stride, double* out, uint64_t n, int sms, cudaStream_t s) {
    k_copy_strided<<<grid_for(n, sms), 256, 0, s>>>(a, stride, out, n);
    return cudaGetLastError();
}

cudaError_t
launch_copy_scaled(const double* a, double* out, uint64_t n, double w, int sms, cudaStream_t s) {
    k_copy_scaled<<<grid_for(n, sms), 256, 0, s>>>(a, out, n, w);
    return cudaGetLastError();
}

}   // namespace mqi_gpu
