// Dij kernels: compaction of the (spot, voxel) hash table, a stable LSD radix sort, the two CSR
// layouts, and the sparse products dose = D.w and grad = D^T.g.
//
// The reference scores Dij into an open-addressing table keyed by (voxel, spot)
// (insert_hashtable, moqui/kernel_functions/mqi_transport.hpp:68-111) and writes it as a
// spot-row CSR npz in table-scan order (save_to_npz, moqui/base/mqi_io.hpp:251-320).  Here the
// table is compacted and sorted on the device, so both layouts come out in a fixed order:
//   spot rows  (the reference's npz layout, shape [n_spots, n_voxels]): indptr / voxel / value,
//              voxels ascending in a row -- the transposed operator, read by D^T.g;
//   voxel rows (only voxels with an entry, "doubly compressed"): row voxel / indptr / spot /
//              value, spots ascending in a row -- read by D.w.
// Both products are gathers with a fixed reduction order: no atomics, reproducible results.
#include <algorithm>
#include <cstdint>
#include <cuda_runtime.h>

#include "mqi_internal.h"

namespace mqi_gpu
{

namespace
{

constexpr int kThreads = 256;   // radix sort block
constexpr int kItems   = 8;     // keys per thread per pass
constexpr int kTile    = kThreads * kItems;
constexpr int kScanTile = 2048;

__device__ inline unsigned
lanemask_lt() {
    return (1u << (threadIdx.x & 31)) - 1u;
}

// ---- compaction -----------------------------------------------------------------------------

/// Append every occupied slot as (spot * n_voxels + voxel, slot index); warp-aggregated cursor.
__global__ void
k_dij_compact(const DijSlot* __restrict__ tab, uint64_t cap, uint64_t n_voxels, unsigned long long* __restrict__ keys,
              uint32_t* __restrict__ idx, uint64_t n_max, unsigned long long* __restrict__ cursor) {
    const uint64_t stride = (uint64_t) gridDim.x * blockDim.x;
    const uint64_t span   = (cap + stride - 1) / stride * stride;   // every lane runs the same trip count
    for (uint64_t i = blockIdx.x * (uint64_t) blockDim.x + threadIdx.x; i < span; i += stride) {
        unsigned long long k = 0;
        if (i < cap) k = tab[i].key;
        const bool     valid = k != 0ull;
        const unsigned b     = __ballot_sync(0xFFFFFFFFu, valid);
        if (!b) continue;
        unsigned long long base = 0;
        const int          lead = __ffs(b) - 1;
        if ((int) (threadIdx.x & 31) == lead) base = atomicAdd(cursor, (unsigned long long) __popc(b));
        base = __shfl_sync(0xFFFFFFFFu, base, lead);
        if (valid) {
            const unsigned long long raw   = k - 1ull;
            const uint64_t           spot  = raw >> 32;
            const uint64_t           voxel = raw & 0xFFFFFFFFull;
            const uint64_t           pos   = base + __popc(b & lanemask_lt());
            if (pos < n_max) {   // the host compares the cursor with n_max afterwards
                keys[pos] = spot * n_voxels + voxel;
                idx[pos]  = (uint32_t) i;
            }
        }
    }
}

/// *out += the number of occupied slots (nonzero keys) of the table: a grid-stride count, one
/// atomic per warp.
__global__ void
k_dij_count(const DijSlot* __restrict__ tab, uint64_t cap, unsigned long long* __restrict__ out) {
    const uint64_t     stride = (uint64_t) gridDim.x * blockDim.x;
    unsigned long long n      = 0;
    for (uint64_t i = blockIdx.x * (uint64_t) blockDim.x + threadIdx.x; i < cap; i += stride) n += tab[i].key != 0ull;
    for (int o = 16; o > 0; o >>= 1) n += __shfl_down_sync(0xFFFFFFFFu, n, o);
    if ((threadIdx.x & 31) == 0 && n) atomicAdd(out, n);
}

// ---- exclusive scan of u32 ------------------------------------------------------------------

__device__ inline uint32_t
block_exclusive_scan(uint32_t v, uint32_t* warp_sums, uint32_t& total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    uint32_t  x    = v;
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_sums[warp] = x;
    __syncthreads();
    if (warp == 0) {
        uint32_t s = lane < nw ? warp_sums[lane] : 0u;
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, s, o);
            if (lane >= o) s += y;
        }
        if (lane < nw) warp_sums[lane] = s;
    }
    __syncthreads();
    const uint32_t warp_off = warp ? warp_sums[warp - 1] : 0u;
    total                   = warp_sums[nw - 1];
    __syncthreads();
    return warp_off + x - v;
}

/// Per-tile exclusive scan (kScanTile elements per 256-thread block, 8 per thread in order);
/// tile totals to `sums`.
__global__ void
k_scan_tiles(const uint32_t* __restrict__ in, uint32_t* __restrict__ out, uint64_t n, uint32_t* __restrict__ sums) {
    __shared__ uint32_t ws[32];
    const uint64_t t0 = (uint64_t) blockIdx.x * kScanTile + (uint64_t) threadIdx.x * 8;
    uint32_t       v[8], s = 0;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        v[k] = (t0 + k < n) ? in[t0 + k] : 0u;
        s += v[k];
    }
    uint32_t total;
    uint32_t run = block_exclusive_scan(s, ws, total);
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        if (t0 + k < n) out[t0 + k] = run;
        run += v[k];
    }
    if (threadIdx.x == 0) sums[blockIdx.x] = total;
}

/// Exclusive scan of the tile totals by one block, in order.
__global__ void
k_scan_sums(uint32_t* __restrict__ sums, uint64_t n) {
    __shared__ uint32_t ws[32];
    uint32_t carry = 0;
    for (uint64_t b = 0; b < n; b += blockDim.x) {
        const uint64_t i = b + threadIdx.x;
        const uint32_t v = i < n ? sums[i] : 0u;
        uint32_t total;
        const uint32_t e = block_exclusive_scan(v, ws, total);
        if (i < n) sums[i] = carry + e;
        carry += total;
        __syncthreads();
    }
}

__global__ void
k_scan_add(uint32_t* __restrict__ out, uint64_t n, const uint32_t* __restrict__ sums) {
    const uint64_t i = (uint64_t) blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] += sums[i / kScanTile];
}

// ---- radix sort -----------------------------------------------------------------------------

__global__ void
k_radix_hist(const unsigned long long* __restrict__ keys, uint64_t n, int shift, uint32_t* __restrict__ hist,
             uint32_t n_tiles) {
    __shared__ uint32_t cnt[256];
    cnt[threadIdx.x] = 0;
    __syncthreads();
    const uint64_t t0 = (uint64_t) blockIdx.x * kTile;
#pragma unroll
    for (int r = 0; r < kItems; ++r) {
        const uint64_t i = t0 + (uint64_t) r * kThreads + threadIdx.x;
        if (i < n) atomicAdd(&cnt[(keys[i] >> shift) & 255u], 1u);
    }
    __syncthreads();
    hist[(uint64_t) threadIdx.x * n_tiles + blockIdx.x] = cnt[threadIdx.x];
}

/// Stable scatter of one 8-bit digit.  The tile is visited in input order (round, warp, lane);
/// an element's destination is its tile's digit offset + the count of equal digits before it in
/// earlier rounds, earlier warps of its round, and lower lanes of its warp.
__global__ void
k_radix_scatter(const unsigned long long* __restrict__ kin, const uint32_t* __restrict__ vin,
                unsigned long long* __restrict__ kout, uint32_t* __restrict__ vout, uint64_t n, int shift,
                const uint32_t* __restrict__ offs, uint32_t n_tiles) {
    constexpr int kWarps = kThreads / 32;
    __shared__ uint32_t base[256];
    __shared__ uint32_t wcnt[kWarps][256];
    __shared__ uint32_t wpre[kWarps][256];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    base[threadIdx.x] = offs[(uint64_t) threadIdx.x * n_tiles + blockIdx.x];
#pragma unroll
    for (int w = 0; w < kWarps; ++w) wcnt[w][threadIdx.x] = 0;
    __syncthreads();
    const uint64_t t0 = (uint64_t) blockIdx.x * kTile;
    for (int r = 0; r < kItems; ++r) {
        const uint64_t i     = t0 + (uint64_t) r * kThreads + threadIdx.x;
        const bool     valid = i < n;
        unsigned long long k = 0;
        uint32_t           v = 0;
        uint32_t           d = 0x100u;   // matches no digit
        if (valid) {
            k = kin[i];
            v = vin[i];
            d = (uint32_t) ((k >> shift) & 255u);
        }
        const unsigned peers = __match_any_sync(0xFFFFFFFFu, d);
        const uint32_t rank  = __popc(peers & lanemask_lt());
        if (valid && lane == __ffs(peers) - 1) wcnt[warp][d] = __popc(peers);
        __syncthreads();
        {
            const int dd  = threadIdx.x;
            uint32_t  run = base[dd];
#pragma unroll
            for (int w = 0; w < kWarps; ++w) {
                const uint32_t c = wcnt[w][dd];
                wpre[w][dd]      = run;
                run += c;
                wcnt[w][dd] = 0;
            }
            base[dd] = run;
        }
        __syncthreads();
        if (valid) {
            const uint32_t pos = wpre[warp][d] + rank;
            kout[pos] = k;
            vout[pos] = v;
        }
        __syncthreads();
    }
}

// ---- CSR assembly ---------------------------------------------------------------------------

/// indptr[r] = lower_bound(keys, r * row_span) for r in [0, n_rows].
__global__ void
k_row_bounds(const unsigned long long* __restrict__ keys, uint64_t n, uint64_t row_span, uint64_t n_rows,
             uint64_t* __restrict__ indptr) {
    const uint64_t r = (uint64_t) blockIdx.x * blockDim.x + threadIdx.x;
    if (r > n_rows) return;
    const unsigned long long target = r * row_span;
    uint64_t lo = 0, hi = n;
    while (lo < hi) {
        const uint64_t mid = (lo + hi) >> 1;
        if (keys[mid] < target) lo = mid + 1; else hi = mid;
    }
    indptr[r] = lo;
}

/// Spot-row CSR entries: voxel column and FP32 value (FP64 tally x scale, rounded once).
__global__ void
k_spot_rows(const unsigned long long* __restrict__ keys, const uint32_t* __restrict__ slot, uint64_t n,
            uint64_t n_voxels, const DijSlot* __restrict__ tab, double scale, uint32_t* __restrict__ vox,
            float* __restrict__ val, unsigned long long* __restrict__ vkeys, uint32_t* __restrict__ vpos) {
    const uint64_t k = (uint64_t) blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const uint32_t v = (uint32_t) (keys[k] % n_voxels);
    vox[k]   = v;
    val[k]   = (float) (tab[slot[k]].value * scale);
    vkeys[k] = v;
    vpos[k]  = (uint32_t) k;
}

__global__ void
k_row_flags(const unsigned long long* __restrict__ vkeys, uint64_t n, uint32_t* __restrict__ flags) {
    const uint64_t j = (uint64_t) blockIdx.x * blockDim.x + threadIdx.x;
    if (j < n) flags[j] = (j == 0 || vkeys[j] != vkeys[j - 1]) ? 1u : 0u;
}

/// Voxel-row entries: spot column and value from the spot-row entry they came from; row starts.
__global__ void
k_voxel_rows(const unsigned long long* __restrict__ vkeys, const uint32_t* __restrict__ vpos, uint64_t n,
             const unsigned long long* __restrict__ skeys, uint64_t n_voxels, const float* __restrict__ sval,
             const uint32_t* __restrict__ flags, const uint32_t* __restrict__ rowid, uint32_t* __restrict__ row_voxel,
             uint64_t* __restrict__ indptr, uint32_t* __restrict__ spot, float* __restrict__ val) {
    const uint64_t j = (uint64_t) blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    const uint32_t p = vpos[j];
    spot[j] = (uint32_t) (skeys[p] / n_voxels);
    val[j]  = sval[p];
    if (flags[j]) {
        row_voxel[rowid[j]] = (uint32_t) vkeys[j];
        indptr[rowid[j]]    = j;
    }
    if (j == n - 1) indptr[rowid[j] + flags[j]] = n;
}

// ---- backward segments: their work order ---------------------------------------------------

/// Sort keys of the backward's work order: the voxel of each segment's first entry (the keys are
/// the sorted spot * n_voxels + voxel pairs).
__global__ void
k_seg_keys(const uint64_t* __restrict__ seg_start, uint32_t n_seg, const unsigned long long* __restrict__ keys,
           uint64_t n_voxels, unsigned long long* __restrict__ okeys, uint32_t* __restrict__ oval) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_seg) return;
    okeys[i] = keys[seg_start[i]] % n_voxels;
    oval[i]  = i;
}

// ---- products -------------------------------------------------------------------------------

/// Block b of the staged forward owns the voxel rows that start in entries [b * kFwdEntries,
/// (b + 1) * kFwdEntries): row_first[b] = the first row r with indptr[r] >= b * kFwdEntries, and
/// run_k[b] = indptr[row_first[b]], the run's first entry.  One thread per block boundary, a binary
/// search over indptr (once per Dij build).
__global__ void
k_fwd_blocks(const uint64_t* __restrict__ indptr, uint64_t n_rows, uint64_t n_blocks, uint32_t* __restrict__ row_first,
             uint64_t* __restrict__ run_k) {
    const uint64_t b = (uint64_t) blockIdx.x * blockDim.x + threadIdx.x;
    if (b > n_blocks) return;
    const uint64_t target = b * kFwdEntries;
    uint64_t lo = 0, hi = n_rows;   // first r in [0, n_rows] with indptr[r] >= target
    while (lo < hi) {
        const uint64_t mid = (lo + hi) >> 1;
        if (indptr[mid] < target) lo = mid + 1; else hi = mid;
    }
    const uint64_t r = b == n_blocks ? n_rows : lo;
    row_first[b]     = (uint32_t) r;
    run_k[b]         = indptr[r];
}

/// dose[row_voxel[r]] = sum_k val[k] * w[spot[k]] over voxel rows (D.w).  A block stages the
/// products of its rows' entries -- a contiguous run of at most kFwdEntries + the longest row,
/// read with coalesced loads -- in shared memory, then each thread sums whole rows from there in
/// entry order (a fixed order: the result does not depend on the launch).  A run longer than the
/// staging buffer (a row of more than kFwdStage - kFwdEntries entries) is summed from global
/// memory instead, in the same order.  Accumulates in T.
template<typename T>
__global__ void __launch_bounds__(256)
k_dij_forward(const uint32_t* __restrict__ row_voxel, const uint64_t* __restrict__ indptr,
              const uint32_t* __restrict__ row_first, const uint32_t* __restrict__ spot, const float* __restrict__ val,
              const T* __restrict__ w, T* __restrict__ dose) {
    extern __shared__ __align__(16) unsigned char fwd_smem[];
    T* prod = reinterpret_cast<T*>(fwd_smem);
    const uint32_t r0 = row_first[blockIdx.x], r1 = row_first[blockIdx.x + 1];
    if (r0 >= r1) return;
    const uint64_t k0 = indptr[r0], k1 = indptr[r1];
    const bool     staged = k1 - k0 <= kFwdStage;
    // the thread's first row is read before the staging, so that its latency overlaps it
    uint32_t r  = r0 + threadIdx.x;
    uint64_t rb = 0, re = 0;
    uint32_t rv = 0;
    if (r < r1) {
        rb = indptr[r];
        re = indptr[r + 1];
        rv = row_voxel[r];
    }
    if (staged) {
        // 16-byte loads of whole groups of four entries (the arrays are padded to whole groups);
        // entries of the group outside [k0, k1) are skipped
        const uint4*   s4 = reinterpret_cast<const uint4*>(spot);
        const float4*  v4 = reinterpret_cast<const float4*>(val);
        const uint64_t q1 = (k1 + 3) >> 2;
#pragma unroll 2
        for (uint64_t q = (k0 >> 2) + threadIdx.x; q < q1; q += blockDim.x) {
            const uint4    ss = s4[q];
            const float4   vv = v4[q];
            const uint64_t k  = q << 2;
            if (k >= k0 && k < k1) prod[k - k0] = (T) vv.x * w[ss.x];
            if (k + 1 >= k0 && k + 1 < k1) prod[k + 1 - k0] = (T) vv.y * w[ss.y];
            if (k + 2 >= k0 && k + 2 < k1) prod[k + 2 - k0] = (T) vv.z * w[ss.z];
            if (k + 3 >= k0 && k + 3 < k1) prod[k + 3 - k0] = (T) vv.w * w[ss.w];
        }
        __syncthreads();
    }
    while (r < r1) {
        T acc = T(0);
        if (staged)
            for (uint64_t k = rb; k < re; ++k) acc += prod[k - k0];
        else
            for (uint64_t k = rb; k < re; ++k) acc += (T) val[k] * w[spot[k]];
        dose[rv] = acc;
        r += blockDim.x;
        if (r < r1) {
            rb = indptr[r];
            re = indptr[r + 1];
            rv = row_voxel[r];
        }
    }
}

// ---- bulk copies: the copy engine (untiled cp.async.bulk) completing on a shared-memory mbarrier

__device__ __forceinline__ uint32_t
smem_u32(const void* p) {
    return (uint32_t) __cvta_generic_to_shared(p);
}

__device__ __forceinline__ void
mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void
mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}

/// Global -> shared copy of `bytes` (a multiple of 16, both addresses 16-byte aligned) that
/// completes its bytes on `bar`.
__device__ __forceinline__ void
bulk_load(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                 ::"r"(smem_u32(dst)), "l"(src), "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}

__device__ __forceinline__ bool
mbar_try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                 "selp.u32 %0, 1, 0, p;\n\t}"
                 : "=r"(ok)
                 : "r"(smem_u32(bar)), "r"(parity)
                 : "memory");
    return ok != 0;
}

/// The rows and entries of one run of the persistent forward, as thread 0 found them.
struct FwdRun {
    unsigned long long k0, k1, a0;   // entries [k0, k1); staged from a0 (k0 rounded down to a group of four)
    uint32_t           r0, r1;       // voxel rows [r0, r1)
    uint32_t           staged, pad;
};
static_assert(sizeof(FwdRun) == 40, "FwdRun layout");

constexpr uint32_t kFwdPipeHeader     = 256;                                  // kFwdStages mbarriers + FwdRuns
constexpr uint32_t kFwdPipeStageBytes = (uint32_t) kFwdPipeStageEntries * 8;  // spots then values
static_assert(kFwdStages * (8 + sizeof(FwdRun)) <= kFwdPipeHeader, "forward header");

/// D.w in FP32, persistent, through a ring of kFwdStages shared-memory stages.  Each CTA walks the
/// runs b = blockIdx.x, blockIdx.x + gridDim.x, ... (run b: the voxel rows that start in entries
/// [b * kFwdEntries, (b + 1) * kFwdEntries), row_first[b] to row_first[b + 1], first entry
/// run_k[b]).  While the block forms and sums run i from one stage, the copy engine fills the
/// others with runs i + 1 .. i + kFwdStages - 1: thread 0 issues two untiled bulk copies per run
/// (its spots and values, rounded out to whole 16-byte groups; the arrays are padded) completing
/// on that stage's mbarrier, so each CTA keeps kFwdStages - 1 runs' bytes in flight while it
/// computes.  In a run the block multiplies each value by w[spot] in place, then each thread sums
/// whole rows from there in entry order (as k_dij_forward does): the result does not depend on
/// the grid.  Waits are bounded: a block whose copies have not landed after ~1 s of polling sets
/// bit 8 of `err`, waits (bounded) for its other stages' copies and returns.  A run longer than a
/// stage (kFwdPipeStageEntries entries: a row of more than ~2000 spots) is summed from global memory.
__global__ void __launch_bounds__(kFwdPipeThreads)
k_dij_forward_pipe(const uint32_t* __restrict__ row_voxel, const uint64_t* __restrict__ indptr,
                   const uint32_t* __restrict__ row_first, const uint64_t* __restrict__ run_k, uint64_t n_blocks,
                   const uint32_t* __restrict__ spot, const float* __restrict__ val, const float* __restrict__ w,
                   float* __restrict__ dose, uint32_t* __restrict__ err) {
    extern __shared__ __align__(16) unsigned char fwd_smem[];
    uint64_t*      bar  = reinterpret_cast<uint64_t*>(fwd_smem);
    FwdRun*        runs = reinterpret_cast<FwdRun*>(fwd_smem + 8 * kFwdStages);
    unsigned char* data = fwd_smem + kFwdPipeHeader;
    const int      tid  = threadIdx.x;
    const uint64_t step = gridDim.x;

    // Thread 0 reads a run's bounds one run before it starts that run's copies, so the loads'
    // latency passes while the block computes.
    uint32_t           pf_r0 = 0, pf_r1 = 0;
    unsigned long long pf_k0 = 0, pf_k1 = 0;
    auto fetch = [&](uint64_t b) {
        pf_r0 = row_first[b];
        pf_r1 = row_first[b + 1];
        pf_k0 = run_k[b];
        pf_k1 = run_k[b + 1];
    };
    // thread 0: describe the fetched run in stage s and start its copies
    auto issue = [&](int s) {
        FwdRun R;
        R.r0  = pf_r0;
        R.r1  = pf_r1;
        R.k0  = pf_k0;
        R.k1  = pf_k1;
        R.a0  = R.k0 & ~3ull;
        R.pad = 0;
        const unsigned long long a1 = (R.k1 + 3ull) & ~3ull;
        R.staged = (R.r0 < R.r1 && a1 - R.a0 <= kFwdPipeStageEntries) ? 1u : 0u;
        if (R.staged) {
            const uint32_t bytes = (uint32_t) ((a1 - R.a0) * sizeof(uint32_t));
            unsigned char* st    = data + (size_t) s * kFwdPipeStageBytes;
            mbar_expect_tx(&bar[s], 2 * bytes);
            bulk_load(st, spot + R.a0, bytes, &bar[s]);
            bulk_load(st + kFwdPipeStageEntries * sizeof(uint32_t), val + R.a0, bytes, &bar[s]);
        }
        runs[s] = R;
    };

    if (tid == 0) {
        for (int s = 0; s < kFwdStages; ++s) mbar_init(&bar[s], 1);
        // the first kFwdStages - 1 runs start at once
        uint64_t b = blockIdx.x;
        for (int s = 0; s < kFwdStages - 1 && b < n_blocks; ++s, b += step) {
            fetch(b);
            issue(s);
        }
        if (b < n_blocks) fetch(b);
    }
    __syncthreads();
    uint32_t parity = 0;   // bit s: the phase of stage s's barrier to wait for next
    bool     failed = false;
    int      s      = 0;   // the stage of run i
    uint64_t b      = blockIdx.x;
    for (; b < n_blocks; b += step) {
        const uint64_t ahead = b + (kFwdStages - 1) * step;     // the run that goes into the stage freed last
        const int      sf    = s == 0 ? kFwdStages - 1 : s - 1;
        if (tid == 0 && ahead < n_blocks) {
            issue(sf);
            if (ahead + step < n_blocks) fetch(ahead + step);
        }
        const FwdRun R = runs[s];
        if (R.r0 < R.r1) {
            uint32_t r  = R.r0 + tid;
            uint64_t rb = 0, re = 0;
            uint32_t rv = 0;
            if (r < R.r1) {
                rb = indptr[r];
                re = indptr[r + 1];
                rv = row_voxel[r];
            }
            uint32_t* s_spot = reinterpret_cast<uint32_t*>(data + (size_t) s * kFwdPipeStageBytes);
            float*    s_val  = reinterpret_cast<float*>(data + (size_t) s * kFwdPipeStageBytes +
                                                       kFwdPipeStageEntries * sizeof(uint32_t));
            if (R.staged) {
                bool     done  = false;
                uint32_t spins = 0;
                while (!(done = mbar_try_wait(&bar[s], (parity >> s) & 1u)) && ++spins < kBulkSpinLimit) {
                }
                parity ^= 1u << s;
                if (__syncthreads_or(!done)) {
                    failed = true;
                    break;
                }
                for (uint64_t k = R.k0 + tid; k < R.k1; k += blockDim.x) s_val[k - R.a0] *= w[s_spot[k - R.a0]];
                __syncthreads();
            }
            while (r < R.r1) {
                float acc = 0.0f;
                if (R.staged)
                    for (uint64_t k = rb; k < re; ++k) acc += s_val[k - R.a0];
                else
                    for (uint64_t k = rb; k < re; ++k) acc += val[k] * w[spot[k]];
                dose[rv] = acc;
                r += blockDim.x;
                if (r < R.r1) {
                    rb = indptr[r];
                    re = indptr[r + 1];
                    rv = row_voxel[r];
                }
            }
        }
        __syncthreads();   // stage s is free: the next iteration refills it
        s = s + 1 == kFwdStages ? 0 : s + 1;
    }
    if (failed && tid == 0) {
        atomicOr(err, 8u);
        // copies started for the other stages may still be landing: wait for them (bounded) before
        // the block's shared memory is released
        for (int k = 1; k < kFwdStages; ++k) {
            const int      so = (s + k) % kFwdStages;
            const uint64_t bo = b + (uint64_t) k * step;
            if (bo < n_blocks && runs[so].staged)
                for (uint32_t spins = 0; !mbar_try_wait(&bar[so], (parity >> so) & 1u) && spins < kBulkSpinLimit; ++spins) {
                }
        }
    }
}

/// grad[s] = sum_k val[k] * g[voxel[k]] over spot rows (the transposed operator), in two passes
/// with a fixed order.  Pass 1 (k_dij_backward_segments): the entries are cut into segments of at
/// most kDijSegment entries that never cross a row; one block sums a segment's products (signed
/// terms of a gradient cancel, so plain FP32 sums lose digits: a double-float accumulator per
/// thread for FP32 g, FP64 for FP64 g; FP64 across the block) into one FP64 partial.  Pass 2
/// (k_dij_backward_rows): one thread per row adds its segments' partials in order.  Rows of very
/// different lengths (1e4 to 3e6 entries at 2000 spots) thereby spread over every SM.
/// s + c += a * b with no rounding error in the product (TwoProd: one FMA gives the product's
/// rounding error) and Knuth's TwoSum for the addition: a double-float accumulator of about 48
/// significant bits on the FP32 pipes.  GB300's FP64 pipe is far narrower than its FP32 pipes,
/// and an FP64 multiply-add per entry (with two conversions) made the backward FP64-bound.
__device__ __forceinline__ void
df_fma(float& s, float& c, float a, float b) {
    const float p   = __fmul_rn(a, b);
    const float pe  = __fmaf_rn(a, b, -p);
    const float t   = __fadd_rn(s, p);
    const float z   = __fsub_rn(t, s);
    const float err = __fadd_rn(__fsub_rn(s, __fsub_rn(t, z)), __fsub_rn(p, z));
    c               = __fadd_rn(c, __fadd_rn(err, pe));
    s               = t;
}

/// A block's share of the products of entries [b, e) of a spot row, per thread, in a fixed order:
/// thread t takes the groups of four q = (b >> 2) + t, + blockDim.x, ... (16-byte loads of voxels
/// and values, four independent gathers of g per group; the arrays are padded to whole groups).
template<typename T>
__device__ __forceinline__ double
segment_sum(uint64_t b, uint64_t e, const uint32_t* __restrict__ vox, const float* __restrict__ val,
            const T* __restrict__ g) {
    const uint4*   v4 = reinterpret_cast<const uint4*>(vox);
    const float4*  a4 = reinterpret_cast<const float4*>(val);
    const uint64_t q1 = (e + 3) >> 2;
    if constexpr (sizeof(T) == sizeof(float)) {
        float s = 0.0f, c = 0.0f;
#pragma unroll 4
        for (uint64_t q = (b >> 2) + threadIdx.x; q < q1; q += blockDim.x) {
            const uint4    vv = v4[q];
            const float4   aa = a4[q];
            const uint64_t k  = q << 2;
            const bool     m0 = k >= b && k < e, m1 = k + 1 >= b && k + 1 < e;
            const bool     m2 = k + 2 >= b && k + 2 < e, m3 = k + 3 >= b && k + 3 < e;
            const float    g0 = m0 ? g[vv.x] : 0.0f, g1 = m1 ? g[vv.y] : 0.0f;
            const float    g2 = m2 ? g[vv.z] : 0.0f, g3 = m3 ? g[vv.w] : 0.0f;
            if (m0) df_fma(s, c, aa.x, g0);
            if (m1) df_fma(s, c, aa.y, g1);
            if (m2) df_fma(s, c, aa.z, g2);
            if (m3) df_fma(s, c, aa.w, g3);
        }
        return (double) s + (double) c;
    } else {
        double d = 0.0;
#pragma unroll 2
        for (uint64_t q = (b >> 2) + threadIdx.x; q < q1; q += blockDim.x) {
            const uint4    vv = v4[q];
            const float4   aa = a4[q];
            const uint64_t k  = q << 2;
            if (k >= b && k < e) d += (double) aa.x * g[vv.x];
            if (k + 1 >= b && k + 1 < e) d += (double) aa.y * g[vv.y];
            if (k + 2 >= b && k + 2 < e) d += (double) aa.z * g[vv.z];
            if (k + 3 >= b && k + 3 < e) d += (double) aa.w * g[vv.w];
        }
        return d;
    }
}

/// Pass 1 of D^T.g.  The blocks take segments from a shared cursor in the order of their first
/// voxel (`order`), so the segments in flight at any moment -- of every spot -- cover a narrow
/// band of depth, and their gathers of g come from a few megabytes that stay in L2 instead of each
/// spot's row sweeping the whole dose-gradient vector (a 4-byte gather then costs a 32-byte DRAM
/// sector).  Each segment's partial is written at its spot-major index; which block computes it
/// does not change it, so the result is reproducible.  The cursor is returned to zero by
/// k_dij_backward_rows, which runs after this kernel on the same stream.
template<typename T>
__global__ void __launch_bounds__(256, 8)
k_dij_backward_segments(const uint32_t* __restrict__ order, uint32_t n_seg, const uint64_t* __restrict__ seg_start,
                        const uint32_t* __restrict__ vox, const float* __restrict__ val, const T* __restrict__ g,
                        double* __restrict__ partial, uint32_t* __restrict__ cursor) {
    __shared__ double   part[32];
    __shared__ uint32_t s_next;
    if (threadIdx.x == 0) s_next = atomicAdd(cursor, 1u);
    __syncthreads();
    uint32_t i = s_next;
    while (i < n_seg) {
        __syncthreads();   // everyone has read s_next
        // the next segment is claimed before this one is summed, so the claim's latency overlaps it
        if (threadIdx.x == 0) s_next = atomicAdd(cursor, 1u);
        const uint32_t sg = order[i];
        double         d  = segment_sum<T>(seg_start[sg], seg_start[sg + 1], vox, val, g);
        for (int o = 16; o > 0; o >>= 1) d += __shfl_down_sync(0xFFFFFFFFu, d, o);
        if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = d;
        __syncthreads();
        if (threadIdx.x < 32) {
            d = threadIdx.x < (blockDim.x >> 5) ? part[threadIdx.x] : 0.0;
            for (int o = 16; o > 0; o >>= 1) d += __shfl_down_sync(0xFFFFFFFFu, d, o);
            if (threadIdx.x == 0) partial[sg] = d;
        }
        __syncthreads();   // part[] is free again; s_next holds the next claim
        i = s_next;
    }
}

template<typename T>
__global__ void
k_dij_backward_rows(const uint32_t* __restrict__ row_seg, uint32_t n_rows, const double* __restrict__ partial,
                    T* __restrict__ grad, uint32_t* __restrict__ cursor) {
    const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r == 0 && cursor) *cursor = 0u;
    if (r >= n_rows) return;
    double d = 0.0;
    for (uint32_t k = row_seg[r]; k < row_seg[r + 1]; ++k) d += partial[k];
    grad[r] = (T) d;
}

__global__ void
k_dij_clear(DijSlot* __restrict__ tab, uint64_t cap) {
    const uint64_t stride = (uint64_t) gridDim.x * blockDim.x;
    for (uint64_t i = blockIdx.x * (uint64_t) blockDim.x + threadIdx.x; i < cap; i += stride) {
        tab[i].key   = 0ull;
        tab[i].value = 0.0;
    }
}

unsigned
blocks_for(uint64_t n, int per_block) {
    return (unsigned) ((n + per_block - 1) / per_block);
}

}   // namespace

cudaError_t
dij_clear(DijSlot* tab, uint64_t cap, int sms, cudaStream_t s) {
    k_dij_clear<<<sms * 8, 256, 0, s>>>(tab, cap);
    return cudaGetLastError();
}

cudaError_t
dij_count(const DijSlot* tab, uint64_t cap, unsigned long long* out, int sms, cudaStream_t s) {
    cudaError_t e = cudaMemsetAsync(out, 0, sizeof(unsigned long long), s);
    if (e != cudaSuccess || cap == 0) return e;
    k_dij_count<<<(unsigned) std::min<uint64_t>((cap + 255) / 256, (uint64_t) sms * 8), 256, 0, s>>>(tab, cap, out);
    return cudaGetLastError();
}

cudaError_t
dij_compact(const DijSlot* tab, uint64_t cap, uint64_t n_voxels, unsigned long long* keys, uint32_t* idx,
            uint64_t n_max, unsigned long long* cursor, int sms, cudaStream_t s) {
    cudaError_t e = cudaMemsetAsync(cursor, 0, sizeof(unsigned long long), s);
    if (e != cudaSuccess) return e;
    k_dij_compact<<<sms * 8, 256, 0, s>>>(tab, cap, n_voxels, keys, idx, n_max, cursor);
    return cudaGetLastError();
}

uint64_t
scan_scratch_words(uint64_t n) {
    return (n + kScanTile - 1) / kScanTile + 1;
}

cudaError_t
scan_exclusive_u32(const uint32_t* in, uint32_t* out, uint64_t n, uint32_t* scratch, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    const uint64_t tiles = (n + kScanTile - 1) / kScanTile;
    k_scan_tiles<<<(unsigned) tiles, 256, 0, s>>>(in, out, n, scratch);
    k_scan_sums<<<1, 1024, 0, s>>>(scratch, tiles);
    k_scan_add<<<blocks_for(n, 256), 256, 0, s>>>(out, n, scratch);
    return cudaGetLastError();
}

uint64_t
radix_hist_words(uint64_t n) {
    return 256ull * ((n + kTile - 1) / kTile);
}

cudaError_t
radix_sort_pairs(unsigned long long*& keys, uint32_t*& vals, unsigned long long*& keys_alt, uint32_t*& vals_alt,
                 uint64_t n, int bits, uint32_t* hist, uint32_t* offs, uint32_t* scan_scratch, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    const uint32_t n_tiles = (uint32_t) ((n + kTile - 1) / kTile);
    const uint64_t words   = 256ull * n_tiles;
    for (int shift = 0; shift < bits; shift += 8) {
        k_radix_hist<<<n_tiles, kThreads, 0, s>>>(keys, n, shift, hist, n_tiles);
        cudaError_t e = scan_exclusive_u32(hist, offs, words, scan_scratch, s);
        if (e != cudaSuccess) return e;
        k_radix_scatter<<<n_tiles, kThreads, 0, s>>>(keys, vals, keys_alt, vals_alt, n, shift, offs, n_tiles);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
        unsigned long long* tk = keys;
        keys                   = keys_alt;
        keys_alt               = tk;
        uint32_t* tv           = vals;
        vals                   = vals_alt;
        vals_alt               = tv;
    }
    return cudaGetLastError();
}

cudaError_t
dij_row_bounds(const unsigned long long* keys, uint64_t n, uint64_t row_span, uint64_t n_rows, uint64_t* indptr,
               cudaStream_t s) {
    k_row_bounds<<<blocks_for(n_rows + 1, 256), 256, 0, s>>>(keys, n, row_span, n_rows, indptr);
    return cudaGetLastError();
}

cudaError_t
dij_spot_rows(const unsigned long long* keys, const uint32_t* slot, uint64_t n, uint64_t n_voxels, const DijSlot* tab,
              double scale, uint32_t* vox, float* val, unsigned long long* vkeys, uint32_t* vpos, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    k_spot_rows<<<blocks_for(n, 256), 256, 0, s>>>(keys, slot, n, n_voxels, tab, scale, vox, val, vkeys, vpos);
    return cudaGetLastError();
}

cudaError_t
dij_row_flags(const unsigned long long* vkeys, uint64_t n, uint32_t* flags, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    k_row_flags<<<blocks_for(n, 256), 256, 0, s>>>(vkeys, n, flags);
    return cudaGetLastError();
}

cudaError_t
dij_voxel_rows(const unsigned long long* vkeys, const uint32_t* vpos, uint64_t n, const unsigned long long* skeys,
               uint64_t n_voxels, const float* sval, const uint32_t* flags, const uint32_t* rowid, uint32_t* row_voxel,
               uint64_t* indptr, uint32_t* spot, float* val, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    k_voxel_rows<<<blocks_for(n, 256), 256, 0, s>>>(vkeys, vpos, n, skeys, n_voxels, sval, flags, rowid, row_voxel,
                                                   indptr, spot, val);
    return cudaGetLastError();
}

cudaError_t
dij_forward_blocks(const uint64_t* indptr, uint64_t n_rows, uint64_t nnz, uint32_t* row_first, uint64_t* run_k,
                   uint64_t* n_blocks, cudaStream_t s) {
    const uint64_t nb = (nnz + kFwdEntries - 1) / kFwdEntries;
    *n_blocks         = nb;
    k_fwd_blocks<<<blocks_for(nb + 1, 256), 256, 0, s>>>(indptr, n_rows, nb, row_first, run_k);
    return cudaGetLastError();
}

cudaError_t
dij_seg_order_keys(const uint64_t* seg_start, uint32_t n_seg, const unsigned long long* keys, uint64_t n_voxels,
                   unsigned long long* okeys, uint32_t* oval, cudaStream_t s) {
    if (n_seg == 0) return cudaSuccess;
    k_seg_keys<<<blocks_for(n_seg, 256), 256, 0, s>>>(seg_start, n_seg, keys, n_voxels, okeys, oval);
    return cudaGetLastError();
}

cudaError_t
dij_forward(const uint32_t* row_voxel, const uint64_t* indptr, const uint32_t* row_first, const uint64_t* run_k,
            uint64_t n_blocks, const uint32_t* spot, const float* val, const void* w, void* dose, int fp64, uint32_t* err,
            int sms, cudaStream_t s) {
    if (n_blocks == 0) return cudaSuccess;
    static_assert(kFwdStage * sizeof(double) <= 227 * 1024, "staging buffer exceeds shared memory");
    if (fp64) {
        const size_t sm = kFwdStage * sizeof(double);
        cudaError_t  e  = cudaFuncSetAttribute(k_dij_forward<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) sm);
        if (e != cudaSuccess) return e;
        k_dij_forward<double><<<(unsigned) n_blocks, 256, sm, s>>>(row_voxel, indptr, row_first, spot, val,
                                                                  (const double*) w, (double*) dose);
    } else {
        constexpr size_t sm = kFwdPipeHeader + kFwdStages * (size_t) kFwdPipeStageBytes;
        static_assert(kFwdPipeBlocksPerSm * (sm + 1024) <= 228 * 1024, "the persistent forward blocks must fit one SM");
        cudaError_t e = cudaFuncSetAttribute(k_dij_forward_pipe, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) sm);
        if (e != cudaSuccess) return e;
        const uint64_t cap  = (uint64_t) sms * kFwdPipeBlocksPerSm;
        const unsigned grid = (unsigned) (n_blocks < cap ? n_blocks : cap);
        k_dij_forward_pipe<<<grid, kFwdPipeThreads, sm, s>>>(row_voxel, indptr, row_first, run_k, n_blocks, spot, val,
                                                            (const float*) w, (float*) dose, err);
    }
    return cudaGetLastError();
}

cudaError_t
dij_backward(const uint32_t* order, const uint64_t* seg_start, uint32_t n_seg, const uint32_t* row_seg, uint32_t n_rows,
             const uint32_t* vox, const float* val, double* partial, uint32_t* cursor, const void* g, void* grad,
             int fp64, int sms, cudaStream_t s) {
    if (n_rows == 0) return cudaSuccess;
    if (n_seg) {
        const uint64_t cap  = (uint64_t) sms * 8;   // 8 blocks of 256 threads per SM
        const unsigned grid = (unsigned) std::min<uint64_t>(n_seg, cap);
        if (fp64)
            k_dij_backward_segments<double><<<grid, 256, 0, s>>>(order, n_seg, seg_start, vox, val, (const double*) g,
                                                                 partial, cursor);
        else
            k_dij_backward_segments<float><<<grid, 256, 0, s>>>(order, n_seg, seg_start, vox, val, (const float*) g,
                                                                partial, cursor);
    }
    const unsigned rb = (n_rows + 255) / 256;
    if (fp64) k_dij_backward_rows<double><<<rb, 256, 0, s>>>(row_seg, n_rows, partial, (double*) grad, cursor);
    else k_dij_backward_rows<float><<<rb, 256, 0, s>>>(row_seg, n_rows, partial, (float*) grad, cursor);
    return cudaGetLastError();
}

}   // namespace mqi_gpu
