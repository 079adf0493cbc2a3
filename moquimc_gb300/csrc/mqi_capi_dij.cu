// C ABI of the Dij scorer: the (voxel, spot) table, its CSR build, and the two sparse products.
#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "mqi_ctx.h"

using namespace mqi_gpu;

namespace
{

int
bit_length(uint64_t v) {
    int b = 0;
    while (v) {
        ++b;
        v >>= 1;
    }
    return b;
}

void
free_csr(DijCsr& m) {
    cudaFree(m.s_indptr); cudaFree(m.s_voxel); cudaFree(m.s_value);
    cudaFree(m.v_row); cudaFree(m.v_indptr); cudaFree(m.v_spot); cudaFree(m.v_value);
    cudaFree(m.seg_start); cudaFree(m.row_seg); cudaFree(m.seg_order); cudaFree(m.bwd_cursor);
    cudaFree(m.partial); cudaFree(m.fwd_row_first); cudaFree(m.fwd_run_k);
    m = DijCsr{};
}

/// Device buffers freed on scope exit unless released.
struct Scratch {
    std::vector<void*> ptrs;
    template<typename T>
    cudaError_t
    alloc(T*& p, uint64_t n) {
        p = nullptr;
        cudaError_t e = cudaMalloc(reinterpret_cast<void**>(&p), std::max<uint64_t>(n, 1) * sizeof(T));
        if (e == cudaSuccess) ptrs.push_back(p);
        return e;
    }
    void
    release(void* p) {
        ptrs.erase(std::remove(ptrs.begin(), ptrs.end(), p), ptrs.end());
    }
    ~Scratch() {
        for (void* p : ptrs) cudaFree(p);
    }
};

ScorerHost*
dij_scorer(mqi_ctx* c, int id, const char* who) {
    if (!valid_ctx(c)) {
        fail(c, MQI_ERR_INVALID, std::string(who) + ": ctx is NULL");
        return nullptr;
    }
    if (id < 0 || id >= (int) c->scorers.size() || c->scorers[id].type != MQI_SCORER_DIJ) {
        fail(c, MQI_ERR_INVALID, std::string(who) + ": not a Dij scorer");
        return nullptr;
    }
    return &c->scorers[id];
}

}   // namespace

namespace mqi_gpu
{

/// Called by mqi_destroy / mqi_reset_tallies.
void
dij_release(ScorerHost& s) {
    cudaFree(s.hit_log);
    cudaFree(s.hit_count);
    s.hit_log   = nullptr;
    s.hit_count = nullptr;
    s.hit_cap   = 0;
    free_csr(s.csr);
    cudaFree(s.dij);
    cudaFree(s.dij_count);
    s.dij = nullptr;
    s.dij_count = nullptr;
}

cudaError_t
dij_reset(ScorerHost& s, int sms, cudaStream_t st) {
    free_csr(s.csr);
    cudaError_t e = dij_clear(s.dij, s.dij_cap, sms, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(s.dij_count, 0, sizeof(unsigned long long), st);
    return e;
}

}   // namespace mqi_gpu

extern "C" {

int
mqi_add_dij_scorer(mqi_ctx* c, int child_id, int roi_method, uint32_t roi_length, const uint32_t* roi_start,
                   const uint32_t* roi_stride, const uint32_t* roi_acc, uint64_t capacity, int* scorer_id) {
    if (!valid_ctx(c)) return fail(c, MQI_ERR_INVALID, "mqi_add_dij_scorer: ctx is NULL");
    if (c->n_scen > 1) return fail(c, MQI_ERR_UNSUPPORTED, "mqi_add_dij_scorer: not with robust scenarios");
    if (capacity == 0) capacity = 1ull << 26;
    if (capacity > (1ull << 32)) return fail(c, MQI_ERR_INVALID, "mqi_add_dij_scorer: at most 2^32 slots");
    uint64_t cap = 1;
    while (cap < capacity) cap <<= 1;
    // the dense-scorer path validates the child and the ROI and allocates the ROI arrays
    int id = -1;
    int rc = mqi_add_scorer(c, child_id, MQI_SCORER_EDEP, roi_method, roi_length, roi_start, roi_stride, roi_acc, &id);
    if (rc != MQI_OK) return rc;
    ScorerHost& s = c->scorers[id];
    DeviceGuard g(c->device);
    cudaFree(s.tally);   // a Dij scorer has no dense tally
    s.tally     = nullptr;
    s.tally_len = 0;
    s.type      = MQI_SCORER_DIJ;
    s.dij_cap   = cap;
    cudaError_t e = cudaMalloc(&s.dij, cap * sizeof(DijSlot));
    if (e == cudaSuccess) e = cudaMalloc(&s.dij_count, sizeof(unsigned long long));
    if (e == cudaSuccess) e = dij_reset(s, c->num_sms, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) {
        dij_release(s);
        cudaFree(s.start); cudaFree(s.stride); cudaFree(s.acc);
        c->scorers.pop_back();
        return cuda_fail(c, e, "mqi_add_dij_scorer");
    }
    if (scorer_id) *scorer_id = id;
    return MQI_OK;
}

int
mqi_dij_record_hits(mqi_ctx* c, int id, uint64_t capacity) {
    ScorerHost* sp = dij_scorer(c, id, "mqi_dij_record_hits");
    if (!sp) return MQI_ERR_INVALID;
    ScorerHost& s = *sp;
    DeviceGuard g(c->device);
    MQI_CUDA(c, cudaStreamSynchronize(c->stream), "mqi_dij_record_hits");
    cudaFree(s.hit_log);
    cudaFree(s.hit_count);
    s.hit_log   = nullptr;
    s.hit_count = nullptr;
    s.hit_cap   = 0;
    if (capacity == 0) return MQI_OK;
    cudaError_t e = cudaMalloc(&s.hit_log, capacity * sizeof(DijHit));
    if (e == cudaSuccess) e = cudaMalloc(&s.hit_count, sizeof(unsigned long long));
    if (e == cudaSuccess) e = cudaMemsetAsync(s.hit_count, 0, sizeof(unsigned long long), c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) {
        cudaFree(s.hit_log);
        cudaFree(s.hit_count);
        s.hit_log   = nullptr;
        s.hit_count = nullptr;
        return cuda_fail(c, e, "mqi_dij_record_hits");
    }
    s.hit_cap = capacity;
    return MQI_OK;
}

int
mqi_dij_get_hits(mqi_ctx* c, int id, uint32_t* voxel, uint32_t* spot, double* value, uint64_t* n_out) {
    ScorerHost* sp = dij_scorer(c, id, "mqi_dij_get_hits");
    if (!sp) return MQI_ERR_INVALID;
    ScorerHost& s = *sp;
    if (!n_out) return fail(c, MQI_ERR_INVALID, "mqi_dij_get_hits: n_out is NULL");
    if (!s.hit_log) return fail(c, MQI_ERR_STATE, "mqi_dij_get_hits: recording is off (mqi_dij_record_hits)");
    DeviceGuard g(c->device);
    unsigned long long count = 0;
    MQI_CUDA(c, cudaMemcpyAsync(&count, s.hit_count, sizeof(count), cudaMemcpyDeviceToHost, c->stream),
             "mqi_dij_get_hits");
    MQI_CUDA(c, cudaStreamSynchronize(c->stream), "mqi_dij_get_hits");
    const uint64_t n = std::min<uint64_t>(count, s.hit_cap);
    *n_out = n;
    if (count > s.hit_cap)
        return fail(c, MQI_ERR_OVERFLOW, "mqi_dij_get_hits: more insertions than the log holds (" +
                                             std::to_string(count) + " > " + std::to_string(s.hit_cap) + ")");
    if (!voxel && !spot && !value) return MQI_OK;
    std::vector<DijHit> h(n);
    if (n) {
        MQI_CUDA(c, cudaMemcpyAsync(h.data(), s.hit_log, n * sizeof(DijHit), cudaMemcpyDeviceToHost, c->stream),
                 "mqi_dij_get_hits");
        MQI_CUDA(c, cudaStreamSynchronize(c->stream), "mqi_dij_get_hits");
    }
    for (uint64_t i = 0; i < n; ++i) {
        if (voxel) voxel[i] = h[i].voxel;
        if (spot) spot[i] = h[i].spot;
        if (value) value[i] = h[i].value;
    }
    return MQI_OK;
}

int
mqi_dij_build(mqi_ctx* c, int id, uint32_t n_spots, double scale, uint64_t* nnz_out) {
    ScorerHost* sp = dij_scorer(c, id, "mqi_dij_build");
    if (!sp) return MQI_ERR_INVALID;
    ScorerHost& s = *sp;
    if (n_spots == 0) n_spots = c->n_plan_spots;
    if (n_spots == 0) return fail(c, MQI_ERR_INVALID, "mqi_dij_build: n_spots is 0 and no spot plan is set");
    const ChildHost& ch = c->children[s.child];
    const uint64_t nvox = (uint64_t) ch.nx * ch.ny * ch.nz;
    DeviceGuard g(c->device);
    cudaStream_t st = c->stream;
    free_csr(s.csr);
    unsigned long long count = 0;
    MQI_CUDA(c, dij_count(s.dij, s.dij_cap, s.dij_count, c->num_sms, st), "mqi_dij_build: count");
    MQI_CUDA(c, cudaMemcpyAsync(&count, s.dij_count, sizeof(count), cudaMemcpyDeviceToHost, st), "mqi_dij_build");
    MQI_CUDA(c, cudaStreamSynchronize(st), "mqi_dij_build");
    const uint64_t n = count;

    Scratch sc;
    unsigned long long *ka, *kb, *kc, *cursor;
    uint32_t *ia, *ib, *ic, *hist, *offs, *scan, *flags, *rowid;
    const uint64_t hw = radix_hist_words(n);
    MQI_CUDA(c, sc.alloc(ka, n), "mqi_dij_build: allocation");
    MQI_CUDA(c, sc.alloc(kb, n), "mqi_dij_build: allocation");
    MQI_CUDA(c, sc.alloc(kc, n), "mqi_dij_build: allocation");
    MQI_CUDA(c, sc.alloc(ia, n), "mqi_dij_build: allocation");
    MQI_CUDA(c, sc.alloc(ib, n), "mqi_dij_build: allocation");
    MQI_CUDA(c, sc.alloc(ic, n), "mqi_dij_build: allocation");
    MQI_CUDA(c, sc.alloc(hist, hw), "mqi_dij_build: allocation");
    MQI_CUDA(c, sc.alloc(offs, hw), "mqi_dij_build: allocation");
    MQI_CUDA(c, sc.alloc(scan, std::max(scan_scratch_words(hw), scan_scratch_words(n))), "mqi_dij_build: allocation");
    MQI_CUDA(c, sc.alloc(flags, n), "mqi_dij_build: allocation");
    MQI_CUDA(c, sc.alloc(rowid, n), "mqi_dij_build: allocation");
    MQI_CUDA(c, sc.alloc(cursor, 1), "mqi_dij_build: allocation");

    DijCsr m;
    m.n_spots  = n_spots;
    m.n_voxels = nvox;
    m.nnz      = n;
    MQI_CUDA(c, sc.alloc(m.s_indptr, (uint64_t) n_spots + 1), "mqi_dij_build: allocation");
    // entry arrays padded to whole groups of four: the products read them with 16-byte loads
    MQI_CUDA(c, sc.alloc(m.s_voxel, n + 4), "mqi_dij_build: allocation");
    MQI_CUDA(c, sc.alloc(m.s_value, n + 4), "mqi_dij_build: allocation");
    MQI_CUDA(c, sc.alloc(m.v_spot, n + 4), "mqi_dij_build: allocation");
    MQI_CUDA(c, sc.alloc(m.v_value, n + 4), "mqi_dij_build: allocation");

    // 1. compact the table to (spot * n_voxels + voxel, slot) pairs
    MQI_CUDA(c, dij_compact(s.dij, s.dij_cap, nvox, ka, ia, n, cursor, c->num_sms, st), "mqi_dij_build: compact");
    unsigned long long got = 0;
    MQI_CUDA(c, cudaMemcpyAsync(&got, cursor, sizeof(got), cudaMemcpyDeviceToHost, st), "mqi_dij_build");
    MQI_CUDA(c, cudaStreamSynchronize(st), "mqi_dij_build");
    if (got != n) return fail(c, MQI_ERR_DEVICE, "mqi_dij_build: occupied slots disagree with the insertion count");

    // 2. sort by (spot, voxel): spot rows, voxels ascending
    unsigned long long* skeys = ka;
    uint32_t*           sslot = ia;
    MQI_CUDA(c, radix_sort_pairs(skeys, sslot, kb, ib, n, bit_length((uint64_t) n_spots * nvox - 1), hist, offs, scan, st),
             "mqi_dij_build: sort");
    MQI_CUDA(c, dij_row_bounds(skeys, n, nvox, n_spots, m.s_indptr, st), "mqi_dij_build");
    std::vector<uint64_t> indptr(n_spots + 1);
    MQI_CUDA(c, cudaMemcpyAsync(indptr.data(), m.s_indptr, indptr.size() * sizeof(uint64_t), cudaMemcpyDeviceToHost, st),
             "mqi_dij_build");
    MQI_CUDA(c, cudaStreamSynchronize(st), "mqi_dij_build");
    if (indptr[n_spots] != n) return fail(c, MQI_ERR_INVALID, "mqi_dij_build: the table holds a spot index >= n_spots");
    // backward segments: each row cut into runs of at most kDijSegment entries, and their work
    // order: by the voxel of their first entry (the free sort buffers are reused below)
    {
        std::vector<uint64_t> seg;
        std::vector<uint32_t> row_seg(n_spots + 1);
        for (uint32_t r = 0; r < n_spots; ++r) {
            row_seg[r] = (uint32_t) seg.size();
            for (uint64_t b = indptr[r]; b < indptr[r + 1]; b += kDijSegment) seg.push_back(b);
        }
        row_seg[n_spots] = (uint32_t) seg.size();
        m.n_seg = seg.size();
        seg.push_back(n);
        MQI_CUDA(c, sc.alloc(m.seg_start, seg.size()), "mqi_dij_build: allocation");
        MQI_CUDA(c, sc.alloc(m.row_seg, row_seg.size()), "mqi_dij_build: allocation");
        MQI_CUDA(c, sc.alloc(m.seg_order, m.n_seg), "mqi_dij_build: allocation");
        MQI_CUDA(c, sc.alloc(m.partial, m.n_seg), "mqi_dij_build: allocation");
        MQI_CUDA(c, sc.alloc(m.bwd_cursor, 1), "mqi_dij_build: allocation");
        MQI_CUDA(c, cudaMemsetAsync(m.bwd_cursor, 0, sizeof(uint32_t), st), "mqi_dij_build");
        MQI_CUDA(c, cudaMemcpyAsync(m.seg_start, seg.data(), seg.size() * sizeof(uint64_t), cudaMemcpyHostToDevice, st),
                 "mqi_dij_build");
        MQI_CUDA(c, cudaMemcpyAsync(m.row_seg, row_seg.data(), row_seg.size() * sizeof(uint32_t), cudaMemcpyHostToDevice,
                                    st), "mqi_dij_build");
        if (m.n_seg) {
            unsigned long long* okeys = (skeys == ka) ? kb : ka;
            unsigned long long* okalt = kc;
            uint32_t*           oval  = (sslot == ia) ? ib : ia;
            uint32_t*           ovalt = ic;
            MQI_CUDA(c, dij_seg_order_keys(m.seg_start, (uint32_t) m.n_seg, skeys, nvox, okeys, oval, st), "mqi_dij_build");
            MQI_CUDA(c, radix_sort_pairs(okeys, oval, okalt, ovalt, m.n_seg, bit_length(nvox - 1), hist, offs, scan, st),
                     "mqi_dij_build: sort");
            MQI_CUDA(c, cudaMemcpyAsync(m.seg_order, oval, m.n_seg * sizeof(uint32_t), cudaMemcpyDeviceToDevice, st),
                     "mqi_dij_build");
        }
        MQI_CUDA(c, cudaStreamSynchronize(st), "mqi_dij_build");   // the host vectors are copied from
    }

    // 3. spot-row entries, and (voxel, position) pairs for the voxel-row layout
    unsigned long long* vkeys = (skeys == ka) ? kb : ka;
    uint32_t*           vpos  = (sslot == ia) ? ib : ia;
    MQI_CUDA(c, dij_spot_rows(skeys, sslot, n, nvox, s.dij, scale, m.s_voxel, m.s_value, vkeys, vpos, st),
             "mqi_dij_build");
    unsigned long long* kalt = kc;
    uint32_t*           ialt = ic;
    MQI_CUDA(c, radix_sort_pairs(vkeys, vpos, kalt, ialt, n, bit_length(nvox - 1), hist, offs, scan, st),
             "mqi_dij_build: sort");

    // 4. voxel rows: row starts by flag + scan
    MQI_CUDA(c, dij_row_flags(vkeys, n, flags, st), "mqi_dij_build");
    MQI_CUDA(c, scan_exclusive_u32(flags, rowid, n, scan, st), "mqi_dij_build");
    uint32_t tail[2] = { 0, 0 };
    if (n) {
        MQI_CUDA(c, cudaMemcpyAsync(&tail[0], rowid + n - 1, sizeof(uint32_t), cudaMemcpyDeviceToHost, st), "mqi_dij_build");
        MQI_CUDA(c, cudaMemcpyAsync(&tail[1], flags + n - 1, sizeof(uint32_t), cudaMemcpyDeviceToHost, st), "mqi_dij_build");
        MQI_CUDA(c, cudaStreamSynchronize(st), "mqi_dij_build");
    }
    m.n_vrows = n ? (uint64_t) tail[0] + tail[1] : 0;
    MQI_CUDA(c, sc.alloc(m.v_row, m.n_vrows), "mqi_dij_build: allocation");
    MQI_CUDA(c, sc.alloc(m.v_indptr, m.n_vrows + 1), "mqi_dij_build: allocation");
    if (n == 0) MQI_CUDA(c, cudaMemsetAsync(m.v_indptr, 0, sizeof(uint64_t), st), "mqi_dij_build");
    MQI_CUDA(c, dij_voxel_rows(vkeys, vpos, n, skeys, nvox, m.s_value, flags, rowid, m.v_row, m.v_indptr, m.v_spot,
                               m.v_value, st), "mqi_dij_build");
    // 5. the forward blocks' first rows
    MQI_CUDA(c, sc.alloc(m.fwd_row_first, (n + kFwdEntries - 1) / kFwdEntries + 1), "mqi_dij_build: allocation");
    MQI_CUDA(c, sc.alloc(m.fwd_run_k, (n + kFwdEntries - 1) / kFwdEntries + 1), "mqi_dij_build: allocation");
    MQI_CUDA(c, dij_forward_blocks(m.v_indptr, m.n_vrows, n, m.fwd_row_first, m.fwd_run_k, &m.n_fwd_blocks, st),
             "mqi_dij_build");
    MQI_CUDA(c, cudaStreamSynchronize(st), "mqi_dij_build");
    for (void* p : { (void*) m.s_indptr, (void*) m.s_voxel, (void*) m.s_value, (void*) m.v_row, (void*) m.v_indptr,
                     (void*) m.v_spot, (void*) m.v_value, (void*) m.seg_start, (void*) m.row_seg, (void*) m.seg_order,
                     (void*) m.bwd_cursor, (void*) m.partial, (void*) m.fwd_row_first, (void*) m.fwd_run_k })
        sc.release(p);
    m.built = true;
    s.csr   = m;
    if (nnz_out) *nnz_out = n;
    return MQI_OK;
}

int
mqi_dij_get_csr(mqi_ctx* c, int id, uint64_t* indptr, uint32_t* indices, float* data, int on_device) {
    ScorerHost* sp = dij_scorer(c, id, "mqi_dij_get_csr");
    if (!sp) return MQI_ERR_INVALID;
    const DijCsr& m = sp->csr;
    if (!m.built) return fail(c, MQI_ERR_STATE, "mqi_dij_get_csr: call mqi_dij_build first");
    DeviceGuard g(c->device);
    const cudaMemcpyKind k = on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
    if (indptr) MQI_CUDA(c, cudaMemcpyAsync(indptr, m.s_indptr, (m.n_spots + 1) * sizeof(uint64_t), k, c->stream), "mqi_dij_get_csr");
    if (indices && m.nnz) MQI_CUDA(c, cudaMemcpyAsync(indices, m.s_voxel, m.nnz * sizeof(uint32_t), k, c->stream), "mqi_dij_get_csr");
    if (data && m.nnz) MQI_CUDA(c, cudaMemcpyAsync(data, m.s_value, m.nnz * sizeof(float), k, c->stream), "mqi_dij_get_csr");
    MQI_CUDA(c, cudaStreamSynchronize(c->stream), "mqi_dij_get_csr");
    return MQI_OK;
}

int
mqi_dij_info(mqi_ctx* c, int id, uint64_t* table_slots, uint64_t* occupied, uint64_t* nnz, uint64_t* n_voxel_rows) {
    ScorerHost* sp = dij_scorer(c, id, "mqi_dij_info");
    if (!sp) return MQI_ERR_INVALID;
    DeviceGuard g(c->device);
    unsigned long long occ = 0;
    MQI_CUDA(c, dij_count(sp->dij, sp->dij_cap, sp->dij_count, c->num_sms, c->stream), "mqi_dij_info");
    MQI_CUDA(c, cudaMemcpyAsync(&occ, sp->dij_count, sizeof(occ), cudaMemcpyDeviceToHost, c->stream), "mqi_dij_info");
    MQI_CUDA(c, cudaStreamSynchronize(c->stream), "mqi_dij_info");
    if (table_slots) *table_slots = sp->dij_cap;
    if (occupied) *occupied = occ;
    if (nnz) *nnz = sp->csr.built ? sp->csr.nnz : 0;
    if (n_voxel_rows) *n_voxel_rows = sp->csr.built ? sp->csr.n_vrows : 0;
    return MQI_OK;
}

int
mqi_dij_matvec(mqi_ctx* c, int id, const void* w, void* dose, int fp64, int on_device) {
    ScorerHost* sp = dij_scorer(c, id, "mqi_dij_matvec");
    if (!sp) return MQI_ERR_INVALID;
    const DijCsr& m = sp->csr;
    if (!m.built) return fail(c, MQI_ERR_STATE, "mqi_dij_matvec: call mqi_dij_build first");
    if (!w || !dose) return fail(c, MQI_ERR_INVALID, "mqi_dij_matvec: NULL buffer");
    DeviceGuard g(c->device);
    const size_t es = fp64 ? sizeof(double) : sizeof(float);
    Scratch sc;
    const void* dw = w;
    void*       dd = dose;
    if (!on_device) {
        char *tw, *td;
        MQI_CUDA(c, sc.alloc(tw, m.n_spots * es), "mqi_dij_matvec");
        MQI_CUDA(c, sc.alloc(td, m.n_voxels * es), "mqi_dij_matvec");
        MQI_CUDA(c, cudaMemcpyAsync(tw, w, m.n_spots * es, cudaMemcpyHostToDevice, c->stream), "mqi_dij_matvec");
        dw = tw;
        dd = td;
    }
    MQI_CUDA(c, cudaMemsetAsync(dd, 0, m.n_voxels * es, c->stream), "mqi_dij_matvec");
    MQI_CUDA(c, dij_forward(m.v_row, m.v_indptr, m.fwd_row_first, m.fwd_run_k, m.n_fwd_blocks, m.v_spot, m.v_value,
                            dw, dd, fp64, c->counters + 3, c->num_sms, c->stream), "mqi_dij_matvec");
    if (!on_device) {
        uint32_t flag = 0;
        MQI_CUDA(c, cudaMemcpyAsync(dose, dd, m.n_voxels * es, cudaMemcpyDeviceToHost, c->stream), "mqi_dij_matvec");
        MQI_CUDA(c, cudaMemcpyAsync(&flag, c->counters + 3, sizeof(flag), cudaMemcpyDeviceToHost, c->stream),
                 "mqi_dij_matvec");
        MQI_CUDA(c, cudaStreamSynchronize(c->stream), "mqi_dij_matvec");
        if (flag & 8u) return fail(c, MQI_ERR_DEVICE, "mqi_dij_matvec: a bulk copy did not complete");
    }
    return MQI_OK;
}

int
mqi_dij_rmatvec(mqi_ctx* c, int id, const void* gin, void* grad, int fp64, int on_device) {
    ScorerHost* sp = dij_scorer(c, id, "mqi_dij_rmatvec");
    if (!sp) return MQI_ERR_INVALID;
    const DijCsr& m = sp->csr;
    if (!m.built) return fail(c, MQI_ERR_STATE, "mqi_dij_rmatvec: call mqi_dij_build first");
    if (!gin || !grad) return fail(c, MQI_ERR_INVALID, "mqi_dij_rmatvec: NULL buffer");
    DeviceGuard g(c->device);
    const size_t es = fp64 ? sizeof(double) : sizeof(float);
    Scratch sc;
    const void* dg = gin;
    void*       dr = grad;
    if (!on_device) {
        char *tg, *tr;
        MQI_CUDA(c, sc.alloc(tg, m.n_voxels * es), "mqi_dij_rmatvec");
        MQI_CUDA(c, sc.alloc(tr, m.n_spots * es), "mqi_dij_rmatvec");
        MQI_CUDA(c, cudaMemcpyAsync(tg, gin, m.n_voxels * es, cudaMemcpyHostToDevice, c->stream), "mqi_dij_rmatvec");
        dg = tg;
        dr = tr;
    }
    MQI_CUDA(c, dij_backward(m.seg_order, m.seg_start, (uint32_t) m.n_seg, m.row_seg, m.n_spots, m.s_voxel, m.s_value,
                             m.partial, m.bwd_cursor, dg, dr, fp64, c->num_sms, c->stream), "mqi_dij_rmatvec");
    if (!on_device) {
        MQI_CUDA(c, cudaMemcpyAsync(grad, dr, m.n_spots * es, cudaMemcpyDeviceToHost, c->stream), "mqi_dij_rmatvec");
        MQI_CUDA(c, cudaStreamSynchronize(c->stream), "mqi_dij_rmatvec");
    }
    return MQI_OK;
}

}   // extern "C"
