// Transport kernels of the GB300 proton engine.
//
// The reference runs one thread per history with a per-thread LIFO stack of secondaries
// (moqui/kernel_functions/mqi_transport.hpp:113-250, moqui/base/mqi_track_stack.hpp:11-67).
// Here every track lives in a structure-of-arrays queue.  A wave kernel drains the queue: each
// lane fetches a track (warp-aggregated cursor), steps it voxel by voxel in registers, scores
// each step with warp-aggregated FP64 atomics, and appends its daughters -- and itself, when its
// step budget for the wave runs out -- to the next queue.  The host (or a captured graph) swaps
// queues until none is left.  Because each track's random stream is keyed by (seed, history,
// track uid) and the 200/10-deep stack limit is emulated from each track's recorded stack depth,
// the result does not depend on the order the queue is drained in.
#include <cstdint>
#include <cuda_runtime.h>

#include "mqi_device.cuh"
#include "mqi_internal.h"

namespace mqi_gpu
{

// meta word layout
constexpr uint32_t kMetaBelowMask = 0xFFFFu;
constexpr uint32_t kMetaPrimary   = 1u << 16;
constexpr uint32_t kMetaKe1Zero   = 1u << 17;
constexpr uint32_t kMetaPhaseStep = 1u << 18;
constexpr int      kMetaChildShift = 19;   // 3 bits
constexpr int      kMetaNpushShift = 22;   // 10 bits

enum StatIdx { ST_HIST = 0, ST_TRACKS, ST_STEPS, ST_SEC, ST_LOCAL, ST_DROP, ST_WAVES, ST_ERR };

constexpr uint32_t kMaxTrackSteps = 1u << 20;

/// A track in registers: track_t<float> (mqi_track.hpp:48-205) reduced to what transport reads.
struct Trk {
    float    ke0, ke1;
    float3   p0, d0, p1, d1;
    float    dE, ldE;
    int3     cell;
    uint64_t uid;
    uint32_t hist;
    uint32_t spot;   // spot of the history (Dij column); inherited by daughters
    uint32_t below, npush;
    int      child;
    float    spr0;   // SPR at (voxel density, ke0) when the step computed it, else < 0
    bool     primary, stopped;
};

/// Per-lane context of a wave.
struct Ctx {
    const WaveParams* P;
    const Tables*     T;
    Grid              g;          // current child grid
    int               child;
    uint32_t          spot;
    bool              dbg;
    float             tcut;
};

/// A block's event counters (indices of mqi_stats: histories, tracks, steps, secondaries queued,
/// secondaries scored in place, secondaries dropped, -, errors), kept in shared memory so that the
/// step loop does not carry them in registers; flushed once per block.
enum { kCntHist = 0, kCntTracks = 1, kCntSteps = 2, kCntSec = 3, kCntLocal = 4, kCntDrop = 5, kCntErr = 7 };
static __shared__ unsigned int s_cnt[8];

__device__ __forceinline__ void
count_event(int k) {
    atomicAdd(&s_cnt[k], 1u);
}

// ------------------------------------------------------------------------------------------
// Calibration plug-in (material_t::compute_rsp_ / compute_rl_, materials/mqi_material.hpp:10-25):
// the default curves, or tables on uniform grids (mqi_set_calibration).
// ------------------------------------------------------------------------------------------

/// Lower node and upper weight of x on a uniform grid of n >= 2 nodes, clamped to the grid.
__device__ inline float
calib_index(float x, float x0, float dx, uint32_t n, int& i) {
    const float f = (x - x0) / dx;
    if (!(f > 0.0f)) {
        i = 0;
        return 0.0f;
    }
    if (f >= (float) (n - 1)) {
        i = (int) n - 2;
        return 1.0f;
    }
    i = (int) f;
    return f - (float) i;
}

/// SPR(rho, E) from the table, bilinear (E first).
__device__ __noinline__ float
spr_table(const CalibDev& c, float rho, float Ek) {
    int         ir, ie;
    const float wr = calib_index(rho, c.rho0, c.drho, c.n_rho, ir);
    const float we = calib_index(Ek, c.e0, c.de, c.n_e, ie);
    const float* r0 = c.spr + (size_t) ir * c.n_e;
    const float* r1 = r0 + c.n_e;
    const float  a  = r0[ie] + we * (r0[ie + 1] - r0[ie]);
    const float  b  = r1[ie] + we * (r1[ie + 1] - r1[ie]);
    return a + wr * (b - a);
}

/// X0(rho) from the table, linear.
__device__ __noinline__ float
x0_table(const CalibDev& c, float rho) {
    int         ir;
    const float wr = calib_index(rho, c.rho0, c.drho, c.n_rho, ir);
    return c.x0[ir] + wr * (c.x0[ir + 1] - c.x0[ir]);
}

/// The run's stopping-power ratio (compute_rsp_): the tables are out of line, so the default
/// curve's step loop carries one uniform branch and a call.
__device__ __forceinline__ float
spr_of(const CalibDev& c, float rho, float Ek, bool dbg) {
    return c.mode ? spr_table(c, rho, Ek) : spr_default(rho, Ek, dbg);
}

/// The run's radiation length (compute_rl_).
__device__ __forceinline__ float
x0_of(const CalibDev& c, float rho, bool dbg) {
    return c.mode ? x0_table(c, rho) : radiation_length_default(rho, dbg);
}

__device__ inline Grid
make_grid(const ChildDev& c, const float* sxe, const float* sye, const float* sze) {
    Grid g;
    g.nx = c.nx; g.ny = c.ny; g.nz = c.nz;
    g.xe = sxe ? sxe : c.xe;
    g.ye = sye ? sye : c.ye;
    g.ze = sze ? sze : c.ze;
    g.rho = c.rho;
    g.rho_scale = 1.0f;
    return g;
}

/// The grid of `child` as the track with spot word `sw` sees it: a robust scenario of the
/// scenario child has its own edges (setup shift) and density scale.
__device__ inline void
apply_scenario(const WaveParams& P, Grid& g, int child, uint32_t sw) {
    if (P.n_scen > 1 && child == P.scen_child) {
        const int    s = (int) (sw >> kScenShift);
        const float* e = P.scen_edges + (size_t) s * P.scen_stride;
        g.xe        = e;
        g.ye        = e + g.nx + 1;
        g.ze        = e + g.nx + g.ny + 2;
        g.rho_scale = P.scen_scale[s];
    }
}

/// Density of voxel cnb in the track's scenario: hu_to_density(hu) * DensityScaling as one FP32
/// product (mqi_tps_env.hpp:766-769); the scale is 1 outside robust runs.
__device__ inline float
voxel_rho(const Grid& g, uint32_t cnb) {
    return __fmul_rn(g.rho[cnb], g.rho_scale);
}

// ------------------------------------------------------------------------------------------
// Scoring (mqi_transport.hpp:204-225 and :342-364; scorer callbacks in
// moqui/base/scorers/mqi_scorer_energy_deposit.hpp:12-177; insert_hashtable :68-111).
// ------------------------------------------------------------------------------------------

/// Add v to tally[key] with one FP64 atomic (a fire-and-forget reduction at L2).  Combining the
/// lanes of a warp that hit the same voxel first (__match_any_sync, shuffles, one atomic per
/// distinct voxel) was measured slower on every workload -- 5.7% on the slab phantom, 6.6% on the
/// synthetic-CT plan, 15% with the statistics pair -- because lanes of a warp run different
/// histories and rarely share a voxel, while the match costs issue slots in an issue-bound kernel.
/// The Dij insertion keeps the aggregation: there it saves hash probes.
__device__ inline void
tally_add(double* tally, uint64_t slot, double v, bool valid) {
    if (valid) atomicAdd(&tally[slot], v);
}

/// Hash of a Dij key: the splitmix64 finalizer (Steele, Lea & Flood, "Fast splittable
/// pseudorandom number generators", OOPSLA 2014).
__device__ inline uint64_t
dij_hash(uint64_t k) {
    k ^= k >> 30;
    k *= 0xBF58476D1CE4E5B9ull;
    k ^= k >> 27;
    k *= 0x94D049BB133111EBull;
    k ^= k >> 31;
    return k;
}

/// Add v to the Dij entry (spot, voxel).  Lanes of the warp with the same table and key are
/// combined first (two match rounds: the key, then the table), so one insertion is issued per
/// distinct entry.  The leader probes linearly from the hashed slot: a slot holding the key takes
/// the add; an empty slot is claimed with one 64-bit CAS.  After kDijMaxProbes probes the table
/// counts as full and the error flag's bit 4 is set.  Claims are not counted here (a counter
/// bumped on every claim, one address for every SM, cost 8% of the Dij transport): the occupied
/// slots are counted by one pass over the table when the count is needed (k_dij_count).
__device__ inline void
dij_add(const ScorerDev& s, uint32_t* error_flag, uint32_t spot, uint32_t voxel, double v, bool valid) {
    DijSlot* const           table      = s.dij;
    const uint64_t           table_mask = s.dij_mask;
    if (s.hit_log && valid) {   // recorded insertions, for checking the table against a replay
        const unsigned long long i = atomicAdd(s.hit_count, 1ull);
        if (i < s.hit_cap) s.hit_log[i] = DijHit{ voxel, spot, v };
    }
    const unsigned           mask  = __activemask();
    const unsigned long long key   = ((((unsigned long long) spot) << 32) | voxel) + 1ull;
    const unsigned           peers = __match_any_sync(mask, valid ? key : 0ull) &
                           __match_any_sync(mask, (unsigned long long) table);
    if (!valid) return;
    double   sum = v;
    if (__popc(peers) > 1) {
        sum = 0.0;
        unsigned m = peers;
        while (m) {
            const int src = __ffs(m) - 1;
            sum += __shfl_sync(peers, v, src);
            m &= m - 1;
        }
        if ((int) (threadIdx.x & 31) != __ffs(peers) - 1) return;
    }
    uint64_t slot = dij_hash(key) & table_mask;
    for (uint32_t probe = 0; probe < kDijMaxProbes; ++probe) {
        DijSlot* e = table + slot;
        unsigned long long k = *reinterpret_cast<volatile unsigned long long*>(&e->key);
        if (k == 0ull) k = atomicCAS(&e->key, 0ull, key);
        if (k == 0ull || k == key) {
            atomicAdd(&e->value, sum);
            return;
        }
        slot = (slot + 1) & table_mask;
    }
    atomicOr(error_flag, 4u);
}

/// roi_t::idx / get_mask_idx for the three mapping methods (mqi_roi.hpp:47-71, 87-160).
__device__ inline int32_t
roi_lower_bound(const ScorerDev& s, uint32_t v) {
    int32_t first = 0, count = (int32_t) s.roi_len;
    while (count > 0) {
        const int32_t step = count / 2;
        const int32_t it   = first + step;
        if (s.start[it] <= v) { first = it + 1; count -= step + 1; }
        else count = step;
    }
    return first;
}

__device__ inline int32_t
roi_idx(const ScorerDev& s, uint32_t v) {
    if (s.roi_method == MQI_ROI_INDIRECT) return (int32_t) s.start[v];
    if (s.roi_method == MQI_ROI_CONTOUR) {
        const int32_t c = roi_lower_bound(s, v) - 1;
        if (c < 0) return -1;
        return (v - s.start[c] < s.stride[c]) ? 1 : -1;
    }
    return (int32_t) v;
}

__device__ inline int32_t
roi_mask_idx(const ScorerDev& s, uint32_t v) {
    if (s.roi_method == MQI_ROI_INDIRECT) return (int32_t) s.start[v];
    if (s.roi_method == MQI_ROI_CONTOUR) {
        const int32_t c = roi_lower_bound(s, v) - 1;
        if (c < 0) return -1;
        uint32_t d = v - s.start[c];
        if (d < s.stride[c]) {
            if (c > 0) d += s.acc[c - 1];
            return (int32_t) d;
        }
        return -1;
    }
    return (int32_t) v;
}

/// fp_compute_hit of the scorers that need nothing beyond the step's deposit and its
/// dose_to_water (mqi_scorer_energy_deposit.hpp:12-77), as the FP32 quantity they are formed from:
/// the deposit, or dose_to_water (squared in FP64 by the caller for dose_to_water_square).  It is
/// never negative, so "value > 0" (insert_hashtable's filter) is decided in FP32.
__device__ inline float
compute_hit_simple(int type, const Trk& t, float dose_w) {
    switch (type) {
    case MQI_SCORER_EDEP: return t.dE + t.ldE;
    case MQI_SCORER_EDEP_PRIMARY: return t.primary ? t.dE : 0.0f;
    case MQI_SCORER_EDEP_SECONDARY: return t.primary ? 0.0f : t.dE;
    // dose_to_water in Gy per history: formed in FP32 (one rounding per step; the reference forms
    // it in double) and accumulated in FP64.  GB300's FP64 pipe is narrow, so the per-step
    // division stays in FP32.
    case MQI_SCORER_DOSE_W:
    case MQI_SCORER_DOSE_W2:
    case MQI_SCORER_DIJ: return dose_w;
    default: return 0.0f;
    }
}

/// fp_compute_hit for every enum'd scorer: the simple ones plus dose_to_medium and the LET weights
/// (FP64 square root and divisions), compiled only into the kernel instance of runs that use them.
__device__ inline double
compute_hit(int type, const Trk& t, float rho, float vol, float dose_w) {
    if (type == MQI_SCORER_DOSE_M)
        return t.primary ? (double) t.dE * 1.60218e-13 * 1000.0 / (double) (vol * rho) : 0.0;
    if (type < MQI_SCORER_LETD_NUM || type > MQI_SCORER_LETT_DEN) {
        const double v = (double) compute_hit_simple(type, t, dose_w);
        return type == MQI_SCORER_DOSE_W2 ? v * v : v;
    }
    // LET scorers (mqi_scorer_energy_deposit.hpp:91-177)
    // the step length as the reference forms it: float differences squared in float, summed in double
    const float  density = rho * 1000.0f;
    const float  lx = t.p1.x - t.p0.x, ly = t.p1.y - t.p0.y, lz = t.p1.z - t.p0.z;
    const double length = sqrt((double) (lx * lx) + (double) (ly * ly) + (double) (lz * lz));
    if (!(length > 0.0)) return 0.0;
    const double let = (double) t.dE / length / (double) density;
    switch (type) {
    case MQI_SCORER_LETD_NUM: return (let >= 25.0) ? 0.0 : (double) t.dE * let;
    case MQI_SCORER_LETD_DEN: return (let >= 25.0) ? 0.0 : (double) t.dE;
    case MQI_SCORER_LETT_NUM: return length * let;
    case MQI_SCORER_LETT_DEN: return length;
    default: return 0.0;
    }
}

/// Score one step of track t in voxel cnb with every scorer of the current child.  The kernel
/// instance's mode (kModeDij | kModeFull | kModeRoi, WaveParams::kernel_mode) compiles in only
/// the scoring code the run uses: the Dij insertion, the dose_to_medium and LET callbacks (FP64
/// square root and divisions), the INDIRECT / CONTOUR ROI mappings.  Code that never runs still
/// costs registers and instruction-cache space in the step loop: carrying all of it cost 30% of
/// the slab-phantom throughput, the ROI mappings alone another 11%.
template<int kMode = kModeAll>
__device__ inline void
score_step(Ctx& C, const Trk& t, uint32_t cnb, float rho, float vol) {
    constexpr bool kDij  = (kMode & kModeDij) != 0;
    constexpr bool kFull = (kMode & kModeFull) != 0;
    constexpr bool kRoi  = (kMode & kModeRoi) != 0;
    if constexpr ((kMode & kModeSingle) != 0) {
        // one scorer: the loop, its per-scorer dispatch and the scenario/stride addressing fold
        // away (measured 5.8% of the step time on the slab phantom)
        const ScorerDev& s  = C.P->scorer[0];
        float            vf = t.dE + t.ldE;
        if (s.type == MQI_SCORER_DOSE_W) {
            const float spr = t.spr0 >= 0.0f ? t.spr0 : spr_of(C.P->calib, rho, t.ke0, C.dbg);
            vf              = (rho < 1.0e-7f) ? 0.0f : vf * 1.60218e-10f / (vol * rho * spr);
        }
        tally_add(s.tally, cnb, (double) vf, cnb > 0 && vf > 0.0f);
        return;
    }
    if constexpr (kMode == kModeStat) {
        // dose_to_water, then the statistics pair of the same value (dose and dose^2 side by side):
        // the generic loop's per-scorer dispatch and addressing fold away
        const ChildDev& ch = C.P->child[C.child];
        if (ch.n_scorers == 0) return;
        const ScorerDev& sd  = C.P->scorer[ch.scorer_begin];
        const ScorerDev& sp  = C.P->scorer[ch.scorer_begin + 1];
        const float      spr = t.spr0 >= 0.0f ? t.spr0 : spr_of(C.P->calib, rho, t.ke0, C.dbg);
        const float dose_w = (rho < 1.0e-7f) ? 0.0f : (t.dE + t.ldE) * 1.60218e-10f / (vol * rho * spr);
        if (!(dose_w > 0.0f)) return;
        const double   v  = (double) dose_w;
        const uint64_t sc = (uint64_t) (C.spot >> kScenShift);
        tally_add(sd.tally, sc * sd.tally_len + cnb, v, cnb > 0);   // DIRECT: idx(cnb) = cnb > 0
        double* pair = sp.tally + (sc * sp.tally_len + cnb) * 2;    // DIRECT: get_mask_idx(cnb) = cnb
        atomicAdd(pair, v);
        atomicAdd(pair + 1, v * v);
        return;
    }
    const WaveParams& P   = *C.P;
    const ChildDev&   ch  = P.child[C.child];
    const float       spr = t.spr0 >= 0.0f ? t.spr0 : spr_of(P.calib, rho, t.ke0, C.dbg);
    // dose_to_water of the step, shared by the dose, dose^2 and Dij scorers (Dw_pointer,
    // mqi_scorer_energy_deposit.hpp:23-40): 0 in vacuum voxels
    const float dose_w = (rho < 1.0e-7f) ? 0.0f : (t.dE + t.ldE) * 1.60218e-10f / (vol * rho * spr);
    for (int si = 0; si < ch.n_scorers; ++si) {
        const ScorerDev& s = P.scorer[ch.scorer_begin + si];
        bool     ok;
        uint32_t key = cnb;
        if (!kRoi) {
            ok = s.stat_mode || cnb > 0;   // DIRECT: idx(cnb) = cnb > 0; get_mask_idx(cnb) = cnb
        } else if (s.stat_mode) {
            const int32_t m = roi_mask_idx(s, cnb);
            ok              = m >= 0;
            key             = (uint32_t) m;
        } else {
            ok = roi_idx(s, cnb) > 0;
        }
        double v;
        bool   pos;
        if (kFull) {
            v   = ok ? compute_hit(s.type, t, rho, vol, dose_w) : 0.0;
            pos = v > 0.0;
        } else {
            // the FP64 pipe is narrow: filter in FP32, convert once, square only for dose^2
            const float vf = ok ? compute_hit_simple(s.type, t, dose_w) : 0.0f;
            pos            = vf > 0.0f;
            v              = (double) vf;
            if (s.type == MQI_SCORER_DOSE_W2) v *= v;
        }
        if (s.double_score) v += v;
        if (kDij && s.type == MQI_SCORER_DIJ) {
            // insert_hashtable(data_, cnb, spot_ind, ...) (mqi_transport.hpp:204-225); a history
            // without a spot index lands in column 0
            const uint32_t col = (C.spot & kSpotMask) == kNoSpot ? 0u : (C.spot & kSpotMask);
            dij_add(s, P.error_flag, col, cnb, v, ok && pos);
            continue;
        }
        const bool valid = ok && pos && key < s.tally_len;
        const uint64_t slot = ((uint64_t) (C.spot >> kScenShift) * s.tally_len + key) * s.tstride;   // scenario's tally
        tally_add(s.tally, slot, v, valid);
    }
}

// ------------------------------------------------------------------------------------------
// Daughters
// ------------------------------------------------------------------------------------------

/// Child-frame -> world-frame transform the reference applies to a daughter's vertex before
/// pushing it (e.g. mqi_pp_elastic.hpp:188-195): R_fwd * (p - T) + T and R_fwd * d.  The child's
/// rotation and translation are read from the kernel parameters (the per-lane grid does not carry
/// them: they are used only at child entry and exit and for daughters).
__device__ inline void
daughter_to_world(const ChildDev& ch, float3& p, float3& d) {
    if (ch.identity) return;
    const float3 q = make_float3(p.x - ch.tr[0], p.y - ch.tr[1], p.z - ch.tr[2]);
    const float3 r = matvec(ch.rf, q);
    p              = make_float3(r.x + ch.tr[0], r.y + ch.tr[1], r.z + ch.tr[2]);
    d              = matvec(ch.rf, d);
}

/// World -> child frame on entry (mqi_transport.hpp:165-168).
__device__ inline void
to_child(const ChildDev& ch, float3& p, float3& d) {
    if (!ch.identity) {
        p = matvec(ch.ri, make_float3(fsub(p.x, ch.tr[0]), fsub(p.y, ch.tr[1]), fsub(p.z, ch.tr[2])));
        d = matvec(ch.ri, d);
    }
    d = normalize3(d);
}

/// Child -> world frame on exit (mqi_transport.hpp:234-237).
__device__ inline void
to_world(const ChildDev& ch, float3& p, float3& d) {
    if (ch.identity) return;
    const float3 r = matvec(ch.rf, p);
    p              = make_float3(fadd(r.x, ch.tr[0]), fadd(r.y, ch.tr[1]), fadd(r.z, ch.tr[2]));
    d              = matvec(ch.rf, d);
}

/// track_t::update_post_vertex_position with the last_step length
/// (p_ionization_tabulated::last_step, mqi_p_ionization.hpp:481-490).
/// The last-step position with the stopping-power ratio at (rho, ke0) given.
__device__ inline float3
last_step_pos_spr(const Tables* T, float3 p0, float3 d0, float ke0, float dE, float rho, float spr) {
    float lw = 0.0f;
    if (dE > 0.0f) lw = -dE / dedx_lookup(*T, ke0);
    const float sl = lw * kWaterDensity / (spr * rho);
    return make_float3(p0.x + d0.x * sl, p0.y + d0.y * sl, p0.z + d0.z * sl);
}

/// The same, out of line and with the ratio computed here (the step loop's cut branch, which ends
/// each track once).
__device__ __noinline__ float3
last_step_pos(const Tables* T, const CalibDev* cal, bool dbg, float3 p0, float3 d0, float ke0, float dE, float rho) {
    return last_step_pos_spr(T, p0, d0, ke0, dE, rho, spr_of(*cal, rho, ke0, dbg));
}

/// What the reference does when it pops a deposit-only daughter (kinetic energy at or below
/// the 0.5 MeV tracking cut) in a single-child world: enter the grid, take the stepping()
/// cut branch (mqi_fippel_physics.hpp:86-94) and score once.  Returns false when the daughter
/// needs the general path (outside the grid or in a vacuum voxel).
template<int kMode>
__device__ inline bool
score_local_daughter(Ctx& C, float3 pw, float3 dw, float ke0, float dE0, uint32_t hint_cnb) {
    float3 p = pw, d = dw;
    to_child(C.P->child[C.child], p, d);
    Trk t;
    const uint32_t nxy  = (uint32_t) C.g.nx * (uint32_t) C.g.ny;
    const int3     hint = make_int3((int) (hint_cnb % nxy % (uint32_t) C.g.nx), (int) (hint_cnb % nxy / (uint32_t) C.g.nx),
                                    (int) (hint_cnb / nxy));
    // the daughter sits where its parent's step started, nearly always well inside the parent's
    // voxel: grid3d::index's answer is then that voxel, and the three edge searches are skipped
    t.cell = make_int3(index_axis_hint(C.g.xe, C.g.nx, p.x, d.x, hint.x), index_axis_hint(C.g.ye, C.g.ny, p.y, d.y, hint.y),
                       index_axis_hint(C.g.ze, C.g.nz, p.z, d.z, hint.z));
    if (!grid_valid(C.g, t.cell)) return false;
    const uint32_t cnb = grid_cnb(C.g, t.cell);
    const float    rho = voxel_rho(C.g, cnb);
    if (rho < 1.0e-7f) return false;
    const float d2b = grid_exit(C.g, p, d, t.cell);
    if (d2b < 0.0f) return true;   // the voxel loop breaks before scoring
    t.p0 = p; t.d0 = d; t.p1 = p; t.d1 = d;
    t.ke0 = ke0 < 0.0f ? 0.0f : ke0;
    t.dE = dE0; t.ldE = 0.0f;
    t.spr0 = -1.0f;
    t.primary = false;
    if (rho <= 99.9f) {
        t.dE += t.ke0;
        t.spr0 = spr_of(C.P->calib, rho, t.ke0, C.dbg);   // computed once for the position and the score
        t.p1   = last_step_pos_spr(C.T, p, d, t.ke0, t.dE, rho, t.spr0);
    }
    score_step<kMode>(C, t, cnb, rho, grid_volume(C.g, t.cell));
    return true;
}

/// Emit one daughter that survived the stack-limit check: move it to the world frame, score it
/// where it stands when it is a deposit-only daughter of a single-child world, else append it to
/// the next queue.  Out of line and by value: it runs on a few percent of the steps and its
/// body would otherwise be inlined at every push site of the four processes.
/// Returns 0 queued, 1 scored locally, 2 queue overflow.
template<int kMode>
static __device__ __noinline__ int
emit_daughter(const WaveParams* P, const Tables* T, int child, uint32_t hint, const float* xe, const float* ye, const float* ze,
              bool dbg, uint32_t below, uint64_t uid, uint32_t hist, uint32_t spot, float ke0, bool ke1_zero, float3 p,
              float3 d, float dE0) {
    Ctx C;
    C.P = P; C.T = T; C.child = child; C.dbg = dbg; C.tcut = 0.0f; C.spot = spot;
    C.g = make_grid(P->child[child], xe, ye, ze);
    apply_scenario(*P, C.g, child, spot);
    daughter_to_world(P->child[child], p, d);
    if (P->inline_local && ke0 <= kTpCut && score_local_daughter<kMode>(C, p, d, ke0, dE0, hint)) return 1;
    const Queue&   q = P->out;
    const uint32_t i = atomicAdd(P->n_out, 1u);
    if (i >= q.capacity) {
        atomicOr(P->error_flag, 2u);
        return 2;
    }
    q.ke[i] = ke0;
    q.px[i] = p.x; q.py[i] = p.y; q.pz[i] = p.z;
    q.dx[i] = d.x; q.dy[i] = d.y; q.dz[i] = d.z;
    q.dE0[i] = dE0;
    q.hist[i] = hist;
    q.uid_lo[i] = (uint32_t) uid;
    q.uid_hi[i] = (uint32_t) (uid >> 32);
    q.ctr[i] = 0;
    q.meta[i] = (below & kMetaBelowMask) | (ke1_zero ? kMetaKe1Zero : 0u);
    q.cell[i] = 0;
    q.spot[i] = spot;
    return 0;
}

/// track_stack_t::push_secondary (mqi_track_stack.hpp:36-41) with the stack depth emulated:
/// a track popped with `below` entries under it pushes its i-th daughter at depth below + i,
/// and the push is dropped when that reaches the limit (200 with debug physics, else 10).
template<int kMode>
__device__ inline void
push_daughter(Ctx& C, Trk& t, float ke0, bool ke1_zero, float3 p, float3 d, float dE0) {
    if (t.below + t.npush >= (uint32_t) C.P->stack_limit) {
        count_event(kCntDrop);
        return;
    }
    const uint32_t below = t.below + t.npush;
    const uint64_t uid   = daughter_uid(t.uid, t.npush);
    ++t.npush;
    const int r = emit_daughter<kMode>(C.P, C.T, C.child, grid_cnb(C.g, t.cell), C.g.xe, C.g.ye, C.g.ze, C.dbg, below, uid, t.hist,
                                t.spot, ke0, ke1_zero,
                                p, d, dE0);
    count_event(r == 0 ? kCntSec : (r == 1 ? kCntLocal : kCntErr));
}

// ------------------------------------------------------------------------------------------
// Physics: p_ionization_tabulated (mqi_p_ionization.hpp:297-490), pp/po elastic, po inelastic
// ------------------------------------------------------------------------------------------

/// energy_loss (mqi_p_ionization.hpp:297-331) with the straggling variance (:334-345).  The
/// range-table walk is guarded at index 0 (the reference's uint16 index wraps there).
__device__ inline float
energy_loss(const Tables& T, const Rel& rel, float rho, float len, float spr, float z) {
    const float lw = len * spr * rho / kWaterDensity;
    int n = (int) ((rel.Ek - 0.1f) / 0.5f);
    if (n > MQI_TABLE_N - 2) n = MQI_TABLE_N - 2;
    if (n < 0) n = 0;
    float x0 = 0.1f + (float) n * 0.5f;
    float x1 = x0 + 0.5f;
    if (x0 > rel.Ek && n > 0) n -= 1;
    if (x1 < rel.Ek && n < MQI_TABLE_N - 2) n += 1;
    float r = intpl1d_grid(rel.Ek, x0, x1, T.range[n], T.range[n + 1]);
    if (r < lw) return rel.Ek;
    r -= lw;
    while (n > 0 && r < T.range[n]) --n;
    x0 = 0.1f + (float) n * 0.5f;
    x1 = x0 + 0.5f;
    const float dE_mean = rel.Ek - intpl1d(r, T.range[n], T.range[n + 1], x0, x1);
    const float Te      = (rel.Te_max >= kTeStragCap) ? kTeStragCap : rel.Te_max;
    float       var     = dedx_term0() * rho / kWaterDensity * lw;
    var *= Te / rel.beta_sq * (1.0f - 0.5f * rel.beta_sq);
    float ret = z * sqrtf(var) + dE_mean;
    if (ret < 0.0f) ret = -ret;
    return ret;
}

/// p_ionization_tabulated::along_step (mqi_p_ionization.hpp:349-420): CSDA loss with Gaussian
/// straggling, Highland-style multiple scattering, position/energy update.  The step's first
/// block of random words is laid out as: [0] free path, [1,2] Box-Muller pair (straggling,
/// scattering angle), [3] azimuth.
__device__ inline void
along_step(Ctx& C, Trk& t, const Rel& rel, float len, float rho, float spr, float z_strag, float z_mcs,
           float u_phi) {
    const float dE = energy_loss(*C.T, rel, rho, len, spr, z_strag);
    float       r  = 1.0f;
    if (dE >= t.ke0) {
        r         = t.ke0 / dE;
        t.stopped = true;
    }
    const float P     = rel.momentum();
    const float X0    = x0_of(C.P->calib, rho, C.dbg);
    const float th_sq = ((kEs / P) * (kEs / P) / rel.beta_sq) * len / X0;
    float       th    = sqrtf(th_sq);
    th                = z_mcs * (sqrtf(2.0f) * th);
    if (th < 0.0f) th = -th;
    const float phi = 2.0f * kPi * u_phi;
    t.d1            = rotate_dir_inline(t.d1, th, phi);
    t.dE += dE * r;
    t.p1 = advance(t.p0, t.d0, r * len);
    t.ke1 -= dE * r;
}

/// Delta-ray production (p_ionization_tabulated::post_step, mqi_p_ionization.hpp:425-477).
template<int kMode>
__device__ inline void
post_delta(Ctx& C, Trk& t, Rng& rng) {
    const Rel rel(t.ke1);
    float     Te = 0.0f;
    for (int it = 0;; ++it) {
        const float n = rng.uniform();
        Te            = C.tcut * rel.Te_max;
        Te /= ((1.0f - n) * rel.Te_max + n * C.tcut);
        if (rng.uniform() < 1.0f - rel.beta_sq * Te / rel.Te_max + Te * Te / (2.0f * rel.Et_sq)) break;
        if (it >= 63) {   // acceptance >= 1 - beta^2 > 0: unreachable in practice, bounded anyway
            count_event(kCntErr);
            break;
        }
    }
    if (C.dbg) push_daughter<kMode>(C, t, 0.0f, true, t.p0, t.d0, Te);
    else t.dE += Te;
    t.ke1 -= Te;
}

/// p-p elastic (pp_elastic_tabulated::post_step, mqi_pp_elastic.hpp:119-219).
template<int kMode>
__device__ inline void
post_pp(Ctx& C, Trk& t, Rng& rng) {
    const Rel   rel(t.ke1);
    const float Mp_sq = kMp * kMp;
    const float minv  = kTpCut / rel.Ek;
    const float u     = rng.uniform() * (1.0f - 2.0f * minv) + minv;
    const float E1    = rel.Et;
    const float dE    = rel.Ek * u;
    const float E3    = (rel.Ek - dE) + kMp;
    const float E4    = dE + kMp;
    const float P1    = rel.momentum();
    const float P3    = sqrtf(E3 * E3 - Mp_sq);
    const float P4    = sqrtf(E4 * E4 - Mp_sq);
    float c3  = E1 * E3 - Mp_sq - kMp * (E1 - E3);
    c3 /= (P1 * P3);
    float c34 = E3 * E4 - E1 * kMp;
    c34 /= (P3 * P4);
    c3  = fminf(fmaxf(c3, -1.0f), 1.0f);
    c34 = fminf(fmaxf(c34, -1.0f), 1.0f);
    const float th3 = acosf(c3);
    const float th4 = th3 - acosf(c34);
    const float phi = 2.0f * kPi * rng.uniform();
    t.ke1 -= dE;
    t.d1 = rotate_dir(t.d1, th3, phi);
    const float3 dd = rotate_dir(t.d1, th4, phi);
    push_daughter<kMode>(C, t, dE, false, t.p1, dd, 0.0f);
}

/// p-O elastic (po_elastic::post_step, mqi_po_elastic.hpp:96-217).  The energy given to the
/// oxygen is a truncated exponential of mean Tp_avg on [0, Tp_max]; it is drawn by inverting
/// its CDF, which has the same law as the reference's redraw-until-below-Tp_max loop
/// (mqi_math.hpp:298-307) without the loop.
template<int kMode>
__device__ inline void
post_poe(Ctx& C, Trk& t, Rng& rng) {
    const Rel rel(t.ke1);
    if (rel.Ek <= 5.5f) {
        const float dE = rel.Ek;
        if (C.dbg) push_daughter<kMode>(C, t, dE, true, t.p1, t.d1, dE);
        else t.ldE += dE;
        t.ke1 -= dE;
        t.stopped = true;
        return;
    }
    const float MoMp    = kMo / kMp;
    const float MoMp_sq = MoMp * MoMp;
    const float Tp_avg  = 0.65f * expf(-0.0013f * rel.Ek) - 0.71f * expf(-0.0177f * rel.Ek);
    const float Tp_max  = (2.0f * kMo * rel.beta_sq * rel.gamma_sq) / (1.0f + 2.0f * rel.gamma * MoMp + MoMp_sq);
    const float u       = rng.uniform();
    float       dE      = -Tp_avg * log1pf(u * expm1f(-Tp_max / Tp_avg));
    if (!(dE >= 0.0f)) dE = 0.0f;
    if (dE > Tp_max) dE = Tp_max;
    const float E1 = rel.Ek * (rel.Ek + 2.0f * kMp);
    const float E3 = (rel.Ek - dE) * (rel.Ek - dE + 2.0f * kMp);
    float c3 = (E1 + E3 - dE * (dE + 2.0f * kMo)) / 2.0f / sqrtf(E1 * E3);
    c3              = fminf(fmaxf(c3, -1.0f), 1.0f);
    const float th3 = acosf(c3);
    const float phi = 2.0f * kPi * rng.uniform();
    if (C.dbg) push_daughter<kMode>(C, t, dE, true, t.p0, t.d0, dE);
    else t.ldE += dE;
    t.ke1 -= dE;
    t.d1 = rotate_dir(t.d1, th3, phi);
}

/// p-O inelastic cascade (po_inelastic_tabulated::post_step, mqi_po_inelastic.hpp:158-288).
template<int kMode>
__device__ inline void
post_poi(Ctx& C, Trk& t, Rng& rng) {
    const float Ek = t.ke1;
    float       Eb = 5.0f, Er = Ek;
    float       P2, PL, pw;
    if (Ek <= 215.0f && Ek > 200.0f) { P2 = 0.78f; PL = P2 + (1.0f - P2) * 0.9f; pw = 0.4f; }
    else if (Ek > 215.0f)            { P2 = 0.78f; PL = P2 + (1.0f - P2) * 1.0f; pw = 0.4f; }
    else if (Ek > 150.0f)            { P2 = 0.72f; PL = P2 + (1.0f - P2) * 0.83f; pw = 0.45f; }
    else                             { P2 = 0.7f;  PL = P2 + (1.0f - P2) * 0.83f; pw = 0.52f; }
    for (int round = 0; (Er - Eb) > 2.0f; ++round) {
        if (round >= 64) { count_event(kCntErr); break; }   // Eb shrinks by 0.65 and Er by >= 2 MeV per round
        Er -= Eb;
        float dE = powf(rng.uniform(), pw) * (Er - 2.0f) + 2.0f;
        if (dE >= Er) dE = Er;
        Er -= dE;
        t.ke1 -= (dE + Eb);
        const float zeta = rng.uniform();
        if (zeta < P2) {
            float c = (2.0f * dE / Ek - 1.0f) + 2.0f * (1.0f - dE / Ek) * rng.uniform();
            c               = fminf(fmaxf(c, -1.0f), 1.0f);
            const float th  = acosf(c);
            const float phi = 2.0f * kPi * rng.uniform();
            const float3 dd = rotate_dir(t.d1, th, phi);
            push_daughter<kMode>(C, t, dE, false, t.p1, dd, 0.0f);
        } else if (zeta < PL) {
            // long-range energy (neutrons, photons) leaves the system
        } else if (C.dbg) {
            push_daughter<kMode>(C, t, dE, true, t.p0, t.d0, dE);
        }
        Eb *= 0.65f;
    }
    t.dE += Er;
    t.ke1 -= Er;
    t.stopped = true;
}

/// The post-step of a nuclear interaction run inside the step loop (kernel instances that do not
/// hand them to the post-step kernel): the track and its stream go in and out by value, which
/// keeps the rarely-taken processes from pinning registers across the loop.
struct PostState {
    Trk t;
    Rng rng;
};

template<int kMode>
__device__ __forceinline__ PostState
post_nuclear(const WaveParams* P, const Tables* T, Grid g, int child, bool dbg, float tcut, int proc, PostState s) {
    Ctx C;
    C.P = P; C.T = T; C.g = g; C.child = child; C.dbg = dbg; C.tcut = tcut;
    C.spot = s.t.spot;
    if (proc == 1) post_pp<kMode>(C, s.t, s.rng);
    else if (proc == 2) post_poe<kMode>(C, s.t, s.rng);
    else post_poi<kMode>(C, s.t, s.rng);
    return s;
}

/// fippel_physics::stepping (mqi_fippel_physics.hpp:67-216).  A delta ray is produced here.  A
/// nuclear interaction (1 p-p elastic, 2 p-O elastic, 3 p-O inelastic) either runs here too
/// (kSplit false) or ends the step early: stepping returns the process and the post-step kernel
/// (k_post) finishes the step after the wave (kSplit true).
template<int kMode, bool kSplit>
__device__ inline int
stepping(Ctx& C, Trk& t, Rng& rng, float rho, float d2b) {
    t.spr0 = -1.0f;
    if (rho < 1.0e-7f) {
        t.p1 = advance(t.p0, t.d0, d2b);
        return 0;
    }
    if (rho > 99.9f) {
        t.stopped = true;
        return 0;
    }
    if (t.ke0 <= kTpCut) {
        if (t.ke0 < 0.0f) t.ke0 = 0.0f;
        t.dE += t.ke0;
        t.ke1 -= t.ke0;
        t.p1      = last_step_pos(C.T, &C.P->calib, C.dbg, t.p0, t.d0, t.ke0, t.dE, rho);
        t.stopped = true;
        return 0;
    }
    const Tables& T = *C.T;
    rng.begin_step();
    const Rel   rel(t.ke0);
    const float spr      = spr_of(C.P->calib, rho, t.ke0, C.dbg);
    const float dedx     = dedx_lookup(T, rel.Ek);
    const float cur_min  = kMaxStep * spr * rho / kWaterDensity;
    const float max_loss = -1.0f * cur_min * dedx;
    const CrossSections k1 = cross_sections(T, rel.Ek, rho);
    const CrossSections k2 = cross_sections(T, t.ke0 - max_loss, rho);
    const float sum1 = k1.ion + k1.pp + k1.poe + k1.poi;
    const float sum2 = k2.ion + k2.pp + k2.poe + k2.poi;
    const bool  pick1 = sum1 >= sum2;
    const float cs_sum = pick1 ? sum1 : sum2;
    const float c0 = pick1 ? k1.ion : k2.ion;
    const float c1 = pick1 ? k1.pp : k2.pp;
    const float c2 = pick1 ? k1.poe : k2.poe;
    const float c3 = pick1 ? k1.poi : k2.poi;
    const float u_mfp      = rng.uniform();
    const float mfp        = -1.0f * logf(u_mfp) / cs_sum;
    const float step_limit = cur_min * kWaterDensity / (spr * rho);
    // Box-Muller pair and azimuth for along_step (words 1..3 of the step's first block)
    const float bm_u1 = rng.uniform();
    const float bm_u2 = rng.uniform();
    const float u_phi = rng.uniform();
    float       s_bm, c_bm;
    sincospif(2.0f * bm_u2, &s_bm, &c_bm);
    const float bm_r  = sqrtf(-2.0f * logf(bm_u1));
    const float z1    = bm_r * c_bm;
    const float z2    = bm_r * s_bm;
    // The three branches of the reference (boundary, interaction, maximum step) differ only in the
    // step length given to along_step and in the post-step process of the interaction branch, so
    // the length is selected first and along_step runs once for every lane of the warp.
    const bool to_boundary = d2b < mfp && d2b < step_limit;
    const bool interaction = !to_boundary && (mfp < d2b || fabsf(mfp - d2b) < kGeoTol) &&
                             (mfp < step_limit || fabsf(mfp - step_limit) < kGeoTol);
    const float len = to_boundary ? d2b : (interaction ? mfp : step_limit);
    along_step(C, t, rel, len, rho, spr, z1, z2, u_phi);
    t.spr0 = spr;
    if (interaction && t.ke1 > kTpCut) {
        const float u = cs_sum * rng.uniform();
        t.d1          = t.d0;
        const int proc = (u < c0) ? 0 : (u < c0 + c1) ? 1 : (u < c0 + c1 + c2) ? 2 : (u < c0 + c1 + c2 + c3) ? 3 : -1;
        if (proc == 0) {
            post_delta<kMode>(C, t, rng);   // ~15% of the steps
        } else if (proc > 0) {       // ~0.2% of the steps
            if constexpr (kSplit) {
                return proc;
            } else {
                PostState ps;
                ps.t   = t;
                ps.rng = rng;
                ps     = post_nuclear<kMode>(C.P, C.T, C.g, C.child, C.dbg, C.tcut, proc, ps);
                t      = ps.t;
                rng    = ps.rng;
            }
        }
    }
    return 0;
}

// ------------------------------------------------------------------------------------------
// The wave kernel
// ------------------------------------------------------------------------------------------

/// Load queue entry i.  A track re-queued mid-grid (step_phase) comes back with the voxel index
/// it stopped in, in `cnb`; the caller turns it into a cell once the child's grid is known.
__device__ inline void
load_track(const Queue& q, uint32_t i, Trk& t, Rng& rng, bool& step_phase, uint32_t& cnb) {
    t.ke0  = q.ke[i];
    const uint32_t meta = q.meta[i];
    t.ke1  = (meta & kMetaKe1Zero) ? 0.0f : t.ke0;
    t.p0   = make_float3(q.px[i], q.py[i], q.pz[i]);
    t.d0   = make_float3(q.dx[i], q.dy[i], q.dz[i]);
    t.p1   = t.p0;
    t.d1   = t.d0;
    t.dE   = q.dE0[i];
    t.ldE  = 0.0f;
    t.hist = q.hist[i];
    t.spot = q.spot[i];
    t.uid  = (uint64_t) q.uid_lo[i] | ((uint64_t) q.uid_hi[i] << 32);
    t.below   = meta & kMetaBelowMask;
    t.primary = (meta & kMetaPrimary) != 0;
    t.child   = (int) ((meta >> kMetaChildShift) & 7u);
    t.npush   = (meta >> kMetaNpushShift) & 1023u;
    t.stopped = false;
    step_phase = (meta & kMetaPhaseStep) != 0;
    cnb = q.cell[i];
    rng.hist   = t.hist;
    rng.uid_lo = (uint32_t) t.uid;
    rng.uid_hi = (uint32_t) (t.uid >> 32);
    rng.ctr    = q.ctr[i];
    rng.pos    = 4;
    rng.has2   = false;
}

/// The queue's meta word of a track (without the phase bit).
__device__ inline uint32_t
track_meta(const Trk& t) {
    return (t.below & kMetaBelowMask) | (t.primary ? kMetaPrimary : 0u) | (t.ke1 != t.ke0 ? kMetaKe1Zero : 0u) |
           ((uint32_t) t.child << kMetaChildShift) | ((t.npush & 1023u) << kMetaNpushShift);
}

/// Queue a track that left a child grid for the entry into child t.child (world frame).
__device__ inline void
requeue_entry(Ctx& C, const Trk& t, const Rng& rng) {
    const Queue& q   = C.P->out;
    const uint32_t i = atomicAdd(C.P->n_out, 1u);
    if (i >= q.capacity) {
        atomicOr(C.P->error_flag, 2u);
        count_event(kCntErr);
        return;
    }
    q.ke[i] = t.ke0;
    q.px[i] = t.p0.x; q.py[i] = t.p0.y; q.pz[i] = t.p0.z;
    q.dx[i] = t.d0.x; q.dy[i] = t.d0.y; q.dz[i] = t.d0.z;
    q.dE0[i] = 0.0f;
    q.hist[i] = t.hist;
    q.uid_lo[i] = (uint32_t) t.uid;
    q.uid_hi[i] = (uint32_t) (t.uid >> 32);
    q.ctr[i] = rng.ctr;
    q.meta[i] = track_meta(t);
    q.cell[i] = 0;
    q.spot[i] = t.spot;
}

/// Hand a track whose step ended in nuclear process `proc` to the post-step kernel.  A track is
/// handed over at most once per wave and every handed-over track was fetched from the wave's
/// input, so the record array (sized like the input queue) cannot run out.
__device__ inline void
defer_track(Ctx& C, const Trk& t, const Rng& rng, uint32_t cnb, int proc) {
    const uint32_t i = atomicAdd(C.P->n_def, 1u);
    if (i >= C.P->in.capacity) {
        atomicOr(C.P->error_flag, 2u);
        count_event(kCntErr);
        return;
    }
    Deferred& d = C.P->def[i];
    d.ke0 = t.ke0;
    d.ke1 = t.ke1;
    d.p0[0] = t.p0.x; d.p0[1] = t.p0.y; d.p0[2] = t.p0.z;
    d.d0[0] = t.d0.x; d.d0[1] = t.d0.y; d.d0[2] = t.d0.z;
    d.p1[0] = t.p1.x; d.p1[1] = t.p1.y; d.p1[2] = t.p1.z;
    d.dE     = t.dE;
    d.spr0   = t.spr0;
    d.cnb    = cnb;
    d.uid_lo = (uint32_t) t.uid;
    d.uid_hi = (uint32_t) (t.uid >> 32);
    d.hist   = t.hist;
    d.spot   = t.spot;
    d.meta   = (t.below & kMetaBelowMask) | (t.primary ? kMetaPrimary : 0u) | ((uint32_t) t.child << kMetaChildShift) |
             ((t.npush & 1023u) << kMetaNpushShift);
    d.ctr  = rng.ctr;
    d.proc = (uint32_t) proc;
}

/// Write a track that used up its step budget back to the next queue, mid-grid.
__device__ inline void
requeue_track(Ctx& C, const Trk& t, const Rng& rng) {
    const Queue& q   = C.P->out;
    const uint32_t i = atomicAdd(C.P->n_out, 1u);
    if (i >= q.capacity) {
        atomicOr(C.P->error_flag, 2u);
        count_event(kCntErr);
        return;
    }
    q.ke[i] = t.ke0;
    q.px[i] = t.p0.x; q.py[i] = t.p0.y; q.pz[i] = t.p0.z;
    q.dx[i] = t.d0.x; q.dy[i] = t.d0.y; q.dz[i] = t.d0.z;
    q.dE0[i] = 0.0f;
    q.hist[i] = t.hist;
    q.uid_lo[i] = (uint32_t) t.uid;
    q.uid_hi[i] = (uint32_t) (t.uid >> 32);
    q.ctr[i] = rng.ctr;
    q.meta[i] = track_meta(t) | kMetaPhaseStep;
    q.cell[i] = grid_cnb(C.g, t.cell);
    q.spot[i] = t.spot;
}

template<int kMode, bool kSplit>
__device__ __forceinline__ void
wave_body(const WaveParams& P) {
    extern __shared__ __align__(16) unsigned char smem[];
    Tables* T = reinterpret_cast<Tables*>(smem);
    {
        const float4* src = reinterpret_cast<const float4*>(P.tables);
        float4*       dst = reinterpret_cast<float4*>(smem);
        for (int i = threadIdx.x; i < 6 * MQI_TABLE_N / 4; i += blockDim.x) dst[i] = src[i];
    }
    // Edges of the children staged after the tables when they fit.
    float* sedges     = reinterpret_cast<float*>(smem + sizeof(Tables));
    __shared__ const float* s_edges[kMaxChildren][3];   // staged edge arrays per child (null: global)
    if (threadIdx.x < kMaxChildren * 3) s_edges[threadIdx.x / 3][threadIdx.x % 3] = nullptr;
    if (threadIdx.x < 8) s_cnt[threadIdx.x] = 0u;
    __syncthreads();
    {
        int off = 0;
        for (int c = 0; c < P.n_children; ++c) {
            const ChildDev& ch = P.child[c];
            const int need     = ch.nx + ch.ny + ch.nz + 3;
            if (P.n_scen > 1 && c == P.scen_child) continue;   // scenario edges are read from global memory
            if (off + need > P.smem_edge_floats) break;
            float* e = sedges + off;
            for (int i = threadIdx.x; i <= ch.nx; i += blockDim.x) e[i] = ch.xe[i];
            for (int i = threadIdx.x; i <= ch.ny; i += blockDim.x) e[ch.nx + 1 + i] = ch.ye[i];
            for (int i = threadIdx.x; i <= ch.nz; i += blockDim.x) e[ch.nx + ch.ny + 2 + i] = ch.ze[i];
            if (threadIdx.x == 0) {
                s_edges[c][0] = e;
                s_edges[c][1] = e + ch.nx + 1;
                s_edges[c][2] = e + ch.nx + ch.ny + 2;
            }
            off += need;
        }
    }
    __syncthreads();

    Ctx C;
    C.P      = &P;
    C.T      = T;
    C.dbg    = P.physics_debug != 0;
    C.tcut   = P.t_cut;
    uint32_t n_steps = 0;

    Rng rng;
    rng.k0 = P.k0;
    rng.k1 = P.k1;
    Trk  t;
    bool have  = false;
    bool in_grid = false;
    uint32_t slice = 0;
    uint32_t track_steps = 0;   // per-track guard: a track is abandoned after kMaxTrackSteps
    // The input count can exceed the queue's capacity only after an overflowed append (the
    // append cursor counts on; nothing was written past the end).  The wave then does nothing:
    // the host reports the overflow, and no entry past the capacity is ever read.
    const uint32_t n_raw = *P.n_in;
    const uint32_t n_in  = (n_raw > P.in.capacity || (*P.error_flag & 2u)) ? 0u : n_raw;
    const int lane = threadIdx.x & 31;

    for (;;) {
        // ---- fetch (one atomic per warp) ----
        const unsigned act   = __activemask();
        const unsigned needm = __ballot_sync(act, !have);
        if (needm) {
            uint32_t base = 0;
            const int leader = __ffs(needm) - 1;
            if (lane == leader) base = atomicAdd(P.head, (uint32_t) __popc(needm));
            base = __shfl_sync(act, base, leader);
            if (!have) {
                const uint32_t idx = base + (uint32_t) __popc(needm & ((1u << lane) - 1u));
                if (idx >= n_in) break;
                bool     step_phase;
                uint32_t cnb0;
                load_track(P.in, idx, t, rng, step_phase, cnb0);
                have    = true;
                in_grid = step_phase;
                slice   = 0;
                track_steps = 0;
                count_event(kCntTracks);
                if (step_phase) {
                    C.child = t.child;
                    C.g     = make_grid(P.child[t.child], s_edges[t.child][0], s_edges[t.child][1], s_edges[t.child][2]);
                    apply_scenario(P, C.g, t.child, t.spot);
                    const uint32_t nxy = (uint32_t) C.g.nx * (uint32_t) C.g.ny;
                    const uint32_t rem = cnb0 % nxy;
                    t.cell = make_int3((int) (rem % (uint32_t) C.g.nx), (int) (rem / (uint32_t) C.g.nx), (int) (cnb0 / nxy));
                }
            }
        }
        if (!in_grid) {
            // ---- child entry (mqi_transport.hpp:161-190) ----
            if (t.stopped || t.child >= P.n_children) {
                if (t.primary) count_event(kCntHist);
                have = false;
                continue;
            }
            C.child = t.child;
            C.g     = make_grid(P.child[t.child], s_edges[t.child][0], s_edges[t.child][1], s_edges[t.child][2]);
            apply_scenario(P, C.g, t.child, t.spot);
            C.spot  = t.spot;
            to_child(P.child[t.child], t.p0, t.d0);
            t.p1 = t.p0;
            t.d1 = t.d0;
            int3 c = grid_index(C.g, t.p0, t.d0);
            if (!grid_valid(C.g, c)) {
                const float dist = grid_entry(C.g, t.p0, t.d0);
                if (dist < 0.0f) {
                    to_world(P.child[t.child], t.p0, t.d0);
                    t.p1 = t.p0;
                    t.d1 = t.d0;
                    ++t.child;
                    continue;
                }
                t.p1 = advance(t.p0, t.d0, dist);
                // move(): vtx0 = vtx1 (including ke), deposits reset
                t.p0  = t.p1;
                t.d0  = t.d1;
                t.ke0 = t.ke1;
                t.dE = t.ldE = 0.0f;
                c = grid_index(C.g, t.p0, t.d0);
            }
            t.cell = c;
            if (!grid_valid(C.g, c)) {
                to_world(P.child[t.child], t.p0, t.d0);
                t.p1 = t.p0;
                t.d1 = t.d0;
                ++t.child;
                continue;
            }
            in_grid = true;
            continue;
        }
        // ---- one voxel step (mqi_transport.hpp:192-233) ----
        C.spot = t.spot;
        const uint32_t cnb = grid_cnb(C.g, t.cell);
        const float    rho = voxel_rho(C.g, cnb);
        const float    d2b = grid_exit(C.g, t.p0, t.d0, t.cell);
        const int      nuclear = stepping<kMode, kSplit>(C, t, rng, rho, d2b);
        ++n_steps;
        if (kSplit && nuclear) {   // the post-step kernel finishes this step and queues the track
            defer_track(C, t, rng, cnb, nuclear);
            have    = false;
            in_grid = false;
            continue;
        }
        if (++track_steps > kMaxTrackSteps) {   // no physical track comes near this; never hang
            t.stopped = true;
            count_event(kCntErr);
        }
        bool leave = false;
        if (d2b < 0.0f) {
            leave = true;
        } else {
            score_step<kMode>(C, t, cnb, rho, grid_volume(C.g, t.cell));
            if (!t.stopped) {
                grid_step_index(C.g, t.p1, t.d1, t.cell);
                t.p0  = t.p1;
                t.d0  = t.d1;
                t.ke0 = t.ke1;
                t.dE = t.ldE = 0.0f;
            }
            leave = t.stopped || !grid_valid(C.g, t.cell);
        }
        if (leave) {
            to_world(P.child[C.child], t.p0, t.d0);
            t.p1 = t.p0;
            t.d1 = t.d0;
            ++t.child;
            in_grid = false;
            continue;
        }
        if (P.max_slice_steps && ++slice >= P.max_slice_steps) {
            requeue_track(C, t, rng);
            have    = false;
            in_grid = false;
        }
    }

    // ---- counters: one global atomic per block and field ----
    if (n_steps) atomicAdd(&s_cnt[kCntSteps], n_steps);
    __syncthreads();
    if (threadIdx.x < 8 && s_cnt[threadIdx.x]) atomicAdd(&P.stats[threadIdx.x], (unsigned long long) s_cnt[threadIdx.x]);
    if (threadIdx.x == 0 && s_cnt[kCntErr]) atomicOr(P.error_flag, 1u);
}

/// The post-step kernel's body: for each track the wave stopped at a nuclear interaction, the rest
/// of its step as the wave would have run it -- the process's post_step (mqi_pp_elastic.hpp:119-219,
/// mqi_po_elastic.hpp:96-217, mqi_po_inelastic.hpp:158-288), the step's scoring, the cell update
/// and move() (mqi_transport.hpp:204-233) -- then the track goes to the next wave's queue: mid-grid,
/// at the entry of the next child, or nowhere when it stopped or left the world.  The random
/// stream resumes where the step left it (the process draw was the first word of the block at
/// counter ctr - 1), so the track draws the same numbers as if the wave had run the process.
template<int kMode>
__device__ __forceinline__ void
post_body(const WaveParams& P) {
    Ctx C;
    C.P     = &P;
    C.T     = reinterpret_cast<const Tables*>(P.tables);
    C.dbg   = P.physics_debug != 0;
    C.tcut  = P.t_cut;
    if (threadIdx.x < 8) s_cnt[threadIdx.x] = 0u;
    __syncthreads();
    const uint32_t n_raw  = *P.n_def;
    const uint32_t n      = n_raw > P.in.capacity ? P.in.capacity : n_raw;   // past it: flagged, not written
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const Deferred& d = P.def[i];
        Trk t;
        t.ke0 = d.ke0;
        t.ke1 = d.ke1;
        t.p0  = make_float3(d.p0[0], d.p0[1], d.p0[2]);
        t.d0  = make_float3(d.d0[0], d.d0[1], d.d0[2]);
        t.p1  = make_float3(d.p1[0], d.p1[1], d.p1[2]);
        t.d1  = t.d0;
        t.dE  = d.dE;
        t.ldE = 0.0f;
        t.spr0 = d.spr0;
        t.uid  = (uint64_t) d.uid_lo | ((uint64_t) d.uid_hi << 32);
        t.hist = d.hist;
        t.spot = d.spot;
        t.below   = d.meta & kMetaBelowMask;
        t.primary = (d.meta & kMetaPrimary) != 0;
        t.child   = (int) ((d.meta >> kMetaChildShift) & 7u);
        t.npush   = (d.meta >> kMetaNpushShift) & 1023u;
        t.stopped = false;
        Rng rng;
        rng.k0     = P.k0;
        rng.k1     = P.k1;
        rng.hist   = d.hist;
        rng.uid_lo = d.uid_lo;
        rng.uid_hi = d.uid_hi;
        rng.ctr    = d.ctr;
        rng.blk    = philox_block(d.ctr - 1u, d.hist, d.uid_lo, d.uid_hi, P.k0, P.k1);
        rng.pos    = 1;
        rng.has2   = false;
        C.child = t.child;
        C.spot  = t.spot;
        C.g     = make_grid(P.child[t.child], nullptr, nullptr, nullptr);
        apply_scenario(P, C.g, t.child, t.spot);
        const uint32_t nxy = (uint32_t) C.g.nx * (uint32_t) C.g.ny;
        const uint32_t rem = d.cnb % nxy;
        t.cell = make_int3((int) (rem % (uint32_t) C.g.nx), (int) (rem / (uint32_t) C.g.nx), (int) (d.cnb / nxy));
        if (d.proc == 1) post_pp<kMode>(C, t, rng);
        else if (d.proc == 2) post_poe<kMode>(C, t, rng);
        else post_poi<kMode>(C, t, rng);
        score_step<kMode>(C, t, d.cnb, voxel_rho(C.g, d.cnb), grid_volume(C.g, t.cell));
        if (!t.stopped) {
            grid_step_index(C.g, t.p1, t.d1, t.cell);
            t.p0  = t.p1;
            t.d0  = t.d1;
            t.ke0 = t.ke1;
            t.dE = t.ldE = 0.0f;
        }
        if (!t.stopped && grid_valid(C.g, t.cell)) {
            requeue_track(C, t, rng);
            continue;
        }
        to_world(P.child[C.child], t.p0, t.d0);
        ++t.child;
        if (t.stopped || t.child >= P.n_children) {
            if (t.primary) count_event(kCntHist);
            continue;
        }
        requeue_entry(C, t, rng);
    }
    __syncthreads();
    if (threadIdx.x < 8 && s_cnt[threadIdx.x]) atomicAdd(&P.stats[threadIdx.x], (unsigned long long) s_cnt[threadIdx.x]);
    if (threadIdx.x == 0 && s_cnt[kCntErr]) atomicOr(P.error_flag, 1u);
}

}   // namespace mqi_gpu
namespace mqi_gpu
{

// ------------------------------------------------------------------------------------------
// Primaries: vertex_t<float> AoS (mqi_vertex.hpp:16-29) -> queue entries
// (track_t::set + push_primary, mqi_track.hpp:124-133, mqi_track_stack.hpp:44-48).
// ------------------------------------------------------------------------------------------
__device__ inline void
write_vertex_entry(const Queue& q, uint32_t i, const mqi_vertex* __restrict__ v, const uint32_t* __restrict__ spot_ids,
                   uint64_t h, uint32_t scen) {
    const mqi_vertex x = v[h];
    q.ke[i]     = x.ke;
    q.px[i]     = x.pos[0];
    q.py[i]     = x.pos[1];
    q.pz[i]     = x.pos[2];
    q.dx[i]     = x.dir[0];
    q.dy[i]     = x.dir[1];
    q.dz[i]     = x.dir[2];
    q.dE0[i]    = 0.0f;
    q.hist[i]   = (uint32_t) h;
    q.uid_lo[i] = 0u;
    q.uid_hi[i] = 0u;
    q.ctr[i]    = 0u;
    q.meta[i]   = kMetaPrimary;
    q.cell[i]   = 0;
    q.spot[i]   = ((spot_ids ? spot_ids[h] : kNoSpot) & kSpotMask) | (scen << kScenShift);
}

__global__ void
k_load_primaries(Queue q, const mqi_vertex* __restrict__ v, const uint32_t* __restrict__ spot_ids, uint64_t h0,
                 uint32_t n, uint32_t n_scen) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n * n_scen) return;
    write_vertex_entry(q, i, v, spot_ids, h0 + i / n_scen, i % n_scen);
}

/// One thread: size the top-up of the queue holding *n_in entries (what the previous wave left).
/// After a queue overflow (error bit 2) nothing more is loaded and the remaining waves of the
/// graph find an empty queue.
__global__ void
k_topup(TopUp* tu, uint32_t* n_in, const uint32_t* error_flag) {
    if (*error_flag & 2u) {
        tu->count = 0;
        *n_in     = 0;
        return;
    }
    const uint32_t have = *n_in;
    uint64_t       want = have < tu->target ? (tu->target - have) / tu->n_scen : 0ull;
    const uint64_t left = tu->end - tu->next;
    if (want > left) want = left;
    tu->base  = tu->next;
    tu->dst   = have;
    tu->count = (uint32_t) (want * tu->n_scen);
    tu->next += want;
    *n_in = have + tu->count;
}

__global__ void
k_load_topup(Queue q, const TopUp* __restrict__ tu, const mqi_vertex* __restrict__ v,
             const uint32_t* __restrict__ spot_ids) {
    const uint32_t n = tu->count, S = tu->n_scen, dst = tu->dst;
    const uint64_t base = tu->base;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        write_vertex_entry(q, dst + i, v, spot_ids, base + i / S, i % S);
}

cudaError_t
launch_load_primaries(const Queue& q, const mqi_vertex* v, const uint32_t* spot_ids, uint64_t h0, uint32_t n,
                      uint32_t n_scen, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    const uint32_t m = n * n_scen;
    k_load_primaries<<<(m + 255) / 256, 256, 0, s>>>(q, v, spot_ids, h0, n, n_scen);
    return cudaGetLastError();
}

/// The wave kernel in the launch shapes the tuner chooses from: (threads per block, minimum
/// resident blocks per SM).  The register budget each shape implies is what differs.  Mode 0
/// (DIRECT ROIs, simple scorer callbacks) comes in every shape; the other modes in 128 x 5.
template<int kBlock, int kMinBlocks, int kMode, bool kSplit>
__global__ void __launch_bounds__(kBlock, kMinBlocks)
k_wave(const __grid_constant__ WaveParams P) {
    wave_body<kMode, kSplit>(P);
}

constexpr int kPostBlock = 128;

template<int kMode>
__global__ void __launch_bounds__(kPostBlock)
k_post(const __grid_constant__ WaveParams P) {
    post_body<kMode>(P);
}

int
wave_smem_bytes(const WaveParams& p) {
    return (int) sizeof(Tables) + p.smem_edge_floats * (int) sizeof(float);
}

int
wave_edge_floats(const ChildDev* c, int n) {
    int f = 0;
    for (int i = 0; i < n; ++i) {
        const int need = c[i].nx + c[i].ny + c[i].nz + 3;
        if (f + need > 3 * 2048 + 12) break;
        f += need;
    }
    return (f + 3) & ~3;
}

/// One wave.  With kSplit: the record count of the post-step kernel cleared, the wave kernel, then
/// the post-step kernel over the tracks the wave stopped at nuclear interactions (a grid-stride
/// loop over a count it reads on the device).  Without: the wave kernel alone.
template<int B, int M, int K, bool S>
static cudaError_t
launch_variant(const WaveParams& p, int grid, cudaStream_t s) {
    const int   smem = wave_smem_bytes(p);
    cudaError_t e    = cudaFuncSetAttribute(k_wave<B, M, K, S>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if constexpr (S) {
        if (e == cudaSuccess) e = cudaMemsetAsync(p.n_def, 0, sizeof(uint32_t), s);
    }
    if (e != cudaSuccess) {
        (void) cudaGetLastError();   // the failed call's error is returned here, not left for the next launch
        return e;
    }
    k_wave<B, M, K, S><<<grid, B, smem, s>>>(p);
    if constexpr (S) k_post<K><<<grid, kPostBlock, 0, s>>>(p);
    return cudaGetLastError();
}

// ------------------------------------------------------------------------------------------
// The queue sorted by energy bin before a wave: a counting sort on 1 MeV bins of the entries'
// kinetic energy, highest first, through a queue-sized scratch and back.  Primaries that have not
// taken a step yet form a class of their own, placed after the sorted tracks: they arrive grouped
// (one spot's histories, one energy, neighbouring voxels) and keep that grouping, which
// interleaving them with other spots of the same energy would break.  Protons are the only
// transported particle type (moqui stacks only protons), so the type key is constant.  Each
// kernel reads the entry count on the device and returns at once below sort_min, so the sort can
// sit in a captured graph.  A warp claims one range per distinct class (one atomic each), so
// entries of one class keep their order within a warp.
// ------------------------------------------------------------------------------------------
constexpr int kFreshPrimaryClass = kSortBins - 1;

__device__ inline int
sort_class(const Queue& q, uint32_t i) {
    if ((q.meta[i] & kMetaPrimary) && q.ctr[i] == 0u) return kFreshPrimaryClass;
    const int b = (int) q.ke[i];
    return b < 0 ? 0 : (b >= kFreshPrimaryClass ? kFreshPrimaryClass - 1 : b);
}

__global__ void
k_sort_count(Queue q, const uint32_t* __restrict__ n_in, uint32_t sort_min, uint32_t* __restrict__ bins) {
    __shared__ uint32_t h[kSortBins];
    const uint32_t n = min(*n_in, q.capacity);
    if (n < sort_min) return;
    for (int i = threadIdx.x; i < kSortBins; i += blockDim.x) h[i] = 0;
    __syncthreads();
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        atomicAdd(&h[sort_class(q, i)], 1u);
    __syncthreads();
    for (int i = threadIdx.x; i < kSortBins; i += blockDim.x)
        if (h[i]) atomicAdd(&bins[i], h[i]);
}

/// Counts -> cursors (highest energy bin first, fresh primaries last), and the counts zeroed for
/// the next sort.
__global__ void
k_sort_scan(const uint32_t* __restrict__ n_in, uint32_t capacity, uint32_t sort_min, uint32_t* __restrict__ bins) {
    __shared__ uint32_t c[kSortBins];
    if (min(*n_in, capacity) < sort_min) return;
    for (int i = threadIdx.x; i < kSortBins; i += blockDim.x) {
        c[i]    = bins[i];
        bins[i] = 0;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t acc = 0;
        for (int i = kFreshPrimaryClass - 1; i >= 0; --i) {
            bins[kSortBins + i] = acc;
            acc += c[i];
        }
        bins[kSortBins + kFreshPrimaryClass] = acc;
    }
}

__device__ inline void
copy_entry(const Queue& from, uint32_t i, const Queue& to, uint32_t j) {
    to.ke[j] = from.ke[i]; to.px[j] = from.px[i]; to.py[j] = from.py[i]; to.pz[j] = from.pz[i];
    to.dx[j] = from.dx[i]; to.dy[j] = from.dy[i]; to.dz[j] = from.dz[i]; to.dE0[j] = from.dE0[i];
    to.hist[j] = from.hist[i]; to.uid_lo[j] = from.uid_lo[i]; to.uid_hi[j] = from.uid_hi[i];
    to.ctr[j] = from.ctr[i]; to.meta[j] = from.meta[i]; to.cell[j] = from.cell[i]; to.spot[j] = from.spot[i];
}

__global__ void
k_sort_scatter(Queue q, Queue t, const uint32_t* __restrict__ n_in, uint32_t sort_min, uint32_t* __restrict__ bins) {
    const uint32_t n = min(*n_in, q.capacity);
    if (n < sort_min) return;
    const int lane = threadIdx.x & 31;
    // the loop bound is the same for every thread of a block, so whole warps take each iteration
    for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += gridDim.x * blockDim.x) {
        const uint32_t i     = base + threadIdx.x;
        const bool     valid = i < n;
        const int      b     = valid ? sort_class(q, i) : -1;
        const unsigned peers = __match_any_sync(0xFFFFFFFFu, b);
        const int      lead  = __ffs(peers) - 1;
        uint32_t       pos   = 0;
        if (valid && lane == lead) pos = atomicAdd(&bins[kSortBins + b], (uint32_t) __popc(peers));
        pos = __shfl_sync(0xFFFFFFFFu, pos, lead);
        if (valid) copy_entry(q, i, t, pos + (uint32_t) __popc(peers & ((1u << lane) - 1u)));
    }
}

__global__ void
k_sort_copy_back(Queue q, Queue t, const uint32_t* __restrict__ n_in, uint32_t sort_min) {
    const uint32_t n = min(*n_in, q.capacity);
    if (n < sort_min) return;
    for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) copy_entry(t, j, q, j);
}

static cudaError_t
launch_sort(const WaveParams& p, int grid, cudaStream_t s) {
    k_sort_count<<<grid, 256, 0, s>>>(p.in, p.n_in, p.sort_min, p.sort_bins);
    k_sort_scan<<<1, 256, 0, s>>>(p.n_in, p.in.capacity, p.sort_min, p.sort_bins);
    k_sort_scatter<<<grid, 256, 0, s>>>(p.in, p.sort_tmp, p.n_in, p.sort_min, p.sort_bins);
    k_sort_copy_back<<<grid, 256, 0, s>>>(p.in, p.sort_tmp, p.n_in, p.sort_min);
    return cudaGetLastError();
}

/// Instances: the split form in every launch shape of the common modes and in 128 x 5 for the
/// others; the inline form in the two leading shapes of the common modes (one dose-like scorer,
/// DIRECT ROIs) and in 128 x 5 for the FP64 callbacks (dose to medium, LET) and for Dij runs with
/// DIRECT ROIs (tps_env's Dij runs are one spot per call: small runs) and for the dose scorer with the
/// statistics pair (per-spot runs with statistical stopping).  A request for an inline
/// instance that is not compiled runs the split one (the results are the same) when the caller
/// gave a record array.
cudaError_t
launch_wave(const WaveParams& p, int grid, int block, int blocks_per_sm, cudaStream_t s) {
    const int grid5 = grid / (blocks_per_sm > 0 ? blocks_per_sm : 1) * 5;
    if (p.sort_bins) {
        const cudaError_t e = launch_sort(p, grid5, s);
        if (e != cudaSuccess) return e;
    }
    if (!p.split && (p.kernel_mode == 0 || p.kernel_mode == kModeSingle)) {
        const bool wide = block != 128;
        if (p.kernel_mode == kModeSingle)
            return wide ? launch_variant<256, 2, kModeSingle, false>(p, grid, s)
                        : launch_variant<128, 5, kModeSingle, false>(p, grid5, s);
        return wide ? launch_variant<256, 2, 0, false>(p, grid, s) : launch_variant<128, 5, 0, false>(p, grid5, s);
    }
    if (!p.split && p.kernel_mode == kModeFull) return launch_variant<128, 5, kModeFull, false>(p, grid5, s);
    if (!p.split && p.kernel_mode == kModeDij) return launch_variant<128, 5, kModeDij, false>(p, grid5, s);
    if (!p.split && p.kernel_mode == kModeStat) return launch_variant<128, 5, kModeStat, false>(p, grid5, s);
    if (p.kernel_mode == kModeStat && p.def && p.n_def) return launch_variant<128, 5, kModeStat, true>(p, grid5, s);
    if (!p.def || !p.n_def) return cudaErrorInvalidValue;   // the split form needs its record array
    switch (p.kernel_mode) {
    case 0: break;
    case kModeSingle:
        if (block == 128) {
            if (blocks_per_sm >= 6) return launch_variant<128, 6, kModeSingle, true>(p, grid, s);
            if (blocks_per_sm == 5) return launch_variant<128, 5, kModeSingle, true>(p, grid, s);
            return launch_variant<128, 4, kModeSingle, true>(p, grid, s);
        }
        return launch_variant<256, 2, kModeSingle, true>(p, grid, s);
    case kModeFull: return launch_variant<128, 5, kModeFull, true>(p, grid5, s);
    case kModeRoi: return launch_variant<128, 5, kModeRoi, true>(p, grid5, s);
    case kModeDij: return launch_variant<128, 5, kModeDij, true>(p, grid5, s);   // Dij (+ dose-like), DIRECT ROIs
    case kModeFull | kModeRoi: return launch_variant<128, 5, kModeFull | kModeRoi, true>(p, grid5, s);
    default: return launch_variant<128, 5, kModeAll, true>(p, grid5, s);   // any mode with Dij
    }
    if (block == 128) {
        if (blocks_per_sm >= 6) return launch_variant<128, 6, 0, true>(p, grid, s);
        if (blocks_per_sm == 5) return launch_variant<128, 5, 0, true>(p, grid, s);
        return launch_variant<128, 4, 0, true>(p, grid, s);
    }
    return launch_variant<256, 2, 0, true>(p, grid, s);
}

// ------------------------------------------------------------------------------------------
// HU -> density (patient_material_t::hu_to_density, mqi_patient_materials.hpp:514-542), then
// the DensityScaling factor (mqi_tps_env.hpp:766-769).  The piecewise line is evaluated in
// double with explicit round-to-nearest operations, as the reference's host code does, so the
// result is bit-identical.
// ------------------------------------------------------------------------------------------
__global__ void
k_hu_to_density(const float* __restrict__ corr, const int16_t* __restrict__ hu, float* __restrict__ rho,
                uint64_t n, float scale) {
    for (uint64_t i = blockIdx.x * (uint64_t) blockDim.x + threadIdx.x; i < n; i += (uint64_t) gridDim.x * blockDim.x) {
        int h = hu[i];
        if (h < -1000) h = -1000;
        else if (h > 2995) h = 2995;
        double r;
        const double hd = (double) h;
        if (h < -98) r = __dadd_rn(0.00121, __dmul_rn(0.001029700665188, __dadd_rn(1000.0, hd)));
        else if (h < 15) r = __dadd_rn(1.018, __dmul_rn(0.000893, hd));
        else if (h < 23) r = 1.03;
        else if (h < 101) r = __dadd_rn(1.003, __dmul_rn(0.001169, hd));
        else if (h < 2001) r = __dadd_rn(1.017, __dmul_rn(0.000592, hd));
        else if (h < 2995) r = __dadd_rn(2.201, __dmul_rn(0.0005, __dadd_rn(-2000.0, hd)));
        else r = 4.54;
        float f = (float) r;
        f       = __fmul_rn(f, corr[h + 1000]);
        f       = (float) __ddiv_rn((double) f, 1000.0);
        rho[i]  = __fmul_rn(f, scale);
    }
}

cudaError_t
launch_hu_to_density(const float* corr, const int16_t* hu, float* rho, uint64_t n, float scale, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    const uint64_t blocks = (n + 255) / 256;
    k_hu_to_density<<<(unsigned) (blocks < 152 * 64 ? blocks : 152 * 64), 256, 0, s>>>(corr, hu, rho, n, scale);
    return cudaGetLastError();
}

// ------------------------------------------------------------------------------------------
// Ray walk: the transport's child entry and voxel loop (mqi_transport.hpp:161-233) with the
// physics step replaced by "advance to the voxel exit".  One thread per ray; ray r writes its
// entries at [r * max_steps, ...) and its count to counts[r].
// ------------------------------------------------------------------------------------------
__global__ void
k_trace_rays(const __grid_constant__ ChildDev c, const float* __restrict__ rays, uint64_t n_rays, uint32_t max_steps,
             uint64_t* __restrict__ cnb, float* __restrict__ dist, int32_t* __restrict__ cells,
             uint32_t* __restrict__ counts) {
    const uint64_t r = blockIdx.x * (uint64_t) blockDim.x + threadIdx.x;
    if (r >= n_rays) return;
    const Grid g = make_grid(c, nullptr, nullptr, nullptr);
    float3 p0 = make_float3(rays[6 * r + 0], rays[6 * r + 1], rays[6 * r + 2]);
    float3 d0 = make_float3(rays[6 * r + 3], rays[6 * r + 4], rays[6 * r + 5]);
    to_child(c, p0, d0);
    float3 d1 = d0;
    int3   cell = grid_index(g, p0, d0);
    uint32_t k = 0;
    bool entered = true;
    if (!grid_valid(g, cell)) {
        const float e = grid_entry(g, p0, d0);
        if (e < 0.0f) {
            entered = false;
        } else {
            p0   = advance(p0, d0, e);
            d0   = d1;
            cell = grid_index(g, p0, d0);
        }
    }
    const uint64_t base = r * (uint64_t) max_steps;
    while (entered && grid_valid(g, cell) && k < max_steps) {
        const uint32_t id  = grid_cnb(g, cell);
        const float    d2b = grid_exit(g, p0, d0, cell);
        cnb[base + k]           = id;
        dist[base + k]          = d2b;
        cells[3 * (base + k)]     = cell.x;
        cells[3 * (base + k) + 1] = cell.y;
        cells[3 * (base + k) + 2] = cell.z;
        ++k;
        if (d2b < 0.0f) break;
        const float3 p1 = advance(p0, d0, d2b);
        grid_step_index(g, p1, d1, cell);
        p0 = p1;
        d0 = d1;
    }
    counts[r] = k;
}

cudaError_t
launch_trace_rays(const ChildDev& c, const float* rays, uint64_t n_rays, uint32_t max_steps, uint64_t* cnb,
                  float* dist, int32_t* cells, uint32_t* counts, cudaStream_t s) {
    if (n_rays == 0) return cudaSuccess;
    k_trace_rays<<<(unsigned) ((n_rays + 127) / 128), 128, 0, s>>>(c, rays, n_rays, max_steps, cnb, dist, cells, counts);
    return cudaGetLastError();
}

// ------------------------------------------------------------------------------------------
// Physics probe for parity tests: the same device functions the transport calls.
// ------------------------------------------------------------------------------------------
__global__ void
k_eval_physics(const float* __restrict__ tables, const float* __restrict__ e, uint64_t n, float* __restrict__ out) {
    __shared__ __align__(16) Tables T;
    for (int i = threadIdx.x; i < 6 * MQI_TABLE_N; i += blockDim.x) reinterpret_cast<float*>(&T)[i] = tables[i];
    __syncthreads();
    for (uint64_t i = blockIdx.x * (uint64_t) blockDim.x + threadIdx.x; i < n; i += (uint64_t) gridDim.x * blockDim.x) {
        const Rel rel(e[i]);
        float*    o = out + 8 * i;
        o[0] = cs_lookup(T.cs_ion, rel.Ek, 0.1f, 299.6f, 1.0f);
        o[1] = cs_lookup(T.cs_pp, rel.Ek, 0.5f, 300.0f, 1.0f);
        o[2] = cs_lookup(T.cs_poe, rel.Ek, 0.5f, 300.0f, 1.0f);
        o[3] = cs_lookup(T.cs_poi, rel.Ek, 0.5f, 300.0f, 1.0f);
        o[4] = dedx_lookup(T, rel.Ek);
        o[5] = rel.beta_sq;
        o[6] = rel.Te_max;
        o[7] = rel.momentum();
    }
}

// ------------------------------------------------------------------------------------------
// Scorer-callback and ROI probes for parity tests: the transport's own device functions on given
// step states and voxels.
// ------------------------------------------------------------------------------------------
__global__ void
k_eval_hits(const __grid_constant__ ChildDev c, const __grid_constant__ CalibDev cal, int dbg, int type,
            const float* __restrict__ steps, const uint32_t* __restrict__ cnb, const int32_t* __restrict__ prim,
            uint64_t n, double* __restrict__ out) {
    const Grid g = make_grid(c, nullptr, nullptr, nullptr);
    for (uint64_t i = blockIdx.x * (uint64_t) blockDim.x + threadIdx.x; i < n; i += (uint64_t) gridDim.x * blockDim.x) {
        const float* st = steps + 9 * i;
        Trk t;
        t.ke0 = st[0];
        t.dE  = st[1];
        t.ldE = st[2];
        t.p0  = make_float3(st[3], st[4], st[5]);
        t.p1  = make_float3(st[6], st[7], st[8]);
        t.primary = prim[i] != 0;
        const uint32_t v   = cnb[i];
        const uint32_t nxy = (uint32_t) g.nx * (uint32_t) g.ny;
        const int3     cell = make_int3((int) (v % nxy % (uint32_t) g.nx), (int) (v % nxy / (uint32_t) g.nx), (int) (v / nxy));
        const float rho = g.rho[v];
        const float vol = grid_volume(g, cell);
        // dose_to_water of the step exactly as score_step forms it
        const float spr    = spr_of(cal, rho, t.ke0, dbg != 0);
        const float dose_w = (rho < 1.0e-7f) ? 0.0f : (t.dE + t.ldE) * 1.60218e-10f / (vol * rho * spr);
        out[i]             = compute_hit(type, t, rho, vol, dose_w);
    }
}

__global__ void
k_eval_roi(const __grid_constant__ ScorerDev s, const uint32_t* __restrict__ vox, uint64_t n, int32_t* __restrict__ idx,
           int32_t* __restrict__ mask) {
    for (uint64_t i = blockIdx.x * (uint64_t) blockDim.x + threadIdx.x; i < n; i += (uint64_t) gridDim.x * blockDim.x) {
        idx[i]  = roi_idx(s, vox[i]);
        mask[i] = roi_mask_idx(s, vox[i]);
    }
}

cudaError_t
launch_eval_hits(const ChildDev& c, const CalibDev& cal, int dbg, int type, const float* steps, const uint32_t* cnb,
                 const int32_t* prim, uint64_t n, double* out, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    k_eval_hits<<<(unsigned) ((n + 127) / 128 < 4096 ? (n + 127) / 128 : 4096), 128, 0, s>>>(c, cal, dbg, type, steps, cnb,
                                                                                            prim, n, out);
    return cudaGetLastError();
}

cudaError_t
launch_eval_roi(const ScorerDev& sc, const uint32_t* vox, uint64_t n, int32_t* idx, int32_t* mask, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    k_eval_roi<<<(unsigned) ((n + 127) / 128 < 4096 ? (n + 127) / 128 : 4096), 128, 0, s>>>(sc, vox, n, idx, mask);
    return cudaGetLastError();
}

cudaError_t
launch_eval_physics(const float* t, const float* e, uint64_t n, float* out, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    k_eval_physics<<<(unsigned) ((n + 255) / 256 < 1024 ? (n + 255) / 256 : 1024), 256, 0, s>>>(t, e, n, out);
    return cudaGetLastError();
}

}   // namespace mqi_gpu

namespace mqi_gpu
{

// ------------------------------------------------------------------------------------------
// Device-side source sampling from a spot plan.  The reference samples every vertex on the host
// with std::default_random_engine (beamlet::operator(), moqui/base/mqi_beamlet.hpp:80-90;
// phsp_6d, moqui/base/distributions/mqi_phsp6d.hpp:61-79; norm_1d,
// moqui/base/distributions/mqi_norm_1d.hpp) and uploads them (upload_vertices).  Here each
// primary is drawn on the device from its own Philox stream (history index, uid all-ones) with
// the same phase-space law, so a plan of any size needs no host vertex array and no H2D copy.
// ------------------------------------------------------------------------------------------
__device__ inline uint32_t
sample_spot_vertex(const mqi_spot* __restrict__ spots, const uint64_t* __restrict__ cum, uint32_t n_spots, uint64_t h,
                   uint32_t k0, uint32_t k1, float3& pos, float3& dir, float& ke) {
    // spot s with cum[s] <= h < cum[s+1]
    uint32_t lo = 0, hi = n_spots;
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (cum[mid] <= h) lo = mid; else hi = mid;
    }
    const mqi_spot& S = spots[lo];
    // six normals (Box-Muller) from two Philox blocks of the history's source stream
    const u32x4 b0 = philox4x32_10(u32x4{ 0u, (uint32_t) h, 0xFFFFFFFFu, 0xFFFFFFFFu }, k0, k1);
    const u32x4 b1 = philox4x32_10(u32x4{ 1u, (uint32_t) h, 0xFFFFFFFFu, 0xFFFFFFFFu }, k0, k1);
    float z[6];
    const uint32_t w[6] = { b0.x, b0.y, b0.z, b0.w, b1.x, b1.y };
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const float r = sqrtf(-2.0f * logf(u01(w[2 * k])));
        float       sn, cs;
        sincospif(2.0f * u01(w[2 * k + 1]), &sn, &cs);
        z[2 * k]     = r * cs;
        z[2 * k + 1] = r * sn;
    }
    const float Ux = z[0], Vx = z[1], Uy = z[2], Vy = z[3], Uz = z[4], Ue = z[5];
    // phsp_6d: position, then direction correlated with position (mqi_phsp6d.hpp:66-78)
    const float x  = S.mean[0] + S.sigma[0] * Ux;
    const float y  = S.mean[1] + S.sigma[1] * Uy;
    const float zz = S.mean[2] + S.sigma[2] * Uz;
    const float xp = S.mean[3] + S.sigma[3] * (S.corr[0] * Ux + Vx * sqrtf(1.0f - S.corr[0] * S.corr[0]));
    const float yp = S.mean[4] + S.sigma[4] * (S.corr[1] * Uy + Vy * sqrtf(1.0f - S.corr[1] * S.corr[1]));
    const float zp = -sqrtf(fmaxf(1.0f - xp * xp - yp * yp, 0.0f));
    // beamlet: pos = R p + T, dir = R d (mqi_beamlet.hpp:80-90)
    const float* R = S.rot;
    pos = make_float3(R[0] * x + R[1] * y + R[2] * zz + S.trans[0], R[3] * x + R[4] * y + R[5] * zz + S.trans[1],
                      R[6] * x + R[7] * y + R[8] * zz + S.trans[2]);
    dir = make_float3(R[0] * xp + R[1] * yp + R[2] * zp, R[3] * xp + R[4] * yp + R[5] * zp,
                      R[6] * xp + R[7] * yp + R[8] * zp);
    ke  = S.energy + S.energy_sigma * Ue;
    return lo;
}

__device__ inline void
write_sampled_entry(const Queue& q, uint32_t i, const mqi_spot* __restrict__ spots, const uint64_t* __restrict__ cum,
                    uint32_t n_spots, uint64_t h, uint32_t scen, uint32_t k0, uint32_t k1) {
    float3 p, d;
    float  ke;
    const uint32_t s = sample_spot_vertex(spots, cum, n_spots, h, k0, k1, p, d, ke);
    q.px[i] = p.x; q.py[i] = p.y; q.pz[i] = p.z;
    q.dx[i] = d.x; q.dy[i] = d.y; q.dz[i] = d.z;
    q.ke[i]     = ke;
    q.dE0[i]    = 0.0f;
    q.hist[i]   = (uint32_t) h;
    q.uid_lo[i] = 0u;
    q.uid_hi[i] = 0u;
    q.ctr[i]    = 0u;
    q.meta[i]   = kMetaPrimary;
    q.cell[i]   = 0;
    q.spot[i]   = (s & kSpotMask) | (scen << kScenShift);
}

__global__ void
k_sample_primaries(Queue q, const mqi_spot* __restrict__ spots, const uint64_t* __restrict__ cum, uint32_t n_spots,
                   uint64_t h0, uint32_t n, uint32_t n_scen, uint32_t k0, uint32_t k1) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n * n_scen) return;
    write_sampled_entry(q, i, spots, cum, n_spots, h0 + i / n_scen, i % n_scen, k0, k1);
}

__global__ void
k_sample_topup(Queue q, const TopUp* __restrict__ tu, const mqi_spot* __restrict__ spots,
               const uint64_t* __restrict__ cum, uint32_t n_spots, uint32_t k0, uint32_t k1) {
    const uint32_t n = tu->count, S = tu->n_scen, dst = tu->dst;
    const uint64_t base = tu->base;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        write_sampled_entry(q, dst + i, spots, cum, n_spots, base + i / S, i % S, k0, k1);
}

__global__ void
k_sample_vertices(mqi_vertex* __restrict__ out, uint32_t* __restrict__ spot_out, const mqi_spot* __restrict__ spots,
                  const uint64_t* __restrict__ cum, uint32_t n_spots, uint64_t h0, uint32_t n, uint32_t k0, uint32_t k1) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float3 p, d;
    float  ke;
    const uint32_t s = sample_spot_vertex(spots, cum, n_spots, h0 + i, k0, k1, p, d, ke);
    mqi_vertex v;
    v.ke = ke;
    v.pos[0] = p.x; v.pos[1] = p.y; v.pos[2] = p.z;
    v.dir[0] = d.x; v.dir[1] = d.y; v.dir[2] = d.z;
    out[i] = v;
    if (spot_out) spot_out[i] = s;
}

cudaError_t
launch_sample_primaries(const Queue& q, const mqi_spot* spots, const uint64_t* cum, uint32_t n_spots, uint64_t h0,
                        uint32_t n, uint32_t n_scen, uint32_t k0, uint32_t k1, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    const uint32_t m = n * n_scen;
    k_sample_primaries<<<(m + 127) / 128, 128, 0, s>>>(q, spots, cum, n_spots, h0, n, n_scen, k0, k1);
    return cudaGetLastError();
}

cudaError_t
launch_sample_vertices(mqi_vertex* out, uint32_t* spot_out, const mqi_spot* spots, const uint64_t* cum, uint32_t n_spots,
                       uint64_t h0, uint32_t n, uint32_t k0, uint32_t k1, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    k_sample_vertices<<<(n + 127) / 128, 128, 0, s>>>(out, spot_out, spots, cum, n_spots, h0, n, k0, k1);
    return cudaGetLastError();
}

cudaError_t
launch_topup(TopUp* tu, uint32_t* n_in, const uint32_t* error_flag, cudaStream_t s) {
    k_topup<<<1, 1, 0, s>>>(tu, n_in, error_flag);
    return cudaGetLastError();
}

cudaError_t
launch_load_topup(const Queue& q, const TopUp* tu, const mqi_vertex* v, const uint32_t* spot_ids, int sms,
                  cudaStream_t s) {
    k_load_topup<<<sms * 8, 256, 0, s>>>(q, tu, v, spot_ids);
    return cudaGetLastError();
}

cudaError_t
launch_sample_topup(const Queue& q, const TopUp* tu, const mqi_spot* spots, const uint64_t* cum, uint32_t n_spots,
                    uint32_t k0, uint32_t k1, int sms, cudaStream_t s) {
    k_sample_topup<<<sms * 8, 128, 0, s>>>(q, tu, spots, cum, n_spots, k0, k1);
    return cudaGetLastError();
}

}   // namespace mqi_gpu
