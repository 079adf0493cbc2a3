// Device-side physics, geometry and random numbers of the GB300 proton transport.
//
// Every function here restates one piece of moqui's condensed-history proton transport for a
// single FP32 track held in registers; the reference file:line each follows is cited beside it.
// The kernels in mqi_kernels.cu drive these functions from an event queue instead of the
// reference's per-thread LIFO stack.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "mqi_gpu.h"
#include "mqi_tables.h"

namespace mqi_gpu
{

// ------------------------------------------------------------------------------------------
// Constants (moqui/base/mqi_physics_constants.hpp:14-38, mqi_physics_list.hpp:24-28,
// mqi_interaction.hpp:24-30, mqi_math.hpp:17-23, mqi_fippel_physics.hpp:20-21)
// ------------------------------------------------------------------------------------------
constexpr float kMp            = 938.272046f;
constexpr float kMe            = 0.510998928f;
constexpr float kMo            = 14903.3460795634f;
constexpr float kWaterDensity  = 0.001f;      // g/mm^3
constexpr float kX0Water       = 360.863f;    // mm
constexpr float kTpCut         = 0.5f;        // MeV, proton tracking cut
constexpr float kTcutDebug     = 0.08511f;    // MeV, delta-ray cut with __PHYSICS_DEBUG__
constexpr float kTcutRelease   = 0.0815f;     // MeV, delta-ray cut otherwise
constexpr float kTeStragCap    = 0.08511f;    // MeV, Te cap in the straggling variance
constexpr float kEs            = 13.9f;       // MeV, MCS constant
constexpr float kNearZero      = 1e-7f;
constexpr float kGeoTol        = 1e-3f;
constexpr float kMaxStep       = 1.0f;        // mm in water
constexpr float kMevToGyMm3    = 1.60218e-10f;
constexpr float kPi            = 3.14159265358979323846f;

// dedx_term0 = 2 pi re^2 me c^2 * n_e(water) (mqi_physics_constants.hpp:29-30), evaluated in
// float exactly as the reference's physics_constants<float> does.
__host__ __device__ inline float
dedx_term0() {
    const float re     = 2.8179403262e-12f;
    const float re_sq  = re * re;
    const float two_pi = (float) (2.0 * 3.14159265358979323846);
    const float t      = (float) ((double) two_pi * (double) re_sq);
    const float t2     = t * kMe;
    const float cm3    = 1000.0f;
    return (float) ((double) t2 * 3.3428e+23 / (double) cm3);
}

// ------------------------------------------------------------------------------------------
// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as easy as 1, 2, 3",
// SC'11), written from the paper: 10 rounds of the 4x32 S-box with the published multipliers
// and Weyl key increments.  It replaces the reference's per-history cuRAND XORWOW state
// (mqi_transport.hpp:148): a track's stream is a pure function of (seed, history, track uid,
// counter), so no state initialisation exists and the result is independent of the order in
// which the queue processes tracks.
// ------------------------------------------------------------------------------------------
struct u32x4 {
    uint32_t x, y, z, w;
};

__host__ __device__ inline void
mulhilo32(uint32_t a, uint32_t b, uint32_t& hi, uint32_t& lo) {
    const uint64_t p = (uint64_t) a * (uint64_t) b;
    hi               = (uint32_t) (p >> 32);
    lo               = (uint32_t) p;
}

__host__ __device__ inline u32x4
philox4x32_10(u32x4 c, uint32_t k0, uint32_t k1) {
    const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u;
    const uint32_t W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        uint32_t hi0, lo0, hi1, lo1;
        mulhilo32(M0, c.x, hi0, lo0);
        mulhilo32(M1, c.z, hi1, lo1);
        c  = u32x4{ hi1 ^ c.y ^ k0, lo1, hi0 ^ c.w ^ k1, lo0 };
        k0 += W0;
        k1 += W1;
    }
    return c;
}

/// u in (0, 1): 24 significant bits, never 0 or 1, so logs of u and 1-u are finite.
__host__ __device__ inline float
u01(uint32_t x) {
    return ((float) (x >> 8) + 0.5f) * (1.0f / 16777216.0f);
}

/// Splitmix64 finaliser; derives a daughter's uid from its parent's uid and push index.
__host__ __device__ inline uint64_t
mix64(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

__host__ __device__ inline uint64_t
daughter_uid(uint64_t parent_uid, uint32_t push_index) {
    return mix64(parent_uid * 0x9E3779B97F4A7C15ull + (uint64_t) (push_index + 1u));
}

/// One Philox block, out of line: the hot step draws its first block inline (begin_step) and
/// only the rare post-step processes need more, so one shared copy of the ten rounds keeps the
/// kernel's instruction footprint small.
static __device__ __noinline__ u32x4
philox_block(uint32_t ctr, uint32_t hist, uint32_t lo, uint32_t hi, uint32_t k0, uint32_t k1) {
    return philox4x32_10(u32x4{ ctr, hist, lo, hi }, k0, k1);
}

/// The random stream of one track.  Each physics step starts on a fresh 4-word block
/// (`begin_step`), so the words a step consumes never depend on where a queue slice ended.  The
/// step's second block (counter + 1) is computed with the first, as a second independent chain:
/// a step that interacts needs a fifth word, and with ~15% of the steps interacting nearly every
/// warp-step has such a lane, so the block was computed anyway, at a fraction of the lanes and
/// behind a call (eagerly: +1% on the slab phantom and the CT plan).  The words are the same.
struct Rng {
    uint32_t k0, k1;     // key: run seed
    uint32_t hist;       // history index
    uint32_t uid_lo, uid_hi;
    uint32_t ctr;        // next block counter
    u32x4    blk;
    u32x4    blk2;       // the step's second block, while has2
    int      pos;        // next word of blk (4 = exhausted)
    bool     has2;

    /// Start a step on a fresh block (generated here, inline).
    __device__ inline void
    begin_step() {
        blk  = philox4x32_10(u32x4{ ctr, hist, uid_lo, uid_hi }, k0, k1);
        blk2 = philox4x32_10(u32x4{ ctr + 1u, hist, uid_lo, uid_hi }, k0, k1);
        ++ctr;
        pos  = 0;
        has2 = true;
    }
    __device__ inline uint32_t
    next() {
        if (pos >= 4) {
            if (has2) {
                blk  = blk2;
                has2 = false;
            } else {
                blk = philox_block(ctr, hist, uid_lo, uid_hi, k0, k1);
            }
            ++ctr;
            pos = 0;
        }
        const uint32_t w = (pos == 0) ? blk.x : (pos == 1) ? blk.y : (pos == 2) ? blk.z : blk.w;
        ++pos;
        return w;
    }
    __device__ inline float
    uniform() {
        return u01(next());
    }
};

// ------------------------------------------------------------------------------------------
// Physics tables staged in shared memory (the reference keeps them in __constant__,
// mqi_p_ionization.hpp:11,74,145; mqi_pp_elastic.hpp:11; mqi_po_elastic.hpp:12;
// mqi_po_inelastic.hpp:11).  Divergent lanes read different energy bins every step, which the
// constant cache serialises; shared memory serves them in one pass.
// ------------------------------------------------------------------------------------------
struct Tables {
    float cs_ion[MQI_TABLE_N];
    float dedx[MQI_TABLE_N];
    float range[MQI_TABLE_N];
    float cs_pp[MQI_TABLE_N];
    float cs_poe[MQI_TABLE_N];
    float cs_poi[MQI_TABLE_N];
};

/// intpl1d (mqi_math.hpp:26-30)
__host__ __device__ inline float
intpl1d(float x, float x0, float x1, float y0, float y1) {
    return (x1 == x0) ? y0 : y0 + (x - x0) * (y1 - y0) / (x1 - x0);
}

/// intpl1d at a node of the 0.1 MeV + 0.5 MeV * i energy grid: there x1 - x0 is exactly 0.5 in FP32
/// except at the four nodes whose interval crosses 2, 8, 32 or 128 MeV (checked exhaustively), and
/// dividing by exactly 0.5 is multiplying by 2, so the division runs only at those four.  The
/// result is intpl1d's, bit for bit.
__host__ __device__ inline float
intpl1d_grid(float x, float x0, float x1, float y0, float y1) {
    const float w   = x1 - x0;
    const float num = (x - x0) * (y1 - y0);
    float       q;
    if (w == 0.5f) q = num * 2.0f;
    else q = num / w;
    return y0 + q;
}

/// relativistic_quantities (mqi_relativistic_quantities.hpp:24-40), FP32.
struct Rel {
    float Ek, Et, Et_sq, gamma, gamma_sq, beta_sq, Te_max;
    __host__ __device__ inline explicit Rel(float ek) {
        const float MeMp    = kMe / kMp;
        const float MeMp_sq = MeMp * MeMp;
        Ek                  = ek;
        Et                  = ek + kMp;
        Et_sq               = Et * Et;
        gamma               = Et / kMp;
        gamma_sq            = gamma * gamma;
        // The reference evaluates 1 - 1/gamma^2 in double (1.0 is a double literal); a float
        // quotient would lose ~1e-3 relative at 0.02 MeV.  r + e*r recovers the quotient to about
        // 2^-46 (e is the exact residual of the rounded reciprocal), and 1 - r is exact.
        const float r       = 1.0f / gamma_sq;
        const float e       = fmaf(-r, gamma_sq, 1.0f);
        beta_sq             = (1.0f - r) - e * r;
        Te_max              = (2.0f * kMe * beta_sq * gamma_sq) / (1.0f + 2.0f * gamma * MeMp + MeMp_sq);
    }
    __host__ __device__ inline float
    momentum() const {
        return sqrtf(Et * Et - kMp * kMp);
    }
};

/// Tabulated cross-section lookup shared by the four processes
/// (mqi_p_ionization.hpp:254-268, mqi_pp_elastic.hpp:221-235, mqi_po_elastic.hpp:243-256,
/// mqi_po_inelastic.hpp:141-155).  The upper node index is clamped to the table; the reference
/// reads one element past the end when Ek sits on the last node.
__device__ inline float
cs_lookup(const float* tab, float Ek, float e_min, float e_max, float rho) {
    float cs = 0.0f;
    if (Ek >= e_min && Ek <= e_max) {
        const int i0 = (int) ((Ek - e_min) / 0.5f);
        const int i1 = min(i0 + 1, MQI_TABLE_N - 1);
        const float x0 = e_min + (float) i0 * 0.5f;
        const float x1 = x0 + 0.5f;
        cs             = intpl1d_grid(Ek, x0, x1, tab[i0], tab[i1]);
    }
    return cs * rho;
}

/// The four macroscopic cross sections at one energy.  p-p, p-O elastic and p-O inelastic share
/// one energy grid (0.5 MeV .. 300 MeV in 0.5 MeV steps), so their node index and interpolation
/// weights are computed once; the arithmetic per table is that of cs_lookup, so the values are
/// identical.
struct CrossSections {
    float ion, pp, poe, poi;
};

__device__ inline CrossSections
cross_sections(const Tables& T, float Ek, float rho) {
    CrossSections c;
    c.ion = cs_lookup(T.cs_ion, Ek, 0.1f, 299.6f, rho);
    c.pp = c.poe = c.poi = 0.0f;
    if (Ek >= 0.5f && Ek <= 300.0f) {
        const int   i0 = (int) ((Ek - 0.5f) / 0.5f);
        const int   i1 = min(i0 + 1, MQI_TABLE_N - 1);
        const float x0 = 0.5f + (float) i0 * 0.5f;
        const float x1 = x0 + 0.5f;
        // On this grid x1 - x0 is exactly 0.5 for every node (checked exhaustively in FP32), so
        // intpl1d's division by it is the exact scaling by 2 written here: identical results.
        (void) x1;
        const float dx = Ek - x0;
        c.pp  = T.cs_pp[i0] + dx * (T.cs_pp[i1] - T.cs_pp[i0]) * 2.0f;
        c.poe = T.cs_poe[i0] + dx * (T.cs_poe[i1] - T.cs_poe[i0]) * 2.0f;
        c.poi = T.cs_poi[i0] + dx * (T.cs_poi[i1] - T.cs_poi[i0]) * 2.0f;
    }
    c.pp *= rho;
    c.poe *= rho;
    c.poi *= rho;
    return c;
}

/// p_ionization_tabulated::dEdx (mqi_p_ionization.hpp:271-286); returns a negative number.
__device__ inline float
dedx_lookup(const Tables& T, float Ek) {
    float pw = 0.0f;
    if (Ek >= 0.1f && Ek <= 299.6f) {
        const int i0 = (int) ((Ek - 0.1f) / 0.5f);
        const int i1 = min(i0 + 1, MQI_TABLE_N - 1);
        const float x0 = 0.1f + (float) i0 * 0.5f;
        const float x1 = x0 + 0.5f;
        pw             = intpl1d_grid(Ek, x0, x1, T.dedx[i0], T.dedx[i1]);
    } else if (Ek < 0.1f && Ek > 0.0f) {
        pw = T.dedx[0];
    }
    return -1.0f * pw;
}

// ------------------------------------------------------------------------------------------
// Calibration: spr_default / radiation_length_default (materials/mqi_patient_materials.hpp:414-473)
// ------------------------------------------------------------------------------------------
__host__ __device__ inline float
spr_default(float rho_mass, float Ek, bool physics_debug) {
    const float d = rho_mass * 1000.0f;
    if (physics_debug && fabsf(d - 1.0f) < 1e-3f) return 1.0f;
    if (d <= 0.26f) {
        if (d < 0.0012f) return 0.0f;
        return intpl1d(d, 0.0012f, 0.26f, 0.8815f, 0.9925f);
    }
    float rsp = 1.0123f - 3.386e-5f * Ek;
    rsp += 0.291f * (1.0f + powf(Ek, -0.3421f)) * (powf(d, -0.7f) - 1.0f);
    if (d >= 0.9f) return rsp;
    return intpl1d(d, 0.26f, 0.9f, 0.9925f, rsp);
}

__host__ __device__ inline float
radiation_length_default(float rho_mass, bool physics_debug) {
    const float d = rho_mass * 1000.0f;
    if (physics_debug && fabsf(d - 1.0f) < 1e-3f) return kX0Water;
    float f = 0.0f;
    if (d <= 0.26f) {
        f = 0.9857f + 0.0085f * d;
    } else if (d <= 0.9f) {
        f = 1.0446f - 0.2180f * d;
    } else {
        f = 1.19f + 0.44f * logf(d - 0.44f);
    }
    return (kWaterDensity * kX0Water) / (d * 0.001f * f);
}

// ------------------------------------------------------------------------------------------
// Geometry (moqui/base/mqi_grid3d.hpp).  All arithmetic that decides a voxel index is written
// with round-to-nearest intrinsics so the compiler cannot contract it into FMAs: the voxel
// index sequence along a ray must be bit-identical to the reference's FP32 host code.
// ------------------------------------------------------------------------------------------
struct Grid {
    int          nx, ny, nz;
    const float* xe;   // nx+1 edges (shared or global memory)
    const float* ye;
    const float* ze;
    const float* rho;  // g/mm^3, x fastest
    float        rho_scale;  // density scale of the track's scenario (1: none)
};

__device__ inline float fadd(float a, float b) { return __fadd_rn(a, b); }
__device__ inline float fsub(float a, float b) { return __fsub_rn(a, b); }
__device__ inline float fmul(float a, float b) { return __fmul_rn(a, b); }
__device__ inline float fdiv(float a, float b) { return __fdiv_rn(a, b); }

/// mat3x3 * vec3 (mqi_matrix.hpp operator*(vec3)), each row as ((a*x + b*y) + c*z).
__device__ inline float3
matvec(const float* m, float3 v) {
    return make_float3(fadd(fadd(fmul(m[0], v.x), fmul(m[1], v.y)), fmul(m[2], v.z)),
                       fadd(fadd(fmul(m[3], v.x), fmul(m[4], v.y)), fmul(m[5], v.z)),
                       fadd(fadd(fmul(m[6], v.x), fmul(m[7], v.y)), fmul(m[8], v.z)));
}

/// vec3::normalize (mqi_vec.hpp:197-205)
__device__ inline float3
normalize3(float3 v) {
    const float n = __fsqrt_rn(fadd(fadd(fmul(v.x, v.x), fmul(v.y, v.y)), fmul(v.z, v.z)));
    return make_float3(fdiv(v.x, n), fdiv(v.y, n), fdiv(v.z, n));
}

/// p + d * len (track_t::update_post_vertex_position, mqi_track.hpp:176-180)
__device__ inline float3
advance(float3 p, float3 d, float len) {
    return make_float3(fadd(p.x, fmul(d.x, len)), fadd(p.y, fmul(d.y, len)), fadd(p.z, fmul(d.z, len)));
}

/// One axis of grid3d::index(p, dir) (mqi_grid3d.hpp:745-844).  The reference scans the edges
/// linearly and returns at the first of: p within tolerance of the lower edge, of the upper
/// edge, or strictly inside.  With edges more than two tolerances apart this is the nearest
/// edge's tie rule, else the containing interval, found here by bisection.
__device__ inline int
index_axis(const float* e, int n, float p, float dir) {
    // largest k with e[k] <= p, clamped to [0, n]
    int lo = 0, hi = n;
    if (p < e[0]) {
        lo = 0;
    } else if (p >= e[n]) {
        lo = n;
    } else {
        while (hi - lo > 1) {
            const int mid = (lo + hi) >> 1;
            if (e[mid] <= p) lo = mid; else hi = mid;
        }
    }
    // nearest edge among e[lo], e[lo+1]
    int m = lo;
    if (lo + 1 <= n && fabsf(fsub(e[lo + 1], p)) < fabsf(fsub(e[lo], p))) m = lo + 1;
    if (fabsf(fsub(e[m], p)) < kGeoTol) {
        if (m == 0) return (dir < 0.0f) ? -1 : 0;        // first-edge branch at ind = 0
        return (dir > 0.0f) ? m : m - 1;                  // upper-edge branch at ind = m-1
    }
    if (lo < n && fsub(e[lo], p) < 0.0f && fsub(e[lo + 1], p) > 0.0f) return lo;
    return -1;
}

/// index_axis when p may lie in interval k: if p is strictly inside [e[k], e[k+1]] and at least the
/// tolerance away from both edges, index_axis returns k (the bisection lands on k and neither edge
/// ties), so k is returned without the search; otherwise the search runs.
__device__ inline int
index_axis_hint(const float* e, int n, float p, float dir, int k) {
    if (k >= 0 && k < n) {
        const float a = fsub(e[k], p), b = fsub(e[k + 1], p);
        if (a < 0.0f && b > 0.0f && fabsf(a) >= kGeoTol && fabsf(b) >= kGeoTol) return k;
    }
    return index_axis(e, n, p, dir);
}

__device__ inline int3
grid_index(const Grid& g, float3 p, float3 d) {
    return make_int3(index_axis(g.xe, g.nx, p.x, d.x), index_axis(g.ye, g.ny, p.y, d.y),
                     index_axis(g.ze, g.nz, p.z, d.z));
}

__device__ inline bool
grid_valid(const Grid& g, int3 c) {
    return !(c.x < 0 || c.y < 0 || c.z < 0 || c.x >= g.nx || c.y >= g.ny || c.z >= g.nz);
}

__device__ inline uint32_t
grid_cnb(const Grid& g, int3 c) {
    return (uint32_t) c.z * (uint32_t) g.nx * (uint32_t) g.ny + (uint32_t) c.y * (uint32_t) g.nx + (uint32_t) c.x;
}

/// One axis of grid3d::intersect(p, d, idx) (mqi_grid3d.hpp:528-605): the distance to the
/// exit plane of the current voxel on this axis.  A plane the particle already sits on (within
/// tolerance) is skipped by a large sentinel, except the grid's lowest plane; a direction
/// component with square below 1e-7 is zeroed in place.
__device__ inline float
exit_axis(float p, float& d, float v1, float v2, int idx) {
    if (fmul(d, d) > kNearZero) {
        if (d < 0.0f) {
            const float t = fdiv(-fsub(p, v1), d);
            return (fabsf(t) < kGeoTol && idx > 0) ? (1.0f / kGeoTol) : t;
        }
        const float t = fdiv(fsub(v2, p), d);
        return (fabsf(t) < kGeoTol) ? (1.0f / kGeoTol) : t;   // idx < dim always holds here
    }
    d = 0.0f;
    return __int_as_float(0x7f800000);   // +inf
}

/// grid3d::intersect(p, d, idx): distance to the voxel exit, or -1 when none is ahead.
__device__ inline float
grid_exit(const Grid& g, float3 p, float3& d, int3 c) {
    const float tx = exit_axis(p.x, d.x, g.xe[c.x], g.xe[c.x + 1], c.x);
    const float ty = exit_axis(p.y, d.y, g.ye[c.y], g.ye[c.y + 1], c.y);
    const float tz = exit_axis(p.z, d.z, g.ze[c.z], g.ze[c.z + 1], c.z);
    float u;
    if (tx < ty) u = (tx < tz) ? tx : tz;
    else u = (ty < tz) ? ty : tz;
    return (u > 0.0f) ? u : -1.0f;
}

/// grid3d::intersect(p, d) for a ray starting outside the grid (mqi_grid3d.hpp:628-743):
/// returns the entry distance (>= 0) or -1 on a miss.  Zeroes tiny direction components in place.
__device__ inline float
grid_entry(const Grid& g, float3 p, float3& d) {
    const float x0 = g.xe[0], x1 = g.xe[g.nx];
    const float y0 = g.ye[0], y1 = g.ye[g.ny];
    const float z0 = g.ze[0], z1 = g.ze[g.nz];
    if (p.x >= x0 && p.x <= x1 && p.y >= y0 && p.y <= y1 && p.z >= z0 && p.z <= z1) return 0.0f;
    const float inf = __int_as_float(0x7f800000);
    float tminx, tmaxx, tminy, tmaxy, tminz, tmaxz;
    if (fmul(d.x, d.x) > kNearZero) {
        if (d.x > 0.0f) { tminx = fdiv(fsub(x0, p.x), d.x); tmaxx = fdiv(fsub(x1, p.x), d.x); }
        else            { tmaxx = fdiv(fsub(x0, p.x), d.x); tminx = fdiv(fsub(x1, p.x), d.x); }
    } else { d.x = 0.0f; tminx = -inf; tmaxx = inf; }
    if (fmul(d.y, d.y) > kNearZero) {
        if (d.y > 0.0f) { tminy = fdiv(fsub(y0, p.y), d.y); tmaxy = fdiv(fsub(y1, p.y), d.y); }
        else            { tmaxy = fdiv(fsub(y0, p.y), d.y); tminy = fdiv(fsub(y1, p.y), d.y); }
    } else { d.y = 0.0f; tminy = -inf; tmaxy = inf; }
    if (fmul(d.z, d.z) > kNearZero) {
        if (d.z > 0.0f) { tminz = fdiv(fsub(z0, p.z), d.z); tmaxz = fdiv(fsub(z1, p.z), d.z); }
        else            { tmaxz = fdiv(fsub(z0, p.z), d.z); tminz = fdiv(fsub(z1, p.z), d.z); }
    } else { d.z = 0.0f; tminz = -inf; tmaxz = inf; }
    float umin, umax;
    if (tminx > tminy) umin = (tminx > tminz) ? tminx : tminz;
    else umin = (tminy > tminz) ? tminy : tminz;
    if (tmaxx < tmaxy) umax = (tmaxx < tmaxz) ? tmaxx : tmaxz;
    else umax = (tmaxy < tmaxz) ? tmaxy : tmaxz;
    if ((umin < umax || fabsf(fsub(umin, umax)) < kGeoTol) && umin >= 0.0f && umax >= 0.0f) return umin;
    return -1.0f;
}

/// grid3d::index(vtx1, dir1, idx): the +-1 cell update after a step (mqi_grid3d.hpp:846-877).
__device__ inline void
grid_step_index(const Grid& g, float3 p, float3 d, int3& c) {
    if (d.x < 0.0f && (fabsf(fsub(p.x, g.xe[c.x])) < kGeoTol || p.x < g.xe[c.x])) c.x -= 1;
    else if (d.x > 0.0f && (fabsf(fsub(p.x, g.xe[c.x + 1])) < kGeoTol || p.x > g.xe[c.x + 1])) c.x += 1;
    if (d.y < 0.0f && (fabsf(fsub(p.y, g.ye[c.y])) < kGeoTol || p.y < g.ye[c.y])) c.y -= 1;
    else if (d.y > 0.0f && (fabsf(fsub(p.y, g.ye[c.y + 1])) < kGeoTol || p.y > g.ye[c.y + 1])) c.y += 1;
    if (d.z < 0.0f && (fabsf(fsub(p.z, g.ze[c.z])) < kGeoTol || p.z < g.ze[c.z])) c.z -= 1;
    else if (d.z > 0.0f && (fabsf(fsub(p.z, g.ze[c.z + 1])) < kGeoTol || p.z > g.ze[c.z + 1])) c.z += 1;
}

/// grid3d::get_volume(cnb) (mqi_grid3d.hpp:470-478)
__device__ inline float
grid_volume(const Grid& g, int3 c) {
    float v = fsub(g.xe[c.x + 1], g.xe[c.x]);
    v       = fmul(v, fsub(g.ye[c.y + 1], g.ye[c.y]));
    return fmul(v, fsub(g.ze[c.z + 1], g.ze[c.z]));
}

// ------------------------------------------------------------------------------------------
// Direction update: track_t::update_post_vertex_direction (mqi_track.hpp:163-172) with the
// Moller-Hughes alignment of mat3x3(f, t) (mqi_matrix.hpp:88-150), ref vector f = (0,0,1).
// ------------------------------------------------------------------------------------------
__device__ __forceinline__ float3
rotate_dir_inline(float3 t, float th, float ph) {
    // dl = mat3x3(0, th, ph) * (0,0,1): the new direction in the frame whose z axis is t.
    float s1, c1, s2, c2;
    sincosf(th, &s1, &c1);
    sincosf(ph, &s2, &c2);
    const float dx = c2 * s1, dy = s2 * s1, dz = c1;
    const float it = rsqrtf(t.x * t.x + t.y * t.y + t.z * t.z);
    const float tx = t.x * it, ty = t.y * it, c = t.z * it;
    // Moller-Hughes, general case: R = c I + [v]x + h v v^T with v = z x t = (-ty, tx, 0) and
    // h = (1 - c) / (1 - c^2) = 1 / (1 + c):  R dl = c dl + v x dl + h (v . dl) v.
    const float vx = -ty, vy = tx;
    const float h  = 1.0f / (1.0f + c);
    const float vd = vx * dx + vy * dy;
    const float gx = c * dx + vy * dz + h * vd * vx;
    const float gy = c * dy - vx * dz + h * vd * vy;
    const float gz = c * dz + (vx * dy - vy * dx);
    // Moller-Hughes near +-z (|c -+ 1| < 1e-3): the product of the reflections about
    // u = (x - z)/|x - z| and w = (x - t)/|x - t|, x = (1,0,0):
    // R dl = dl - 2 (u.dl) u - 2 (w.dl) w + 4 (u.w)(u.dl) w.
    const float r2 = 0.70710678f;
    float       wx = 1.0f - tx, wy = -ty, wz = -c;
    const float iw = rsqrtf(wx * wx + wy * wy + wz * wz);
    wx *= iw; wy *= iw; wz *= iw;
    const float ud = r2 * (dx - dz);
    const float wd = wx * dx + wy * dy + wz * dz;
    const float uw = r2 * (wx - wz);
    const float k  = 4.0f * uw * ud - 2.0f * wd;
    const float rx = dx - 2.0f * ud * r2 + k * wx;
    const float ry = dy + k * wy;
    const float rz = dz + 2.0f * ud * r2 + k * wz;
    // both forms are evaluated and one selected: lanes of a warp near and away from the beam
    // axis then run one instruction stream
    const bool  refl = fabsf(c - 1.0f) < kGeoTol || fabsf(c + 1.0f) < kGeoTol;
    const float ox = refl ? rx : gx, oy = refl ? ry : gy, oz = refl ? rz : gz;
    const float io = rsqrtf(ox * ox + oy * oy + oz * oz);
    return make_float3(ox * io, oy * io, oz * io);
}

/// Out-of-line copy for the rare post-step processes (one copy instead of one per call site).
static __device__ __noinline__ float3
rotate_dir(float3 t, float th, float ph) {
    return rotate_dir_inline(t, th, ph);
}

}   // namespace mqi_gpu
