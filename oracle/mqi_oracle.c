/* mqi_oracle.c - CPU restatement of moqui's proton transport (TEST INFRASTRUCTURE ONLY).
 *
 * See mqi_oracle.h.  Each function cites the reference file:line it restates.  The stepping
 * arithmetic is of type `real`: FP32 by default, as in moqui's float instantiation, or FP64 when
 * built with -DMQO_FP64 -- the all-FP64 oracle, moqui instantiated with R = double.  Its inputs stay
 * what they are in both builds: FP32 tables (mqi_p_ionization.hpp:11 and the other process headers
 * declare them `const float`), FP32 grid edges, densities and vertices, and the same 24-bit uniform
 * draws, so the two builds differ only in the precision of the arithmetic.  Build with
 * -ffp-contract=off so x86 and Arm builds agree.
 */
#include "mqi_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "../moquimc_gb300/csrc/mqi_tables.h"

#ifdef MQO_FP64
typedef double real;
#define RC(x) x
#define RABS fabs
#define RSQRT sqrt
#define RMIN fmin
#define RMAX fmax
#define RACOS acos
#define RSIN sin
#define RCOS cos
#define RPOW pow
#define RLOG log
#define REXP exp
#define RLOG1P log1p
#define REXPM1 expm1
#define RHUGE HUGE_VAL
#else
typedef float real;
#define RC(x) x##f
#define RABS fabsf
#define RSQRT sqrtf
#define RMIN fminf
#define RMAX fmaxf
#define RACOS acosf
#define RSIN sinf
#define RCOS cosf
#define RPOW powf
#define RLOG logf
#define REXP expf
#define RLOG1P log1pf
#define REXPM1 expm1f
#define RHUGE HUGE_VALF
#endif

/* ---- constants (mqi_physics_constants.hpp:14-38, mqi_interaction.hpp:24-30) ---------------- */
#define MP RC(938.272046)
#define ME RC(0.510998928)
#define MO RC(14903.3460795634)
#define WATER_DENSITY RC(0.001)
#define X0_WATER RC(360.863)
#define TP_CUT RC(0.5)
#define ES RC(13.9)
#define NEAR_ZERO RC(1e-7)
#define GEO_TOL RC(1e-3)
#define PI_F RC(3.14159265358979323846)

typedef struct { real x, y, z; } v3;

static v3 mk(real x, real y, real z) { v3 r = { x, y, z }; return r; }

/* ---- Philox4x32-10 (Salmon et al., SC'11) and the per-track stream ------------------------- */
typedef struct { uint32_t x, y, z, w; } u4;

static u4 philox(u4 c, uint32_t k0, uint32_t k1) {
    for (int r = 0; r < 10; ++r) {
        uint64_t p0 = (uint64_t) 0xD2511F53u * c.x;
        uint64_t p1 = (uint64_t) 0xCD9E8D57u * c.z;
        u4 n = { (uint32_t) (p1 >> 32) ^ c.y ^ k0, (uint32_t) p1, (uint32_t) (p0 >> 32) ^ c.w ^ k1, (uint32_t) p0 };
        c = n;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    return c;
}

void mqo_philox(const uint32_t* counter, const uint32_t* key, uint32_t* out) {
    u4 c = { counter[0], counter[1], counter[2], counter[3] };
    u4 r = philox(c, key[0], key[1]);
    out[0] = r.x; out[1] = r.y; out[2] = r.z; out[3] = r.w;
}

static uint64_t mix64(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

static uint64_t daughter_uid(uint64_t parent, uint32_t k) {
    return mix64(parent * 0x9E3779B97F4A7C15ull + (uint64_t) (k + 1u));
}

typedef struct {
    uint32_t k0, k1, hist, lo, hi, ctr, pos;
    u4       blk;
} rng_t;

static void rng_begin_step(rng_t* r) { r->pos = 4; }

static uint32_t rng_next(rng_t* r) {
    if (r->pos >= 4) {
        u4 c = { r->ctr, r->hist, r->lo, r->hi };
        r->blk = philox(c, r->k0, r->k1);
        r->ctr++;
        r->pos = 0;
    }
    uint32_t w = r->pos == 0 ? r->blk.x : r->pos == 1 ? r->blk.y : r->pos == 2 ? r->blk.z : r->blk.w;
    r->pos++;
    return w;
}

static real rng_u(rng_t* r) { return ((real) (rng_next(r) >> 8) + RC(0.5)) * (RC(1.0) / RC(16777216.0)); }

/* ---- helpers (mqi_math.hpp:26-30, mqi_relativistic_quantities.hpp:24-40) ------------------ */
static real intpl1d(real x, real x0, real x1, real y0, real y1) {
    return (x1 == x0) ? y0 : y0 + (x - x0) * (y1 - y0) / (x1 - x0);
}

typedef struct { real Ek, Et, Et_sq, gamma, gamma_sq, beta_sq, Te_max; } rel_t;

static rel_t rel_of(real ek) {
    rel_t r;
    const real MeMp = ME / MP, MeMp_sq = MeMp * MeMp;
    r.Ek = ek;
    r.Et = ek + MP;
    r.Et_sq = r.Et * r.Et;
    r.gamma = r.Et / MP;
    r.gamma_sq = r.gamma * r.gamma;
    r.beta_sq = (real) (1.0 - 1.0 / (double) r.gamma_sq);   /* double intermediate, as the reference */
    r.Te_max = (RC(2.0) * ME * r.beta_sq * r.gamma_sq) / (RC(1.0) + RC(2.0) * r.gamma * MeMp + MeMp_sq);
    return r;
}

static real momentum(const rel_t* r) { return RSQRT(r->Et * r->Et - MP * MP); }

/* ---- cross sections and stopping power (mqi_p_ionization.hpp:254-286, mqi_pp_elastic.hpp:221-235,
 *      mqi_po_elastic.hpp:243-256, mqi_po_inelastic.hpp:141-155) ---------------------------- */
static real cs_tab(const float* t, real Ek, real lo, real hi, real rho) {
    real cs = RC(0.0);
    if (Ek >= lo && Ek <= hi) {
        int i0 = (int) ((Ek - lo) / RC(0.5));
        int i1 = i0 + 1 < MQI_TABLE_N ? i0 + 1 : MQI_TABLE_N - 1;
        real x0 = lo + (real) i0 * RC(0.5);
        real x1 = x0 + RC(0.5);
        cs = intpl1d(Ek, x0, x1, t[i0], t[i1]);
    }
    return cs * rho;
}

static real dedx(real Ek) {
    real pw = RC(0.0);
    if (Ek >= RC(0.1) && Ek <= RC(299.6)) {
        int i0 = (int) ((Ek - RC(0.1)) / RC(0.5));
        int i1 = i0 + 1 < MQI_TABLE_N ? i0 + 1 : MQI_TABLE_N - 1;
        real x0 = RC(0.1) + (real) i0 * RC(0.5);
        real x1 = x0 + RC(0.5);
        pw = intpl1d(Ek, x0, x1, mqi_tab_dedx[i0], mqi_tab_dedx[i1]);
    } else if (Ek < RC(0.1) && Ek > RC(0.0)) {
        pw = mqi_tab_dedx[0];
    }
    return -RC(1.0) * pw;
}

/* ---- calibration (materials/mqi_patient_materials.hpp:414-473, 514-542) -------------------- */
static real spr_of(real rho, real Ek, int dbg) {
    const real d = rho * RC(1000.0);
    if (dbg && RABS(d - RC(1.0)) < RC(1e-3)) return RC(1.0);
    if (d <= RC(0.26)) {
        if (d < RC(0.0012)) return RC(0.0);
        return intpl1d(d, RC(0.0012), RC(0.26), RC(0.8815), RC(0.9925));
    }
    real rsp = RC(1.0123) - RC(3.386e-5) * Ek;
    rsp += RC(0.291) * (RC(1.0) + RPOW(Ek, -RC(0.3421))) * (RPOW(d, -RC(0.7)) - RC(1.0));
    if (d >= RC(0.9)) return rsp;
    return intpl1d(d, RC(0.26), RC(0.9), RC(0.9925), rsp);
}

static real x0_of(real rho, int dbg) {
    const real d = rho * RC(1000.0);
    real f;
    if (dbg && RABS(d - RC(1.0)) < RC(1e-3)) return X0_WATER;
    if (d <= RC(0.26)) f = RC(0.9857) + RC(0.0085) * d;
    else if (d <= RC(0.9)) f = RC(1.0446) - RC(0.2180) * d;
    else f = RC(1.19) + RC(0.44) * RLOG(d - RC(0.44));
    return (WATER_DENSITY * X0_WATER) / (d * RC(0.001) * f);
}

/* The tabulated calibration (the material plug-in, materials/mqi_material.hpp:10-25, as tables):
 * lower node and upper weight of x on a uniform grid of n >= 2 nodes, clamped to the grid. */
static real calib_index(real x, real x0, real dx, uint32_t n, int* i) {
    const real f = (x - x0) / dx;
    if (!(f > RC(0.0))) { *i = 0; return RC(0.0); }
    if (f >= (real) (n - 1)) { *i = (int) n - 2; return RC(1.0); }
    *i = (int) f;
    return f - (real) *i;
}

static real spr_table(const mqo_calib* c, real rho, real Ek) {
    int ir, ie;
    const real wr = calib_index(rho, c->rho0, c->drho, c->n_rho, &ir);
    const real we = calib_index(Ek, c->e0, c->de, c->n_e, &ie);
    const float* r0 = c->spr + (size_t) ir * c->n_e;
    const float* r1 = r0 + c->n_e;
    const real a = r0[ie] + we * ((real) r0[ie + 1] - (real) r0[ie]);
    const real b = r1[ie] + we * ((real) r1[ie + 1] - (real) r1[ie]);
    return a + wr * (b - a);
}

static real x0_table(const mqo_calib* c, real rho) {
    int ir;
    const real wr = calib_index(rho, c->rho0, c->drho, c->n_rho, &ir);
    return c->x0[ir] + wr * ((real) c->x0[ir + 1] - (real) c->x0[ir]);
}

static real spr_cal(const mqo_calib* c, real rho, real Ek, int dbg) { return c ? spr_table(c, rho, Ek) : spr_of(rho, Ek, dbg); }

static real x0_cal(const mqo_calib* c, real rho, int dbg) { return c ? x0_table(c, rho) : x0_of(rho, dbg); }

float mqo_spr(float rho, float Ek, int dbg) { return (float) spr_of(rho, Ek, dbg); }

float mqo_x0(float rho, int dbg) { return (float) x0_of(rho, dbg); }

float mqo_hu_to_density(int hu) {
    double r;
    float  f;
    if (hu < -1000) hu = -1000;
    else if (hu > 2995) hu = 2995;
    if (hu < -98) r = 0.00121 + 0.001029700665188 * (1000.0 + hu);
    else if (hu < 15) r = 1.018 + 0.000893 * hu;
    else if (hu < 23) r = 1.03;
    else if (hu < 101) r = 1.003 + 0.001169 * hu;
    else if (hu < 2001) r = 1.017 + 0.000592 * hu;
    else if (hu < 2995) r = 2.201 + 0.0005 * (-2000.0 + hu);
    else r = 4.54;
    f = (float) r;
    f = f * mqi_tab_density_correction[hu + 1000];
    f = (float) ((double) f / 1000.0);
    return f;
}

void mqo_eval_physics(const float* e, uint64_t n, float* out) {
    for (uint64_t i = 0; i < n; ++i) {
        rel_t r = rel_of(e[i]);
        float* o = out + 8 * i;
        o[0] = cs_tab(mqi_tab_cs_p_ion, r.Ek, RC(0.1), RC(299.6), RC(1.0));
        o[1] = cs_tab(mqi_tab_cs_pp_e, r.Ek, RC(0.5), RC(300.0), RC(1.0));
        o[2] = cs_tab(mqi_tab_cs_po_e, r.Ek, RC(0.5), RC(300.0), RC(1.0));
        o[3] = cs_tab(mqi_tab_cs_po_i, r.Ek, RC(0.5), RC(300.0), RC(1.0));
        o[4] = dedx(r.Ek);
        o[5] = r.beta_sq;
        o[6] = r.Te_max;
        o[7] = momentum(&r);
    }
}

/* ---- geometry (moqui/base/mqi_grid3d.hpp:488-889) ------------------------------------------ */

/* grid3d::index(p, dir) for one axis: the reference's linear scan, restated literally
 * (mqi_grid3d.hpp:751-780). */
static int index_scan(const float* e, int n, real p, real dir) {
    int idx = -1;
    for (int ind = 0; ind < n; ind++) {
        if (RABS(e[ind] - p) < GEO_TOL) {
            if (dir > 0) return ind;
            if (dir < 0) return ind - 1;
            return ind;
        } else if (RABS(e[ind + 1] - p) < GEO_TOL) {
            if (dir > 0) return ind + 1;
            if (dir < 0) return ind;
            return ind;
        } else if (e[ind] - p < 0 && e[ind + 1] - p > 0) {
            return ind;
        } else {
            idx = -1;
        }
    }
    return idx;
}

static int valid(const mqo_grid* g, int x, int y, int z) {
    return !(x < 0 || y < 0 || z < 0 || x >= g->nx || y >= g->ny || z >= g->nz);
}

/* intersect(p, d, idx) per axis (mqi_grid3d.hpp:528-605) */
static real exit_axis(real p, real* d, real v1, real v2, int idx, int dim) {
    if ((*d) * (*d) > NEAR_ZERO) {
        if (*d < 0) {
            real t = -(p - v1) / *d;
            if (RABS(t) < GEO_TOL && idx > 0) return RC(1.0) / GEO_TOL;
            return t;
        } else {
            real t = (v2 - p) / *d;
            if (RABS(t) < GEO_TOL && idx < dim) return RC(1.0) / GEO_TOL;
            return t;
        }
    }
    *d = RC(0.0);
    return RHUGE;
}

static real intersect_voxel(const mqo_grid* g, v3 p, v3* d, int cx, int cy, int cz) {
    real tx = exit_axis(p.x, &d->x, g->xe[cx], g->xe[cx + 1], cx, g->nx);
    real ty = exit_axis(p.y, &d->y, g->ye[cy], g->ye[cy + 1], cy, g->ny);
    real tz = exit_axis(p.z, &d->z, g->ze[cz], g->ze[cz + 1], cz, g->nz);
    real u;
    if (tx < ty) u = (tx < tz) ? tx : tz;
    else u = (ty < tz) ? ty : tz;
    return (u > 0) ? u : -RC(1.0);
}

/* intersect(p, d) from outside (mqi_grid3d.hpp:628-743); returns entry distance or -1 */
static real intersect_box(const mqo_grid* g, v3 p, v3* d) {
    real x0 = g->xe[0], x1 = g->xe[g->nx], y0 = g->ye[0], y1 = g->ye[g->ny], z0 = g->ze[0], z1 = g->ze[g->nz];
    real tminx, tmaxx, tminy, tmaxy, tminz, tmaxz, umin, umax;
    if (p.x >= x0 && p.x <= x1 && p.y >= y0 && p.y <= y1 && p.z >= z0 && p.z <= z1) return RC(0.0);
    if (d->x * d->x > NEAR_ZERO) {
        if (d->x > 0) { tminx = (x0 - p.x) / d->x; tmaxx = (x1 - p.x) / d->x; }
        else { tmaxx = (x0 - p.x) / d->x; tminx = (x1 - p.x) / d->x; }
    } else { d->x = 0; tminx = -RHUGE; tmaxx = RHUGE; }
    if (d->y * d->y > NEAR_ZERO) {
        if (d->y > 0) { tminy = (y0 - p.y) / d->y; tmaxy = (y1 - p.y) / d->y; }
        else { tmaxy = (y0 - p.y) / d->y; tminy = (y1 - p.y) / d->y; }
    } else { d->y = 0; tminy = -RHUGE; tmaxy = RHUGE; }
    if (d->z * d->z > NEAR_ZERO) {
        if (d->z > 0) { tminz = (z0 - p.z) / d->z; tmaxz = (z1 - p.z) / d->z; }
        else { tmaxz = (z0 - p.z) / d->z; tminz = (z1 - p.z) / d->z; }
    } else { d->z = 0; tminz = -RHUGE; tmaxz = RHUGE; }
    if (tminx > tminy) umin = (tminx > tminz) ? tminx : tminz;
    else umin = (tminy > tminz) ? tminy : tminz;
    if (tmaxx < tmaxy) umax = (tmaxx < tmaxz) ? tmaxx : tmaxz;
    else umax = (tmaxy < tmaxz) ? tmaxy : tmaxz;
    if ((umin < umax || RABS(umin - umax) < GEO_TOL) && umin >= 0 && umax >= 0) return umin;
    return -RC(1.0);
}

/* index(vtx1, dir1, idx) (mqi_grid3d.hpp:846-877) */
static void index_update(const mqo_grid* g, v3 p, v3 d, int* cx, int* cy, int* cz) {
    if (d.x < 0 && (RABS(p.x - g->xe[*cx]) < GEO_TOL || p.x < g->xe[*cx])) *cx -= 1;
    else if (d.x > 0 && (RABS(p.x - g->xe[*cx + 1]) < GEO_TOL || p.x > g->xe[*cx + 1])) *cx += 1;
    if (d.y < 0 && (RABS(p.y - g->ye[*cy]) < GEO_TOL || p.y < g->ye[*cy])) *cy -= 1;
    else if (d.y > 0 && (RABS(p.y - g->ye[*cy + 1]) < GEO_TOL || p.y > g->ye[*cy + 1])) *cy += 1;
    if (d.z < 0 && (RABS(p.z - g->ze[*cz]) < GEO_TOL || p.z < g->ze[*cz])) *cz -= 1;
    else if (d.z > 0 && (RABS(p.z - g->ze[*cz + 1]) < GEO_TOL || p.z > g->ze[*cz + 1])) *cz += 1;
}

static v3 normalize(v3 v) {
    real n = RSQRT(v.x * v.x + v.y * v.y + v.z * v.z);
    return mk(v.x / n, v.y / n, v.z / n);
}

static v3 advance(v3 p, v3 d, real len) { return mk(p.x + d.x * len, p.y + d.y * len, p.z + d.z * len); }

int mqo_trace_ray(const mqo_grid* g, const float ray[6], int max_steps, uint64_t* cnb, float* dist, int32_t* cells) {
    v3 p0 = mk(ray[0], ray[1], ray[2]);
    v3 d0 = normalize(mk(ray[3], ray[4], ray[5]));
    v3 d1 = d0;
    int cx = index_scan(g->xe, g->nx, p0.x, d0.x);
    int cy = index_scan(g->ye, g->ny, p0.y, d0.y);
    int cz = index_scan(g->ze, g->nz, p0.z, d0.z);
    int k = 0;
    if (!valid(g, cx, cy, cz)) {
        real e = intersect_box(g, p0, &d0);
        if (e < 0) return 0;
        p0 = advance(p0, d0, e);
        d0 = d1;
        cx = index_scan(g->xe, g->nx, p0.x, d0.x);
        cy = index_scan(g->ye, g->ny, p0.y, d0.y);
        cz = index_scan(g->ze, g->nz, p0.z, d0.z);
    }
    while (valid(g, cx, cy, cz) && k < max_steps) {
        real d2b = intersect_voxel(g, p0, &d0, cx, cy, cz);
        cnb[k] = (uint64_t) cz * g->nx * g->ny + (uint64_t) cy * g->nx + cx;
        dist[k] = (float) d2b;
        cells[3 * k] = cx; cells[3 * k + 1] = cy; cells[3 * k + 2] = cz;
        ++k;
        if (d2b < 0) break;
        v3 p1 = advance(p0, d0, d2b);
        index_update(g, p1, d1, &cx, &cy, &cz);
        p0 = p1;
        d0 = d1;
    }
    return k;
}

/* ---- tracks and the LIFO stack (mqi_track.hpp:48-205, mqi_track_stack.hpp:11-67) ----------- */
typedef struct {
    real    ke0, ke1;
    v3       p0, d0, p1, d1;
    real    dE, ldE;
    int      primary, stopped;
    uint64_t uid;
    uint32_t npush;
} trk_t;

typedef struct {
    trk_t*  t;
    int     idx, limit;
    uint64_t pushed, dropped;
} stack_t_;

typedef struct {
    const mqo_grid*  g;
    int              dbg;
    const mqo_calib* calib;
    real            tcut;
    stack_t_*        stk;
    rng_t            rng;
} env_t;

static void push(env_t* E, trk_t* parent, real ke0, real ke1, v3 p, v3 d, real dE0) {
    stack_t_* s = E->stk;
    if (s->idx >= s->limit) {   /* push_secondary silently drops (mqi_track_stack.hpp:36-41) */
        s->dropped++;
        return;
    }
    trk_t* n = &s->t[s->idx++];
    memset(n, 0, sizeof(*n));
    n->ke0 = ke0;
    n->ke1 = ke1;
    n->p0 = p; n->p1 = p; n->d0 = d; n->d1 = d;
    n->dE = dE0;
    n->primary = 0;
    n->uid = daughter_uid(parent->uid, parent->npush);
    parent->npush++;
    s->pushed++;
}

/* Möller-Hughes alignment + track_t::update_post_vertex_direction (mqi_track.hpp:163-172,
 * mqi_matrix.hpp:88-150) */
static v3 rotate_dir(v3 t, real th, real ph) {
    real s1 = RSIN(th), c1 = RCOS(th), s2 = RSIN(ph), c2 = RCOS(ph);
    v3 dl = normalize(mk(c2 * s1, s2 * s1, c1));
    real tn = RSQRT(t.x * t.x + t.y * t.y + t.z * t.z);
    real c = t.z / tn;
    real m[9];
    if (RABS(c - RC(1.0)) < GEO_TOL || RABS(c + RC(1.0)) < GEO_TOL) {
        real r2 = RC(1.0) / RSQRT(RC(2.0));
        real ux = r2, uy = RC(0.0), uz = -r2;
        real vx = RC(1.0) - t.x, vy = -t.y, vz = -t.z;
        real vn = RSQRT(vx * vx + vy * vy + vz * vz);
        vx /= vn; vy /= vn; vz /= vn;
        real du = ux * ux + uy * uy + uz * uz, dv = vx * vx + vy * vy + vz * vz, duv = vx * ux + vy * uy + vz * uz;
        real a = RC(2.0) / du, b = RC(2.0) / dv, k = RC(4.0) * duv / (du * dv);
        m[0] = RC(1.0) - a * ux * ux - b * vx * vx + k * vx * ux;
        m[1] = RC(0.0) - a * ux * uy - b * vx * vy + k * vx * uy;
        m[2] = RC(0.0) - a * ux * uz - b * vx * vz + k * vx * uz;
        m[3] = RC(0.0) - a * uy * ux - b * vy * vx + k * vy * ux;
        m[4] = RC(1.0) - a * uy * uy - b * vy * vy + k * vy * uy;
        m[5] = RC(0.0) - a * uy * uz - b * vy * vz + k * vy * uz;
        m[6] = RC(0.0) - a * uz * ux - b * vz * vx + k * vz * ux;
        m[7] = RC(0.0) - a * uz * uy - b * vz * vy + k * vz * uy;
        m[8] = RC(1.0) - a * uz * uz - b * vz * vz + k * vz * uz;
    } else {
        real vx = -t.y, vy = t.x, vz = RC(0.0);
        real h = (RC(1.0) - c) / (RC(1.0) - c * c);
        m[0] = c + h * vx * vx; m[1] = h * vx * vy - vz; m[2] = h * vx * vz + vy;
        m[3] = h * vx * vy + vz; m[4] = c + h * vy * vy; m[5] = h * vy * vz - vx;
        m[6] = h * vx * vz - vy; m[7] = h * vy * vz + vx; m[8] = c + h * vz * vz;
    }
    return normalize(mk(m[0] * dl.x + m[1] * dl.y + m[2] * dl.z, m[3] * dl.x + m[4] * dl.y + m[5] * dl.z,
                        m[6] * dl.x + m[7] * dl.y + m[8] * dl.z));
}

/* energy_loss + energy_straggling (mqi_p_ionization.hpp:297-345), range walk guarded at 0 */
static real energy_loss(rel_t* rel, real rho, real len, real spr, real z) {
    real lw = len * spr * rho / WATER_DENSITY;
    int n = (int) ((rel->Ek - RC(0.1)) / RC(0.5));
    real x0, x1, r, dE_mean, Te, var, ret;
    if (n > MQI_TABLE_N - 2) n = MQI_TABLE_N - 2;
    if (n < 0) n = 0;
    x0 = RC(0.1) + (real) n * RC(0.5);
    x1 = x0 + RC(0.5);
    if (x0 > rel->Ek && n > 0) n -= 1;
    if (x1 < rel->Ek && n < MQI_TABLE_N - 2) n += 1;
    r = intpl1d(rel->Ek, x0, x1, mqi_tab_range[n], mqi_tab_range[n + 1]);
    if (r < lw) return rel->Ek;
    r -= lw;
    while (n > 0 && r < mqi_tab_range[n]) --n;
    x0 = RC(0.1) + (real) n * RC(0.5);
    x1 = x0 + RC(0.5);
    dE_mean = rel->Ek - intpl1d(r, mqi_tab_range[n], mqi_tab_range[n + 1], x0, x1);
    Te = (rel->Te_max >= RC(0.08511)) ? RC(0.08511) : rel->Te_max;
    {
        /* dedx_term0 (mqi_physics_constants.hpp:29-30) in the stepping type */
        const real re = RC(2.8179403262e-12), re_sq = re * re;
        const real two_pi = (real) (2.0 * 3.14159265358979323846);
        const real t = (real) ((double) two_pi * (double) re_sq);
        const real t2 = t * ME;
        const real term0 = (real) ((double) t2 * 3.3428e+23 / 1000.0);
        var = term0 * rho / WATER_DENSITY * lw;
    }
    var *= Te / rel->beta_sq * (RC(1.0) - RC(0.5) * rel->beta_sq);
    ret = z * RSQRT(var) + dE_mean;
    if (ret < 0) ret = -ret;
    return ret;
}

/* last_step (mqi_p_ionization.hpp:481-490) */
static void last_step(env_t* E, trk_t* t, real rho) {
    real lw = RC(0.0), sl;
    if (t->dE > 0) lw = -t->dE / dedx(t->ke0);
    sl = lw * WATER_DENSITY / (spr_cal(E->calib, rho, t->ke0, E->dbg) * rho);
    t->p1 = advance(t->p0, t->d0, sl);
}

/* along_step (mqi_p_ionization.hpp:349-420) */
static void along_step(env_t* E, trk_t* t, real len, real rho, real spr, real z1, real z2, real u_phi) {
    rel_t rel = rel_of(t->ke0);
    real dE = energy_loss(&rel, rho, len, spr, z1);
    real r = RC(1.0), P, X0, th_sq, th, phi;
    if (dE >= t->ke0) {
        r = t->ke0 / dE;
        t->stopped = 1;
    }
    P = momentum(&rel);
    X0 = x0_cal(E->calib, rho, E->dbg);
    th_sq = ((ES / P) * (ES / P) / rel.beta_sq) * len / X0;
    th = RSQRT(th_sq);
    th = z2 * (RSQRT(RC(2.0)) * th);
    if (th < 0) th = -th;
    phi = RC(2.0) * PI_F * u_phi;
    t->d1 = rotate_dir(t->d1, th, phi);
    t->dE += dE * r;
    t->p1 = advance(t->p0, t->d0, r * len);
    t->ke1 -= dE * r;
}

/* p_ionization post_step (mqi_p_ionization.hpp:425-477) */
static void post_delta(env_t* E, trk_t* t) {
    rel_t rel = rel_of(t->ke1);
    real Te = RC(0.0);
    for (int it = 0; it < 64; ++it) {
        real n = rng_u(&E->rng);
        Te = E->tcut * rel.Te_max;
        Te /= ((RC(1.0) - n) * rel.Te_max + n * E->tcut);
        if (rng_u(&E->rng) < RC(1.0) - rel.beta_sq * Te / rel.Te_max + Te * Te / (RC(2.0) * rel.Et_sq)) break;
    }
    if (E->dbg) push(E, t, RC(0.0), RC(0.0), t->p0, t->d0, Te);
    else t->dE += Te;
    t->ke1 -= Te;
}

/* pp_elastic post_step (mqi_pp_elastic.hpp:119-219) */
static void post_pp(env_t* E, trk_t* t) {
    rel_t rel = rel_of(t->ke1);
    const real Mp_sq = MP * MP;
    real minv = TP_CUT / rel.Ek;
    real u = rng_u(&E->rng) * (RC(1.0) - RC(2.0) * minv) + minv;
    real E1 = rel.Et, dE = rel.Ek * u, E3 = (rel.Ek - dE) + MP, E4 = dE + MP;
    real P1 = momentum(&rel), P3 = RSQRT(E3 * E3 - Mp_sq), P4 = RSQRT(E4 * E4 - Mp_sq);
    real c3 = E1 * E3 - Mp_sq - MP * (E1 - E3), c34 = E3 * E4 - E1 * MP, th3, th4, phi;
    v3 dd;
    c3 /= (P1 * P3);
    c34 /= (P3 * P4);
    c3 = RMIN(RMAX(c3, -RC(1.0)), RC(1.0));
    c34 = RMIN(RMAX(c34, -RC(1.0)), RC(1.0));
    th3 = RACOS(c3);
    th4 = th3 - RACOS(c34);
    phi = RC(2.0) * PI_F * rng_u(&E->rng);
    t->ke1 -= dE;
    t->d1 = rotate_dir(t->d1, th3, phi);
    dd = rotate_dir(t->d1, th4, phi);
    push(E, t, dE, dE, t->p1, dd, RC(0.0));
}

/* po_elastic post_step (mqi_po_elastic.hpp:96-217); truncated exponential by inverse CDF */
static void post_poe(env_t* E, trk_t* t) {
    rel_t rel = rel_of(t->ke1);
    if (rel.Ek <= RC(5.5)) {
        real dE = rel.Ek;
        if (E->dbg) push(E, t, dE, RC(0.0), t->p1, t->d1, dE);
        else t->ldE += dE;
        t->ke1 -= dE;
        t->stopped = 1;
        return;
    }
    {
        const real MoMp = MO / MP, MoMp_sq = MoMp * MoMp;
        real Tp_avg = RC(0.65) * REXP(-RC(0.0013) * rel.Ek) - RC(0.71) * REXP(-RC(0.0177) * rel.Ek);
        real Tp_max = (RC(2.0) * MO * rel.beta_sq * rel.gamma_sq) / (RC(1.0) + RC(2.0) * rel.gamma * MoMp + MoMp_sq);
        real u = rng_u(&E->rng);
        real dE = -Tp_avg * RLOG1P(u * REXPM1(-Tp_max / Tp_avg));
        real E1, E3, c3, th3, phi;
        if (!(dE >= RC(0.0))) dE = RC(0.0);
        if (dE > Tp_max) dE = Tp_max;
        E1 = rel.Ek * (rel.Ek + RC(2.0) * MP);
        E3 = (rel.Ek - dE) * (rel.Ek - dE + RC(2.0) * MP);
        c3 = (E1 + E3 - dE * (dE + RC(2.0) * MO)) / RC(2.0) / RSQRT(E1 * E3);
        c3 = RMIN(RMAX(c3, -RC(1.0)), RC(1.0));
        th3 = RACOS(c3);
        phi = RC(2.0) * PI_F * rng_u(&E->rng);
        if (E->dbg) push(E, t, dE, RC(0.0), t->p0, t->d0, dE);
        else t->ldE += dE;
        t->ke1 -= dE;
        t->d1 = rotate_dir(t->d1, th3, phi);
    }
}

/* po_inelastic post_step (mqi_po_inelastic.hpp:158-288) */
static void post_poi(env_t* E, trk_t* t) {
    const real Ek = t->ke1;
    real Eb = RC(5.0), Er = Ek, P2, PL, pw;
    if (Ek <= RC(215.0) && Ek > RC(200.0)) { P2 = RC(0.78); PL = P2 + (RC(1.0) - P2) * RC(0.9); pw = RC(0.4); }
    else if (Ek > RC(215.0)) { P2 = RC(0.78); PL = P2 + (RC(1.0) - P2) * RC(1.0); pw = RC(0.4); }
    else if (Ek > RC(150.0)) { P2 = RC(0.72); PL = P2 + (RC(1.0) - P2) * RC(0.83); pw = RC(0.45); }
    else { P2 = RC(0.7); PL = P2 + (RC(1.0) - P2) * RC(0.83); pw = RC(0.52); }
    while ((Er - Eb) > RC(2.0)) {
        real dE, zeta;
        Er -= Eb;
        dE = RPOW(rng_u(&E->rng), pw) * (Er - RC(2.0)) + RC(2.0);
        if (dE >= Er) dE = Er;
        Er -= dE;
        t->ke1 -= (dE + Eb);
        zeta = rng_u(&E->rng);
        if (zeta < P2) {
            real c = (RC(2.0) * dE / Ek - RC(1.0)) + RC(2.0) * (RC(1.0) - dE / Ek) * rng_u(&E->rng);
            real th, phi;
            c = RMIN(RMAX(c, -RC(1.0)), RC(1.0));
            th = RACOS(c);
            phi = RC(2.0) * PI_F * rng_u(&E->rng);
            push(E, t, dE, dE, t->p1, rotate_dir(t->d1, th, phi), RC(0.0));
        } else if (zeta < PL) {
        } else if (E->dbg) {
            push(E, t, dE, RC(0.0), t->p0, t->d0, dE);
        }
        Eb *= RC(0.65);
    }
    t->dE += Er;
    t->ke1 -= Er;
    t->stopped = 1;
}

/* fippel_physics::stepping (mqi_fippel_physics.hpp:67-216) */
static void stepping(env_t* E, trk_t* t, real rho, real d2b) {
    rel_t rel, rel2;
    real spr, dd, cur_min, max_loss, cs1[4], cs2[4], sum1, sum2, cs_sum, c[4], u_mfp, mfp, step_limit;
    real bm_u1, bm_u2, u_phi, bm_r, z1, z2;
    if (rho < RC(1.0e-7)) { t->p1 = advance(t->p0, t->d0, d2b); return; }
    if (rho > RC(99.9)) { t->stopped = 1; return; }
    if (t->ke0 <= TP_CUT) {
        if (t->ke0 < 0) t->ke0 = 0;
        t->dE += t->ke0;
        t->ke1 -= t->ke0;
        last_step(E, t, rho);
        t->stopped = 1;
        return;
    }
    rng_begin_step(&E->rng);
    rel = rel_of(t->ke0);
    spr = spr_cal(E->calib, rho, t->ke0, E->dbg);
    dd = dedx(rel.Ek);
    cur_min = RC(1.0) * spr * rho / WATER_DENSITY;
    max_loss = -RC(1.0) * cur_min * dd;
    cs1[0] = cs_tab(mqi_tab_cs_p_ion, rel.Ek, RC(0.1), RC(299.6), rho);
    cs1[1] = cs_tab(mqi_tab_cs_pp_e, rel.Ek, RC(0.5), RC(300.0), rho);
    cs1[2] = cs_tab(mqi_tab_cs_po_e, rel.Ek, RC(0.5), RC(300.0), rho);
    cs1[3] = cs_tab(mqi_tab_cs_po_i, rel.Ek, RC(0.5), RC(300.0), rho);
    rel2 = rel_of(t->ke0 - max_loss);
    cs2[0] = cs_tab(mqi_tab_cs_p_ion, rel2.Ek, RC(0.1), RC(299.6), rho);
    cs2[1] = cs_tab(mqi_tab_cs_pp_e, rel2.Ek, RC(0.5), RC(300.0), rho);
    cs2[2] = cs_tab(mqi_tab_cs_po_e, rel2.Ek, RC(0.5), RC(300.0), rho);
    cs2[3] = cs_tab(mqi_tab_cs_po_i, rel2.Ek, RC(0.5), RC(300.0), rho);
    sum1 = cs1[0] + cs1[1] + cs1[2] + cs1[3];
    sum2 = cs2[0] + cs2[1] + cs2[2] + cs2[3];
    cs_sum = (sum1 >= sum2) ? sum1 : sum2;
    for (int k = 0; k < 4; ++k) c[k] = (sum1 >= sum2) ? cs1[k] : cs2[k];
    u_mfp = rng_u(&E->rng);
    mfp = -RC(1.0) * RLOG(u_mfp) / cs_sum;
    step_limit = cur_min * WATER_DENSITY / (spr * rho);
    bm_u1 = rng_u(&E->rng);
    bm_u2 = rng_u(&E->rng);
    u_phi = rng_u(&E->rng);
    bm_r = RSQRT(-RC(2.0) * RLOG(bm_u1));
    z1 = bm_r * RCOS(RC(2.0) * PI_F * bm_u2);
    z2 = bm_r * RSIN(RC(2.0) * PI_F * bm_u2);
    if (d2b < mfp && d2b < step_limit) {
        along_step(E, t, d2b, rho, spr, z1, z2, u_phi);
    } else if ((mfp < d2b || RABS(mfp - d2b) < GEO_TOL) && (mfp < step_limit || RABS(mfp - step_limit) < GEO_TOL)) {
        real u;
        along_step(E, t, mfp, rho, spr, z1, z2, u_phi);
        if (t->ke1 <= TP_CUT) return;
        u = cs_sum * rng_u(&E->rng);
        t->d1 = t->d0;
        if (u < c[0]) post_delta(E, t);
        else if (u < c[0] + c[1]) post_pp(E, t);
        else if (u < c[0] + c[1] + c[2]) post_poe(E, t);
        else if (u < c[0] + c[1] + c[2] + c[3]) post_poi(E, t);
    } else {
        along_step(E, t, step_limit, rho, spr, z1, z2, u_phi);
    }
}

/* scorer callbacks (scorers/mqi_scorer_energy_deposit.hpp:12-177): 1 energy_deposit, 2 dose_to_water,
 * 3 dose_to_water_square, 4 dose_to_medium, 5/6 LETd_weight1/2, 7/8 LETt_weight1/2,
 * 9/10 energy_deposit_primary/secondary */
static double hit(const mqo_config* cfg, const trk_t* t, real rho, real vol, int dbg) {
    real edep = t->dE + t->ldE;
    switch (cfg->scorer) {
    case 1: return (double) edep;
    case 9: return t->primary ? (double) t->dE : 0.0;
    case 10: return t->primary ? 0.0 : (double) t->dE;
    case 2:
    case 3: {
        double d;
        if (rho < RC(1.0e-7)) return 0.0;
        d = (double) (edep * RC(1.60218e-10) / (vol * rho * spr_cal(cfg->calib, rho, t->ke0, dbg)));
        return cfg->scorer == 3 ? d * d : d;
    }
    case 4: return t->primary ? (double) t->dE * 1.60218e-13 * 1000.0 / (double) (vol * rho) : 0.0;
    default: break;
    }
    {
        /* the LET weights: the step length from differences squared in the stepping type, summed in double */
        const real density = rho * RC(1000.0);
        const real dx = t->p1.x - t->p0.x, dy = t->p1.y - t->p0.y, dz = t->p1.z - t->p0.z;
        double length = (double) (dx * dx);
        double let;
        length += (double) (dy * dy);
        length += (double) (dz * dz);
        length = sqrt(length);
        if (length <= 0.0) return 0.0;
        let = (double) t->dE / length / (double) density;
        switch (cfg->scorer) {
        case 5: return (let >= 25.0) ? 0.0 : (double) t->dE * let;
        case 6: return (let >= 25.0) ? 0.0 : (double) t->dE;
        case 7: return length * let;
        case 8: return length;
        default: return 0.0;
        }
    }
}

/* The history loop (mqi_transport.hpp:146-249), one child, DIRECT ROI. */
int mqo_transport(const mqo_grid* g, const mqo_config* cfg, const float* V, uint64_t h0, uint64_t h1, uint64_t seed,
                  double* tally, double* per_hist, mqo_stats* st) {
    env_t    E;
    stack_t_ S;
    memset(&E, 0, sizeof(E));
    memset(&S, 0, sizeof(S));
    S.limit = cfg->physics_debug ? 200 : 10;
    S.t = (trk_t*) calloc((size_t) S.limit, sizeof(trk_t));
    if (!S.t) return -3;
    E.g = g;
    E.dbg = cfg->physics_debug;
    E.calib = cfg->calib;
    E.tcut = cfg->physics_debug ? RC(0.08511) : RC(0.0815);
    E.stk = &S;
    E.rng.k0 = (uint32_t) seed;
    E.rng.k1 = (uint32_t) (seed >> 32);
    for (uint64_t h = h0; h < h1; ++h) {
        const float* v = V + 7 * h;
        double hsum = 0.0;
        trk_t* p = &S.t[0];
        memset(p, 0, sizeof(*p));
        p->ke0 = p->ke1 = v[0];
        p->p0 = p->p1 = mk(v[1], v[2], v[3]);
        p->d0 = p->d1 = mk(v[4], v[5], v[6]);
        p->primary = 1;
        p->uid = 0;
        S.idx = 1;
        while (S.idx > 0) {
            trk_t t = S.t[--S.idx];
            int cx, cy, cz;
            if (st) st->tracks++;
            E.rng.hist = (uint32_t) h;
            E.rng.lo = (uint32_t) t.uid;
            E.rng.hi = (uint32_t) (t.uid >> 32);
            E.rng.ctr = 0;
            E.rng.pos = 4;
            /* child entry (mqi_transport.hpp:165-190), identity transform */
            t.d0 = normalize(t.d0);
            t.p1 = t.p0;
            t.d1 = t.d0;
            cx = index_scan(g->xe, g->nx, t.p0.x, t.d0.x);
            cy = index_scan(g->ye, g->ny, t.p0.y, t.d0.y);
            cz = index_scan(g->ze, g->nz, t.p0.z, t.d0.z);
            if (!valid(g, cx, cy, cz)) {
                real e = intersect_box(g, t.p0, &t.d0);
                if (e < 0) continue;
                t.p1 = advance(t.p0, t.d0, e);
                t.p0 = t.p1; t.d0 = t.d1; t.ke0 = t.ke1; t.dE = t.ldE = RC(0.0);
                cx = index_scan(g->xe, g->nx, t.p0.x, t.d0.x);
                cy = index_scan(g->ye, g->ny, t.p0.y, t.d0.y);
                cz = index_scan(g->ze, g->nz, t.p0.z, t.d0.z);
            }
            while (valid(g, cx, cy, cz) && !t.stopped) {
                uint64_t cnb = (uint64_t) cz * g->nx * g->ny + (uint64_t) cy * g->nx + cx;
                real rho = g->rho[cnb];
                real d2b = intersect_voxel(g, t.p0, &t.d0, cx, cy, cz);
                stepping(&E, &t, rho, d2b);
                if (st) st->steps++;
                if (d2b < 0) break;
                if (cnb > 0) {   /* DIRECT ROI: roi_->idx(cnb) > 0 */
                    real vol = ((real) g->xe[cx + 1] - (real) g->xe[cx]) * ((real) g->ye[cy + 1] - (real) g->ye[cy]) *
                               ((real) g->ze[cz + 1] - (real) g->ze[cz]);
                    double val = hit(cfg, &t, rho, vol, E.dbg);
                    if (val > 0) {
                        tally[cnb] += val;
                        hsum += val;
                    }
                }
                if (!t.stopped) {
                    index_update(g, t.p1, t.d1, &cx, &cy, &cz);
                    t.p0 = t.p1; t.d0 = t.d1; t.ke0 = t.ke1; t.dE = t.ldE = RC(0.0);
                }
            }
        }
        if (per_hist) per_hist[h - h0] = hsum;
        if (st) st->histories++;
    }
    if (st) { st->pushed += S.pushed; st->dropped += S.dropped; }
    free(S.t);
    return 0;
}

/* Sampling probes, mirroring the reference driver's `sample` mode: n independent draws of each
 * process at kinetic energy ke in a medium of density rho (g/mm^3) with default calibration, track
 * along -z from the origin.  Draw i uses the Philox stream (seed, history i, uid 0) from block 0,
 * the words laid out as in stepping(): the along-step probe takes its Box-Muller pair and azimuth
 * from words 1..3 of the first block, the post-step probes draw from the stream's start.
 * process: 0 along_step over 1 mm -> out[2n] = {dE, cos theta}; 1 delta ray -> out[n] = {Te};
 * 2 p-p elastic -> out[3n] = {dE, cos theta_3, cos theta_4 (2 without a daughter)};
 * 3 p-O elastic -> out[2n] = {dE, cos theta_3}; 4 p-O inelastic -> out[3n] = {proton daughters,
 * their summed kinetic energy, energy deposited by the primary}.  Each quantity is a block of n. */
int mqo_sample(int process, float ke, float rho, uint64_t n, uint64_t seed, int physics_debug, float* out) {
    env_t    E;
    stack_t_ S;
    memset(&E, 0, sizeof(E));
    memset(&S, 0, sizeof(S));
    S.limit = 200;
    S.t = (trk_t*) calloc((size_t) S.limit, sizeof(trk_t));
    if (!S.t) return -3;
    E.dbg = physics_debug;
    E.tcut = physics_debug ? RC(0.08511) : RC(0.0815);
    E.stk = &S;
    E.rng.k0 = (uint32_t) seed;
    E.rng.k1 = (uint32_t) (seed >> 32);
    for (uint64_t i = 0; i < n; ++i) {
        trk_t t;
        memset(&t, 0, sizeof(t));
        t.ke0 = t.ke1 = ke;
        t.p0 = t.p1 = mk(RC(0.0), RC(0.0), RC(0.0));
        t.d0 = t.d1 = mk(RC(0.0), RC(0.0), -RC(1.0));
        t.primary = 1;
        S.idx = 0;
        E.rng.hist = (uint32_t) i;
        E.rng.lo = E.rng.hi = 0;
        E.rng.ctr = 0;
        E.rng.pos = 4;
        if (process == 0) {
            real bm_u1, bm_u2, u_phi, r;
            (void) rng_u(&E.rng);   /* word 0: the free path in stepping() */
            bm_u1 = rng_u(&E.rng);
            bm_u2 = rng_u(&E.rng);
            u_phi = rng_u(&E.rng);
            r = RSQRT(-RC(2.0) * RLOG(bm_u1));
            along_step(&E, &t, RC(1.0), rho, spr_of(rho, ke, physics_debug), r * RCOS(RC(2.0) * PI_F * bm_u2),
                       r * RSIN(RC(2.0) * PI_F * bm_u2), u_phi);
            out[i] = (float) (t.ke0 - t.ke1);
            out[n + i] = (float) -t.d1.z;
        } else if (process == 1) {
            post_delta(&E, &t);
            out[i] = (float) (t.ke0 - t.ke1);
        } else if (process == 2) {
            post_pp(&E, &t);
            out[i] = (float) (t.ke0 - t.ke1);
            out[n + i] = (float) -t.d1.z;
            out[2 * n + i] = S.idx > 0 ? (float) -S.t[S.idx - 1].d1.z : 2.0f;
        } else if (process == 3) {
            post_poe(&E, &t);
            out[i] = (float) (t.ke0 - t.ke1);
            out[n + i] = (float) -t.d1.z;
        } else if (process == 4) {
            int   np = 0;
            real  e2 = RC(0.0);
            post_poi(&E, &t);
            for (int k = 0; k < S.idx; ++k)
                if (S.t[k].ke1 > RC(0.0)) {
                    ++np;
                    e2 += S.t[k].ke1;
                }
            out[i] = (float) np;
            out[n + i] = (float) e2;
            out[2 * n + i] = (float) t.dE;
        } else {
            free(S.t);
            return -1;
        }
    }
    free(S.t);
    return 0;
}
