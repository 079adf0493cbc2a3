// Reference CPU oracle driver: test infrastructure only.
//
// This translation unit is compiled against the staged, patched copy of the reference headers
// (oracle/stage_ref.py) and runs the reference's OWN CPU code path.  It is the checker that pins
// the C restatement (oracle/mqi_oracle.c) and the CUDA path; nothing in the product links it.
//
// Modes (argv[1]):
//   phantom <phantom_env CLI> [--beam uniform|gaussian] [--json <file>] [--beamline <file>]
//       Runs mqi::phantom_env<float> (moqui/base/environments/mqi_phantom_env.hpp:37-428) on the CPU:
//       initialize -> run -> save_reshaped_files.  run() is overridden only to (a) seed the CPU
//       transport RNG from --random_seed (the stock CPU branch default-constructs it, so every
//       process would share one stream, mqi_transport.hpp:147-149 / mqi_phantom_env.hpp:420-422)
//       and (b) time the transport call alone.  --beam gaussian swaps phsp_6d_uniform for the
//       Gaussian phsp_6d (moqui/base/distributions/mqi_phsp6d.hpp) with sigma = --spot_size.
//       --beamline puts beamline children before the phantom, built as tps_env builds them
//       (mqi_tps_env.hpp:735-758, 1605-1737); one device per line:
//         rangeshifter xmin xmax ymin ymax zmin zmax density_g_cm3 ax ay az tx ty tz
//         aperture cx cy cz vx vy vz ax ay az tx ty tz n_openings {n_vertices x y ...}...
//       (angles in radians for mat3x3(ax, ay, az), translation in mm).  The children's rotation
//       matrices go to the --json record and each aperture's densities to aperture<k>.bin in the
//       output directory.
//   raywalk <rays.bin> <out.bin>
//       Walks rays through a grid3d exactly as the transport kernel's voxel loop does
//       (mqi_transport.hpp:161-239) with the physics replaced by a pure boundary step.
//   physics <out.bin>
//       Tabulates the deterministic physics functions on fixed input grids.
//   sample <out.bin> <n> <seed>
//       Draws n samples from each sampling routine at fixed inputs (along_step, the four
//       post_step processes) for distribution tests.
//   vertices <out.bin> <n> <seed> <gaussian> x y z sx sy energy colli gantry couch iec
//       Samples phantom_env's beam source with the reference's own distribution classes.
//   dij <hits.bin> <capacity> <n_spots> <nx> <ny> <nz> <scale> <out_dir> <name>
//       Replays recorded Dij insertions through insert_hashtable and writes save_to_npz's file.
//   hits <in.bin> <out.bin>
//       Evaluates the scorer callbacks (dose, LET weights, ...) on given step states.
//   roi <in.bin> <out.bin>
//       Evaluates roi_t::idx and get_mask_idx on given voxels.
#include <moqui/base/environments/mqi_phantom_env.hpp>
#include <moqui/kernel_functions/mqi_transport.hpp>

#include "ref_beams.hpp"

#include <chrono>
#include <csignal>
#include <cstdio>
#include <execinfo.h>
#include <unistd.h>
#include <cstring>
#include <fstream>
#include <iomanip>
#include <sstream>
#include <string>
#include <vector>

// Shim: the reference's print_materials reads members that no longer exist
// (moqui/kernel_functions/mqi_print_data.hpp:20-24).  An empty specialisation lets
// x_environment<float>::initialize instantiate; it only printed diagnostics.
template<>
void
mc::print_materials<float>(mqi::material_t<float>*, uint16_t) {}

namespace
{

template<typename T>
void
write_vec(std::ofstream& f, const std::vector<T>& v) {
    uint64_t n = v.size();
    f.write(reinterpret_cast<const char*>(&n), sizeof(n));
    if (n) f.write(reinterpret_cast<const char*>(v.data()), n * sizeof(T));
}

template<typename T>
std::vector<T>
read_vec(std::ifstream& f) {
    uint64_t n = 0;
    f.read(reinterpret_cast<char*>(&n), sizeof(n));
    std::vector<T> v(n);
    if (n) f.read(reinterpret_cast<char*>(v.data()), n * sizeof(T));
    return v;
}

/// phantom_env with a seeded CPU transport RNG, a timed transport phase and an optional
/// Gaussian spot.  Everything else is the stock reference class.
/// One beamline device read from a --beamline file.
struct beamline_device {
    std::string                      kind;
    float                            a[6] = { 0, 0, 0, 0, 0, 0 };   // rangeshifter: box; aperture: centre, volume
    float                            density = 0.0f;
    float                            ang[3] = { 0, 0, 0 };
    float                            tr[3]  = { 0, 0, 0 };
    std::vector<std::vector<float>>  openings;                       // x, y pairs
};

std::vector<beamline_device>
read_beamline(const std::string& path) {
    std::vector<beamline_device> out;
    std::ifstream                f(path);
    std::string                  line;
    while (std::getline(f, line)) {
        std::istringstream in(line);
        beamline_device    d;
        if (!(in >> d.kind)) continue;
        for (float& v : d.a) in >> v;
        if (d.kind == "rangeshifter") in >> d.density;
        for (float& v : d.ang) in >> v;
        for (float& v : d.tr) in >> v;
        if (d.kind == "aperture") {
            int n_open = 0;
            in >> n_open;
            for (int k = 0; k < n_open; ++k) {
                int nv = 0;
                in >> nv;
                std::vector<float> poly(2 * nv);
                for (float& v : poly) in >> v;
                d.openings.push_back(poly);
            }
        }
        out.push_back(d);
    }
    return out;
}

/// tps_env::sol1_1 (mqi_tps_env.hpp:1753-1770): crossing-number point-in-polygon test.
bool
inside_polygon(const mqi::vec3<float>& pos, const std::vector<mqi::vec2<float>>& seg) {
    int c = 0;
    const int n = (int) seg.size();
    for (int i = 0, j = n - 1; i < n; j = i++) {
        const mqi::vec2<float> p0 = seg[i], p1 = seg[j];
        if ((((p0.y <= pos.y) && (pos.y < p1.y)) || ((p1.y <= pos.y) && (pos.y < p0.y))) &&
            (pos.x < (p1.x - p0.x) * (pos.y - p0.y) / (p1.y - p0.y) + p0.x))
            c = !c;
    }
    return c;
}

/// The child of a range shifter, as tps_env::create_rangeshifter (mqi_tps_env.hpp:1605-1650).
mqi::node_t<float>*
make_rangeshifter(const beamline_device& d) {
    auto* n       = new mqi::node_t<float>;
    n->n_scorers  = 0;
    n->n_children = 0;
    n->scorers    = nullptr;
    n->children   = nullptr;
    n->geo = new mqi::grid3d<mqi::density_t, float>(d.a[0], d.a[1], 2, d.a[2], d.a[3], 2, d.a[4], d.a[5], 2,
                                                    mqi::mat3x3<float>(d.ang[0], d.ang[1], d.ang[2]));
    n->geo->fill_data(d.density * 1e-3);
    n->geo->translation_vector = mqi::vec3<float>(d.tr[0], d.tr[1], d.tr[2]);
    return n;
}

/// The child of a voxelised aperture, as tps_env::create_voxelized_aperture
/// (mqi_tps_env.hpp:1652-1737) with 1 mm voxels; the last opening decides (is_inside, :1739-1750).
mqi::node_t<float>*
make_aperture(const beamline_device& d, std::vector<float>& rho_out) {
    const mqi::vec3<float> pos(d.a[0], d.a[1], d.a[2]), vol(d.a[3], d.a[4], d.a[5]), vox(1, 1, 1);
    std::vector<std::vector<mqi::vec2<float>>> segs;
    for (const auto& poly : d.openings) {
        std::vector<mqi::vec2<float>> s;
        for (size_t j = 0; j + 1 < poly.size(); j += 2) {
            mqi::vec2<float> v;
            v.x = poly[j] + pos.x;
            v.y = poly[j + 1] + pos.y;
            s.push_back(v);
        }
        segs.push_back(s);
    }
    const size_t nx = (size_t) mqi::mqi_ceil(vol.x / vox.x), ny = (size_t) mqi::mqi_ceil(vol.y / vox.y),
                 nz = (size_t) mqi::mqi_ceil(vol.z / vox.z);
    float* xe = new float[nx + 1];
    float* ye = new float[ny + 1];
    float* ze = new float[nz + 1];
    for (size_t i = 0; i < nx + 1; i++) xe[i] = (pos.x - vol.x / 2) + i * vox.x;
    for (size_t i = 0; i < ny + 1; i++) ye[i] = (pos.y - vol.y / 2) + i * vox.y;
    for (size_t i = 0; i < nz + 1; i++) ze[i] = (pos.z - vol.z / 2) + i * vox.z;
    auto* n       = new mqi::node_t<float>;
    n->n_scorers  = 0;
    n->n_children = 0;
    n->scorers    = nullptr;
    n->children   = nullptr;
    n->geo = new mqi::grid3d<mqi::density_t, float>(xe, nx + 1, ye, ny + 1, ze, nz + 1,
                                                    mqi::mat3x3<float>(d.ang[0], d.ang[1], d.ang[2]));
    auto* data = new mqi::density_t[nx * ny * nz];
    mqi::vec3<float> p(0, 0, 0);
    for (size_t i = 0; i < nx; i++) {
        p.x = xe[i] + vox.x * 0.5;
        for (size_t j = 0; j < ny; j++) {
            p.y = ye[j] + vox.y * 0.5;
            bool inside = false;
            for (const auto& s : segs) inside = inside_polygon(p, s);
            for (size_t k = 0; k < nz; k++) data[k * nx * ny + j * nx + i] = inside ? 1e-8 : 100.0;
        }
    }
    n->geo->set_data(data);
    n->geo->translation_vector = mqi::vec3<float>(d.tr[0], d.tr[1], d.tr[2]);
    rho_out.assign(data, data + nx * ny * nz);
    return n;
}

class oracle_phantom_env : public mqi::phantom_env<float>
{
public:
    bool        gaussian = false;
    double      transport_seconds = 0.0;
    uint32_t    tracked = 0;
    std::vector<beamline_device>      beamline;
    std::vector<std::vector<float>>   aperture_rho;
    std::vector<std::array<float, 9>> beamline_rot;

    oracle_phantom_env(mqi::cli& c, bool g) : mqi::phantom_env<float>(c), gaussian(g) {}

    void
    setup_world() override {
        mqi::phantom_env<float>::setup_world();
        if (beamline.empty()) return;
        // beamline children first, the phantom last (mqi_tps_env.hpp:735-758)
        mqi::node_t<float>*  phantom = this->world->children[0];
        const int            n       = (int) beamline.size() + 1;
        mqi::node_t<float>** kids    = new mqi::node_t<float>*[n];
        for (size_t i = 0; i < beamline.size(); ++i) {
            if (beamline[i].kind == "rangeshifter") {
                kids[i] = make_rangeshifter(beamline[i]);
            } else {
                aperture_rho.emplace_back();
                kids[i] = make_aperture(beamline[i], aperture_rho.back());
            }
            const auto& r = kids[i]->geo->rotation_matrix_fwd;
            beamline_rot.push_back({ r.xx, r.xy, r.xz, r.yx, r.yy, r.yz, r.zx, r.zy, r.zz });
        }
        kids[n - 1]              = phantom;
        this->world->children    = kids;
        this->world->n_children  = n;
    }

    void
    setup_beamsource() override {
        if (gaussian)
            gaussian_phantom_beamsource(*this);
        else
            mqi::phantom_env<float>::setup_beamsource();
    }

    void
    run() override {
        // CPU branch of phantom_env::run (mqi_phantom_env.hpp:302-323, 416-423).
        uint32_t h1     = this->beamsource.total_histories();
        this->num_spots = this->beamsource.total_beamlets();
        uint32_t tp[1]  = { 0 };
        std::vector<int32_t> transport_seed(h1);
        std::default_random_engine tmp_rng;
        tmp_rng.seed(this->random_seed);
        for (uint32_t i = 0; i < h1; ++i)
            transport_seed[i] = tmp_rng();
        mc::mc_world     = this->world;
        mc::mc_vertices  = this->vertices;
        mc::mc_materials = this->materials;
        mqi::thrd_t* worker_threads = new mqi::thrd_t[1];
        worker_threads[0].rnd_generator.seed(static_cast<unsigned long>(this->random_seed) * 2654435761UL + 12345UL);
        auto t0 = std::chrono::steady_clock::now();
        mc::transport_particles_patient<float>(
          worker_threads, mc::mc_world, mc::mc_vertices, mc::mc_materials, h1, tp, transport_seed.data());
        auto t1 = std::chrono::steady_clock::now();
        transport_seconds = std::chrono::duration<double>(t1 - t0).count();
        tracked           = tp[0];
        delete[] worker_threads;
    }
};

int
run_phantom(int argc, char** argv) {
    bool        gaussian = false;
    std::string json, beamline;
    std::vector<char*> rest;
    rest.push_back(argv[0]);
    for (int i = 2; i < argc; ++i) {
        if (!std::strcmp(argv[i], "--beam") && i + 1 < argc) {
            gaussian = !std::strcmp(argv[++i], "gaussian");
        } else if (!std::strcmp(argv[i], "--json") && i + 1 < argc) {
            json = argv[++i];
        } else if (!std::strcmp(argv[i], "--beamline") && i + 1 < argc) {
            beamline = argv[++i];
        } else {
            rest.push_back(argv[i]);
        }
    }
    mqi::cli cl;
    cl.read(static_cast<int>(rest.size()), rest.data());
    oracle_phantom_env env(cl, gaussian);
    if (!beamline.empty()) env.beamline = read_beamline(beamline);
    env.initialize();
    env.run();
    env.finalize();
    env.save_reshaped_files();
    if (!json.empty()) {
        std::ofstream f(json);
        f << "{\"transport_seconds\": " << env.transport_seconds << ", \"histories\": "
          << env.beamsource.total_histories() << ", \"tracked\": " << env.tracked
#ifdef __PHYSICS_DEBUG__
          << ", \"physics_debug\": 1"
#else
          << ", \"physics_debug\": 0"
#endif
          << ", \"beamline_rot\": [";
        for (size_t i = 0; i < env.beamline_rot.size(); ++i) {
            f << (i ? ", [" : "[");
            for (int k = 0; k < 9; ++k) f << (k ? ", " : "") << std::setprecision(9) << env.beamline_rot[i][k];
            f << "]";
        }
        f << "]}\n";
        for (size_t k = 0; k < env.aperture_rho.size(); ++k) {
            std::ofstream a(env.output_path + "/aperture" + std::to_string(k) + ".bin", std::ios::binary);
            a.write(reinterpret_cast<const char*>(env.aperture_rho[k].data()), env.aperture_rho[k].size() * sizeof(float));
        }
    }
    return 0;
}

/// Ray walk through a grid built with the reference's uniform-edge constructor
/// (mqi_grid3d.hpp grid3d(xmin,xmax,nx+1,...)).  Input layout (all little-endian):
///   f32[9] grid: xmin xmax ymin ymax zmin zmax, i32[3] n, u32 max_steps, then vec<f32> rays
///   (6 floats per ray: pos, dir).  Output: vec<i64> offsets (n_rays+1), vec<u64> cnb,
///   vec<f32> dist, vec<i32> cell (3 per entry).
int
run_raywalk(const char* in_path, const char* out_path) {
    std::ifstream fin(in_path, std::ios::binary);
    float  g[6];
    int32_t n[3];
    uint32_t max_steps;
    fin.read(reinterpret_cast<char*>(g), sizeof(g));
    fin.read(reinterpret_cast<char*>(n), sizeof(n));
    fin.read(reinterpret_cast<char*>(&max_steps), sizeof(max_steps));
    std::vector<float> rays = read_vec<float>(fin);
    mqi::grid3d<mqi::density_t, float> geo(
      g[0], g[1], n[0] + 1, g[2], g[3], n[1] + 1, g[4], g[5], n[2] + 1);
    std::vector<int64_t>  off(1, 0);
    std::vector<uint64_t> cnbs;
    std::vector<float>    dists;
    std::vector<int32_t>  cells;
    const size_t n_rays = rays.size() / 6;
    for (size_t r = 0; r < n_rays; ++r) {
        mqi::track_t<float> track;
        mqi::vertex_t<float> v;
        v.ke  = 100.0f;
        v.pos = mqi::vec3<float>(rays[6 * r + 0], rays[6 * r + 1], rays[6 * r + 2]);
        v.dir = mqi::vec3<float>(rays[6 * r + 3], rays[6 * r + 4], rays[6 * r + 5]);
        track.set(v);
        // Child entry (mqi_transport.hpp:165-190).
        track.vtx0.pos = geo.rotation_matrix_inv * (track.vtx0.pos - geo.translation_vector);
        track.vtx0.dir = geo.rotation_matrix_inv * (track.vtx0.dir);
        track.vtx0.dir.normalize();
        track.vtx1.pos = track.vtx0.pos;
        track.vtx1.dir = track.vtx0.dir;
        mqi::vec3<mqi::ijk_t> chk = geo.index(track.vtx0.pos, track.vtx0.dir);
        bool entered = true;
        if (!geo.is_valid(chk)) {
            track.its = geo.intersect(track.vtx0.pos, track.vtx0.dir);
            if (track.its.dist < 0) {
                entered = false;
            } else {
                track.update_post_vertex_position(track.its.dist);
                track.move();
                track.its.cell = geo.index(track.vtx0.pos, track.vtx0.dir);
            }
        } else {
            track.its.dist = 0.0;
            track.its.cell = chk;
        }
        uint32_t steps = 0;
        // Voxel loop (mqi_transport.hpp:192-233) with a boundary-only step.
        while (entered && geo.is_valid(track.its.cell) && steps < max_steps) {
            mqi::cnb_t cnb = geo.ijk2cnb(track.its.cell);
            track.its      = geo.intersect(track.vtx0.pos, track.vtx0.dir, track.its.cell);
            cnbs.push_back(cnb);
            dists.push_back(track.its.dist);
            cells.push_back(track.its.cell.x);
            cells.push_back(track.its.cell.y);
            cells.push_back(track.its.cell.z);
            ++steps;
            if (track.its.dist < 0) break;
            track.update_post_vertex_position(track.its.dist);
            geo.index(track.vtx1.pos, track.vtx1.dir, track.its.cell);
            track.move();
        }
        off.push_back(static_cast<int64_t>(cnbs.size()));
    }
    std::ofstream fout(out_path, std::ios::binary);
    write_vec(fout, off);
    write_vec(fout, cnbs);
    write_vec(fout, dists);
    write_vec(fout, cells);
    return 0;
}

/// Deterministic physics tables.  Output: a sequence of named f32 vectors.
int
run_physics(const char* out_path) {
    mqi::fippel_physics<float>       fp;
    mqi::patient_material_t<float>   pm;
    mqi::material_t<float>*          mat = &pm;
    std::ofstream                    fout(out_path, std::ios::binary);
    // Energy grid: dense regular grid plus the table nodes themselves and values just around them.
    std::vector<float> E;
    for (int i = 0; i <= 6100; ++i)
        E.push_back(0.02f + 0.05f * i);   // 0.02 .. 305.02 MeV
    for (int i = 0; i < 600; ++i) {
        E.push_back(0.1f + 0.5f * i);
        E.push_back(0.5f + 0.5f * i);
        E.push_back(std::nextafter(0.5f + 0.5f * i, 0.0f));
    }
    const float rhos[] = { 0.0000012f, 0.00026f, 0.0003068f, 0.0009f, 0.00098822f, 0.001f,
                           0.0010005f, 0.00103f, 0.0017939f, 0.0025f };
    std::vector<float> rho_v(std::begin(rhos), std::end(rhos));
    write_vec(fout, E);
    write_vec(fout, rho_v);
    std::vector<float> beta_sq, gamma, te_max, et, mom;
    std::vector<float> cs_ion, cs_pp, cs_poe, cs_poi, dedx;
    for (float e : E) {
        mqi::relativistic_quantities<float> rel(e, 938.272046f);
        beta_sq.push_back(rel.beta_sq);
        gamma.push_back(rel.gamma);
        te_max.push_back(rel.Te_max);
        et.push_back(rel.Et);
        mom.push_back(rel.momentum());
        cs_ion.push_back(fp.p_ion.cross_section(rel, mat, 1.0f));
        cs_pp.push_back(fp.pp_e.cross_section(rel, mat, 1.0f));
        cs_poe.push_back(fp.po_e.cross_section(rel, mat, 1.0f));
        cs_poi.push_back(fp.po_i.cross_section(rel, mat, 1.0f));
        dedx.push_back(fp.p_ion.dEdx(rel, mat));
    }
    write_vec(fout, beta_sq);
    write_vec(fout, gamma);
    write_vec(fout, te_max);
    write_vec(fout, et);
    write_vec(fout, mom);
    write_vec(fout, cs_ion);
    write_vec(fout, cs_pp);
    write_vec(fout, cs_poe);
    write_vec(fout, cs_poi);
    write_vec(fout, dedx);
    // SPR(rho, E) and X0(rho) on the rho set x energy grid (every 10th energy).
    std::vector<float> spr, x0, strag;
    for (float r : rho_v) {
        for (size_t i = 0; i < E.size(); i += 10) {
            spr.push_back(mat->compute_rsp_(r, E[i]));
        }
        x0.push_back(mat->compute_rl_(r, 0.001f, 360.863f));
        for (size_t i = 0; i < E.size(); i += 10) {
            mqi::relativistic_quantities<float> rel(E[i], 938.272046f);
            strag.push_back(fp.p_ion.energy_straggling(rel, mat, 1.0f, r));
        }
    }
    write_vec(fout, spr);
    write_vec(fout, x0);
    write_vec(fout, strag);
    // HU -> density for every HU in [-1100, 3100].
    std::vector<float> hu_rho;
    for (int hu = -1100; hu <= 3100; ++hu)
        hu_rho.push_back(pm.hu_to_density(static_cast<int16_t>(hu)));
    write_vec(fout, hu_rho);
    return 0;
}

/// Sampling probes.  A small water grid hosts the track so that the daughters' coordinate
/// transforms have a node.  Output: named f32 vectors (see the list at the end).
int
run_sample(const char* out_path, long n, unsigned seed) {
    mqi::fippel_physics<float>     fp;
    mqi::patient_material_t<float> pm;
    mqi::material_t<float>*        mat = &pm;
    mqi::grid3d<mqi::density_t, float> geo(-50.f, 50.f, 101, -50.f, 50.f, 101, -50.f, 50.f, 101);
    mqi::node_t<float> node;
    node.geo = &geo;
    mqi::mqi_rng rng;
    rng.seed(seed);
    const float rho = 0.001f;
    std::ofstream fout(out_path, std::ios::binary);
    auto make_track = [&](float ke) {
        mqi::vertex_t<float> v;
        v.ke  = ke;
        v.pos = mqi::vec3<float>(0.f, 0.f, 0.f);
        v.dir = mqi::vec3<float>(0.f, 0.f, -1.f);
        mqi::track_t<float> t(v);
        t.c_node = &node;
        return t;
    };
    const float energies[] = { 10.0f, 50.0f, 150.0f };
    for (float ke : energies) {
        // along_step over 1 mm: energy loss and polar deflection.
        std::vector<float> dE, cth;
        for (long i = 0; i < n; ++i) {
            mqi::track_t<float>       t = make_track(ke);
            mqi::track_stack_t<float> stk;
            fp.p_ion.along_step(t, stk, &rng, 1.0f, mat, rho);
            dE.push_back(t.vtx0.ke - t.vtx1.ke);
            cth.push_back(-t.vtx1.dir.z);
        }
        write_vec(fout, dE);
        write_vec(fout, cth);
        // Delta-ray energy (p_ion post_step).
        std::vector<float> te;
        for (long i = 0; i < n; ++i) {
            mqi::track_t<float>       t = make_track(ke);
            mqi::track_stack_t<float> stk;
            fp.p_ion.post_step(t, stk, &rng, 1.0f, mat, true);
            te.push_back(t.vtx0.ke - t.vtx1.ke);
        }
        write_vec(fout, te);
        // p-p elastic: energy transfer, primary polar cosine, daughter polar cosine.
        std::vector<float> pp_de, pp_c3, pp_c4;
        for (long i = 0; i < n; ++i) {
            mqi::track_t<float>       t = make_track(ke);
            mqi::track_stack_t<float> stk;
            fp.pp_e.post_step(t, stk, &rng, 1.0f, mat, true);
            pp_de.push_back(t.vtx0.ke - t.vtx1.ke);
            pp_c3.push_back(-t.vtx1.dir.z);
            pp_c4.push_back(stk.idx > 0 ? -stk.tracks[stk.idx - 1].vtx1.dir.z : 2.0f);
        }
        write_vec(fout, pp_de);
        write_vec(fout, pp_c3);
        write_vec(fout, pp_c4);
        // p-O elastic: energy transfer and primary polar cosine.
        std::vector<float> poe_de, poe_c3;
        for (long i = 0; i < n; ++i) {
            mqi::track_t<float>       t = make_track(ke);
            mqi::track_stack_t<float> stk;
            fp.po_e.post_step(t, stk, &rng, 1.0f, mat, true);
            poe_de.push_back(t.vtx0.ke - t.vtx1.ke);
            poe_c3.push_back(-t.vtx1.dir.z);
        }
        write_vec(fout, poe_de);
        write_vec(fout, poe_c3);
        // p-O inelastic: number of proton secondaries, their summed energy, energy deposited
        // by the primary (Er).
        std::vector<float> poi_n, poi_e2, poi_dep;
        for (long i = 0; i < n; ++i) {
            mqi::track_t<float>       t = make_track(ke);
            mqi::track_stack_t<float> stk;
            fp.po_i.post_step(t, stk, &rng, 1.0f, mat, true);
            int   np = 0;
            float e2 = 0.f;
            for (int k = 0; k < stk.idx; ++k) {
                if (stk.tracks[k].vtx1.ke > 0.f) {   // proton secondaries carry ke in vtx1
                    ++np;
                    e2 += stk.tracks[k].vtx1.ke;
                }
            }
            poi_n.push_back(static_cast<float>(np));
            poi_e2.push_back(e2);
            poi_dep.push_back(t.dE);
        }
        write_vec(fout, poi_n);
        write_vec(fout, poi_e2);
        write_vec(fout, poi_dep);
    }
    return 0;
}

/// The beam source of phantom_env (mqi_phantom_env.hpp:204-232) built from the reference's own
/// classes -- coordinate_transform, phsp_6d_uniform or phsp_6d, const_1d, beamlet, beamsource --
/// and sampled with std::default_random_engine seeded like phantom_env's beam_rng.  Arguments:
/// out n seed gaussian x y z sx sy energy colli gantry couch iec.  Output: vec<f32> of 7 floats
/// per vertex (ke, pos, dir).
int
run_vertices(int argc, char** argv) {
    if (argc < 16) return 2;
    const char* out  = argv[2];
    const long  n    = std::atol(argv[3]);
    const int   seed = std::atoi(argv[4]);
    const bool  gaus = std::atoi(argv[5]) != 0;
    std::array<float, 3> pos  = { std::stof(argv[6]), std::stof(argv[7]), std::stof(argv[8]) };
    std::array<float, 2> size = { std::stof(argv[9]), std::stof(argv[10]) };
    const float energy        = std::stof(argv[11]);
    std::array<float, 4> ang  = { std::stof(argv[12]), std::stof(argv[13]), std::stof(argv[14]), std::stof(argv[15]) };
    mqi::coordinate_transform<float> p_coord(ang, { 0, 0, 0 });
    mqi::vec3<float>                 dir(0, 0, -1);
    std::array<float, 6> mean = { pos[0], pos[1], pos[2], dir.x, dir.y, dir.z };
    std::array<float, 6> sigm = { size[0], size[1], 0, 0, 0, 0 };
    std::array<float, 2> corr = { 0.0, 0.0 };
    mqi::pdf_Md<float, 6>* phsp;
    if (gaus) phsp = new mqi::phsp_6d<float>(mean, sigm, corr);
    else phsp = new mqi::phsp_6d_uniform<float>(mean, sigm, corr);
    auto* e = new mqi::const_1d<float>({ energy }, { 0.0f });
    mqi::beamsource<float> src;
    src.append_beamlet(mqi::beamlet<float>(e, phsp), static_cast<size_t>(n), p_coord);
    std::default_random_engine rng;
    rng.seed(seed);
    std::vector<float> v;
    v.reserve(7 * n);
    for (long i = 0; i < n; ++i) {
        auto             bl = src(i);
        mqi::vertex_t<float> x = bl(&rng);
        v.insert(v.end(), { x.ke, x.pos.x, x.pos.y, x.pos.z, x.dir.x, x.dir.y, x.dir.z });
    }
    std::ofstream fout(out, std::ios::binary);
    write_vec(fout, v);
    return 0;
}

/// Dij table replay: the recorded insertions of a GPU run, in the order they were made, go
/// through the reference's own insert_hashtable (CPU branch, mqi_transport.hpp:68-111) into a
/// scorer's key_value table (init_table, mqi_hash_table.hpp), which the reference's
/// save_to_npz (mqi_io.hpp:249-320) then writes.  Arguments: hits.bin (vec<u32> voxel,
/// vec<u32> spot, vec<f64> value) capacity n_spots nx ny nz scale out_dir name.
int
run_dij(int argc, char** argv) {
    if (argc < 11) return 2;
    std::ifstream fin(argv[2], std::ios::binary);
    const std::vector<uint32_t> vox  = read_vec<uint32_t>(fin);
    const std::vector<uint32_t> spot = read_vec<uint32_t>(fin);
    const std::vector<double>   val  = read_vec<double>(fin);
    if (!fin || vox.size() != spot.size() || vox.size() != val.size()) return 3;
    const uint32_t cap     = static_cast<uint32_t>(std::stoul(argv[3]));
    const uint32_t n_spots = static_cast<uint32_t>(std::stoul(argv[4]));
    const mqi::vec3<mqi::ijk_t> dim(std::atoi(argv[5]), std::atoi(argv[6]), std::atoi(argv[7]));
    const float scale = std::stof(argv[8]);
    mqi::scorer<float> sc("Dij", cap, nullptr);
    sc.data_ = new mqi::key_value[cap];
    mqi::init_table(sc.data_, cap);
    for (size_t i = 0; i < vox.size(); ++i) mc::insert_hashtable<float>(sc.data_, vox[i], spot[i], val[i], 0, cap);
    mqi::io::save_to_npz<float>(&sc, scale, argv[9], argv[10], dim, n_spots);
    return 0;
}

/// Scorer callbacks on given step states: the reference's own fp_compute_hit functions
/// (moqui/base/scorers/mqi_scorer_energy_deposit.hpp:12-177) over a grid3d of the given edges and
/// densities with the patient material's stopping-power ratio.  Input: vec<i32> {nx, ny, nz},
/// vec<f32> xe, ye, ze, rho, vec<f32> steps (9 per step: vtx0.ke, dE, local_dE, vtx0.pos, vtx1.pos),
/// vec<u32> cnb, vec<i32> primary.  Output: ten vec<f64>, in the order energy_deposit,
/// energy_deposit_primary, energy_deposit_secondary, dose_to_water, dose_to_water_square,
/// dose_to_medium, LETd_weight1, LETd_weight2, LETt_weight1, LETt_weight2.
int
run_hits(const char* in_path, const char* out_path) {
    std::ifstream fin(in_path, std::ios::binary);
    const auto dims  = read_vec<int32_t>(fin);
    const auto xe    = read_vec<float>(fin);
    const auto ye    = read_vec<float>(fin);
    const auto ze    = read_vec<float>(fin);
    auto       rho   = read_vec<float>(fin);
    const auto steps = read_vec<float>(fin);
    const auto cnb   = read_vec<uint32_t>(fin);
    const auto prim  = read_vec<int32_t>(fin);
    if (!fin || dims.size() != 3) return 3;
    mqi::grid3d<mqi::density_t, float> geo(xe.data(), dims[0] + 1, ye.data(), dims[1] + 1, ze.data(), dims[2] + 1);
    geo.set_data(rho.data());
    mqi::patient_material_t<float> pm;
    mqi::material_t<float>*        mat = &pm;
    using fn_t = double (*)(const mqi::track_t<float>&, const mqi::cnb_t&, mqi::grid3d<mqi::density_t, float>&,
                            mqi::material_t<float>*&);
    const fn_t fns[10] = { mqi::energy_deposit<float>, mqi::energy_deposit_primary<float>,
                           mqi::energy_deposit_secondary<float>, mqi::dose_to_water<float>,
                           mqi::dose_to_water_square<float>, mqi::dose_to_medium<float>, mqi::LETd_weight1<float>,
                           mqi::LETd_weight2<float>, mqi::LETt_weight1<float>, mqi::LETt_weight2<float> };
    std::ofstream fout(out_path, std::ios::binary);
    for (const fn_t f : fns) {
        std::vector<double> out(cnb.size());
        for (size_t i = 0; i < cnb.size(); ++i) {
            const float*        st = &steps[9 * i];
            mqi::track_t<float> t;
            t.vtx0.ke  = st[0];
            t.dE       = st[1];
            t.local_dE = st[2];
            t.vtx0.pos = mqi::vec3<float>(st[3], st[4], st[5]);
            t.vtx1.pos = mqi::vec3<float>(st[6], st[7], st[8]);
            t.primary  = prim[i] != 0;
            const mqi::cnb_t c = cnb[i];
            out[i]             = f(t, c, geo, mat);
        }
        write_vec(fout, out);
    }
    return 0;
}

/// roi_t::idx and roi_t::get_mask_idx (moqui/base/mqi_roi.hpp:47-71, 87-160) of given voxels.
/// Input: vec<i32> {method, original length}, vec<u32> start, stride, acc, voxels.  Output:
/// vec<i32> idx, vec<i32> mask_idx.
int
run_roi(const char* in_path, const char* out_path) {
    std::ifstream fin(in_path, std::ios::binary);
    const auto hdr    = read_vec<int32_t>(fin);
    auto       start  = read_vec<uint32_t>(fin);
    auto       stride = read_vec<uint32_t>(fin);
    auto       acc    = read_vec<uint32_t>(fin);
    const auto vox    = read_vec<uint32_t>(fin);
    if (!fin || hdr.size() != 2) return 3;
    const auto method = static_cast<mqi::roi_mapping_t>(hdr[0]);
    const int32_t len = static_cast<int32_t>(start.size());
    mqi::roi_t roi(method, static_cast<uint32_t>(hdr[1]), len, start.data(), stride.empty() ? nullptr : stride.data(),
                   acc.empty() ? nullptr : acc.data());
    std::vector<int32_t> idx(vox.size()), mask(vox.size());
    for (size_t i = 0; i < vox.size(); ++i) {
        idx[i]  = roi.idx(vox[i]);
        mask[i] = roi.get_mask_idx(vox[i]);
    }
    std::ofstream fout(out_path, std::ios::binary);
    write_vec(fout, idx);
    write_vec(fout, mask);
    return 0;
}

}   // namespace

void
on_fatal_signal(int sig) {
    void* frames[64];
    const int n = backtrace(frames, 64);
    const char msg[] = "ref_driver: fatal signal, backtrace:\n";
    (void) !write(2, msg, sizeof(msg) - 1);
    backtrace_symbols_fd(frames, n, 2);
    std::signal(sig, SIG_DFL);
    std::raise(sig);
}

int
main(int argc, char** argv) {
    std::signal(SIGSEGV, on_fatal_signal);
    std::signal(SIGABRT, on_fatal_signal);
    if (argc < 2) {
        std::fprintf(stderr, "usage: %s phantom|raywalk|physics|sample ...\n", argv[0]);
        return 2;
    }
    const std::string mode = argv[1];
    if (mode == "phantom") return run_phantom(argc, argv);
    if (mode == "raywalk" && argc >= 4) return run_raywalk(argv[2], argv[3]);
    if (mode == "physics" && argc >= 3) return run_physics(argv[2]);
    if (mode == "vertices") return run_vertices(argc, argv);
    if (mode == "dij") return run_dij(argc, argv);
    if (mode == "hits" && argc >= 4) return run_hits(argv[2], argv[3]);
    if (mode == "roi" && argc >= 4) return run_roi(argv[2], argv[3]);
    if (mode == "sample" && argc >= 5)
        return run_sample(argv[2], std::atol(argv[3]), static_cast<unsigned>(std::atol(argv[4])));
    std::fprintf(stderr, "bad arguments\n");
    return 2;
}
