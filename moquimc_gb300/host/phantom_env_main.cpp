// phantom_env on the GB300 engine: the command-line driver of moqui's water-phantom example
// (moqui/base/environments/mqi_phantom_env.hpp:37-428, tests/mc/phantom) rebuilt over the C ABI
// of libmqigpu.so.  The options, defaults, beam model and output files are the reference's:
//
//   --lxyz Lx Ly Lz        phantom size, mm                     (default 512 512 400)
//   --pxyz Px Py Pz        phantom centre, mm                   (default -256 0 0)
//   --nxyz Nx Ny Nz        voxels                               (default 512 512 200)
//   --spot_position X Y Z  beam-frame spot position, mm         (default 1 0 0)
//   --spot_size Sx Sy      half-widths of the uniform spot, mm  (default 0 0)
//   --spot_energy E dE     energy, MeV (dE unused: const_1d)    (default 230 0)
//   --spot_angles C G P I  collimator, gantry, couch, iec2dicom (default 0 0 0 0)
//   --histories N                                               (default 10000)
//   --phantom_path FILE    int16 HU volume, x fastest           (required)
//   --output_prefix DIR                                         (required)
//   --output_format raw|mhd|mha                                 (default raw)
//   --random_seed S        beam sampling and transport seed     (default: clock)
//   --gpu_id G                                                  (default 0)
//   --threads T [B]        accepted; the engine sizes its own launches
//
// Additions: --beam uniform|gaussian (phsp_6d_uniform as the example, or the Gaussian phsp_6d
// with sigma = --spot_size), --physics debug|release (the example is built with
// -D__PHYSICS_DEBUG__: debug is the default), --json FILE (a run record), --dump_vertices FILE
// (write the sampled source vertices, 7 floats each, and exit before any GPU work).
//
// The source vertices are drawn on the host exactly as phantom_env::setup_beamsource draws them:
// std::default_random_engine seeded with the random seed, the phase-space distribution's draws in
// its order, then the beamlet's coordinate transform.  The dose is written as
// <output_prefix>/0_water_dE_total.{raw,mhd,mha} (x_environment::save_reshaped_files).
#include <array>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iomanip>
#include <map>
#include <random>
#include <stdexcept>
#include <string>
#include <vector>

#include "mqi_gpu.h"

namespace
{

/// moqui's cli: "--name v1 v2 ..." (moqui/base/mqi_cli.hpp).
class Cli
{
public:
    Cli(int argc, char** argv) {
        std::string key;
        for (int i = 1; i < argc; ++i) {
            const std::string a = argv[i];
            if (a.size() > 2 && a[0] == '-' && a[1] == '-' && !is_number(a)) {
                key = a;
                opts_[key];
            } else if (!key.empty()) {
                opts_[key].push_back(a);
            } else {
                throw std::runtime_error("unexpected argument " + a);
            }
        }
    }
    const std::vector<std::string>&
    operator[](const std::string& k) const {
        static const std::vector<std::string> none;
        auto it = opts_.find(k);
        return it == opts_.end() ? none : it->second;
    }

private:
    static bool
    is_number(const std::string& s) {
        char* end = nullptr;
        std::strtod(s.c_str(), &end);
        return end && *end == '\0';
    }
    std::map<std::string, std::vector<std::string>> opts_;
};

struct Mat3 {
    float m[9] = { 1, 0, 0, 0, 1, 0, 0, 0, 1 };
};

/// mat3x3<float>(a, b, c): identity, then rotations about x, y and z in that order, each applied
/// as the reference's rotate_x/_y/_z updates (moqui/base/mqi_matrix.hpp:69-76, 213-272).
Mat3
euler(float a, float b, float c) {
    Mat3 r;
    float& xx = r.m[0]; float& xy = r.m[1]; float& xz = r.m[2];
    float& yx = r.m[3]; float& yy = r.m[4]; float& yz = r.m[5];
    float& zx = r.m[6]; float& zy = r.m[7]; float& zz = r.m[8];
    if (a != 0) {
        const float c1 = std::cos(a), s1 = std::sin(a);
        const float x1 = yx, y1 = yy, z1 = yz;
        yx = c1 * x1 - s1 * zx; yy = c1 * y1 - s1 * zy; yz = c1 * z1 - s1 * zz;
        zx = s1 * x1 + c1 * zx; zy = s1 * y1 + c1 * zy; zz = s1 * z1 + c1 * zz;
    }
    if (b != 0) {
        const float c1 = std::cos(b), s1 = std::sin(b);
        const float x1 = zx, y1 = zy, z1 = zz;
        zx = c1 * x1 - s1 * xx; zy = c1 * y1 - s1 * xy; zz = c1 * z1 - s1 * xz;
        xx = s1 * x1 + c1 * xx; xy = s1 * y1 + c1 * xy; xz = s1 * z1 + c1 * xz;
    }
    if (c != 0) {
        const float c1 = std::cos(c), s1 = std::sin(c);
        const float x1 = xx, y1 = xy, z1 = xz;
        xx = c1 * x1 - s1 * yx; xy = c1 * y1 - s1 * yy; xz = c1 * z1 - s1 * yz;
        yx = s1 * x1 + c1 * yx; yy = s1 * y1 + c1 * yy; yz = s1 * z1 + c1 * yz;
    }
    return r;
}

Mat3
mul(const Mat3& a, const Mat3& b) {
    Mat3 r;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
            r.m[3 * i + j] = a.m[3 * i] * b.m[j] + a.m[3 * i + 1] * b.m[3 + j] + a.m[3 * i + 2] * b.m[6 + j];
    return r;
}

/// coordinate_transform: rotation = iec2dicom * couch * gantry * collimator
/// (moqui/base/mqi_coordinate_transform.hpp:52-58).
Mat3
beam_rotation(const std::array<float, 4>& ang) {
    const float d2r = (float) (3.14159265358979323846 / 180.0);   // coordinate_transform::deg2rad
    const Mat3 col = euler(0, 0, ang[0] * d2r);
    const Mat3 gan = euler(0, ang[1] * d2r, 0);
    const Mat3 cou = euler(0, 0, ang[2] * d2r);
    const Mat3 iec = euler(ang[3] * d2r, 0, 0);
    return mul(mul(mul(iec, cou), gan), col);
}

/// grid3d's uniform edges from phantom_env::setup_world's corners (mqi_phantom_env.hpp:256-264):
/// corners pos -/+ 0.5 l in double stored as float, then edge_i = min + i * ((max - min) / n).
std::vector<float>
edges(float pos, float len, int n) {
    const float lo = (float) (pos - 0.5 * len);
    const float hi = (float) (pos + 0.5 * len);
    const float d  = (hi - lo) / (float) n;
    std::vector<float> e(n + 1);
    for (int i = 0; i <= n; ++i) e[i] = lo + (float) i * d;
    return e;
}

float
to_f(const std::vector<std::string>& v, size_t i, float dflt) {
    return v.size() > i ? std::stof(v[i]) : dflt;
}

void
write_outputs(const std::string& dir, const std::string& name, const std::string& fmt, const std::vector<double>& d,
              const std::vector<float>& xe, const std::vector<float>& ye, const std::vector<float>& ze) {
    const int   nx = (int) xe.size() - 1, ny = (int) ye.size() - 1, nz = (int) ze.size() - 1;
    const float dx = xe[1] - xe[0], dy = ye[1] - ye[0], dz = ze[1] - ze[0];
    const float x0 = xe[0] + dx * 0.5f, y0 = ye[0] + dy * 0.5f, z0 = ze[0] + dz * 0.5f;
    if (fmt == "mha") {
        std::ofstream f(dir + "/" + name + ".mha", std::ios::binary);
        f << "ObjectType = Image\nNDims = 3\nBinaryData = True\nBinaryDataByteOrderMSB = False\n"
          << "CompressedData = False\nTransformMatrix = 1 0 0 0 1 0 0 0 1\n"
          << "Origin = " << std::setprecision(9) << x0 << " " << y0 << " " << z0 << "\n"
          << "CenterOfRotation = 0 0 0\nAnatomicOrientation = RAI\n"
          << "DimSize = " << nx << " " << ny << " " << nz << "\nElementType = MET_DOUBLE\nHeaderSize = -1\n"
          << "ElementSpacing = " << std::setprecision(9) << dx << " " << dy << " " << dz << "\n"
          << "ElementDataFile = LOCAL\n";
        f.write(reinterpret_cast<const char*>(d.data()), d.size() * sizeof(double));
        if (!f) throw std::runtime_error("cannot write " + dir + "/" + name + ".mha");
        return;
    }
    if (fmt == "mhd") {
        std::ofstream h(dir + "/" + name + ".mhd");
        h << "ObjectType = Image\nNDims = 3\nBinaryData = True\nBinaryDataByteOrderMSB = False\n"
          << "CompressedData = False\nTransformMatrix 1 0 0 0 1 0 0 0 1\n"
          << "Offset " << x0 << " " << y0 << " " << z0 << "\nCenterOfRotation 0 0 0\n"
          << "AnatomicOrientation = RAI\nDimSize = " << nx << " " << ny << " " << nz << "\n"
          << "ElementType = MET_DOUBLE\nElementSpacing = " << dx << " " << dy << " " << dz << "\n"
          << "ElementDataFile = " << name << ".raw\n";
        if (!h) throw std::runtime_error("cannot write " + dir + "/" + name + ".mhd");
    }
    std::ofstream r(dir + "/" + name + ".raw", std::ios::binary);
    r.write(reinterpret_cast<const char*>(d.data()), d.size() * sizeof(double));
    if (!r) throw std::runtime_error("cannot write " + dir + "/" + name + ".raw");
}

/// The beam source of setup_beamsource (mqi_phantom_env.hpp:204-232): std::default_random_engine
/// seeded with the random seed; per history the phase-space draws Ux Vx Uy Vy Uz in the
/// distribution's order (phsp_6d_uniform: U(-1, 1), mqi_phsp6d_uniform.hpp:64-78; phsp_6d: N(0, 1),
/// mqi_phsp6d.hpp:61-79), position = mean + size * U on x/y, direction (0, 0, -1), constant
/// energy, then pos = R p and dir = R d (beamlet::operator(), mqi_beamlet.hpp:80-90).
std::vector<mqi_vertex>
sample_vertices(uint64_t n, int seed, bool gaussian, const std::array<float, 3>& spot_pos,
                const std::array<float, 2>& spot_size, float energy, const std::array<float, 4>& ang) {
    std::default_random_engine beam_rng;
    beam_rng.seed(seed);
    const Mat3 R = beam_rotation(ang);
    std::vector<mqi_vertex> v(n);
    std::uniform_real_distribution<float> uni(-1.0f, 1.0f);
    std::normal_distribution<float>       nrm(0.0f, 1.0f);
    for (uint64_t i = 0; i < n; ++i) {
        float u[5];
        for (float& x : u) x = gaussian ? nrm(beam_rng) : uni(beam_rng);
        const float Ux = u[0], Uy = u[2];
        const float p[3] = { spot_pos[0] + spot_size[0] * Ux, spot_pos[1] + spot_size[1] * Uy, spot_pos[2] };
        const float d[3] = { 0.0f, 0.0f, -1.0f };
        mqi_vertex& x = v[i];
        x.ke = energy;
        for (int r = 0; r < 3; ++r) {
            x.pos[r] = R.m[3 * r] * p[0] + R.m[3 * r + 1] * p[1] + R.m[3 * r + 2] * p[2] + 0.0f;   // + translation
            x.dir[r] = R.m[3 * r] * d[0] + R.m[3 * r + 1] * d[1] + R.m[3 * r + 2] * d[2];
        }
    }
    return v;
}

void
check(int rc, mqi_ctx* ctx, const char* what) {
    if (rc != MQI_OK) throw std::runtime_error(std::string(what) + ": " + mqi_last_error(ctx));
}

int
run(const Cli& cli) {
    const int gpu_id = cli["--gpu_id"].empty() ? 0 : std::stoi(cli["--gpu_id"][0]);
    const auto& L = cli["--lxyz"];
    const auto& Pp = cli["--pxyz"];
    const auto& Nn = cli["--nxyz"];
    const float lx = to_f(L, 0, 512.0f), ly = to_f(L, 1, 512.0f), lz = to_f(L, 2, 400.0f);
    const float px = Pp.empty() ? -256.0f : to_f(Pp, 0, 0), py = to_f(Pp, 1, 0.0f), pz = to_f(Pp, 2, 0.0f);
    const int   nx = Nn.empty() ? 512 : std::stoi(Nn[0]), ny = Nn.empty() ? 512 : std::stoi(Nn[1]),
              nz = Nn.empty() ? 200 : std::stoi(Nn[2]);
    const auto& SP = cli["--spot_position"];
    const std::array<float, 3> spot_pos = { SP.empty() ? 1.0f : to_f(SP, 0, 0), to_f(SP, 1, 0.0f), to_f(SP, 2, 0.0f) };
    const std::array<float, 2> spot_size = { to_f(cli["--spot_size"], 0, 0.0f), to_f(cli["--spot_size"], 1, 0.0f) };
    const float energy = to_f(cli["--spot_energy"], 0, 230.0f);
    const auto& SA = cli["--spot_angles"];
    const std::array<float, 4> ang = { to_f(SA, 0, 0), to_f(SA, 1, 0), to_f(SA, 2, 0), to_f(SA, 3, 0) };
    const uint64_t n_hist = cli["--histories"].empty() ? 10000 : std::stoull(cli["--histories"][0]);
    if (cli["--output_prefix"].empty()) throw std::runtime_error("output_path is required.");
    if (cli["--phantom_path"].empty()) throw std::runtime_error("phantom_path is required.");
    const std::string out_dir = cli["--output_prefix"][0];
    const std::string ph_path = cli["--phantom_path"][0];
    const std::string fmt     = cli["--output_format"].empty() ? "raw" : cli["--output_format"][0];
    const int seed = cli["--random_seed"].empty()
                       ? (int) std::chrono::system_clock::now().time_since_epoch().count()
                       : std::stoi(cli["--random_seed"][0]);
    const bool gaussian = !cli["--beam"].empty() && cli["--beam"][0] == "gaussian";
    const bool debug    = cli["--physics"].empty() || cli["--physics"][0] != "release";

    const uint64_t nvox = (uint64_t) nx * ny * nz;
    const std::vector<float> xe = edges(px, lx, nx), ye = edges(py, ly, ny), ze = edges(pz, lz, nz);
    const std::vector<mqi_vertex> v = sample_vertices(n_hist, seed, gaussian, spot_pos, spot_size, energy, ang);
    if (!cli["--dump_vertices"].empty()) {
        std::ofstream f(cli["--dump_vertices"][0], std::ios::binary);
        f.write(reinterpret_cast<const char*>(v.data()), v.size() * sizeof(mqi_vertex));
        return f ? 0 : 1;
    }

    // ---- world: one phantom child with the HU volume
    std::vector<int16_t> hu(nvox);
    {
        std::ifstream f(ph_path, std::ios::binary);
        if (!f) throw std::runtime_error("cannot open phantom " + ph_path);
        f.read(reinterpret_cast<char*>(hu.data()), nvox * sizeof(int16_t));
        if ((uint64_t) f.gcount() != nvox * sizeof(int16_t)) throw std::runtime_error("phantom file is too short");
    }
    mqi_ctx* ctx = nullptr;
    check(mqi_create(gpu_id, &ctx), nullptr, "mqi_create");
    int child = -1, scorer = -1;
    check(mqi_set_physics(ctx, debug ? 1 : 0, 1), ctx, "mqi_set_physics");
    check(mqi_add_child(ctx, nx, ny, nz, xe.data(), ye.data(), ze.data(), nullptr, nullptr, &child), ctx, "mqi_add_child");
    check(mqi_set_hu(ctx, child, hu.data(), 1.0f, 0), ctx, "mqi_set_hu");
    check(mqi_add_scorer(ctx, child, MQI_SCORER_DOSE_W, MQI_ROI_DIRECT, 0, nullptr, nullptr, nullptr, &scorer), ctx,
          "mqi_add_scorer");

    check(mqi_set_vertices(ctx, v.data(), nullptr, n_hist, 0), ctx, "mqi_set_vertices");

    // ---- run
    const auto t0 = std::chrono::steady_clock::now();
    check(mqi_transport(ctx, 0, n_hist, (uint64_t) (uint32_t) seed), ctx, "mqi_transport");
    const auto t1 = std::chrono::steady_clock::now();
    const double secs = std::chrono::duration<double>(t1 - t0).count();
    mqi_stats st{};
    check(mqi_get_stats(ctx, &st), ctx, "mqi_get_stats");
    std::printf("Number of particles tracked %llu\n", (unsigned long long) st.histories);
    std::printf("Run done %f s\n", secs);

    // ---- outputs: 0_water_dE_total
    std::vector<double> dose(nvox);
    uint64_t n_out = 0;
    check(mqi_get_tally(ctx, scorer, dose.data(), &n_out, 0), ctx, "mqi_get_tally");
    write_outputs(out_dir, "0_water_dE_total", fmt, dose, xe, ye, ze);
    if (!cli["--json"].empty()) {
        std::ofstream j(cli["--json"][0]);
        j << "{\"transport_seconds\": " << secs << ", \"histories\": " << n_hist << ", \"tracked\": " << st.histories
          << ", \"steps\": " << st.steps << ", \"physics_debug\": " << (debug ? 1 : 0) << "}\n";
    }
    mqi_destroy(ctx);
    return 0;
}

}   // namespace

int
main(int argc, char** argv) {
    try {
        return run(Cli(argc, argv));
    } catch (const std::exception& e) {
        std::fprintf(stderr, "phantom_env: %s\n", e.what());
        return 1;
    }
}
