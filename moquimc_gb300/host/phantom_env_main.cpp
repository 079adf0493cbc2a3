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
#include "mqi_host.hpp"

namespace
{

using namespace mqi_host;

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
    write_outputs(out_dir, "0_water_dE_total", fmt, dose, 1.0, xe, ye, ze);
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
