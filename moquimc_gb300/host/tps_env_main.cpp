// tps_env on the GB300 engine: moqui's treatment-planning environment (moqui/base/environments/
// mqi_tps_env.hpp) driven by its own input file, over the C ABI of libmqigpu.so, with the CT and the
// beams read from plain files where tps_env reads a DICOM directory.
//
//   tps_env <input file> --ct <int16 HU raw, x fastest> --ct_nxyz NX NY NZ --ct_lxyz LX LY LZ
//           --ct_pxyz PX PY PZ --beams <beams file> [--json <run record>]
//
// The input file follows mqi::file_parser (moqui/base/mqi_file_handler.hpp:220-420) and tps_env's
// keys and defaults (mqi_tps_env.hpp:155-360): GPUID, RandomSeed, Scorer (Dose, LETd, LETt, Dij;
// EnergyDeposition and TrackLength create no scorer, as in tps_env), SimulationType,
// ParticlesPerHistory, UnitWeights, RBE, NumberOfFraction, RangeshifterDensity, Machine
// (PBS:<beam model file>, read as pbs::load_beamdata reads it), Calibration (default),
// DensityScaling, XShift/YShift/ZShift, OutputDir, OutputFormat (raw, mhd, mha), OverwriteResults,
// StoppingStatistics, StoppingCriteria (percent), StatThreshold, BeamNumbers, MaxHistoriesPerBatch.
// Outputs: <OutputDir>/<beam>_<child>_<scorer>.{raw,mhd,mha} scaled by ParticlesPerHistory x RBE x
// NumberOfFraction (save_reshaped_files, :1851-1900); a Dij (scored alone, as tps_env requires) as
// <beam>_<child>_Dij.npz, the spot-row CSR of save_to_npz (moqui/base/mqi_io.hpp:251-320) with the
// same scale.
//
// Beams file, one item per line ('#' comments):
//   beam <name> <gantry> <couch> <collimator> <iso x> <iso y> <iso z> <source-to-isocentre mm>
//   spot <nominal E MeV> <x mm> <y mm> <meterset>           (spots of the last beam)
//   rangeshifter <lo x y z> <hi x y z>                      (beam frame; RangeshifterDensity)
//   aperture <cx cy cz> <vx vy vz> <n> <x1 y1 ... xn yn>     (beam frame; one opening, 1 mm voxels)
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <ctime>
#include <fstream>
#include <map>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>
#include <strings.h>
#include <sys/stat.h>

#include "mqi_gpu.h"
#include "mqi_host.hpp"

namespace
{

using namespace mqi_host;


/// The generic PBS beam model (mqi_treatment_machine_pbs.hpp): load_beamdata's geometry and spot
/// sections, and characterize_beamlet / characterize_history for MODULATED spots, in FP32.
struct Machine {
    struct Row {
        float E, dE, x, y, xp, yp, ratio;
    };
    std::map<float, Row> rows;
    float                sad[2] = { INFINITY, INFINITY };

    explicit Machine(const std::string& path) {
        std::ifstream f(path);
        if (!f) throw std::runtime_error("cannot open beam model " + path);
        std::string line, section;
        while (std::getline(f, line)) {
            line = trim(line.substr(0, line.find('#')));
            if (line.empty()) continue;
            if (line.front() == '[' && line.back() == ']') {
                section = line;
                continue;
            }
            std::istringstream in(line);
            if (section == "[geometry]") {
                std::string key;
                float       a = 0, b = 0;
                in >> key >> a >> b;
                if (key == "SAD(mm)") {
                    sad[0] = a == 0 ? INFINITY : a;
                    sad[1] = b == 0 ? INFINITY : b;
                }
            } else if (section == "[spot]") {
                float e;
                Row   r;
                in >> e >> r.E >> r.dE >> r.x >> r.y >> r.xp >> r.yp >> r.ratio;
                rows[e] = r;
            }
        }
        if (rows.size() < 2) throw std::runtime_error("beam model " + path + " needs at least two spot rows");
    }
    static float
    intpl(float x, float x0, float x1, float y0, float y1) {
        return (x1 == x0) ? y0 : y0 + (x - x0) * (y1 - y0) / (x1 - x0);
    }
    void
    bracket(float e, std::map<float, Row>::const_iterator& down, std::map<float, Row>::const_iterator& up) const {
        up = rows.lower_bound(e);
        if (up == rows.begin() || up == rows.end()) throw std::runtime_error("spot energy outside the beam model");
        down = std::prev(up);
    }
    mqi_spot
    spot(float e, float x, float y, float sid, const float rot[9], const float iso[3]) const {
        std::map<float, Row>::const_iterator d, u;
        bracket(e, d, u);
        const Row& D = d->second;
        const Row& U = u->second;
        mqi_spot s{};
        s.energy       = intpl(e, d->first, u->first, D.E, U.E);
        s.energy_sigma = intpl(e, D.E, U.E, D.dE, U.dE);
        // beam_starting_position (mqi_treatment_machine_ion.hpp:324-333); an infinite SAD is a
        // parallel beam
        float b[3] = { x, y, sid };
        for (int a = 0; a < 2; ++a)
            if (std::isfinite(sad[a])) b[a] = (a == 0 ? x : y) * (sad[a] - sid) / sad[a];
        float dir[3] = { x - b[0], y - b[1], 0.0f - b[2] };
        const float n = std::sqrt(dir[0] * dir[0] + dir[1] * dir[1] + dir[2] * dir[2]);
        for (float& c : dir) c /= n;
        const float m[5] = { b[0], b[1], b[2], dir[0], dir[1] };
        const float sg[5] = { intpl(e, D.E, U.E, D.x, U.x), intpl(e, D.E, U.E, D.y, U.y), 0.0f,
                              intpl(e, D.E, U.E, D.xp, U.xp), intpl(e, D.E, U.E, D.yp, U.yp) };
        std::memcpy(s.mean, m, sizeof(m));
        std::memcpy(s.sigma, sg, sizeof(sg));
        std::memcpy(s.rot, rot, 9 * sizeof(float));
        std::memcpy(s.trans, iso, 3 * sizeof(float));
        return s;
    }
    uint64_t
    histories(float e, float meterset, float scale) const {
        std::map<float, Row>::const_iterator d, u;
        bracket(e, d, u);
        const float ratio = intpl(e, d->first, u->first, d->second.ratio, u->second.ratio);
        return (uint64_t) (meterset * ratio / scale);
    }
};

struct Device {
    std::string        kind;
    float              a[6] = { 0, 0, 0, 0, 0, 0 };
    std::vector<float> poly;   // aperture opening, x y pairs relative to the centre
};

struct Beam {
    std::string                       name;
    float                             gantry = 0, couch = 0, collimator = 0, iso[3] = { 0, 0, 0 }, sid = 390;
    std::vector<std::array<float, 4>> spots;
    std::vector<Device>               devices;
};

std::vector<Beam>
read_beams(const std::string& path) {
    std::ifstream f(path);
    if (!f) throw std::runtime_error("cannot open beams file " + path);
    std::vector<Beam> beams;
    std::string       line;
    while (std::getline(f, line)) {
        line = trim(line.substr(0, line.find('#')));
        if (line.empty()) continue;
        std::istringstream in(line);
        std::string        what;
        in >> what;
        if (what == "beam") {
            Beam b;
            in >> b.name >> b.gantry >> b.couch >> b.collimator >> b.iso[0] >> b.iso[1] >> b.iso[2] >> b.sid;
            beams.push_back(b);
            continue;
        }
        if (beams.empty()) throw std::runtime_error("beams file: '" + what + "' before any beam");
        if (what == "spot") {
            std::array<float, 4> s{};
            in >> s[0] >> s[1] >> s[2] >> s[3];
            beams.back().spots.push_back(s);
        } else if (what == "rangeshifter" || what == "aperture") {
            Device d;
            d.kind = what;
            for (float& v : d.a) in >> v;
            if (what == "aperture") {
                int n = 0;
                in >> n;
                d.poly.resize(2 * n);
                for (float& v : d.poly) in >> v;
            }
            beams.back().devices.push_back(d);
        } else {
            throw std::runtime_error("beams file: unknown item '" + what + "'");
        }
    }
    return beams;
}

/// tps_env::sol1_1 (mqi_tps_env.hpp:1753-1770): crossing-number point-in-polygon test.
bool
inside(float px, float py, const std::vector<float>& poly, float cx, float cy) {
    const int n = (int) poly.size() / 2;
    int       c = 0;
    for (int i = 0, j = n - 1; i < n; j = i++) {
        const float x0 = poly[2 * i] + cx, y0 = poly[2 * i + 1] + cy;
        const float x1 = poly[2 * j] + cx, y1 = poly[2 * j + 1] + cy;
        if ((((y0 <= py) && (py < y1)) || ((y1 <= py) && (py < y0))) && (px < (x1 - x0) * (py - y0) / (y1 - y0) + x0))
            c = !c;
    }
    return c != 0;
}

/// Add a beamline device as a child in the beam frame (create_rangeshifter,
/// create_voxelized_aperture: mqi_tps_env.hpp:1605-1737).
void
add_device(mqi_ctx* ctx, const Device& d, const Mat3& R, const float iso[3], float rs_density) {
    int cid = -1;
    if (d.kind == "rangeshifter") {
        const float xe[2] = { d.a[0], d.a[3] }, ye[2] = { d.a[1], d.a[4] }, ze[2] = { d.a[2], d.a[5] };
        check(mqi_add_child(ctx, 1, 1, 1, xe, ye, ze, R.m, iso, &cid), ctx, "mqi_add_child (range shifter)");
        const float rho = (float) (rs_density * 1e-3);
        check(mqi_set_density(ctx, cid, &rho, 0), ctx, "mqi_set_density");
        return;
    }
    int   n[3];
    std::vector<float> e[3];
    for (int a = 0; a < 3; ++a) {
        n[a] = (int) std::ceil(d.a[3 + a] / 1.0f);
        e[a].resize(n[a] + 1);
        for (int i = 0; i <= n[a]; ++i) e[a][i] = (d.a[a] - d.a[3 + a] / 2) + i * 1.0f;
    }
    std::vector<float> rho((size_t) n[0] * n[1] * n[2]);
    for (int i = 0; i < n[0]; ++i) {
        const float px = e[0][i] + 1.0f * 0.5;
        for (int j = 0; j < n[1]; ++j) {
            const float py   = e[1][j] + 1.0f * 0.5;
            const bool  open = inside(px, py, d.poly, d.a[0], d.a[1]);
            for (int k = 0; k < n[2]; ++k) rho[(size_t) k * n[0] * n[1] + (size_t) j * n[0] + i] = open ? 1e-8f : 100.0f;
        }
    }
    check(mqi_add_child(ctx, n[0], n[1], n[2], e[0].data(), e[1].data(), e[2].data(), R.m, iso, &cid), ctx,
          "mqi_add_child (aperture)");
    check(mqi_set_density(ctx, cid, rho.data(), 0), ctx, "mqi_set_density");
}

int
run(const std::string& input, const Cli& cli) {
    const InputFile p(input);
    const int       gpu_id = p.get_int("GPUID", 0);
    int             seed   = p.get_int("RandomSeed", -1);
    if (seed == -1) seed = (int) std::time(nullptr);
    std::vector<std::string> scorers = p.get_vector("Scorer", ',');
    const bool score_dij = std::any_of(scorers.begin(), scorers.end(),
                                       [](const std::string& s) { return strcasecmp(s.c_str(), "Dij") == 0; });
    if (score_dij && scorers.size() > 1) throw std::runtime_error("Dij cannot be scored with the other quantities");
    for (const auto& s : scorers) {
        static const char* known[] = { "Dose", "LETd", "LETt", "EnergyDeposition", "TrackLength", "Dij" };
        if (std::none_of(std::begin(known), std::end(known), [&](const char* k) { return strcasecmp(k, s.c_str()) == 0; }))
            throw std::runtime_error("Unrecognized scorer name");
    }
    const bool  per_spot   = strcasecmp(p.get_string("SimulationType", "perBeam").c_str(), "perSpot") == 0;
    const float pph        = p.get_float("ParticlesPerHistory", -1.0f);
    const float rbe        = p.get_float("RBE", 1.1f);
    int         fractions  = p.get_int("NumberOfFraction", -1);
    const float rs_density = p.get_float("RangeshifterDensity", 1.19f);
    const int   unit_w     = p.get_int("UnitWeights", -1);
    const float dens_scale = p.get_float("DensityScaling", 1.0f);
    const float shift[3]   = { p.get_float("XShift", 0), p.get_float("YShift", 0), p.get_float("ZShift", 0) };
    const std::string out_dir = p.get_string("OutputDir", "");
    const std::string fmt     = p.get_string("OutputFormat", "raw");
    const bool        use_stat = p.get_bool("StoppingStatistics", false);
    const uint64_t    max_b   = (uint64_t) std::max(0, p.get_int("MaxHistoriesPerBatch", 0));
    float             criteria = -1.0f;
    const float       threshold = p.get_float("StatThreshold", 0.0f);
    if (out_dir.empty()) throw std::runtime_error("Output directory is not provided.");
    if (use_stat) {
        criteria = p.get_float("StoppingCriteria", -1.0f);
        if (criteria < 0) throw std::runtime_error("Statistical criteria must be positive float");
        if (threshold <= 0) throw std::runtime_error("If no contour or mask is selected, the statistical threshold cannot be zero");
    }
    if (strcasecmp(p.get_string("Calibration", "default").c_str(), "default") != 0)
        throw std::runtime_error("Unknown calibration method");
    const std::string machine = p.get_string("Machine", "");
    const size_t      colon   = machine.find(':');
    if (colon == std::string::npos || strcasecmp(machine.substr(0, colon).c_str(), "pbs") != 0)
        throw std::runtime_error("Machine must be PBS:<beam model file>");
    const Machine model(machine.substr(colon + 1));
    if (fractions <= 0) fractions = 1;   // tps_env takes the plan's number of fractions
    struct stat info;
    if (::stat(out_dir.c_str(), &info) != 0) {
        mkdir(out_dir.c_str(), 0755);
    } else if (!p.get_bool("OverwriteResults", false)) {
        throw std::runtime_error("Output directory exists.");
    }

    // ---- CT
    if (cli["--ct"].empty() || cli["--ct_nxyz"].size() < 3 || cli["--ct_lxyz"].size() < 3 || cli["--ct_pxyz"].size() < 3)
        throw std::runtime_error("--ct, --ct_nxyz, --ct_lxyz and --ct_pxyz are required");
    const int nx = std::stoi(cli["--ct_nxyz"][0]), ny = std::stoi(cli["--ct_nxyz"][1]), nz = std::stoi(cli["--ct_nxyz"][2]);
    std::vector<float> xe = edges(to_f(cli["--ct_pxyz"], 0, 0), to_f(cli["--ct_lxyz"], 0, 0), nx);
    std::vector<float> ye = edges(to_f(cli["--ct_pxyz"], 1, 0), to_f(cli["--ct_lxyz"], 1, 0), ny);
    std::vector<float> ze = edges(to_f(cli["--ct_pxyz"], 2, 0), to_f(cli["--ct_lxyz"], 2, 0), nz);
    for (float& v : xe) v += shift[0];   // X/Y/ZShift move the CT (mqi_tps_env.hpp:475-477)
    for (float& v : ye) v += shift[1];
    for (float& v : ze) v += shift[2];
    const uint64_t       nvox = (uint64_t) nx * ny * nz;
    std::vector<int16_t> hu(nvox);
    {
        std::ifstream f(cli["--ct"][0], std::ios::binary);
        f.read(reinterpret_cast<char*>(hu.data()), nvox * sizeof(int16_t));
        if ((uint64_t) f.gcount() != nvox * sizeof(int16_t)) throw std::runtime_error("CT file is too short");
    }
    if (cli["--beams"].empty()) throw std::runtime_error("--beams is required");
    std::vector<Beam> beams = read_beams(cli["--beams"][0]);
    std::vector<int>  chosen;
    for (const auto& t : p.get_vector("BeamNumbers", ',')) chosen.push_back(std::atoi(t.c_str()));
    if (chosen.empty() || (chosen.size() == 1 && chosen[0] == 0)) {
        chosen.clear();
        for (size_t k = 0; k < beams.size(); ++k)
            if (beams[k].name != "Setup") chosen.push_back((int) k + 1);
    }
    std::ofstream json;
    if (!cli["--json"].empty()) json.open(cli["--json"][0]);
    if (json) json << "{";

    for (size_t q = 0; q < chosen.size(); ++q) {
        if (chosen[q] < 1 || chosen[q] > (int) beams.size()) throw std::runtime_error("BeamNumbers out of range");
        const Beam& b = beams[chosen[q] - 1];
        mqi_ctx*    ctx = nullptr;
        check(mqi_create(gpu_id, &ctx), nullptr, "mqi_create");
        check(mqi_set_physics(ctx, 0, 1), ctx, "mqi_set_physics");
        const Mat3 R = beam_rotation({ b.collimator, b.gantry, b.couch, 90.0f });   // iec2dicom, :978
        for (const auto& d : b.devices) add_device(ctx, d, R, b.iso, rs_density);
        int cid = -1;
        check(mqi_add_child(ctx, nx, ny, nz, xe.data(), ye.data(), ze.data(), nullptr, nullptr, &cid), ctx, "mqi_add_child");
        check(mqi_set_hu(ctx, cid, hu.data(), dens_scale, 0), ctx, "mqi_set_hu");
        std::vector<std::pair<std::string, int>> out;
        auto add = [&](const char* name, int type) {
            int sid = -1;
            check(mqi_add_scorer(ctx, cid, type, MQI_ROI_DIRECT, 0, nullptr, nullptr, nullptr, &sid), ctx, "mqi_add_scorer");
            out.emplace_back(name, sid);
        };
        for (const auto& s : scorers) {
            if (strcasecmp(s.c_str(), "Dose") == 0) add(s.c_str(), MQI_SCORER_DOSE_W);
            if (strcasecmp(s.c_str(), "LETd") == 0) { add("LETd_numer", MQI_SCORER_LETD_NUM); add("LETd_denom", MQI_SCORER_LETD_DEN); }
            if (strcasecmp(s.c_str(), "LETt") == 0) { add("LETt_numer", MQI_SCORER_LETT_NUM); add("LETt_denom", MQI_SCORER_LETT_DEN); }
        }
        int dij = -1;
        if (score_dij)   // the (voxel, spot) table; DOSE_Dij values
            check(mqi_add_dij_scorer(ctx, cid, MQI_ROI_DIRECT, 0, nullptr, nullptr, nullptr, 1ull << 28, &dij), ctx,
                  "mqi_add_dij_scorer");
        int d1 = -1, d2 = -1;
        if (use_stat)
            check(mqi_add_stat_scorers(ctx, cid, MQI_ROI_DIRECT, 0, nullptr, nullptr, nullptr, &d1, &d2), ctx,
                  "mqi_add_stat_scorers");
        // the spot plan: characterize_beamlet per spot; histories from the machine's ratio
        // (create_beamsource from the plan, mqi_treatment_machine_ion.hpp:84-133) or UnitWeights
        std::vector<mqi_spot> plan;
        for (const auto& s : b.spots) {
            mqi_spot sp   = model.spot(s[0], s[1], s[2], b.sid, R.m, b.iso);
            sp.histories  = unit_w > 0 ? (uint64_t) unit_w : (pph == -1.0f ? 1 : model.histories(s[0], s[3], pph));
            plan.push_back(sp);
        }
        uint64_t total = 0;
        check(mqi_set_spot_plan(ctx, plan.data(), (uint32_t) plan.size(), &total), ctx, "mqi_set_spot_plan");
        const uint64_t bseed = (uint64_t) (uint32_t) (seed + 10000 * (int) q);
        const auto     t0    = std::chrono::steady_clock::now();
        uint64_t       passes = 1;
        double         achieved = 0.0;
        if (use_stat) {
            check(mqi_run_plan_until_stat(ctx, d1, d2, criteria / 100.0f, threshold, 1000, bseed, &passes, &achieved), ctx,
                  "mqi_run_plan_until_stat");
        } else {
            std::vector<std::pair<uint64_t, uint64_t>> ranges;
            if (per_spot && !score_dij) {   // a Dij run is batched: its table keys carry the spot
                uint64_t h = 0;
                for (const auto& sp : plan) { ranges.emplace_back(h, h + sp.histories); h += sp.histories; }
            } else {
                const uint64_t step = max_b ? max_b : std::max<uint64_t>(total, 1);
                for (uint64_t h = 0; h < total; h += step) ranges.emplace_back(h, std::min(total, h + step));
            }
            for (const auto& r : ranges)
                if (r.second > r.first) check(mqi_transport_plan(ctx, r.first, r.second, bseed), ctx, "mqi_transport_plan");
        }
        const double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        const double scale = (unit_w > 0 ? 1.0f : pph) * rbe * (float) fractions;
        for (const auto& o : out) {
            std::vector<double> vol(nvox);
            uint64_t            n = 0;
            check(mqi_get_tally(ctx, o.second, vol.data(), &n, 0), ctx, "mqi_get_tally");
            write_outputs(out_dir, b.name + "_" + std::to_string(b.devices.size()) + "_" + o.first, fmt, vol, scale, xe,
                          ye, ze);
        }
        if (dij >= 0) {
            uint64_t nnz = 0;
            check(mqi_dij_build(ctx, dij, 0, scale, &nnz), ctx, "mqi_dij_build");
            std::vector<uint64_t> indptr(plan.size() + 1);
            std::vector<uint32_t> indices(nnz);
            std::vector<float>    value(nnz);
            check(mqi_dij_get_csr(ctx, dij, indptr.data(), indices.data(), value.data(), 0), ctx, "mqi_dij_get_csr");
            if (nnz >= (1ull << 32) || nvox >= (1ull << 32))
                throw std::runtime_error("Dij: the npz layout holds uint32 indices and row offsets");
            const std::vector<uint32_t> ptr32(indptr.begin(), indptr.end());
            const std::vector<double>   data(value.begin(), value.end());
            const uint32_t              shape[2] = { (uint32_t) plan.size(), (uint32_t) nvox };
            const std::string           n1 = "(" + std::to_string(ptr32.size()) + ",)", n2 = "(" + std::to_string(nnz) + ",)";
            write_npz(out_dir + "/" + b.name + "_" + std::to_string(b.devices.size()) + "_Dij.npz",
                      { { "indices", "<u4", n2, indices.data(), indices.size() * sizeof(uint32_t) },
                        { "indptr", "<u4", n1, ptr32.data(), ptr32.size() * sizeof(uint32_t) },
                        { "shape", "<u4", "(2,)", shape, sizeof(shape) },
                        { "data", "<f8", n2, data.data(), data.size() * sizeof(double) },
                        { "format", "|S3", "()", "csr", 3 } });
        }
        std::printf("beam %s: %llu histories, %.3f s\n", b.name.c_str(), (unsigned long long) (total * passes), secs);
        if (json)
            json << (q ? ", " : "") << "\"" << b.name << "\": {\"histories\": " << total << ", \"passes\": " << passes
                 << ", \"uncertainty\": " << achieved << ", \"seconds\": " << secs << "}";
        mqi_destroy(ctx);
    }
    if (json) json << "}\n";
    return 0;
}

}   // namespace

int
main(int argc, char** argv) {
    try {
        if (argc < 2) throw std::runtime_error("usage: tps_env <input file> --ct ... --beams ...");
        return run(argv[1], Cli(argc - 1, argv + 1));
    } catch (const std::exception& e) {
        std::fprintf(stderr, "tps_env: %s\n", e.what());
        return 1;
    }
}
