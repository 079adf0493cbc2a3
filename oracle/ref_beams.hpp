// Beam sources shared by the reference oracle drivers (test infrastructure only).
#pragma once

#include <moqui/base/environments/mqi_phantom_env.hpp>

/// phantom_env::setup_beamsource (moqui/base/environments/mqi_phantom_env.hpp:204-232) with the
/// Gaussian 6-D phase space (moqui/base/distributions/mqi_phsp6d.hpp) instead of the uniform one:
/// sigma = --spot_size, same coordinate transform, energy distribution, draw order and generator.
inline void
gaussian_phantom_beamsource(mqi::phantom_env<float>& env) {
    mqi::coordinate_transform<float> p_coord(env.spot_angles, { 0, 0, 0 });
    mqi::vec3<float>                 dir(0, 0, -1);
    std::array<float, 6> beamlet_mean = { env.spot_position[0], env.spot_position[1],
                                          env.spot_position[2], dir.x, dir.y, dir.z };
    std::array<float, 6> beamlet_sigm = { env.spot_size[0], env.spot_size[1], 0, 0, 0, 0 };
    std::array<float, 2> corr         = { 0.0, 0.0 };
    auto phsp   = new mqi::phsp_6d<float>(beamlet_mean, beamlet_sigm, corr);
    auto energy = new mqi::const_1d<float>({ env.spot_energy[0] }, { env.spot_energy[1] });
    env.beamsource.append_beamlet(mqi::beamlet<float>(energy, phsp), env.n_histories, p_coord);
    uint32_t h1   = env.beamsource.total_histories();
    env.vertices  = new mqi::vertex_t<float>[h1];
    for (size_t i = 0; i < h1; ++i) {
        auto bl         = env.beamsource(i);
        env.vertices[i] = bl(&env.beam_rng);
    }
}
