// phantom_env_gb300<R>: moqui's phantom_env (moqui/base/environments/mqi_phantom_env.hpp:17-428)
// with its run()/finalize() on libmqigpu.so.  The constructor (the example's command line),
// setup_world / setup_beamsource (the world, densities and the host-sampled vertices) and
// save_reshaped_files() (the output files) are moqui's own.
#pragma once

#include <moqui/base/environments/mqi_phantom_env.hpp>

#include "mqi_gb300_binding.hpp"

template<typename R>
class phantom_env_gb300 : public mqi::phantom_env<R>
{
    mqi_ctx*         ctx_ = nullptr;
    std::vector<int> scorers_;   // per world child: its scorer ids, in the node's order
    std::vector<int> first_;     // first entry of each child in scorers_

public:
    using mqi::phantom_env<R>::phantom_env;

    ~phantom_env_gb300() {
        if (ctx_) mqi_destroy(ctx_);
    }

    /// transport_particles_patient over the environment's vertices, through the C ABI.
    void
    run() override {
        using mqi_binding::check;
        if (ctx_) mqi_destroy(ctx_);
        check(mqi_create(this->gpu_id, &ctx_), nullptr, "mqi_create");
#if defined(__PHYSICS_DEBUG__)
        check(mqi_set_physics(ctx_, 1, 1), ctx_, "mqi_set_physics");
#else
        check(mqi_set_physics(ctx_, 0, 1), ctx_, "mqi_set_physics");
#endif
        scorers_.clear();
        first_.clear();
        for (int c = 0; c < this->world->n_children; ++c) {
            first_.push_back((int) scorers_.size());
            mqi_binding::add_node(ctx_, this->world->children[c], scorers_);
        }
        const uint64_t h = this->beamsource.total_histories();
        // mqi::vertex_t<float> and mqi_vertex share their layout (ke, pos[3], dir[3])
        static_assert(sizeof(mqi::vertex_t<R>) == sizeof(mqi_vertex), "vertex layout");
        check(mqi_set_vertices(ctx_, reinterpret_cast<const mqi_vertex*>(this->vertices), nullptr, h, 0), ctx_,
              "mqi_set_vertices");
        check(mqi_transport(ctx_, 0, h, (uint64_t) (uint32_t) this->random_seed), ctx_, "mqi_transport");
    }

    /// download_node: the dense tallies into the scorers' key_value tables.
    void
    finalize() override {
        for (int c = 0; c < this->world->n_children; ++c) {
            auto* node = this->world->children[c];
            for (int s = 0; s < node->n_scorers; ++s) {
                uint64_t n = 0;
                mqi_binding::check(mqi_get_tally(ctx_, scorers_[first_[c] + s], nullptr, &n, 0), ctx_, "mqi_get_tally");
                std::vector<double> dense(n);
                mqi_binding::check(mqi_get_tally(ctx_, scorers_[first_[c] + s], dense.data(), &n, 0), ctx_,
                                   "mqi_get_tally");
                mqi_binding::fill_table(node->scorers[s], dense);
            }
        }
    }
};
