// Helpers for moqui subclasses that run their transport through libmqigpu.so (include/mqi_gpu.h).
//
// moqui (MGHPhysicsResearch/moquimc) keeps its user-facing environments -- phantom_env, tps_env
// and user subclasses of x_environment<R> -- and launches transport_particles_patient on the
// node tree it built (moqui/base/environments/mqi_xenvironment.hpp:89-146).  A subclass that
// includes this header hands the same node tree to the C ABI instead:
//   * scorer_type_of(): a scorer's fp_compute_hit pointer -> the ABI's scorer enum, resolved the
//     way moqui obtains the pointers (device symbols in a CUDA build, host functions otherwise);
//   * add_node(): a child node's grid3d (edges, densities, rotation, translation) and its scorers;
//   * fill_table(): a dense tally written into the scorer's key_value table the way moqui's
//     reshape_data() reads it (key1 = voxel), so save_reshaped_files() writes the result.
#pragma once

#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

#include <moqui/base/mqi_node.hpp>
#include <moqui/base/mqi_scorer.hpp>
#include <moqui/base/scorers/mqi_scorer_energy_deposit.hpp>

#include "mqi_gpu.h"

namespace mqi_binding
{

inline void
check(int rc, mqi_ctx* ctx, const char* what) {
    if (rc != MQI_OK) throw std::runtime_error(std::string(what) + ": " + mqi_last_error(ctx));
}

/// The callbacks moqui installs, as the pointers its environments store in scorer::compute_hit_.
template<typename R>
struct callbacks {
    mqi::fp_compute_hit<R> edep, edep_primary, edep_secondary, dose_m, dose_w, dose_w2, letd1, letd2, lett1, lett2;
    callbacks() {
#if defined(__CUDACC__)
        // moqui's CUDA build stores the device addresses it reads from these symbols
        // (e.g. mqi_tps_env.hpp:826-837); energy_deposit_secondary has no such symbol
        cudaMemcpyFromSymbol(&edep, mqi::energy_deposit_pointer, sizeof(edep));
        cudaMemcpyFromSymbol(&edep_primary, mqi::energy_deposit_primary_pointer, sizeof(edep_primary));
        cudaMemcpyFromSymbol(&dose_m, mqi::Dm_pointer, sizeof(dose_m));
        cudaMemcpyFromSymbol(&dose_w, mqi::Dw_pointer, sizeof(dose_w));
        cudaMemcpyFromSymbol(&dose_w2, mqi::Dw_square_pointer, sizeof(dose_w2));
        cudaMemcpyFromSymbol(&letd1, mqi::LETd_weight1_pointer, sizeof(letd1));
        cudaMemcpyFromSymbol(&letd2, mqi::LETd_weight2_pointer, sizeof(letd2));
        cudaMemcpyFromSymbol(&lett1, mqi::LETt_weight1_pointer, sizeof(lett1));
        cudaMemcpyFromSymbol(&lett2, mqi::LETt_weight2_pointer, sizeof(lett2));
        edep_secondary = nullptr;
#else
        edep           = mqi::energy_deposit<R>;
        edep_primary   = mqi::energy_deposit_primary<R>;
        edep_secondary = mqi::energy_deposit_secondary<R>;
        dose_m         = mqi::dose_to_medium<R>;
        dose_w         = mqi::dose_to_water<R>;
        dose_w2        = mqi::dose_to_water_square<R>;
        letd1          = mqi::LETd_weight1<R>;
        letd2          = mqi::LETd_weight2<R>;
        lett1          = mqi::LETt_weight1<R>;
        lett2          = mqi::LETt_weight2<R>;
#endif
    }
};

/// The ABI's enum for a scorer's callback, or MQI_ERR_UNSUPPORTED for a user-written one (it has
/// no device counterpart here: the C ABI cannot take a function pointer).
template<typename R>
int
scorer_type_of(const mqi::scorer<R>* sc, const callbacks<R>& cb = callbacks<R>()) {
    const mqi::fp_compute_hit<R> f = sc->compute_hit_;
    if (!f) return MQI_ERR_UNSUPPORTED;
    if (f == cb.dose_w) return MQI_SCORER_DOSE_W;
    if (f == cb.dose_w2) return MQI_SCORER_DOSE_W2;
    if (f == cb.dose_m) return MQI_SCORER_DOSE_M;
    if (f == cb.letd1) return MQI_SCORER_LETD_NUM;
    if (f == cb.letd2) return MQI_SCORER_LETD_DEN;
    if (f == cb.lett1) return MQI_SCORER_LETT_NUM;
    if (f == cb.lett2) return MQI_SCORER_LETT_DEN;
    if (f == cb.edep) return MQI_SCORER_EDEP;
    if (f == cb.edep_primary) return MQI_SCORER_EDEP_PRIMARY;
    if (cb.edep_secondary && f == cb.edep_secondary) return MQI_SCORER_EDEP_SECONDARY;
    return MQI_ERR_UNSUPPORTED;
}

/// Add `node` (a child of moqui's world) to the context with its densities and scorers; returns
/// the child id and appends one scorer id per node scorer to `scorer_ids`, in the node's order.
/// The roi_t arrays are passed as they are (DIRECT needs none).  tps_env's statistics pair
/// ("Dose_stat", "DoseSquare_stat", mqi_tps_env.hpp:936-960) becomes mqi_add_stat_scorers; with
/// `dij` set (tps_env's DOSE_Dij run, whose scorer carries the dose_to_water callback) a dose
/// scorer becomes a Dij scorer of `dij_capacity` slots.
template<typename R>
int
add_node(mqi_ctx* ctx, mqi::node_t<R>* node, std::vector<int>& scorer_ids, bool dij = false,
         uint64_t dij_capacity = 0) {
    auto*       geo = node->geo;
    const auto  n   = geo->get_nxyz();
    const auto& f   = geo->rotation_matrix_fwd;
    const float rot[9] = { (float) f.xx, (float) f.xy, (float) f.xz, (float) f.yx, (float) f.yy,
                           (float) f.yz, (float) f.zx, (float) f.zy, (float) f.zz };
    const float tr[3]  = { (float) geo->translation_vector.x, (float) geo->translation_vector.y,
                           (float) geo->translation_vector.z };
    int cid = -1;
    check(mqi_add_child(ctx, n.x, n.y, n.z, geo->get_x_edges(), geo->get_y_edges(), geo->get_z_edges(), rot, tr,
                        &cid),
          ctx, "mqi_add_child");
    check(mqi_set_density(ctx, cid, geo->get_data(), 0), ctx, "mqi_set_density");
    const callbacks<R> cb;
    for (int s = 0; s < node->n_scorers; ++s) {
        const mqi::scorer<R>* sc     = node->scorers[s];
        const mqi::roi_t*     roi    = sc->roi_;
        const int             method = roi ? (int) roi->method_ : MQI_ROI_DIRECT;
        const uint32_t        len    = roi ? (uint32_t) roi->length_ : 0;
        const uint32_t*       start  = roi ? roi->start_ : nullptr;
        const uint32_t*       stride = roi ? roi->stride_ : nullptr;
        const uint32_t*       acc    = roi ? roi->acc_stride_ : nullptr;
        if (std::string(sc->name_) == "Dose_stat" && s + 1 < node->n_scorers &&
            std::string(node->scorers[s + 1]->name_) == "DoseSquare_stat") {
            int d1 = -1, d2 = -1;
            check(mqi_add_stat_scorers(ctx, cid, method, len, start, stride, acc, &d1, &d2), ctx, "mqi_add_stat_scorers");
            scorer_ids.push_back(d1);
            scorer_ids.push_back(d2);
            ++s;
            continue;
        }
        const int type = scorer_type_of(sc, cb);
        if (type < 0) throw std::runtime_error(std::string("scorer ") + sc->name_ + ": a callback without an enum");
        int sid = -1;
        if (dij && type == MQI_SCORER_DOSE_W)
            check(mqi_add_dij_scorer(ctx, cid, method, len, start, stride, acc, dij_capacity, &sid), ctx,
                  "mqi_add_dij_scorer");
        else
            check(mqi_add_scorer(ctx, cid, type, method, len, start, stride, acc, &sid), ctx, "mqi_add_scorer");
        scorer_ids.push_back(sid);
    }
    return cid;
}

/// Write a dense tally into the scorer's key_value table as moqui's reshape_data reads it:
/// slot v holds (key1 = v, key2 = 0, value) for every voxel with a positive value.
template<typename R>
void
fill_table(mqi::scorer<R>* sc, const std::vector<double>& dense) {
    const uint64_t n = dense.size() < sc->max_capacity_ ? dense.size() : sc->max_capacity_;
    for (uint64_t v = 0; v < n; ++v)
        if (dense[v] > 0) {
            sc->data_[v].key1  = (mqi::key_t) v;
            sc->data_[v].key2  = 0;
            sc->data_[v].value = dense[v];
        }
}

}   // namespace mqi_binding
