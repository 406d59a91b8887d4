// cast_common.cuh -- definitions shared by the ray (k_rays.cu) and frustum
// (k_frustum.cu) casts: the set of functions of funcs_tuple with their weights resident
// side by side in shared memory, and the cast options as the kernels read them.
#pragma once
#include "niq_host.cuh"

namespace niq {

constexpr int kMaxFuncs = 8;

struct ModelSet {
    NiqModelRef m[kMaxFuncs];
    int woff[kMaxFuncs];   // float offset of each model's weights in the resident buffer
    int n;
};

struct CastDev {
    float hit_eps, max_dist, safety, grow, shrink, init_step;
    int n_max_step, n_substeps;
};

inline int make_set(const niq_model* const* models, int nfunc, ModelSet& S, int& maxw, int& wfloats, int& maxlayer) {
    NIQ_REQUIRE(models && nfunc >= 1 && nfunc <= kMaxFuncs, NIQ_ERR_INVALID_ARG, "nfunc must be in [1, %d]", kMaxFuncs);
    S.n = nfunc;
    maxw = 0; wfloats = 0; maxlayer = 0;
    for (int f = 0; f < nfunc; ++f) {
        NIQ_REQUIRE(models[f], NIQ_ERR_INVALID_ARG, "null model %d", f);
        S.m[f] = models[f]->ref();
        S.woff[f] = wfloats;
        wfloats += models[f]->hdr.n_weight_floats;
        maxw = maxw > models[f]->hdr.max_width ? maxw : models[f]->hdr.max_width;
        const int ml = max_layer_floats(models[f]->hdr);
        maxlayer = maxlayer > ml ? maxlayer : ml;
    }
    return NIQ_OK;
}

inline CastDev to_dev(const niq_cast_opts& c) {
    CastDev d;
    d.hit_eps = c.hit_eps;
    d.max_dist = c.max_dist;
    d.safety = c.safety_factor;
    d.grow = c.interval_grow_fac;
    d.shrink = c.interval_shrink_fac;
    // src/queries.py:148: ones(N) * interval_init_size * max_dist, in float32
    volatile float a = 1.0f * c.interval_init_size;
    d.init_step = a * c.max_dist;
    d.n_max_step = c.n_max_step;
    d.n_substeps = c.n_substeps;
    return d;
}

}  // namespace niq
