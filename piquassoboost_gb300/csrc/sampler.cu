// Clifford & Clifford boson sampler (generalised B form) on the GPU pmf
// layers.
//
// Replaces CGeneralizedCliffordsBSimulationStrategy::simulate / fill_r_sample
// (piquassoboost/sampling/simulation_strategies/source/
// CGeneralizedCliffordsBSimulationStrategy.cpp:137-316, the branch without
// MPI) and, with uniform losses, CGeneralizedCliffordsBUniformLossesSimulation
// Strategy (CGeneralizedCliffordsBUniformLossesSimulationStrategy.cpp:110-328).
// The random stream is the reference's: a std::mt19937 (fully specified by the
// C++ standard, so identical on every platform) seeded with the low 32 bits of
// the seed (samplingHelperFunctions.cpp:58-62), with
//   * the next photon of the working input list picked by generator() % size
//     and removed from the list in order (update_input_by_single_photon,
//     samplingHelperFunctions.cpp:68-74, 378-405);
//   * the output mode drawn as the first index whose running pmf sum reaches
//     generator() / (2^32 - 1), index 0 when none does (sample_from_pmf,
//     :351-375);
//   * with uniform losses, the number of surviving photons drawn first per
//     sample from the binomial law with eta = transmissivity^2
//     (calculate_current_photon_number / calculate_particle_number_
//     probabilities, CGeneralizedCliffordsBUniformLossesSimulationStrategy
//     .cpp:280-322).
// Each layer's pmf is one gbperm_compute_pmf launch sequence (all
// leave-one-out permanents of the layer in one Gray sweep on the GPU).
//
// Deliberate deviation: the reference keeps ONE generator for the whole
// process, shared by every strategy object; here each sampler owns its
// generator, so interleaving two samplers does not couple their streams.
#include <cmath>
#include <cstring>
#include <random>
#include <vector>

#include "gbperm.h"
#include "gbperm_capi_internal.h"

struct gbperm_sampler {
    std::vector<double> U;  // m x m complex128 (interleaved), row-major, ld = m
    int64_t m = 0;
    int arith = GBPERM_ARITH_FP64;
    bool uniform_losses = false;
    double transmissivity = 1.0;
    std::mt19937 rng;
};

namespace gbperm {
namespace {

int copy_matrix(gbperm_sampler* s, const double* U, int64_t m, int64_t ld) {
    if (!U || m <= 0) return fail(GBPERM_ERR_ARG, "gbperm_sampler: empty interferometer");
    if (ld < m) return fail(GBPERM_ERR_ARG, "gbperm_sampler: ld < m");
    if (!all_finite(U, m, m, ld)) return fail(GBPERM_ERR_ARG, "gbperm_sampler: non-finite interferometer");
    s->U.assign((size_t)(2 * m * m), 0.0);
    for (int64_t i = 0; i < m; ++i) std::memcpy(&s->U[(size_t)(2 * i * m)], U + 2 * i * ld, (size_t)(2 * m) * sizeof(double));
    s->m = m;
    return GBPERM_OK;
}

// binomial(n, i) eta^i (1 - eta)^(n - i) for i = 0..n, evaluated as the
// reference does (int64 binomial times two pow calls)
std::vector<double> photon_number_law(int64_t n, double transmissivity) {
    const double eta = transmissivity * transmissivity;
    std::vector<double> p((size_t)(n + 1));
    for (int64_t i = 0; i <= n; ++i) {
        long long b = 1;
        for (int64_t k = 1; k <= i; ++k) b = b * (n - i + k) / k;
        p[(size_t)i] = (double)b * std::pow(eta, (double)i) * std::pow(1.0 - eta, (double)(n - i));
    }
    return p;
}

}  // namespace
}  // namespace gbperm

using namespace gbperm;

extern "C" {

int gbperm_sampler_create(const double* U, int64_t m, int64_t ld, uint64_t seed, int arith, gbperm_sampler** out) {
    if (!out) return fail(GBPERM_ERR_ARG, "gbperm_sampler_create: null output");
    *out = nullptr;
    if (arith != GBPERM_ARITH_FP64 && arith != GBPERM_ARITH_DF32 && arith != GBPERM_ARITH_FX64)
        return fail(GBPERM_ERR_ARG, "gbperm_sampler_create: unknown arithmetic");
    gbperm_sampler* s = new gbperm_sampler();
    int rc = copy_matrix(s, U, m, ld);
    if (rc) {
        delete s;
        return rc;
    }
    s->arith = arith;
    s->rng.seed((std::mt19937::result_type)seed);
    *out = s;
    return GBPERM_OK;
}

int gbperm_sampler_set_matrix(gbperm_sampler* s, const double* U, int64_t m, int64_t ld) {
    if (!s) return fail(GBPERM_ERR_ARG, "gbperm_sampler_set_matrix: null sampler");
    return copy_matrix(s, U, m, ld);
}

int gbperm_sampler_seed(gbperm_sampler* s, uint64_t seed) {
    if (!s) return fail(GBPERM_ERR_ARG, "gbperm_sampler_seed: null sampler");
    s->rng.seed((std::mt19937::result_type)seed);
    return GBPERM_OK;
}

int gbperm_sampler_set_uniform_losses(gbperm_sampler* s, double transmissivity) {
    if (!s) return fail(GBPERM_ERR_ARG, "gbperm_sampler_set_uniform_losses: null sampler");
    if (!(transmissivity >= 0.0 && transmissivity <= 1.0))
        return fail(GBPERM_ERR_ARG, "gbperm_sampler_set_uniform_losses: transmissivity must be in [0, 1]");
    s->uniform_losses = true;
    s->transmissivity = transmissivity;
    return GBPERM_OK;
}

int gbperm_sampler_simulate(gbperm_sampler* s, const int64_t* input_state, int64_t m, int64_t nsamples, int64_t* out,
                            gbperm_stats* stats) {
    if (stats) std::memset(stats, 0, sizeof(*stats));
    if (!s) return fail(GBPERM_ERR_ARG, "gbperm_sampler_simulate: null sampler");
    if (nsamples < 0) return fail(GBPERM_ERR_ARG, "gbperm_sampler_simulate: negative sample count");
    if (nsamples == 0) return GBPERM_OK;
    if (!input_state || !out) return fail(GBPERM_ERR_ARG, "gbperm_sampler_simulate: null argument");
    if (m != s->m)
        return fail(GBPERM_ERR_ARG, "gbperm_sampler_simulate: the input state must have one entry per mode");
    // particle basis: photon k sits in mode particles[k], modes ascending
    // (modes_state_to_particle_state, CGeneralizedCliffordsBSimulationStrategy.cpp:322-340)
    std::vector<int64_t> particles;
    for (int64_t i = 0; i < m; ++i) {
        if (input_state[i] < 0) return fail(GBPERM_ERR_ARG, "gbperm_sampler_simulate: negative occupation");
        for (int64_t c = 0; c < input_state[i]; ++c) particles.push_back(i);
    }
    const int64_t np = (int64_t)particles.size();
    std::vector<double> law;
    if (s->uniform_losses) law = photon_number_law(np, s->transmissivity);
    std::vector<int64_t> working, current((size_t)m), sample((size_t)m);
    std::vector<double> pmf((size_t)m);
    const double rmax = (double)std::mt19937::max();
    for (int64_t smp = 0; smp < nsamples; ++smp) {
        std::fill(sample.begin(), sample.end(), 0);
        std::fill(current.begin(), current.end(), 0);
        working = particles;
        int64_t target = np;
        if (s->uniform_losses) {
            // the first k with a running law sum reaching the draw (or a sum
            // of 1), as calculate_current_photon_number does
            const double u = (double)s->rng() / rmax;
            int64_t k = 0;
            double w = law[0];
            while (w < u && w < 1.0 && k < np) {
                ++k;
                w += law[(size_t)k];
            }
            target = k;
        }
        int64_t ns = 0;
        while (target > ns) {
            if (working.empty())
                return fail(GBPERM_ERR_ARG, "gbperm_sampler_simulate: the working input state is empty");
            const size_t r = (size_t)(s->rng() % (std::mt19937::result_type)working.size());
            current[(size_t)working[r]]++;
            working.erase(working.begin() + (ptrdiff_t)r);
            gbperm_stats st;
            int rc = gbperm_compute_pmf(s->U.data(), m, m, sample.data(), current.data(), s->arith, pmf.data(),
                                        nullptr, &st);
            if (rc) return rc;
            if (stats) {
                stats->kernel_ms += st.kernel_ms;
                stats->steps += st.steps;
                stats->flops += st.flops;
                stats->launches += st.launches;
                if (st.err_est > stats->err_est) stats->err_est = st.err_est;
                stats->arith = st.arith > stats->arith ? st.arith : stats->arith;
            }
            const double u = (double)s->rng() / rmax;
            size_t pick = 0;
            double acc = 0.0;
            for (size_t i = 0; i < (size_t)m; ++i) {
                acc = acc + pmf[i];
                if (acc >= u) {
                    pick = i;
                    break;
                }
            }
            sample[pick]++;
            ns++;
        }
        std::memcpy(out + smp * m, sample.data(), (size_t)m * sizeof(int64_t));
    }
    return GBPERM_OK;
}

void gbperm_sampler_destroy(gbperm_sampler* s) { delete s; }

}  // extern "C"
