// C entry points over the reference's own permanent calculators.
//
// Oracle-only test infrastructure.  This file is compiled together with the
// reference's hot-path sources (read in place from the reference tree, never
// copied) by oracle/build_ref.sh into oracle/_ref/libpqbref.so.  It is used
// in this development container to generate golden fixtures and to pin the
// C restatement in oracle/perm_oracle.c; nothing in the product links it.
//
// Library ids follow the reference's Python wrappers:
//   plain    (GlynnPermanentCalculator_Wrapper.hpp:34-44):   0 GlynnLongDouble,
//            6 GlynnDouble, 7 BBFG double, 8 BBFG long double,
//            10 GlynnSimpleDouble, 11 GlynnSimpleLongDouble
//   repeated (ChinHuhPermanentCalculator_Wrapper.hpp:36-47): 0 ChinHuh,
//            1 GlynnRep long double, 6 GlynnRep double,
//            7 BBFG repeated double, 8 BBFG repeated long double
#include <cstdint>
#include <cstring>
#include <string>

#include "BBFGPermanentCalculator.h"
#include "BBFGPermanentCalculatorRepeated.h"
#include "BatchedPermanentCalculator.h"
#include "CChinHuhPermanentCalculator.h"
#include "GlynnPermanentCalculator.h"
#include "GlynnPermanentCalculatorRepeated.h"
#include "GlynnPermanentCalculatorSimple.h"
#include "CGeneralizedCliffordsBSimulationStrategy.h"
#include "CGeneralizedCliffordsBUniformLossesSimulationStrategy.h"
#include "samplingHelperFunctions.h"

static thread_local std::string g_err;

extern "C" {

const char* ref_last_error() { return g_err.c_str(); }

// A: row-major complex128 (interleaved re, im), rows x cols, stride = cols.
int ref_perm(int lib, const double* A, int64_t rows, int64_t cols, double* out) {
    try {
        pic::matrix m((pic::Complex16*)A, (size_t)rows, (size_t)cols);
        pic::Complex16 r;
        switch (lib) {
            case 0: { pic::GlynnPermanentCalculatorLongDouble c; r = c.calculate(m); break; }
            case 6: { pic::GlynnPermanentCalculatorDouble c; r = c.calculate(m); break; }
            case 7: { pic::BBFGPermanentCalculator c; r = c.calculate(m, false); break; }
            case 8: { pic::BBFGPermanentCalculator c; r = c.calculate(m, true); break; }
            case 10: { pic::GlynnPermanentCalculatorSimpleDouble c; r = c.calculate(m); break; }
            case 11: { pic::GlynnPermanentCalculatorSimpleLongDouble c; r = c.calculate(m); break; }
            default: g_err = "Wrong value set for permanent library."; return 1;
        }
        out[0] = r.real();
        out[1] = r.imag();
        return 0;
    } catch (std::string& e) {
        g_err = e;
        return 2;
    }
}

// input_state = column multiplicities, output_state = row multiplicities,
// as in ChinHuhPermanentCalculator_Wrapper.hpp:367-375.
int ref_perm_repeated(int lib, const double* A, int64_t rows, int64_t cols,
                      const int64_t* input_state, int64_t n_in,
                      const int64_t* output_state, int64_t n_out, double* out) {
    try {
        pic::matrix m((pic::Complex16*)A, (size_t)rows, (size_t)cols);
        pic::PicState_int64 in((int64_t*)input_state, (size_t)n_in);
        pic::PicState_int64 outs((int64_t*)output_state, (size_t)n_out);
        pic::Complex16 r;
        switch (lib) {
            case 0: { pic::CChinHuhPermanentCalculator c; r = c.calculate(m, in, outs); break; }
            case 1: { pic::GlynnPermanentCalculatorRepeatedLongDouble c; r = c.calculate(m, in, outs); break; }
            case 6: { pic::GlynnPermanentCalculatorRepeatedDouble c; r = c.calculate(m, in, outs); break; }
            case 7: { pic::BBFGPermanentCalculatorRepeated c; r = c.calculate(m, in, outs, false); break; }
            case 8: { pic::BBFGPermanentCalculatorRepeated c; r = c.calculate(m, in, outs, true); break; }
            default: g_err = "Wrong value set for permanent library."; return 1;
        }
        out[0] = r.real();
        out[1] = r.imag();
        return 0;
    } catch (std::string& e) {
        g_err = e;
        return 2;
    }
}

// adaptInterferometer (BatchedPermanentCalculator.cpp:412-451): out must hold
// (#nonzero outputs) x (#nonzero inputs) complex values.
int ref_adapt_interferometer(const double* U, int64_t m, const int64_t* input_state,
                             const int64_t* output_state, double* out,
                             int64_t* out_rows, int64_t* out_cols) {
    pic::matrix u((pic::Complex16*)U, (size_t)m, (size_t)m);
    pic::PicState_int64 in((int64_t*)input_state, (size_t)m);
    pic::PicState_int64 outs((int64_t*)output_state, (size_t)m);
    pic::matrix r = pic::adaptInterferometer(u, in, outs);
    *out_rows = (int64_t)r.rows;
    *out_cols = (int64_t)r.cols;
    if (out) std::memcpy(out, r.get_data(), r.rows * r.cols * sizeof(pic::Complex16));
    return 0;
}

// adaptInterferometerGlynnMultiplied (BatchedPermanentCalculator.cpp:367-399):
// rows/cols physically repeated; out must hold N x N values, N = sum(input).
int ref_adapt_interferometer_multiplied(const double* U, int64_t m, const int64_t* input_state,
                                        const int64_t* output_state, double* out) {
    pic::matrix u((pic::Complex16*)U, (size_t)m, (size_t)m);
    pic::PicState_int64 in((int64_t*)input_state, (size_t)m);
    pic::PicState_int64 outs((int64_t*)output_state, (size_t)m);
    int64_t n = 0;
    for (int64_t i = 0; i < m; ++i) n += input_state[i];
    in.number_of_photons = n;
    pic::matrix r = pic::adaptInterferometerGlynnMultiplied(u, &in, &outs);
    std::memcpy(out, r.get_data(), r.rows * r.cols * sizeof(pic::Complex16));
    return 0;
}

// compute_pmf (sampling/simulation_strategies/source/samplingHelperFunctions
// .cpp:78-342): the probability of the next output mode given the sample so
// far and the current input.  pmf must hold m doubles.
int ref_compute_pmf(const double* U, int64_t m, const int64_t* sample, const int64_t* current_input, double* pmf) {
    try {
        pic::matrix u((pic::Complex16*)U, (size_t)m, (size_t)m);
        pic::PicState_int64 smp((int64_t*)sample, (size_t)m);
        pic::PicState_int64 inp((int64_t*)current_input, (size_t)m);
        int64_t ns = 0, ni = 0;
        for (int64_t i = 0; i < m; ++i) { ns += sample[i]; ni += current_input[i]; }
        smp.number_of_photons = ns;
        inp.number_of_photons = ni;
        pic::matrix_real r = pic::compute_pmf(u, smp, inp);
        std::memcpy(pmf, r.get_data(), (size_t)m * sizeof(double));
        return 0;
    } catch (std::string& e) {
        g_err = e;
        return 2;
    }
}

// The reference's Clifford & Clifford B sampler
// (CGeneralizedCliffordsBSimulationStrategy.cpp:137-316, without MPI):
// seeded with `seed`, `nsamples` samples of the input occupation
// `input_state` (m modes) written row by row into out (nsamples x m).
int ref_sample_b(const double* U, int64_t m, const int64_t* input_state, int64_t nsamples, uint64_t seed,
                 int64_t* out) {
    try {
        pic::matrix u((pic::Complex16*)U, (size_t)m, (size_t)m);
        pic::CGeneralizedCliffordsBSimulationStrategy strategy(u, 0);
        strategy.seed(seed);
        pic::PicState_int64 inp((int64_t*)input_state, (size_t)m);
        int64_t np = 0;
        for (int64_t i = 0; i < m; ++i) np += input_state[i];
        inp.number_of_photons = np;
        std::vector<pic::PicState_int64> samples = strategy.simulate(inp, (int)nsamples);
        if ((int64_t)samples.size() != nsamples) {
            g_err = "ref_sample_b: fewer samples than asked";
            return 3;
        }
        for (int64_t s = 0; s < nsamples; ++s)
            std::memcpy(out + s * m, samples[s].get_data(), (size_t)m * sizeof(int64_t));
        return 0;
    } catch (std::string& e) {
        g_err = e;
        return 2;
    }
}

// The reference's uniform-losses sampler
// (CGeneralizedCliffordsBUniformLossesSimulationStrategy.cpp:110-322).
int ref_sample_b_uniform_losses(const double* U, int64_t m, double transmissivity, const int64_t* input_state,
                                int64_t nsamples, uint64_t seed, int64_t* out) {
    try {
        pic::matrix u((pic::Complex16*)U, (size_t)m, (size_t)m);
        pic::CGeneralizedCliffordsBUniformLossesSimulationStrategy strategy(u, transmissivity, 0);
        strategy.seed(seed);
        pic::PicState_int64 inp((int64_t*)input_state, (size_t)m);
        int64_t np = 0;
        for (int64_t i = 0; i < m; ++i) np += input_state[i];
        inp.number_of_photons = np;
        std::vector<pic::PicState_int64> samples = strategy.simulate(inp, (int)nsamples);
        if ((int64_t)samples.size() != nsamples) {
            g_err = "ref_sample_b_uniform_losses: fewer samples than asked";
            return 3;
        }
        for (int64_t s = 0; s < nsamples; ++s)
            std::memcpy(out + s * m, samples[s].get_data(), (size_t)m * sizeof(int64_t));
        return 0;
    } catch (std::string& e) {
        g_err = e;
        return 2;
    }
}

}  // extern "C"
