/*
 * gbperm.h -- C ABI of the GB300 permanent library (libgbperm.so).
 *
 * Every function returns an int status (GBPERM_OK == 0); on failure
 * gbperm_last_error() returns a message for the calling thread.  Nothing is
 * thrown across the ABI and nothing calls exit().
 *
 * Matrices are complex128: interleaved (re, im) doubles, row-major, with a
 * leading dimension `ld` counted in complex elements (ld >= cols).  Results
 * are complex128 written as two doubles {re, im}; where an `out_dd` pointer is
 * accepted it receives {re_hi, im_hi, re_lo, im_lo}, the double-double value
 * of the result before rounding to double.
 *
 * Functions without a `_dev` suffix take HOST pointers: the library copies the
 * inputs to the current CUDA device, computes, copies the result back and
 * synchronises.  `_dev` functions take DEVICE pointers, a caller-provided
 * device workspace and a cudaStream_t (passed as void*), enqueue the work and
 * return without synchronising.
 *
 * Thread safety: host-pointer functions use a per-thread stream and a
 * per-thread device workspace, so concurrent calls from different threads
 * do not share buffers.
 */
#ifndef GBPERM_H
#define GBPERM_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GBPERM_OK 0
#define GBPERM_ERR_ARG 1         /* bad pointer, shape, stride or option */
#define GBPERM_ERR_STATE_SUM 2   /* sum(input_state) != sum(output_state) */
#define GBPERM_ERR_TOO_LARGE 3   /* beyond the supported sizes */
#define GBPERM_ERR_CUDA 4        /* a CUDA runtime call failed */
#define GBPERM_ERR_LIB 5         /* unknown calculator library id */
#define GBPERM_ERR_NO_DEVICE 6   /* no CUDA device visible */

/* Arithmetic of the n-term product (column sums are exact 64-bit fixed
 * point in both; the cross-thread reduction is double-double in both). */
#define GBPERM_ARITH_FP64 0  /* IEEE double product on the FP64 pipe */
#define GBPERM_ARITH_DF32 1  /* double-float product on the FP32 pipe (~2^-46 per
                                complex multiply), tried first for up to 48 columns
                                within the size rules ("df.max_rows",
                                "df.max_photons") when the matrix's dynamic range
                                allows; the integer-mantissa product recomputes on
                                the device when the range check fails or the error
                                estimate exceeds 1e-10, and runs alone beyond the
                                size rules (plain and repeated; pmf and the batched
                                plans recompute in FP64) */
#define GBPERM_ARITH_FX64 2  /* integer-mantissa product on the integer pipes: 64-bit
                                mantissas in 31-bit limbs, 55-57 significant bits per
                                complex multiply (the FP64 product keeps 53); any
                                dynamic range, no FP64 fallback needed.  Plain and
                                repeated permanents, the gradient sweep, the
                                repeated batch plans, pmf layers and the sampler */

/* Largest supported matrix side (columns of the product, rows of the Gray code). */
#define GBPERM_MAX_DIM 64

typedef struct gbperm_stats {
    double kernel_ms;      /* device time of the compute launches (CUDA events) */
    double steps;          /* Gray-code steps evaluated (terms of the sum) */
    double flops;          /* algorithmic FP64 flops: 8 n per plain step (2n column-sum adds,
                              6(n-1) for the product, 2 for the accumulate) */
    int32_t launches;      /* kernels launched by the call */
    int32_t grid;          /* blocks of the main launch */
    int32_t seg_log2;      /* log2 of the Gray segment length (plain / grad) */
    int32_t arith;         /* arithmetic actually used (GBPERM_ARITH_*) */
    double err_est;        /* when the double-float product ran (plain, repeated, pmf, batched):
                              estimated relative rounding error of its result,
                              sqrt(n) 2^-46 sqrt(sum |term|^2) / |perm| (pmf: the largest over the
                              layer's permanents; batched: the largest over the results kept in
                              double-float).  Above 1e-10 the result was recomputed on the device
                              by the integer-mantissa product (plain, repeated, gradient; arith
                              reports FX64) or the FP64 product (pmf, batched: per instance, in a
                              second pass of the plan; arith reports FP64).  0 when the
                              double-float product did not run */
} gbperm_stats;

/* ------------------------------------------------------------- library */
int gbperm_version(void);
const char* gbperm_last_error(void);
/* Number of visible CUDA devices (0 when none); never fails. */
int gbperm_device_count(void);
/* Tuning knobs (process-wide).  Keys:
 *   "plain.seg_log2"      force log2 segment length of the plain kernel (-1 = auto;
 *                         at most 31 is used)
 *   "plain.grid"          force the plain grid size (0 = auto)
 *   "repeated.low_digits" force the digits handled inside a repeated segment (-1 = auto)
 *   "batched.threads"     lanes sharing one Gray segment in a double-float batch plan
 *                         (2 or 4; 0 = 2), read when a plan is created; the autotuner
 *                         tries both
 *   "batched.item_log2"   force the log2 work-item target of new batch plans (0 = by
 *                         the batch's total work)
 *   "plain.df_group"      lanes sharing one Gray segment in the double-float kernel
 *                         (1, 2, 4 or 8; 0 = by column count)
 *   "plain.fx_group"      lanes sharing one Gray segment in the integer-mantissa kernel
 *                         (0 = by column count: pairs up to 40 columns; 4 = quads from 22)
 *   "df.escalate"         1 (default): a double-float result whose error estimate exceeds
 *                         1e-10 is recomputed on the device (integer-mantissa twin for
 *                         plain, repeated and gradient; FP64 for pmf and batched); 0: keep
 *                         it (stats.err_est still reports the estimate)
 *   "df.max_rows"         GBPERM_ARITH_DF32 on a square plain matrix with more rows runs the
 *                         integer-mantissa product alone (default 36)
 *   "df.max_photons"      GBPERM_ARITH_DF32 on a repeated permanent with more photons runs
 *                         the integer-mantissa product alone (default 24)
 *   "df.pmf_max_photons"  GBPERM_ARITH_DF32 on a pmf layer whose sample has more photons
 *                         runs the integer-mantissa layer (default 0: the double-float
 *                         layer measured no faster than FP64 up to 20 photons and
 *                         escalates from 24 on)
 *   "grad.arith"          product of the gradient sweep: 1 (default, double-float with the
 *                         integer-mantissa twin) or 2 (integer-mantissa throughout)
 */
int gbperm_set_option(const char* key, int64_t value);
int64_t gbperm_get_option(const char* key);

/* ------------------------------------------------------ plain permanent */
/* Glynn / BBFG permanent of a rows x cols matrix.  Replaces
 * BBFGPermanentCalculator::calculate (piquassoboost/sampling/source/
 * BBFGPermanentCalculator.cpp:89-126) and GlynnPermanentCalculator::calculate
 * (GlynnPermanentCalculator.hpp:47-57); semantics: rows == 0 or cols == 0 -> 1,
 * rows >= cols + 2 -> 0. */
int gbperm_perm(const double* A, int64_t rows, int64_t cols, int64_t ld, int arith, double* out,
                double* out_dd, gbperm_stats* stats);

/* Device-pointer form.  dA: device complex128 matrix; d_out: 2 doubles on
 * the device; d_out_dd: NULL or 4 doubles on the device.  The workspace must
 * hold gbperm_perm_workspace_size(rows, cols) bytes, 256-byte aligned.  With
 * GBPERM_ARITH_DF32 the range check runs on the device and the
 * integer-mantissa product takes over when it fails, or when the
 * double-float result's estimated relative rounding error exceeds 1e-10
 * (decided on the device, no host round trip). */
size_t gbperm_perm_workspace_size(int64_t rows, int64_t cols);
int gbperm_perm_dev(const void* dA, int64_t rows, int64_t cols, int64_t ld, int arith, void* d_out,
                    void* d_out_dd, void* workspace, size_t workspace_bytes, void* stream);

/* --------------------------------------------------- repeated permanent */
/* Permanent of the matrix whose row i is repeated row_mult[i] times and
 * column j col_mult[j] times (without expanding it).  Replaces
 * BBFGPermanentCalculatorRepeated::calculate (piquassoboost/sampling/source/
 * BBFGPermanentCalculatorRepeated.cpp:75-98) and GlynnPermanentCalculator
 * Repeated::calculate (GlynnPermanentCalculatorRepeated.hpp:48-74).
 * col_mult is the INPUT state and row_mult the OUTPUT state, as in the
 * reference wrapper (ChinHuhPermanentCalculator_Wrapper.hpp:367-375).
 * Only the first nrow rows / ncol columns take part (nrow <= rows,
 * ncol <= cols).  rows == 0 or a zero photon count -> 1;
 * sum(col_mult) != sum(row_mult) -> GBPERM_ERR_STATE_SUM. */
int gbperm_perm_repeated(const double* A, int64_t rows, int64_t cols, int64_t ld,
                         const int64_t* col_mult, int64_t ncol, const int64_t* row_mult,
                         int64_t nrow, int arith, double* out, double* out_dd,
                         gbperm_stats* stats);

/* The same permanent by the Chin-Huh form of the sum (CChinHuhPermanent
 * Calculator::calculate, piquassoboost/sampling/source/CChinHuhPermanent
 * Calculator.cpp:48-201; repeated lib 0): the digits run over the INPUT
 * multiplicities with no fixed copy and the prefactor is 2^-N, the product
 * over the output modes.  A second, independently ordered evaluation of the
 * repeated permanent, on the same kernels; same arguments and errors as
 * gbperm_perm_repeated. */
int gbperm_perm_chinhuh(const double* A, int64_t rows, int64_t cols, int64_t ld, const int64_t* col_mult,
                        int64_t ncol, const int64_t* row_mult, int64_t nrow, int arith, double* out, double* out_dd,
                        gbperm_stats* stats);

/* Many repeated permanents of one matrix: pair i is the input state
 * col_mults[i*ncol .. i*ncol+ncol) and the output state
 * row_mults[i*nrow .. i*nrow+nrow).  Replaces BatchednPermanentCalculator::
 * calculate (piquassoboost/sampling/source/BatchedPermanentCalculator.cpp:
 * 109-296) and the list branch of the repeated wrapper
 * (ChinHuhPermanentCalculator_Wrapper.hpp:233-323).  Pairs whose plain
 * expansion is not much longer than their mixed-radix Gray code are expanded
 * and share one persistent batched launch; the others run as repeated
 * launches.  With GBPERM_ARITH_FX64 every pair runs in one persistent
 * multiplicity launch (gbperm_rep_batch_*) when each has at most 40
 * occupied modes on its product side.  out: 2 * count doubles.  Any invalid
 * pair fails the call. */
int gbperm_perm_repeated_batched(const double* A, int64_t rows, int64_t cols, int64_t ld, const int64_t* col_mults,
                                 int64_t ncol, const int64_t* row_mults, int64_t nrow, int64_t count, int arith,
                                 double* out, gbperm_stats* stats);

/* A reusable plan for many repeated permanents of one interferometer, all
 * in one persistent launch (the same inputs as gbperm_perm_repeated_batched;
 * replaces BatchednPermanentCalculator::calculate, BatchedPermanentCalculator
 * .cpp:109-296, which evaluates each pair through adaptInterferometer and the
 * repeated calculator, :118-143).  Every pair keeps its multiplicities: the
 * mixed-radix Gray code of its cheaper side, so a pair with repeated modes
 * walks far fewer steps than its expanded matrix would.  Integer-mantissa
 * product only (arith must be GBPERM_ARITH_FX64); at most 40 occupied modes
 * on a pair's product side (GBPERM_ERR_TOO_LARGE otherwise).  create plans
 * every pair on the host, uploads the interferometer's submatrices and
 * tables, and captures the host run as a CUDA graph.  run: host output
 * (2 * count doubles, caller's order); run_dev: the same kernels enqueued on
 * `stream` writing 2 * count doubles to device memory.  info: Gray steps,
 * algorithmic flops (as gbperm_stats.flops counts them), 32x32->64 integer
 * multiply-adds of the products (12 per complex multiply, photons - 1
 * multiplies per step) and work items of the plan; any pointer may be null. */
typedef struct gbperm_rep_batch gbperm_rep_batch;
int gbperm_rep_batch_create(const double* A, int64_t rows, int64_t cols, int64_t ld, const int64_t* col_mults,
                            int64_t ncol, const int64_t* row_mults, int64_t nrow, int64_t count, int arith,
                            gbperm_rep_batch** out);
int gbperm_rep_batch_run(gbperm_rep_batch* plan, double* out, gbperm_stats* stats);
int gbperm_rep_batch_run_dev(gbperm_rep_batch* plan, void* d_out, void* stream);
int gbperm_rep_batch_info(const gbperm_rep_batch* plan, double* steps, double* flops, double* mul_ops,
                          int64_t* items);
void gbperm_rep_batch_destroy(gbperm_rep_batch* plan);

/* ------------------------------------------------- batched permanents */
/* Many plain permanents of uneven sizes in one persistent launch (a CUDA
 * graph per plan).  Replaces the list branch of the plain wrapper
 * (piquassoboost/sampling/GlynnPermanentCalculator_Wrapper.hpp:204-294) and
 * BatchednPermanentCalculator::calculate (BatchedPermanentCalculator.cpp:
 * 109-296).  Instance i is a rows[i] x cols[i] complex128 matrix, dense
 * (ld = cols[i]); the instances are packed back to back in index order.
 * A plan holds the instance sizes, the work list and the device buffers; it
 * belongs to the device current at creation.  arith: FP64, DF32 (with the
 * per-instance FP64 redo pass) or FX64 (integer-mantissa worker, lane
 * groups with each instance's columns split evenly).  out: 2 * count
 * doubles. */
typedef struct gbperm_batch_plan gbperm_batch_plan;
int gbperm_batch_plan_create(const int64_t* rows, const int64_t* cols, int64_t count, int arith,
                             gbperm_batch_plan** out_plan);
void gbperm_batch_plan_destroy(gbperm_batch_plan* plan);
int gbperm_batch_plan_run(gbperm_batch_plan* plan, const double* packed, double* out, gbperm_stats* stats);
/* Device-pointer form: d_packed and d_out on the device, enqueued on
 * stream (a copy into the plan's buffer, the kernels and one scatter launch
 * into the caller's slot order; trivial instances -- an empty side, or
 * rows >= cols + 2 -- get 1 or 0). */
int gbperm_batch_plan_run_dev(gbperm_batch_plan* plan, const void* d_packed, void* d_out, void* stream);
/* log2 of the Gray steps in one work item (the load-balancing grain);
 * setting it rebuilds the work list and the graph. */
int gbperm_batch_plan_set_item_log2(gbperm_batch_plan* plan, int64_t item_log2);
int64_t gbperm_batch_plan_get_item_log2(gbperm_batch_plan* plan);
/* Autotuner: plans, captures and times each candidate shape -- lanes per
 * Gray segment (2 or 4 for the double-float product, 1 for FP64) times work
 * items of 1/4, 1 and 4 times the size-based default -- on this batch
 * (`packed`, host buffer; reps timed launches each after one warm-up), keeps
 * the fastest and returns its time per batch in best_ms.  Results do not
 * depend on the choice beyond rounding of the fixed-order partial sums. */
int gbperm_batch_plan_autotune(gbperm_batch_plan* plan, const double* packed, int reps, double* best_ms);
/* The plan's current shape: lanes sharing one Gray segment, columns per lane. */
int gbperm_batch_plan_get_shape(gbperm_batch_plan* plan, int64_t* lanes_per_segment, int64_t* columns_per_lane);
/* One-shot: create, run, destroy. */
int gbperm_perm_batched(const double* packed, const int64_t* rows, const int64_t* cols, int64_t count, int arith,
                        double* out, gbperm_stats* stats);

/* ------------------------------------------ boson-sampling pmf layer */
/* One probability layer of the generalized Clifford & Clifford sampler.
 * Replaces compute_pmf (piquassoboost/sampling/simulation_strategies/source/
 * samplingHelperFunctions.cpp:78-342).  U: m x m complex128 interferometer
 * (leading dimension ld); sample: m output occupations (the photons placed so
 * far); current_input: m input occupations holding exactly one photon more.
 * pmf (m doubles) receives, normalised to sum 1,
 *   pmf[k] ~ | sum_l current_input[l] * perm_l * U[k][l] |^2
 * with perm_l the repeated permanent of the sample rows against the input
 * with one photon removed from mode l; addends (NULL or 2 m doubles)
 * receives the perm_l as complex128 (0 for empty input modes).  All perm_l
 * come from one Gray-code sweep over the sample.  arith as for the
 * permanents: GBPERM_ARITH_FX64 runs every product on integer mantissas
 * (no twin); GBPERM_ARITH_DF32 runs the double-float product up to 32
 * occupied input modes within the "df.pmf_max_photons" rule (recomputed in
 * FP64 on the device when the range check fails or an estimate is above
 * 1e-10) and the integer-mantissa layer otherwise.  Up to
 * 64 sample photons and 64 occupied input modes; a photon-count mismatch ->
 * GBPERM_ERR_STATE_SUM. */
int gbperm_compute_pmf(const double* U, int64_t m, int64_t ld, const int64_t* sample, const int64_t* current_input,
                       int arith, double* pmf, double* addends, gbperm_stats* stats);

/* ------------------------------------------------ boson sampler (B form) */
/* The generalised Clifford & Clifford sampler over gbperm_compute_pmf
 * layers.  Replaces CGeneralizedCliffordsBSimulationStrategy::simulate and
 * fill_r_sample (piquassoboost/sampling/simulation_strategies/source/
 * CGeneralizedCliffordsBSimulationStrategy.cpp:137-316, the branch without
 * MPI) with the reference's random stream: std::mt19937 seeded with the low
 * 32 bits of `seed` (samplingHelperFunctions.cpp:58-74), so a given seed
 * yields the reference's samples.  After gbperm_sampler_set_uniform_losses
 * it is CGeneralizedCliffordsBUniformLossesSimulationStrategy
 * (CGeneralizedCliffordsBUniformLossesSimulationStrategy.cpp:110-322): each
 * sample first draws its surviving photon count from the binomial law with
 * eta = transmissivity^2.  The sampler keeps its own copy of U (m x m,
 * leading dimension ld) and its own generator (the reference shares one
 * generator across all strategy objects).  arith selects the pmf layers'
 * product (gbperm_compute_pmf).  simulate writes nsamples rows of m
 * occupations (int64) into out; the input state has m entries. */
typedef struct gbperm_sampler gbperm_sampler;
int gbperm_sampler_create(const double* U, int64_t m, int64_t ld, uint64_t seed, int arith, gbperm_sampler** out);
int gbperm_sampler_set_matrix(gbperm_sampler* s, const double* U, int64_t m, int64_t ld);
int gbperm_sampler_seed(gbperm_sampler* s, uint64_t seed);
int gbperm_sampler_set_uniform_losses(gbperm_sampler* s, double transmissivity);
int gbperm_sampler_simulate(gbperm_sampler* s, const int64_t* input_state, int64_t m, int64_t nsamples,
                            int64_t* out, gbperm_stats* stats);
void gbperm_sampler_destroy(gbperm_sampler* s);

/* ----------------------------------------------- permanent + gradient */
/* Permanent of an n x n matrix and its full gradient G[k][l] = dperm/da_kl
 * (= perm of A without row k and column l) in one Gray-code sweep, for
 * n <= 32.  No reference counterpart: this is the adjoint of
 * BBFGPermanentCalculator::calculate (BBFGPermanentCalculator.hpp:87-235).
 * grad receives n x n complex128, row-major.  Product ("grad.arith"): the
 * double-float sweep, recomputed on the device by the integer-mantissa sweep
 * when the matrix's dynamic range fails the double-float range check or the
 * permanent's error estimate exceeds 1e-10 (stats.arith then reports FX64);
 * or the integer-mantissa sweep alone.  GBPERM_ERR_TOO_LARGE when n > 32. */
int gbperm_perm_grad(const double* A, int64_t n, int64_t ld, double* perm, double* perm_dd, double* grad,
                     gbperm_stats* stats);
size_t gbperm_perm_grad_workspace_size(int64_t n);
/* Device-pointer form: the same products and the same on-device
 * recomputation, with no host round trip. */
int gbperm_perm_grad_dev(const void* dA, int64_t n, int64_t ld, void* d_perm, void* d_perm_dd, void* d_grad,
                         void* workspace, size_t workspace_bytes, void* stream);
/* Batch of `count` n x n matrices in one set of launches (no reference
 * counterpart; the per-term gradients of a sampler log-likelihood).  Host
 * form: A holds the matrices densely, count x n x n complex128; perms
 * receives count x 2 doubles and grads count x n x n complex128.  A
 * non-finite matrix gives NaN for its own outputs only.  Device form: matrix
 * b starts at dA + b * stride complex elements (leading dimension ld). */
int gbperm_perm_grad_batched(const double* A, int64_t n, int64_t count, double* perms, double* grads,
                             gbperm_stats* stats);
size_t gbperm_perm_grad_batched_workspace_size(int64_t n, int64_t count);
int gbperm_perm_grad_batched_dev(const void* dA, int64_t n, int64_t count, int64_t ld, int64_t stride, void* d_perm,
                                 void* d_grad, void* workspace, size_t workspace_bytes, void* stream);

/* ------------------------------------------------------- Clements mesh */
/* No reference counterpart: the differentiable interferometer in front of
 * the batched gradient.  An m-mode Clements rectangular mesh (1 <= m <= 64)
 * of m(m-1)/2 interferometers; layer l = 0..m-1 holds the pairs (i, i+1),
 * i = l mod 2, l mod 2 + 2, ..., and interferometer t (layer by layer, then
 * by i) with phases (theta, phi) = (phases[2t], phases[2t+1]) maps rows
 * (i, i+1) by [[e^{i phi} cos theta, -sin theta], [e^{i phi} sin theta,
 * cos theta]]; U = L_{m-1} ... L_0 (m x m complex128, row-major).
 * The forward call keeps the layer states in the workspace
 * (gbperm_mesh_workspace_size(m) bytes, 256-byte aligned); the backward
 * call, given gU = dL/dRe(U) + i dL/dIm(U) for a real L, reads them back and
 * writes dL/dphases (m(m-1) doubles), so the same workspace must pass
 * unchanged from one to the other.  Both enqueue on `stream` and return. */
size_t gbperm_mesh_workspace_size(int64_t m);
int gbperm_mesh_unitary_dev(const void* d_phases, int64_t m, void* d_U, void* workspace, size_t workspace_bytes,
                            void* stream);
int gbperm_mesh_unitary_backward_dev(const void* d_phases, int64_t m, const void* d_gU, void* d_gphases,
                                     void* workspace, size_t workspace_bytes, void* stream);

/* ---------------------------------------- allocation-free plain permanent */
/* No counterpart in the reference.  The plain permanent for callers that
 * cannot allocate device memory (their pool belongs to another allocator, or
 * they must not pay cudaMalloc's device-wide synchronisation): same inputs,
 * outputs and arithmetics as gbperm_perm_dev, but the scratch lives in one
 * library-owned device array of gbperm_perm_noalloc_scratch_bytes() bytes
 * (256 KiB) that every GPU loading the library keeps until exit; sizes whose
 * scratch would not fit return GBPERM_ERR_TOO_LARGE.  The first call on a
 * device looks the array's device address up (cudaGetSymbolAddress) with that
 * device current; make that first call before any stream capture, and do
 * not cudaDeviceReset() a device while the library is in use (the looked-up
 * address would go stale).  Trivial shapes are written by a small kernel on
 * the stream, without a host copy or a synchronisation.  All calls share
 * the array: calls that overlap on the GPU race, so serialise them. */
int gbperm_perm_noalloc(const void* dA, int64_t rows, int64_t cols, int64_t ld, int arith, void* d_out,
                        void* d_out_dd, void* stream);
size_t gbperm_perm_noalloc_scratch_bytes(void);

/* ------------------------------------------------------------- probes */
/* Measured pipe peak of the current device: kind 0 = FP64 FMA, kind 1 =
 * FP32 FMA, kind 2 = FP64 tensor MMA (mma.sync m8n8k4), all in TFLOP/s
 * (FMA = 2 flops); kind 3 = 32x32->64-bit integer multiply-add
 * (mad.wide.s32), kind 4 = 32-bit integer multiply-add (mad.lo.s32),
 * kind 5 = variable funnel shift (shf.l.wrap.b32), kind 6 = 64-bit add
 * (add.s64), kind 7 = leading-bit search (bfind.s32), kind 8 = 32-bit add
 * (add.s32), kinds 3-8 in tera lane-operations/s.  Runs ~0.1 s of probe
 * kernels. */
int gbperm_probe_peak(int kind, double* tflops);

#ifdef __cplusplus
}
#endif

#endif /* GBPERM_H */
