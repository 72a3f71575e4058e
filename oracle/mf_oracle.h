/* CPU oracle for the MoreFit likelihood hot path (TEST INFRASTRUCTURE ONLY).
 *
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load
 * this library, and only as the checker or the timed CPU baseline; the CUDA
 * product never calls it. Every function restates the reference's algorithm
 * in plain C and cites the reference file:line it follows.
 *
 * Pinning: the generators and the closed-form densities are checked against
 * golden vectors produced by the reference's own generator, fitter and
 * Minuit2 (oracle/refkit, frozen under tests/golden/).
 */
#ifndef MF_ORACLE_H
#define MF_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* xoshiro128++ state seeded like Xoshiro128pp::setSeed(uint64_t)
 * (random.hh:355-362): four Splitmix64 outputs, upper 32 bits each. */
void mfo_xoshiro_seed(uint64_t seed, uint32_t state[4]);
/* One xoshiro128++ step (random.hh:371-383); returns the raw 32-bit output. */
uint32_t mfo_xoshiro_next(uint32_t state[4]);
/* Xoshiro128pp::jump() (random.hh:395-420): advance by 2^64 steps. */
void mfo_xoshiro_jump(uint32_t state[4]);

/* Seed rows for generator::generate (generator.hh:95-135): row t is the
 * stream state after t jumps; seeds is SoA [4][nrows] (seeds[k*nrows+t]). */
void mfo_seed_rows(uint64_t seed, uint32_t nrows, uint32_t* seeds);

/* Accept-reject generation on one stream per chunk, as the reference's
 * generate kernel does (compute_llvm.hh:362-533): thread t of nthreads takes
 * events [t*(n/nthreads), ...) with its own seed row. Output SoA [ndim][n].
 * workload: 0 = mass fit (truth vector mb, sigma, fsig, alpha; m range
 * [lo, hi]), 1 = K*mumu P-wave (Fl, S3, S4, S5, Afb, S7, S8, S9).
 * Returns 0 on success. */
int mfo_generate(int workload, const double* truth, const double* range_lo, const double* range_hi,
                 uint64_t seed, uint32_t n, uint32_t nthreads, double* out);

/* Accept-reject generation with the accelerator work partition of the
 * reference's OpenCL generate kernel (include/compute_opencl.hh:505-515,
 * 541-580): generator thread t (seed row t of mfo_seed_rows) produces events
 * [t*nper, min((t+1)*nper, n)). nseeds rows are used. */
int mfo_generate_partitioned(int workload, const double* truth, const double* range_lo, const double* range_hi,
                             uint64_t seed, uint32_t n, uint32_t nper, uint32_t nseeds, double* out);

/* Closed-form normalised densities (restating pdf.hh:139-194,423-651 and
 * physicspdfs.hh:39-81) evaluated per event. */
double mfo_mass_prob(double m, const double* theta, double lo, double hi);
double mfo_pwave_prob(double ctl, double ctk, double phi, const double* theta);
double mfo_pwave_max(const double* theta);
double mfo_mass_max(const double* theta, double lo, double hi);

/* The 11 hoisted P-wave angular basis columns in the order the reference's
 * event-buffer hoisting produces them (fitter.hh:345-375 applied to
 * physicspdfs.hh:39-77): out SoA [11][n]. */
void mfo_pwave_basis(const double* events, uint32_t n, double* out);

/* Sum over events of log p and its gradient for the P-wave from the 11
 * basis columns (theta = 8 parameters), with the reference's summation:
 * 4-lane interleaved Kahan per chunk, chunks combined by Kahan in order
 * (compute_llvm.hh:556-568,656-709,751-932). sums[0] = sum log p,
 * sums[1+k] = sum dlogp/dtheta_k. nthreads >= 1. */
void mfo_pwave_nll_grad(const double* basis, uint32_t n, const double* theta, uint32_t nthreads, double* sums);

/* Same for the mass fit from the raw m column (theta = mb, sigma, fsig, alpha). */
void mfo_mass_nll_grad(const double* m, uint32_t n, const double* theta, double lo, double hi, uint32_t nthreads,
                       double* sums);

/* Kahan sum in order (utils.hh:14-26). */
double mfo_kahan(const double* v, uint32_t n);

/* FNV-1a 64 over bytes (used to compare event buffers). */
uint64_t mfo_fnv1a(const void* p, uint64_t nbytes);

#ifdef __cplusplus
}
#endif
#endif
