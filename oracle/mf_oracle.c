/* CPU oracle for the MoreFit likelihood hot path (TEST INFRASTRUCTURE ONLY).
 * See mf_oracle.h for the contract and the reference lines each function
 * restates. Compiled with -ffp-contract=off so that the Kahan steps and the
 * evaluation order are what the C source says. */
#define _GNU_SOURCE
#include "mf_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

/* ---------------- random numbers (random.hh) ---------------- */

/* Splitmix64 output function (random.hh:160-186). */
static uint64_t splitmix64_next(uint64_t* s) {
  uint64_t z = (*s += 0x9e3779b97f4a7c15ULL);
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
  return z ^ (z >> 31);
}

void mfo_xoshiro_seed(uint64_t seed, uint32_t st[4]) {
  uint64_t s = seed;
  for (int k = 0; k < 4; k++) st[k] = (uint32_t)(splitmix64_next(&s) >> 32);
}

static inline uint32_t rotl32(uint32_t x, int k) { return (x << k) | (x >> (32 - k)); }

uint32_t mfo_xoshiro_next(uint32_t s[4]) {
  const uint32_t r = rotl32(s[0] + s[3], 7) + s[0];
  const uint32_t t = s[1] << 9;
  s[2] ^= s[0];
  s[3] ^= s[1];
  s[1] ^= s[2];
  s[0] ^= s[3];
  s[2] ^= t;
  s[3] = rotl32(s[3], 11);
  return r;
}

void mfo_xoshiro_jump(uint32_t s[4]) {
  /* The published xoshiro128 jump polynomial (Blackman & Vigna), as used
   * by Xoshiro128pp::jump. */
  static const uint32_t J[4] = {0x8764000bu, 0xf542d2d3u, 0x6fa035c3u, 0x77f2db5bu};
  uint32_t a = 0, b = 0, c = 0, d = 0;
  for (int i = 0; i < 4; i++)
    for (int bit = 0; bit < 32; bit++) {
      if (J[i] & (1u << bit)) {
        a ^= s[0];
        b ^= s[1];
        c ^= s[2];
        d ^= s[3];
      }
      mfo_xoshiro_next(s);
    }
  s[0] = a;
  s[1] = b;
  s[2] = c;
  s[3] = d;
}

void mfo_seed_rows(uint64_t seed, uint32_t nrows, uint32_t* seeds) {
  uint32_t st[4];
  mfo_xoshiro_seed(seed, st);
  for (uint32_t t = 0; t < nrows; t++) {
    for (int k = 0; k < 4; k++) seeds[(uint64_t)k * nrows + t] = st[k];
    mfo_xoshiro_jump(st);
  }
}

/* The generate kernel's uniform (compute_llvm.hh:383-397): the raw output
 * times 2^-32, in double (not the float-cast host random()). */
static inline double uniform(uint32_t s[4]) { return mfo_xoshiro_next(s) * 2.3283064365386963e-10; }

/* ---------------- densities ---------------- */

double mfo_mass_prob(double m, const double* th, double lo, double hi) {
  const double mb = th[0], sigma = th[1], fsig = th[2], alpha = th[3];
  const double g = 1.0 / sqrt(2.0 * M_PI) / sigma * exp(-((m - mb) * (m - mb) / (2.0 * sigma * sigma)));
  const double ng = 0.5 * (erf((hi - mb) / (sqrt(2.0) * sigma)) - erf((lo - mb) / (sqrt(2.0) * sigma)));
  const double e = exp(alpha * m);
  const double ne = alpha == 0.0 ? (hi - lo) : (exp(alpha * hi) - exp(alpha * lo)) / alpha;
  return fsig * g / ng + (1.0 - fsig) * e / ne;
}

double mfo_mass_max(const double* th, double lo, double hi) {
  /* SumPDF::get_max (pdf.hh:628-640) over GaussianPDF::get_max (:186-190)
   * and ExponentialPDF::get_max (:471-480). */
  const double mb = th[0], sigma = th[1], fsig = th[2], alpha = th[3];
  const double n = 0.5 * (erf((hi - mb) / (sqrt(2.0) * sigma)) - erf((lo - mb) / (sqrt(2.0) * sigma)));
  const double gmax = 1.0 / sqrt(2.0 * M_PI) / sigma / n;
  double emax;
  const double ne = exp(alpha * hi) - exp(alpha * lo);
  if (alpha == 0.0)
    emax = 1.0 / (hi - lo);
  else if (alpha > 0.0)
    emax = alpha * exp(alpha * hi) / ne;
  else
    emax = alpha * exp(alpha * lo) / ne;
  return fsig * gmax + (1.0 - fsig) * emax;
}

/* 9/(32 pi), the P-wave prefactor (physicspdfs.hh:46). */
#define PWAVE_C (9.0 / 32.0 / M_PI)

/* Basis columns in reference hoisting order: index 0..10 correspond to
 * morefit_eventbuffer_3..13 and multiply S9, S8, S7, Afb, S5, S4, S3, -Fl,
 * (1-Fl), (1-Fl), Fl respectively. */
static inline void pwave_basis_one(double ctl, double ctk, double phi, double b[11]) {
  const double c = PWAVE_C;
  const double sl2 = 1.0 - ctl * ctl, sk2 = 1.0 - ctk * ctk;
  const double sl = sqrt(sl2), sk = sqrt(sk2);
  const double c2l = 2.0 * ctl * ctl - 1.0;
  b[0] = c * sin(2.0 * phi) * sl2 * sk2;               /* S9  */
  b[1] = 4.0 * c * sin(phi) * ctk * sk * ctl * sl;     /* S8  */
  b[2] = 2.0 * c * sin(phi) * sl * ctk * sk;           /* S7  */
  b[3] = 4.0 / 3.0 * c * ctl * sk2;                    /* Afb */
  b[4] = 2.0 * c * cos(phi) * sl * ctk * sk;           /* S5  */
  b[5] = 4.0 * c * cos(phi) * ctk * sk * ctl * sl;     /* S4  */
  b[6] = c * cos(2.0 * phi) * sl2 * sk2;               /* S3  */
  b[7] = c * c2l * ctk * ctk;                          /* -Fl */
  b[8] = 0.25 * c * c2l * sk2;                         /* 1-Fl */
  b[9] = 0.75 * c * sk2;                               /* 1-Fl */
  b[10] = c * ctk * ctk;                               /* Fl  */
}

static inline double pwave_p_from_basis(const double b[11], const double* th) {
  const double Fl = th[0], S3 = th[1], S4 = th[2], S5 = th[3], Afb = th[4], S7 = th[5], S8 = th[6], S9 = th[7];
  return b[0] * S9 + b[1] * S8 + b[2] * S7 + b[3] * Afb + b[4] * S5 + b[5] * S4 + b[6] * S3 - b[7] * Fl +
         (b[8] + b[9]) * (1.0 - Fl) + b[10] * Fl;
}

double mfo_pwave_prob(double ctl, double ctk, double phi, const double* th) {
  double b[11];
  pwave_basis_one(ctl, ctk, phi, b);
  return pwave_p_from_basis(b, th);
}

double mfo_pwave_max(const double* th) {
  /* KstarmumuAngularPDF::get_max (physicspdfs.hh:209-213). */
  return 9.0 / 32.0 / M_PI *
         (4.0 + fabs(th[1]) + fabs(th[2]) + fabs(th[3]) + 4.0 / 3.0 * fabs(th[4]) + fabs(th[5]) + fabs(th[6]) +
          fabs(th[7]));
}

void mfo_pwave_basis(const double* ev, uint32_t n, double* out) {
  for (uint32_t i = 0; i < n; i++) {
    double b[11];
    pwave_basis_one(ev[i], ev[(uint64_t)n + i], ev[2 * (uint64_t)n + i], b);
    for (int k = 0; k < 11; k++) out[(uint64_t)k * n + i] = b[k];
  }
}

/* ---------------- generation ---------------- */

/* Same rounding of range constants as the reference's generated text, which
 * prints min and max-min with "%.15e" (compute_llvm.hh:472-478). */
static double printed15(double v) {
  char buf[64];
  snprintf(buf, sizeof buf, "%.15e", v);
  return strtod(buf, NULL);
}

typedef struct {
  int workload;
  const double* th;
  double lo[3], delta[3], mlo, mhi;
  double maxprob;
  const uint32_t* seeds;
  uint32_t nthreads, tid, from, to, n;
  double* out;
} gen_job;

static void* gen_chunk(void* arg) {
  gen_job* j = (gen_job*)arg;
  uint32_t st[4];
  for (int k = 0; k < 4; k++) st[k] = j->seeds[(uint64_t)k * j->nthreads + j->tid];
  const int ndim = j->workload == 0 ? 1 : 3;
  double x[3];
  for (uint32_t i = j->from; i < j->to; i++) {
    for (;;) {
      for (int d = 0; d < ndim; d++) x[d] = j->lo[d] + j->delta[d] * uniform(st);
      const double p = j->workload == 0 ? mfo_mass_prob(x[0], j->th, j->mlo, j->mhi)
                                        : mfo_pwave_prob(x[0], x[1], x[2], j->th);
      if (j->maxprob * uniform(st) < p) {
        for (int d = 0; d < ndim; d++) j->out[(uint64_t)d * j->n + i] = x[d];
        break;
      }
    }
  }
  return NULL;
}

int mfo_generate(int workload, const double* th, const double* lo, const double* hi, uint64_t seed, uint32_t n,
                 uint32_t nthreads, double* out) {
  if (nthreads == 0 || (workload != 0 && workload != 1)) return 1;
  const int ndim = workload == 0 ? 1 : 3;
  uint32_t* seeds = (uint32_t*)malloc(sizeof(uint32_t) * 4 * nthreads);
  mfo_seed_rows(seed, nthreads, seeds);
  gen_job* jobs = (gen_job*)calloc(nthreads, sizeof(gen_job));
  pthread_t* tids = (pthread_t*)calloc(nthreads, sizeof(pthread_t));
  const uint32_t size = n / nthreads;
  for (uint32_t t = 0; t < nthreads; t++) {
    gen_job* j = &jobs[t];
    j->workload = workload;
    j->th = th;
    for (int d = 0; d < ndim; d++) {
      j->lo[d] = printed15(lo[d]);
      j->delta[d] = printed15(hi[d] - lo[d]);
    }
    j->mlo = lo[0];
    j->mhi = hi[0];
    j->maxprob = printed15(workload == 0 ? mfo_mass_max(th, lo[0], hi[0]) : mfo_pwave_max(th));
    j->seeds = seeds;
    j->nthreads = nthreads;
    j->tid = t;
    j->from = t * size;
    j->to = (t == nthreads - 1) ? n : t * size + size;
    j->n = n;
    j->out = out;
  }
  if (nthreads == 1) {
    gen_chunk(&jobs[0]);
  } else {
    for (uint32_t t = 0; t < nthreads; t++) pthread_create(&tids[t], NULL, gen_chunk, &jobs[t]);
    for (uint32_t t = 0; t < nthreads; t++) pthread_join(tids[t], NULL);
  }
  free(tids);
  free(jobs);
  free(seeds);
  return 0;
}

int mfo_generate_partitioned(int workload, const double* th, const double* lo, const double* hi, uint64_t seed,
                             uint32_t n, uint32_t nper, uint32_t nseeds, double* out) {
  if (nseeds == 0 || nper == 0 || (workload != 0 && workload != 1)) return 1;
  const int ndim = workload == 0 ? 1 : 3;
  uint32_t* seeds = (uint32_t*)malloc(sizeof(uint32_t) * 4 * (size_t)nseeds);
  mfo_seed_rows(seed, nseeds, seeds);
  gen_job j;
  memset(&j, 0, sizeof j);
  j.workload = workload;
  j.th = th;
  for (int d = 0; d < ndim; d++) {
    j.lo[d] = printed15(lo[d]);
    j.delta[d] = printed15(hi[d] - lo[d]);
  }
  j.mlo = lo[0];
  j.mhi = hi[0];
  j.maxprob = printed15(workload == 0 ? mfo_mass_max(th, lo[0], hi[0]) : mfo_pwave_max(th));
  j.seeds = seeds;
  j.nthreads = nseeds;
  j.n = n;
  j.out = out;
  for (uint32_t t = 0; t < nseeds; t++) {
    uint64_t from = (uint64_t)t * nper, to = from + nper;
    if (from >= n) break;
    if (to > n) to = n;
    j.tid = t;
    j.from = (uint32_t)from;
    j.to = (uint32_t)to;
    gen_chunk(&j);
  }
  free(seeds);
  return 0;
}

/* ---------------- compensated sums ---------------- */

double mfo_kahan(const double* v, uint32_t n) {
  double s = 0.0, c = 0.0;
  for (uint32_t i = 0; i < n; i++) {
    const double y = v[i] - c;
    volatile double t = s + y;
    c = (t - s) - y;
    s = t;
  }
  return s;
}

/* Per chunk: 4 interleaved Kahan lanes per output (lane = event % 4), lanes
 * combined by Kahan in lane order. */
typedef struct {
  int workload;
  const double* cols;
  const double* th;
  double lo, hi;
  uint32_t n, from, to, nout;
  double sums[16];
} nll_job;

static void mass_terms(double m, const double* th, double lo, double hi, double r[5]) {
  const double mb = th[0], sigma = th[1], fsig = th[2], alpha = th[3];
  const double s2 = sqrt(2.0) * sigma;
  const double zh = (hi - mb) / s2, zl = (lo - mb) / s2;
  const double ng = 0.5 * (erf(zh) - erf(zl));
  const double dng_dmb = -(exp(-zh * zh) - exp(-zl * zl)) / (sqrt(2.0 * M_PI) * sigma);
  const double dng_ds = -(zh * exp(-zh * zh) - zl * exp(-zl * zl)) / (sqrt(M_PI) * sigma);
  const double g = exp(-((m - mb) * (m - mb)) / (2.0 * sigma * sigma)) / (sqrt(2.0 * M_PI) * sigma);
  const double G = g / ng;
  const double eh = exp(alpha * hi), el = exp(alpha * lo);
  const double ne = alpha == 0.0 ? (hi - lo) : (eh - el) / alpha;
  const double dne = alpha == 0.0 ? 0.0 : (hi * eh - lo * el) / alpha - (eh - el) / (alpha * alpha);
  const double E = exp(alpha * m) / ne;
  const double p = fsig * G + (1.0 - fsig) * E;
  const double dG_dmb = G * ((m - mb) / (sigma * sigma) - dng_dmb / ng);
  const double dG_ds = G * ((m - mb) * (m - mb) / (sigma * sigma * sigma) - 1.0 / sigma - dng_ds / ng);
  const double dE_da = E * (m - dne / ne);
  r[0] = log(p);
  r[1] = fsig * dG_dmb / p;
  r[2] = fsig * dG_ds / p;
  r[3] = (G - E) / p;
  r[4] = (1.0 - fsig) * dE_da / p;
}

static void* nll_chunk(void* arg) {
  nll_job* j = (nll_job*)arg;
  double ls[16 * 4], lc[16 * 4];
  memset(ls, 0, sizeof ls);
  memset(lc, 0, sizeof lc);
  double r[16];
  for (uint32_t i = j->from; i < j->to; i++) {
    if (j->workload == 0) {
      mass_terms(j->cols[i], j->th, j->lo, j->hi, r);
    } else {
      double b[11];
      for (int k = 0; k < 11; k++) b[k] = j->cols[(uint64_t)k * j->n + i];
      const double p = pwave_p_from_basis(b, j->th);
      r[0] = log(p);
      /* dp/dtheta in parameter order Fl, S3, S4, S5, Afb, S7, S8, S9 */
      r[1] = (-b[7] - b[8] - b[9] + b[10]) * (1.0 / p);
      r[2] = b[6] * (1.0 / p);
      r[3] = b[5] * (1.0 / p);
      r[4] = b[4] * (1.0 / p);
      r[5] = b[3] * (1.0 / p);
      r[6] = b[2] * (1.0 / p);
      r[7] = b[1] * (1.0 / p);
      r[8] = b[0] * (1.0 / p);
    }
    const uint32_t lane = i % 4u;
    for (uint32_t o = 0; o < j->nout; o++) {
      const uint32_t q = 4u * o + lane;
      const double y = r[o] - lc[q];
      const double t = ls[q] + y;
      lc[q] = (t - ls[q]) - y;
      ls[q] = t;
    }
  }
  for (uint32_t o = 0; o < j->nout; o++) {
    double s = 0.0, c = 0.0;
    for (int l = 0; l < 4; l++) {
      const double y = ls[4 * o + l] - c;
      const double t = s + y;
      c = (t - s) - y;
      s = t;
    }
    j->sums[o] = s;
  }
  return NULL;
}

static void nll_run(int workload, const double* cols, uint32_t n, const double* th, double lo, double hi,
                    uint32_t nthreads, uint32_t nout, double* sums) {
  if (nthreads == 0) nthreads = 1;
  nll_job* jobs = (nll_job*)calloc(nthreads, sizeof(nll_job));
  pthread_t* tt = (pthread_t*)calloc(nthreads, sizeof(pthread_t));
  const uint32_t size = n / nthreads;
  for (uint32_t t = 0; t < nthreads; t++) {
    nll_job* j = &jobs[t];
    j->workload = workload;
    j->cols = cols;
    j->th = th;
    j->lo = lo;
    j->hi = hi;
    j->n = n;
    j->nout = nout;
    j->from = t * size;
    j->to = (t == nthreads - 1) ? n : t * size + size;
  }
  if (nthreads == 1)
    nll_chunk(&jobs[0]);
  else {
    for (uint32_t t = 0; t < nthreads; t++) pthread_create(&tt[t], NULL, nll_chunk, &jobs[t]);
    for (uint32_t t = 0; t < nthreads; t++) pthread_join(tt[t], NULL);
  }
  double col[4096];
  for (uint32_t o = 0; o < nout; o++) {
    for (uint32_t t = 0; t < nthreads && t < 4096; t++) col[t] = jobs[t].sums[o];
    sums[o] = mfo_kahan(col, nthreads < 4096 ? nthreads : 4096);
  }
  free(tt);
  free(jobs);
}

void mfo_pwave_nll_grad(const double* basis, uint32_t n, const double* th, uint32_t nthreads, double* sums) {
  nll_run(1, basis, n, th, 0, 0, nthreads, 9, sums);
}

void mfo_mass_nll_grad(const double* m, uint32_t n, const double* th, double lo, double hi, uint32_t nthreads,
                       double* sums) {
  nll_run(0, m, n, th, lo, hi, nthreads, 5, sums);
}

uint64_t mfo_fnv1a(const void* p, uint64_t nbytes) {
  const unsigned char* b = (const unsigned char*)p;
  uint64_t h = 1469598103934665603ULL;
  for (uint64_t i = 0; i < nbytes; i++) {
    h ^= b[i];
    h *= 1099511628211ULL;
  }
  return h;
}
