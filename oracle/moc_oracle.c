/*
 * moc_oracle.c -- TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C restatement of OpenMOC's CPUSolver flat-source source iteration
 * (the hot path the GB300 solver replaces), used as the checker for the CUDA
 * path and as the timed CPU baseline.  It is never linked into, called by or
 * shipped with the product library; only tests/, the package's smoke check and
 * the CPU-baseline leg of bench.py load it.
 *
 * Compiled twice by oracle/build.sh: ORACLE_REAL=float (mirrors the
 * FP_PRECISION=float CPUSolver) and ORACLE_REAL=double (the FP64 oracle).
 * Parity of this restatement is pinned against OpenMOC itself: the golden
 * fixtures in tests/golden/ are produced by the reference library
 * (tests/golden/make_fixtures.cpp), including the reference test suite's
 * tests/test_forward_pin_cell and tests/test_forward_pin_cell_70g.
 *
 * One deliberate difference: the exponential term (1 - exp(-x))/x is evaluated
 * in double precision from its definition (expm1) instead of the reference's
 * 5/6 rational approximation (src/exponentials.h:156-193, quoted there as
 * accurate to 2e-6), then rounded to ORACLE_REAL.
 *
 * Data layout: the packed structure-of-arrays of include/openmoc_gb300.h.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#ifndef ORACLE_REAL
#define ORACLE_REAL float
#endif
typedef ORACLE_REAL real;

#define FLUX_EPSILON ((real) 1.0E-25)      /* src/constants.h:15 */
#define ZERO_VOLUME 1.0E-12                /* src/constants.h:12 (FLT_EPSILON) */
#define FOUR_PI 12.566370614359172         /* src/constants.h:27 */
#define ONE_OVER_FOUR_PI 0.07957747154594767

enum { RES_SCALAR_FLUX = 0, RES_FISSION_SOURCE = 1, RES_TOTAL_SOURCE = 2 };

typedef struct {
  int32_t num_groups, num_polar_half, num_angles, num_materials;
  int64_t num_fsrs, num_tracks, num_segments;
  const float* seg_len;     /* [S] */
  const int32_t* seg_fsr;   /* [S] */
  const int64_t* seg_off;   /* [T+1] */
  const int32_t* track_ang; /* [T] */
  const int64_t* next;      /* [2T] */
  const uint8_t* flags;     /* [T] */
  const float* weights;     /* [A][Ph] */
  const float* inv_sin;     /* [A][Ph] */
  const float* sigma_t;     /* [M][G] */
  const float* sigma_s;     /* [M][G dest][G orig] */
  const float* nu_sigma_f;  /* [M][G] */
  const float* chi;         /* [M][G] */
  const int32_t* fsr_mat;   /* [R] */
  const float* fsr_vol;     /* [R] */
  int32_t solve_3d;
  int32_t num_threads;
} oracle_problem;

typedef struct {
  real* phi;        /* [R][G] scalar flux */
  real* phi_old;    /* [R][G] stored flux */
  real* reduced;    /* [R][G] reduced source Q/(4 pi) */
  real* fixed;      /* [R][G] fixed source or NULL */
  float* boundary;  /* [T][2][F] incoming angular flux of this sweep */
  float* start;     /* [T][2][F] outgoing angular flux for the next sweep */
  double keff;
} oracle_state;

/* ------------------------------------------------------------ utilities */

/* Double-accumulating pairwise sum, src/pairwise_sum.h:18-39. */
static double pairwise_sum_d(const double* v, long n) {
  if (n < 8) {
    double s = 0.0;
    for (long i = 0; i < n; i++) s += v[i];
    return s;
  }
  long h = n / 2;
  return pairwise_sum_d(v, h) + pairwise_sum_d(v + h, n - h);
}

static double pairwise_sum_r(const real* v, long n) {
  if (n < 8) {
    double s = 0.0;
    for (long i = 0; i < n; i++) s += v[i];
    return s;
  }
  long h = n / 2;
  return pairwise_sum_r(v, h) + pairwise_sum_r(v + h, n - h);
}

static int mat_fissile(const oracle_problem* p, int m) {
  for (int g = 0; g < p->num_groups; g++)
    if (p->nu_sigma_f[(long) m * p->num_groups + g] > 0.f) return 1;
  return 0;
}

static int fluxes_per_track(const oracle_problem* p) {
  return p->num_groups * p->num_polar_half;
}

/* (1 - exp(-x)) / x from its definition, in double. */
static double exp_f1(double x) {
  if (x < 1e-6) return 1.0 - 0.5 * x;
  return -expm1(-x) / x;
}

static void set_threads(const oracle_problem* p) {
#ifdef _OPENMP
  if (p->num_threads > 0) omp_set_num_threads(p->num_threads);
#else
  (void) p;
#endif
}

/* ------------------------------------------------------------ hooks */

/* CPUSolver::flattenFSRFluxes, src/CPUSolver.cpp:1816-1823 */
void oracle_flatten(const oracle_problem* p, oracle_state* s, double value) {
  long n = p->num_fsrs * p->num_groups;
  for (long i = 0; i < n; i++) s->phi[i] = (real) value;
}

/* CPUSolver::storeFSRFluxes, src/CPUSolver.cpp:1846-1853 */
void oracle_store(const oracle_problem* p, oracle_state* s) {
  memcpy(s->phi_old, s->phi, sizeof(real) * p->num_fsrs * p->num_groups);
}

/* CPUSolver::zeroTrackFluxes, src/CPUSolver.cpp:463-478 */
void oracle_zero_track_fluxes(const oracle_problem* p, oracle_state* s) {
  long n = 2 * p->num_tracks * fluxes_per_track(p);
  memset(s->boundary, 0, sizeof(float) * n);
  memset(s->start, 0, sizeof(float) * n);
}

/* CPUSolver::normalizeFluxes, src/CPUSolver.cpp:1860-1933 */
double oracle_normalize(const oracle_problem* p, oracle_state* s) {
  const long R = p->num_fsrs;
  const int G = p->num_groups;
  double* fs = (double*) malloc(sizeof(double) * R);
  set_threads(p);
#pragma omp parallel for schedule(static)
  for (long r = 0; r < R; r++) {
    real grp[1024];
    const float* nf = p->nu_sigma_f + (long) p->fsr_mat[r] * G;
    real vol = (real) p->fsr_vol[r];
    for (int g = 0; g < G; g++)
      grp[g] = (real) nf[g] * s->phi[r * G + g] * vol;
    fs[r] = pairwise_sum_r(grp, G);
  }
  double total = pairwise_sum_d(fs, R);
  free(fs);
  double factor = (double) R / total;
  long n = R * G;
  for (long i = 0; i < n; i++) s->phi[i] *= factor;
  long nb = 2 * p->num_tracks * fluxes_per_track(p);
  for (long i = 0; i < nb; i++) {
    s->start[i] *= factor;
    s->boundary[i] *= factor;
  }
  return factor;
}

/* CPUSolver::computeFSRSources, src/CPUSolver.cpp:1939-2025.  Returns the
 * number of negative sources found. */
long oracle_compute_sources(const oracle_problem* p, oracle_state* s,
                            int iteration, int negative_fluxes_allowed) {
  const long R = p->num_fsrs;
  const int G = p->num_groups;
  long num_negative = 0;
  set_threads(p);
#pragma omp parallel for schedule(static) reduction(+:num_negative)
  for (long r = 0; r < R; r++) {
    real fis[1024], sca[1024];
    int m = p->fsr_mat[r];
    const float* ss = p->sigma_s + (long) m * G * G;
    const float* nf = p->nu_sigma_f + (long) m * G;
    const float* ch = p->chi + (long) m * G;
    int fissile = mat_fissile(p, m);
    for (int gd = 0; gd < G; gd++) {
      for (int g = 0; g < G; g++) {
        /* fission matrix entry chi[dest]*nu_sigma_f[orig], rounded like
         * Material::buildFissionMatrix (src/Material.cpp:956-985) */
        real fm = fissile ? (real) ch[gd] * (real) nf[g] : (real) 0;
        sca[g] = (real) ss[gd * G + g] * s->phi[r * G + g];
        fis[g] = s->phi[r * G + g] * fm;
      }
      double scatter = pairwise_sum_r(sca, G);
      double fission = pairwise_sum_r(fis, G) / s->keff;
      real q = (real) fission;
      q += (real) scatter;
      if (s->fixed) q += s->fixed[r * G + gd];
      q *= (real) ONE_OVER_FOUR_PI;
      if (q < (real) 0) {
        num_negative++;
        if (iteration < 30 && !negative_fluxes_allowed) q = FLUX_EPSILON;
      }
      s->reduced[r * G + gd] = q;
    }
  }
  return num_negative;
}

/* Flat-source attenuation along one segment for all groups and polar angles,
 * CPUSolver::tallyScalarFlux, src/CPUSolver.cpp:2402-2498 (2D branch; the 3D
 * branch is the same with one polar value, inv_sin = 1 and the track weight
 * applied at accumulation). */
static void tally_segment(const oracle_problem* p, const oracle_state* s,
                          long fsr, real length, int mat, int ang,
                          real* fsr_buf, float* psi) {
  const int G = p->num_groups;
  const int Ph = p->num_polar_half;
  const float* st = p->sigma_t + (long) mat * G;
  for (int pp = 0; pp < Ph; pp++) {
    real wgt = p->solve_3d ? (real) 1 : (real) p->weights[ang * Ph + pp];
    real inv_sin = (real) p->inv_sin[ang * Ph + pp];
    for (int g = 0; g < G; g++) {
      int pe = pp * G + g;
      real tau = (real) st[g] * length;
      real e = (real) (inv_sin * exp_f1((double) (tau * inv_sin)));
      real delta = (tau * (real) psi[pe] - length * s->reduced[fsr * G + g]) * e;
      psi[pe] = (float) ((real) psi[pe] - delta);
      fsr_buf[g] += delta * wgt;
    }
  }
}

/* CPUSolver::accumulateScalarFluxContribution, src/CPUSolver.cpp:2507-2527 */
static void flush(const oracle_problem* p, oracle_state* s, long fsr,
                  real weight, real* buf, void* locks) {
  const int G = p->num_groups;
#ifdef _OPENMP
  omp_set_lock(&((omp_lock_t*) locks)[fsr]);
#else
  (void) locks;
#endif
  for (int g = 0; g < G; g++) s->phi[fsr * G + g] += weight * buf[g];
#ifdef _OPENMP
  omp_unset_lock(&((omp_lock_t*) locks)[fsr]);
#endif
  memset(buf, 0, sizeof(real) * G);
}

/* CPUSolver::transferBoundaryFlux, src/CPUSolver.cpp:2560-2600 */
static void transfer(const oracle_problem* p, oracle_state* s, long t, int fwd,
                     const float* psi) {
  const int F = fluxes_per_track(p);
  uint8_t f = p->flags[t];
  int moves = fwd ? (f & 4) : (f & 8);
  if (!moves) return;
  long next = p->next[2 * t + (fwd ? 0 : 1)];
  int next_is_fwd = fwd ? (f & 1) : (f & 2);
  float* dst = s->start + (next * 2 + (next_is_fwd ? 0 : 1)) * (long) F;
  memcpy(dst, psi, sizeof(float) * F);
}

/* CPUSolver::transportSweep + TransportSweep::onTrack
 * (src/CPUSolver.cpp:2338-2398, src/TrackTraversingAlgorithms.cpp:890-1052):
 * zero the scalar flux, copy the start fluxes into the boundary fluxes, then
 * sweep every track forward and backward, tallying FSR contributions in a
 * buffer that is flushed whenever the FSR changes. */
void oracle_sweep(const oracle_problem* p, oracle_state* s) {
  const long R = p->num_fsrs;
  const int G = p->num_groups;
  const long T = p->num_tracks;
  const int F = fluxes_per_track(p);
  memset(s->phi, 0, sizeof(real) * R * G);
  memcpy(s->boundary, s->start, sizeof(float) * 2 * T * F);
  set_threads(p);
  void* locks = NULL;
#ifdef _OPENMP
  omp_lock_t* lk = (omp_lock_t*) malloc(sizeof(omp_lock_t) * R);
  for (long r = 0; r < R; r++) omp_init_lock(&lk[r]);
  locks = lk;
#endif
#pragma omp parallel
  {
    real* buf = (real*) calloc(G, sizeof(real));
#pragma omp for schedule(dynamic)
    for (long t = 0; t < T; t++) {
      long b = p->seg_off[t];
      int n = (int) (p->seg_off[t + 1] - b);
      int ang = p->track_ang[t];
      real weight = p->solve_3d ? (real) p->weights[ang] : (real) 1;
      float* psi = s->boundary + (t * 2) * (long) F;
      for (int k = 0; k < n; k++) {
        long fsr = p->seg_fsr[b + k];
        tally_segment(p, s, fsr, (real) p->seg_len[b + k],
                      p->fsr_mat[fsr], ang, buf, psi);
        if (k < n - 1 && fsr != p->seg_fsr[b + k + 1])
          flush(p, s, fsr, weight, buf, locks);
      }
      transfer(p, s, t, 1, psi);
      psi = s->boundary + (t * 2 + 1) * (long) F;
      for (int k = n - 1; k >= 0; k--) {
        long fsr = p->seg_fsr[b + k];
        tally_segment(p, s, fsr, (real) p->seg_len[b + k],
                      p->fsr_mat[fsr], ang, buf, psi);
        if (k == 0 || fsr != p->seg_fsr[b + k - 1])
          flush(p, s, fsr, weight, buf, locks);
      }
      transfer(p, s, t, 0, psi);
    }
    free(buf);
  }
#ifdef _OPENMP
  for (long r = 0; r < R; r++) omp_destroy_lock(&lk[r]);
  free(lk);
#endif
}

/* CPUSolver::addSourceToScalarFlux, src/CPUSolver.cpp:2608-2660 */
long oracle_add_source(const oracle_problem* p, oracle_state* s,
                       int negative_fluxes_allowed) {
  const long R = p->num_fsrs;
  const int G = p->num_groups;
  long neg = 0;
  set_threads(p);
#pragma omp parallel for schedule(static) reduction(+:neg)
  for (long r = 0; r < R; r++) {
    real vol = (real) p->fsr_vol[r];
    const float* st = p->sigma_t + (long) p->fsr_mat[r] * G;
    if (vol < (real) ZERO_VOLUME) vol = (real) 1e30;
    for (int g = 0; g < G; g++) {
      real v = s->phi[r * G + g];
      v /= ((real) st[g] * vol);
      v += (real) FOUR_PI * s->reduced[r * G + g] / (real) st[g];
      if (v < (real) 0 && !negative_fluxes_allowed) {
        v = FLUX_EPSILON;
        neg++;
      }
      s->phi[r * G + g] = v;
    }
  }
  return neg;
}

/* CPUSolver::computeKeff with keff from fission rates,
 * src/CPUSolver.cpp:2258-2333 */
void oracle_compute_keff(const oracle_problem* p, oracle_state* s) {
  const long R = p->num_fsrs;
  const int G = p->num_groups;
  double* rates = (double*) malloc(sizeof(double) * R);
  set_threads(p);
#pragma omp parallel for schedule(static)
  for (long r = 0; r < R; r++) {
    real grp[1024];
    const float* nf = p->nu_sigma_f + (long) p->fsr_mat[r] * G;
    for (int g = 0; g < G; g++) grp[g] = (real) nf[g] * s->phi[r * G + g];
    rates[r] = pairwise_sum_r(grp, G);
    rates[r] *= (real) p->fsr_vol[r];
  }
  double fission = pairwise_sum_d(rates, R);
  free(rates);
  s->keff *= fission / (double) R;
}

/* CPUSolver::computeResidual, src/CPUSolver.cpp:2113-2255 */
double oracle_residual(const oracle_problem* p, oracle_state* s, int res_type) {
  const long R = p->num_fsrs;
  const int G = p->num_groups;
  double* res = (double*) calloc(R, sizeof(double));
  long norm = R;
  if (res_type == RES_FISSION_SOURCE) {
    norm = 0;
    for (long r = 0; r < R; r++) norm += mat_fissile(p, p->fsr_mat[r]);
  }
  set_threads(p);
#pragma omp parallel for schedule(static)
  for (long r = 0; r < R; r++) {
    int m = p->fsr_mat[r];
    const float* nf = p->nu_sigma_f + (long) m * G;
    if (res_type == RES_SCALAR_FLUX) {
      for (int g = 0; g < G; g++) {
        real o = s->phi_old[r * G + g];
        if (o > (real) 0) {
          double d = ((double) s->phi[r * G + g] - o) / o;
          res[r] += d * d;
        }
      }
    } else if (res_type == RES_FISSION_SOURCE) {
      if (!mat_fissile(p, m)) continue;
      double nw = 0.0, od = 0.0;
      for (int g = 0; g < G; g++) {
        nw += (double) s->phi[r * G + g] * nf[g];
        od += (double) s->phi_old[r * G + g] * nf[g];
      }
      if (od > 0.0) res[r] = ((nw - od) / od) * ((nw - od) / od);
    } else {
      double nw = 0.0, od = 0.0;
      if (mat_fissile(p, m)) {
        for (int g = 0; g < G; g++) {
          nw += (double) s->phi[r * G + g] * nf[g];
          od += (double) s->phi_old[r * G + g] * nf[g];
        }
        nw /= s->keff;
        od /= s->keff;
      }
      const float* ss = p->sigma_s + (long) m * G * G;
      for (int gd = 0; gd < G; gd++)
        for (int g = 0; g < G; g++) {
          nw += (double) ss[gd * G + g] * s->phi[r * G + g];
          od += (double) ss[gd * G + g] * s->phi_old[r * G + g];
        }
      if (od > 0.0) res[r] = ((nw - od) / od) * ((nw - od) / od);
    }
  }
  double total = pairwise_sum_d(res, R);
  free(res);
  if (total < 0.0) total = 0.0;
  if (norm <= 0) norm = 1;
  return sqrt(total / (double) norm);
}

/* ------------------------------------------------------------ drivers */

/* Solver::computeEigenvalue without CMFD or stabilisation
 * (src/Solver.cpp:1542-1700; initial guess src/Solver.cpp:1710-1757).
 * Returns the number of iterations. */
int oracle_compute_eigenvalue(const oracle_problem* p, oracle_state* s,
                              int max_iters, int res_type, double threshold,
                              double* residual_out) {
  s->keff = 1.0;
  oracle_zero_track_fluxes(p, s);
  oracle_flatten(p, s, 1.0);
  oracle_normalize(p, s);
  oracle_store(p, s);
  double k_prev = s->keff;
  double residual = 0.0;
  int iters = 0;
  for (int i = 0; i < max_iters; i++) {
    oracle_compute_sources(p, s, i, 0);
    oracle_sweep(p, s);
    oracle_add_source(p, s, 0);
    oracle_compute_keff(p, s);
    oracle_normalize(p, s);
    residual = oracle_residual(p, s, res_type);
    int dk = (int) (1e5 * (s->keff - k_prev));
    k_prev = s->keff;
    oracle_store(p, s);
    iters++;
    if (residual < threshold && abs(dk) < 1) break;
  }
  if (residual_out) *residual_out = residual;
  return iters;
}

/* Solver::computeSource (src/Solver.cpp:1459-1535). */
int oracle_compute_source(const oracle_problem* p, oracle_state* s,
                          int max_iters, double k_eff, int res_type,
                          double threshold, double* residual_out) {
  s->keff = k_eff;
  oracle_zero_track_fluxes(p, s);
  oracle_flatten(p, s, 1.0);
  oracle_store(p, s);
  double residual = 0.0;
  for (int i = 0; i < max_iters; i++) {
    oracle_compute_sources(p, s, i, 0);
    oracle_sweep(p, s);
    oracle_add_source(p, s, 0);
    residual = oracle_residual(p, s, res_type);
    oracle_store(p, s);
    if (i > 1 && residual < threshold) {
      if (residual_out) *residual_out = residual;
      return i;
    }
  }
  if (residual_out) *residual_out = residual;
  return max_iters;
}

/* Solver::computeFlux with only_fixed_source (src/Solver.cpp:1352-1456). */
int oracle_compute_flux(const oracle_problem* p, oracle_state* s,
                        int max_iters, double threshold, double* residual_out) {
  s->keff = 1.0;
  oracle_zero_track_fluxes(p, s);
  oracle_flatten(p, s, 0.0);
  oracle_store(p, s);
  oracle_compute_sources(p, s, 0, 0);
  double residual = 0.0;
  for (int i = 0; i < max_iters; i++) {
    oracle_sweep(p, s);
    oracle_add_source(p, s, 0);
    residual = oracle_residual(p, s, RES_SCALAR_FLUX);
    oracle_store(p, s);
    if (i > 1 && residual < threshold) {
      if (residual_out) *residual_out = residual;
      return i;
    }
  }
  if (residual_out) *residual_out = residual;
  return max_iters;
}

int oracle_real_size(void) { return (int) sizeof(real); }
