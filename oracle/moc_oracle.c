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
  /* [T] leakage tallied at vacuum track ends, or NULL: keff from the ratio
   * of fission sources (Solver::setKeffFromNeutronBalance switches to
   * fission / (absorption + leakage)) */
  real* leakage;
  /* [R][G] stabilizing flux, or NULL: no transport stabilization
   * (Solver::stabilizeTransport with stab_type 0 DIAGONAL, 1 YAMAMOTO,
   * 2 GLOBAL and stab_factor) */
  real* stab_flux;
  int32_t stab_type;
  double stab_factor;
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

/* CPUSolver::transferBoundaryFlux, src/CPUSolver.cpp:2560-2600; the
 * leakage at a vacuum end takes the quadrature weight of the track's polar
 * index for every polar value, the index being 0 for 2D tracks
 * (src/TrackTraversingAlgorithms.cpp:895-905). */
static void transfer(const oracle_problem* p, oracle_state* s, long t, int fwd,
                     const float* psi) {
  const int F = fluxes_per_track(p);
  uint8_t f = p->flags[t];
  int moves = fwd ? (f & 4) : (f & 8);
  if (!moves && s->leakage) {
    real weight = (real) p->weights[(long) p->track_ang[t] * p->num_polar_half];
    for (int pe = 0; pe < F; pe++) s->leakage[t] += weight * (real) psi[pe];
  }
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
/* CMFD partial currents (Cmfd::tallyCurrent, src/Cmfd.h:572-660): where a
 * track leaves a coarse cell, sum_p w_p psi_p of the outgoing angular flux
 * is added to [cell][face][group] (faces 0 x-min, 1 y-min, 2 x-max,
 * 3 y-max); a crossing through a corner goes half by way of each
 * neighbouring cell (Cmfd::splitEdgeCurrents, src/Cmfd.cpp:2249-2345).
 * Track ends on the boundary add to the face given in end_face. */
typedef struct {
  const int* cell;              /* [R] coarse cell of every FSR */
  const signed char* end_face;  /* [T][2] */
  int nx;
  double* cur;                  /* [cells][4][G] */
} oracle_cmfd_tally;

static void add_current(const oracle_problem* p, const oracle_cmfd_tally* cm,
                        int cell, int face, double frac, int ang,
                        const float* psi) {
  const int G = p->num_groups, Ph = p->num_polar_half;
  double* dst = cm->cur + ((long) cell * 4 + face) * G;
  for (int g = 0; g < G; g++) {
    double j = 0.0;
    for (int pp = 0; pp < Ph; pp++)
      j += (double) p->weights[ang * Ph + pp] * (double) psi[pp * G + g];
#pragma omp atomic
    dst[g] += frac * j;
  }
}

static void tally_crossing(const oracle_problem* p,
                           const oracle_cmfd_tally* cm, long fsr,
                           long fsr_next, int end_face, int ang,
                           const float* psi) {
  const int c0 = cm->cell[fsr];
  if (fsr_next < 0) {
    if (end_face >= 0) add_current(p, cm, c0, end_face, 1.0, ang, psi);
    return;
  }
  const int c1 = cm->cell[fsr_next];
  if (c1 == c0) return;
  const int dx = c1 % cm->nx - c0 % cm->nx, dy = c1 / cm->nx - c0 / cm->nx;
  const int fx = dx > 0 ? 2 : 0, fy = dy > 0 ? 3 : 1;
  if (dx != 0 && dy != 0) {
    add_current(p, cm, c0, fx, 0.5, ang, psi);
    add_current(p, cm, c0 + dx, fy, 0.5, ang, psi);
    add_current(p, cm, c0, fy, 0.5, ang, psi);
    add_current(p, cm, c0 + dy * cm->nx, fx, 0.5, ang, psi);
  } else {
    add_current(p, cm, c0, dx != 0 ? fx : fy, 1.0, ang, psi);
  }
}

/* CPUSolver::transportSweep + TransportSweep::onTrack
 * (src/CPUSolver.cpp:2338-2398, src/TrackTraversingAlgorithms.cpp:890-1052):
 * zero the scalar flux, copy the start fluxes into the boundary fluxes, then
 * sweep every track forward and backward, tallying FSR contributions in a
 * buffer that is flushed whenever the FSR changes; with cm, also the CMFD
 * partial currents (2D). */
static void sweep_impl(const oracle_problem* p, oracle_state* s,
                       const oracle_cmfd_tally* cm) {
  const long R = p->num_fsrs;
  const int G = p->num_groups;
  const long T = p->num_tracks;
  const int F = fluxes_per_track(p);
  memset(s->phi, 0, sizeof(real) * R * G);
  if (s->leakage) memset(s->leakage, 0, sizeof(real) * T);
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
        if (cm)
          tally_crossing(p, cm, fsr, k < n - 1 ? p->seg_fsr[b + k + 1] : -1,
                         cm->end_face[2 * t], ang, psi);
        if (k < n - 1 && fsr != p->seg_fsr[b + k + 1])
          flush(p, s, fsr, weight, buf, locks);
      }
      transfer(p, s, t, 1, psi);
      psi = s->boundary + (t * 2 + 1) * (long) F;
      for (int k = n - 1; k >= 0; k--) {
        long fsr = p->seg_fsr[b + k];
        tally_segment(p, s, fsr, (real) p->seg_len[b + k],
                      p->fsr_mat[fsr], ang, buf, psi);
        if (cm)
          tally_crossing(p, cm, fsr, k > 0 ? p->seg_fsr[b + k - 1] : -1,
                         cm->end_face[2 * t + 1], ang, psi);
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

void oracle_sweep(const oracle_problem* p, oracle_state* s) {
  sweep_impl(p, s, NULL);
}

/* The sweep with the CMFD current tallies added into cur [cells][4][G]
 * (zeroed by the caller). */
void oracle_sweep_currents(const oracle_problem* p, oracle_state* s,
                           const int* cell, const signed char* end_face,
                           int nx, double* cur) {
  oracle_cmfd_tally cm = {cell, end_face, nx, cur};
  sweep_impl(p, s, &cm);
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
  if (!s->leakage) {
    free(rates);
    s->keff *= fission / (double) R;
    return;
  }
  /* absorption = sigma_t less the scattering out of each group, formed as
   * Material::getSigmaA does (src/Material.cpp:230-252) */
#pragma omp parallel for schedule(static)
  for (long r = 0; r < R; r++) {
    real grp[1024];
    const int m = p->fsr_mat[r];
    const float* st = p->sigma_t + (long) m * G;
    const float* ss = p->sigma_s + (long) m * G * G;
    for (int g = 0; g < G; g++) {
      real sa = (real) st[g];
      for (int gd = 0; gd < G; gd++) sa -= (real) ss[gd * G + g];
      grp[g] = sa * s->phi[r * G + g];
    }
    rates[r] = pairwise_sum_r(grp, G);
    rates[r] *= (real) p->fsr_vol[r];
  }
  double absorption = pairwise_sum_d(rates, R);
  free(rates);
  double leakage = pairwise_sum_r(s->leakage, p->num_tracks);
  s->keff = fission / (absorption + leakage);
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

/* The largest |sigma_s,gg / sigma_t,g| over the FSRs' materials times the
 * factor (the YAMAMOTO ratio of group g, src/CPUSolver.cpp:2697-2712). */
static real yamamoto_ratio(const oracle_problem* p, const oracle_state* s,
                           int g) {
  const int G = p->num_groups;
  float max_ratio = 0.0f;
  for (long r = 0; r < p->num_fsrs; r++) {
    const int m = p->fsr_mat[r];
    const float scat = p->sigma_s[((long) m * G + g) * G + g];
    const float total = p->sigma_t[(long) m * G + g];
    const float ratio = fabsf(scat / total);
    if (ratio > max_ratio) max_ratio = ratio;
  }
  return (real) (max_ratio * s->stab_factor);
}

/* CPUSolver::computeStabilizingFlux, src/CPUSolver.cpp:2665-2730 */
void oracle_compute_stabilizing_flux(const oracle_problem* p, oracle_state* s) {
  const long R = p->num_fsrs;
  const int G = p->num_groups;
  if (s->stab_type == 0) {
    for (long r = 0; r < R; r++) {
      const int m = p->fsr_mat[r];
      for (int e = 0; e < G; e++) {
        const real sigma_s = (real) p->sigma_s[((long) m * G + e) * G + e];
        const real sigma_t = (real) p->sigma_t[(long) m * G + e];
        if (sigma_s < 0)
          s->stab_flux[r * G + e] = (real) (-s->phi[r * G + e] *
                                            s->stab_factor * sigma_s / sigma_t);
      }
    }
  } else if (s->stab_type == 1) {
    for (int e = 0; e < G; e++) {
      const real max_ratio = yamamoto_ratio(p, s, e);
      for (long r = 0; r < R; r++)
        s->stab_flux[r * G + e] = s->phi[r * G + e] * max_ratio;
    }
  } else {
    const real mult = (real) (1.0 / s->stab_factor - 1.0);
    for (long i = 0; i < R * G; i++) s->stab_flux[i] = mult * s->phi[i];
  }
}

/* CPUSolver::stabilizeFlux, src/CPUSolver.cpp:2736-2810 */
void oracle_stabilize_flux(const oracle_problem* p, oracle_state* s) {
  const long R = p->num_fsrs;
  const int G = p->num_groups;
  if (s->stab_type == 0) {
    for (long r = 0; r < R; r++) {
      const int m = p->fsr_mat[r];
      for (int e = 0; e < G; e++) {
        const real sigma_s = (real) p->sigma_s[((long) m * G + e) * G + e];
        const real sigma_t = (real) p->sigma_t[(long) m * G + e];
        if (sigma_s < 0) {
          s->phi[r * G + e] += s->stab_flux[r * G + e];
          s->phi[r * G + e] = (real) (s->phi[r * G + e] /
                                      (1.0 - s->stab_factor * sigma_s / sigma_t));
        }
      }
    }
  } else if (s->stab_type == 1) {
    for (int e = 0; e < G; e++) {
      const real max_ratio = yamamoto_ratio(p, s, e);
      for (long r = 0; r < R; r++) {
        s->phi[r * G + e] += s->stab_flux[r * G + e];
        s->phi[r * G + e] /= (1 + max_ratio);
      }
    }
  } else {
    for (long i = 0; i < R * G; i++) {
      s->phi[i] += s->stab_flux[i];
      s->phi[i] = (real) (s->phi[i] * s->stab_factor);
    }
  }
}

/* ------------------------------------------------------------ drivers */

/* Solver::computeEigenvalue without CMFD (src/Solver.cpp:1542-1700;
 * initial guess src/Solver.cpp:1710-1757), with transport stabilization
 * when s->stab_flux is set.  Returns the number of iterations. */
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
  if (s->stab_flux)
    memset(s->stab_flux, 0, sizeof(real) * p->num_fsrs * p->num_groups);
  for (int i = 0; i < max_iters; i++) {
    if (i > 0 && s->stab_flux) oracle_compute_stabilizing_flux(p, s);
    oracle_compute_sources(p, s, i, 0);
    oracle_sweep(p, s);
    oracle_add_source(p, s, 0);
    oracle_compute_keff(p, s);
    if (i > 0 && s->stab_flux) oracle_stabilize_flux(p, s);
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

/* ================================================================ linear
 * source.  CPULSSolver (src/CPULSSolver.cpp) restated for 2D and explicit 3D
 * tracks: the same source iteration with flux and source moments along x
 * and y (and z in 3D) about each FSR centroid.  Layouts follow the
 * reference: moments [R][3][G] (x, y, z; z stays 0 in 2D),
 * src/CPULSSolver.h:20-23; the linear expansion matrix inverse [R][NC] and
 * the source constants [R][NC][G], NC = 3 in 2D (xx, yy, xy) and 6 in 3D
 * (xx, yy, xy, xz, yz, zz), src/TrackTraversingAlgorithms.cpp:470-490.
 *
 * The exponential terms are evaluated in double from their definitions
 * (series below x = 1, closed forms above), where the reference uses
 * rational approximations (src/exponentials.h:101-323, accurate to 2e-7 and
 * 1e-6), then rounded to ORACLE_REAL. */

typedef struct {
  const float* seg_x;     /* [S] segment start relative to its FSR centroid */
  const float* seg_y;     /* [S] */
  const double* ang_dir;  /* [A][2] cos(phi), sin(phi) */
  const double* ang_wgt;  /* [A] azimuthal spacing x azimuthal weight */
  const double* pol_sin;  /* [A][Ph] sin(theta_p) */
  const double* pol_wgt;  /* [A][Ph] polar weight; 3D: polar spacing x
                             polar weight */
  const float* seg_z;     /* 3D: [S] z of the start; NULL in 2D */
  const double* pol_cos;  /* 3D: [A] cos(theta) of each angle row */
} oracle_ls_geometry;

typedef struct {
  double* ilem;           /* [R][NC] */
  real* src_const;        /* [R][NC][G] */
  real* mom;              /* [R][3][G] flux moments */
  real* red_xyz;          /* [R][3][G] reduced source moments */
  const real* fixed_xy;   /* [R][2][G] fixed source moments, or NULL (2D) */
  int32_t negative_allowed;
  int32_t num_flat;       /* FSRs whose expansion matrix is singular */
  real* stab_xyz;         /* [R][3][G] stabilizing flux moments, or NULL:
                             the moments are not stabilized */
} oracle_ls_state;

#define MIN_DET 1E-10     /* src/constants.h:70 */

/* G(x) = (x - 1 + exp(-x)) / x^2 = sum_k (-x)^k / (k+2)! */
static double exp_g(double x) {
  if (x < 1.0) {
    double term = 0.5, sum = 0.5;
    for (int k = 1; k < 24; k++) {
      term *= -x / (double) (k + 2);
      sum += term;
    }
    return sum;
  }
  return (x + expm1(-x)) / (x * x);
}

/* G2(x) = 2/3 - (1 + 2/x) (1/x + 1/2 - (1 + 1/x)(1 - exp(-x))/x)
 *       = sum_{m>=1} (-x)^m [(m+1)/(m+2)! - 2(m+2)/(m+3)!]
 * (the quantity of src/exponentials.h:283-292). */
static double exp_g2(double x) {
  if (x < 1.0) {
    double sum = 0.0, xm = 1.0, f2 = 2.0;   /* f2 = (m+2)!, m = 0 */
    for (int m = 1; m < 26; m++) {
      xm *= -x;
      f2 *= (double) (m + 2);               /* (m+2)! */
      double c = (double) (m + 1) / f2 - 2.0 * (double) (m + 2) /
                                             (f2 * (double) (m + 3));
      sum += c * xm;
    }
    return sum;
  }
  double f1 = -expm1(-x) / x;
  return 2.0 / 3.0 - (1.0 + 2.0 / x) * (1.0 / x + 0.5 - (1.0 + 1.0 / x) * f1);
}

/* LinearExpansionGenerator::onTrack + execute for 2D tracks
 * (src/TrackTraversingAlgorithms.cpp:543-640, :716-826): the volume
 * moments of every FSR, their 2x2 inverse, and the source constants.
 * Returns the number of FSRs left with a flat source (singular matrix). */
static int ls_constants_3d(const oracle_problem* p, const oracle_ls_geometry* g,
                           oracle_ls_state* s);

int oracle_ls_constants(const oracle_problem* p, const oracle_ls_geometry* g,
                        oracle_ls_state* s) {
  if (p->solve_3d) return ls_constants_3d(p, g, s);
  const long R = p->num_fsrs;
  const int G = p->num_groups, Ph = p->num_polar_half;
  double* lem = (double*) calloc((size_t) R * 3, sizeof(double));
  double* sc = (double*) calloc((size_t) R * 3 * G, sizeof(double));
  for (long t = 0; t < p->num_tracks; t++) {
    const int a = p->track_ang[t];
    const double cph = g->ang_dir[2 * a], sph = g->ang_dir[2 * a + 1];
    const double wgt = g->ang_wgt[a];
    for (long k = p->seg_off[t]; k < p->seg_off[t + 1]; k++) {
      const long r = p->seg_fsr[k];
      const float* st = p->sigma_t + (long) p->fsr_mat[r] * G;
      const double len = p->seg_len[k], vol = p->fsr_vol[r];
      const double xc = (double) g->seg_x[k] + 0.5 * len * cph;
      const double yc = (double) g->seg_y[k] + 0.5 * len * sph;
      const double vol_impact = wgt * len / vol;
      const double src_constant = vol_impact * len / 2.0;
      for (int e = 0; e < G; e++) {
        double c0 = vol_impact * xc * xc, c1 = vol_impact * yc * yc;
        double c2 = vol_impact * xc * yc;
        const double tau = len * (double) st[e];
        for (int pp = 0; pp < Ph; pp++) {
          const double sn = g->pol_sin[a * Ph + pp];
          const double g2 = len * exp_g2(tau / sn) * src_constant * 2.0 *
                            g->pol_wgt[a * Ph + pp] * sn;
          c0 += cph * cph * g2;
          c1 += sph * sph * g2;
          c2 += sph * cph * g2;
        }
        sc[(r * 3 + 0) * G + e] += c0;
        sc[(r * 3 + 1) * G + e] += c1;
        sc[(r * 3 + 2) * G + e] += c2;
      }
      lem[r * 3 + 0] += wgt * len / vol * (xc * xc + cph * cph * len * len / 12.0);
      lem[r * 3 + 1] += wgt * len / vol * (yc * yc + sph * sph * len * len / 12.0);
      lem[r * 3 + 2] += wgt * len / vol * (xc * yc + sph * cph * len * len / 12.0);
    }
  }
  int flat = 0;
  for (long r = 0; r < R; r++) {
    const double det = lem[r * 3] * lem[r * 3 + 1] - lem[r * 3 + 2] * lem[r * 3 + 2];
    if (fabs(det) < MIN_DET) {
      s->ilem[r * 3] = s->ilem[r * 3 + 1] = s->ilem[r * 3 + 2] = 0.0;
      flat++;
    } else {
      s->ilem[r * 3 + 0] = lem[r * 3 + 1] / det;
      s->ilem[r * 3 + 1] = lem[r * 3 + 0] / det;
      s->ilem[r * 3 + 2] = -lem[r * 3 + 2] / det;
    }
  }
  for (long i = 0; i < R * 3 * G; i++) s->src_const[i] = (real) sc[i];
  free(lem);
  free(sc);
  s->num_flat = flat;
  return flat;
}

/* The 3D branch of LinearExpansionGenerator::onTrack and execute
 * (src/TrackTraversingAlgorithms.cpp:543-640, :716-781): direction
 * (cos phi sin theta, sin phi sin theta, cos theta), the row weight
 * w_a d_a w_p d_p, G2 at the segment's optical length, six moments and
 * their 3x3 inverse; flat where the determinant is below 1e-10 or the
 * volume below 1e-6. */
static int ls_constants_3d(const oracle_problem* p, const oracle_ls_geometry* g,
                           oracle_ls_state* s) {
  const long R = p->num_fsrs;
  const int G = p->num_groups;
  double* lem = (double*) calloc((size_t) R * 6, sizeof(double));
  double* sc = (double*) calloc((size_t) R * 6 * G, sizeof(double));
  for (long t = 0; t < p->num_tracks; t++) {
    const int a = p->track_ang[t];
    const double cph = g->ang_dir[2 * a], sph = g->ang_dir[2 * a + 1];
    const double sth = g->pol_sin[a], cth = g->pol_cos[a];
    double wgt = g->ang_wgt[a];
    wgt *= g->pol_wgt[a];
    for (long k = p->seg_off[t]; k < p->seg_off[t + 1]; k++) {
      const long r = p->seg_fsr[k];
      const float* st = p->sigma_t + (long) p->fsr_mat[r] * G;
      const double len = p->seg_len[k], vol = p->fsr_vol[r];
      const double xc = (double) g->seg_x[k] + len * 0.5 * cph * sth;
      const double yc = (double) g->seg_y[k] + len * 0.5 * sph * sth;
      const double zc = (double) g->seg_z[k] + len * 0.5 * cth;
      const double vol_impact = wgt * len / vol;
      const double src_constant = vol_impact * len / 2.0;
      for (int e = 0; e < G; e++) {
        const double tau = len * (double) st[e];
        const double g2 = exp_g2(tau) * len * src_constant;
        double* c = sc + r * 6 * G + e;
        c[0] += vol_impact * xc * xc + cph * cph * g2 * sth * sth;
        c[G] += vol_impact * yc * yc + sph * sph * g2 * sth * sth;
        c[2 * G] += vol_impact * xc * yc + sph * cph * g2 * sth * sth;
        c[3 * G] += vol_impact * xc * zc + cph * cth * g2 * sth;
        c[4 * G] += vol_impact * yc * zc + sph * cth * g2 * sth;
        c[5 * G] += vol_impact * zc * zc + cth * cth * g2;
      }
      const double w = wgt * len / vol, l2 = len * len;
      lem[r * 6 + 0] += w * (xc * xc + cph * sth * len * cph * sth * len / 12.0);
      lem[r * 6 + 1] += w * (yc * yc + sph * sth * len * sph * sth * len / 12.0);
      lem[r * 6 + 2] += w * (xc * yc + sph * cph * sth * len * sth * len / 12.0);
      lem[r * 6 + 3] += w * (xc * zc + cph * cth * sth * l2 / 12.0);
      lem[r * 6 + 4] += w * (yc * zc + sph * cth * sth * l2 / 12.0);
      lem[r * 6 + 5] += w * (zc * zc + cth * len * cth * len / 12.0);
    }
  }
  int flat = 0;
  for (long r = 0; r < R; r++) {
    const double* m = lem + r * 6;
    double* il = s->ilem + r * 6;
    const double det = m[0] * m[1] * m[5] + m[2] * m[4] * m[3] +
                       m[3] * m[2] * m[4] - m[0] * m[4] * m[4] -
                       m[3] * m[1] * m[3] - m[2] * m[2] * m[5];
    if (fabs(det) < MIN_DET || p->fsr_vol[r] < 1e-6) {
      for (int i = 0; i < 6; i++) il[i] = 0.0;
      flat++;
    } else {
      il[0] = (m[1] * m[5] - m[4] * m[4]) / det;
      il[1] = (m[0] * m[5] - m[3] * m[3]) / det;
      il[2] = (m[3] * m[4] - m[2] * m[5]) / det;
      il[3] = (m[2] * m[4] - m[3] * m[1]) / det;
      il[4] = (m[3] * m[2] - m[0] * m[4]) / det;
      il[5] = (m[0] * m[1] - m[2] * m[2]) / det;
    }
  }
  for (long i = 0; i < R * 6 * G; i++) s->src_const[i] = (real) sc[i];
  free(lem);
  free(sc);
  s->num_flat = flat;
  return flat;
}

/* CPULSSolver::flattenFSRFluxes, src/CPULSSolver.cpp:343-353 */
void oracle_ls_flatten(const oracle_problem* p, oracle_state* s,
                       oracle_ls_state* ls, double value) {
  oracle_flatten(p, s, value);
  memset(ls->mom, 0, sizeof(real) * p->num_fsrs * 3 * p->num_groups);
}

/* CPULSSolver::normalizeFluxes, src/CPULSSolver.cpp:362-378 */
double oracle_ls_normalize(const oracle_problem* p, oracle_state* s,
                           oracle_ls_state* ls) {
  double f = oracle_normalize(p, s);
  long n = p->num_fsrs * 3 * p->num_groups;
  for (long i = 0; i < n; i++) ls->mom[i] *= f;
  return f;
}

/* CPULSSolver::computeFSRSources (2D branch), src/CPULSSolver.cpp:386-527:
 * the flat source of CPUSolver, then the x and y source moments through the
 * inverse expansion matrix.  Returns the negative flat sources found. */
/* The 3D branch: the x, y and z source moments through the 3x3 inverse
 * (src/CPULSSolver.cpp:466-487). */
static void ls_sources_3d(const oracle_problem* p, oracle_state* s,
                          oracle_ls_state* ls, int iteration) {
  const long R = p->num_fsrs;
  const int G = p->num_groups;
  set_threads(p);
#pragma omp parallel for schedule(static)
  for (long r = 0; r < R; r++) {
    real buf[1024];
    const int m = p->fsr_mat[r];
    const float* ss = p->sigma_s + (long) m * G * G;
    const float* nf = p->nu_sigma_f + (long) m * G;
    const float* ch = p->chi + (long) m * G;
    const int fissile = mat_fissile(p, m);
    const double* il = ls->ilem + r * 6;
    for (int gd = 0; gd < G; gd++) {
      real src[3];
      for (int i = 0; i < 3; i++) {
        const real* mi = ls->mom + (r * 3 + i) * G;
        double fis = 0.0;
        if (fissile) {
          for (int g = 0; g < G; g++) buf[g] = ((real) ch[gd] * (real) nf[g]) * mi[g];
          fis = pairwise_sum_r(buf, G) / s->keff;
        }
        for (int g = 0; g < G; g++) buf[g] = (real) ss[gd * G + g] * mi[g];
        src[i] = (real) (pairwise_sum_r(buf, G) + fis);
      }
      real* q = ls->red_xyz + r * 3 * G + gd;
      if (ls->negative_allowed || s->reduced[r * G + gd] > 10 * FLUX_EPSILON ||
          iteration > 29) {
        q[0] = (real) (ONE_OVER_FOUR_PI / 2 *
                       (il[0] * src[0] + il[2] * src[1] + il[3] * src[2]));
        q[G] = (real) (ONE_OVER_FOUR_PI / 2 *
                       (il[2] * src[0] + il[1] * src[1] + il[4] * src[2]));
        q[2 * G] = (real) (ONE_OVER_FOUR_PI / 2 *
                           (il[3] * src[0] + il[4] * src[1] + il[5] * src[2]));
      } else {
        q[0] = q[G] = q[2 * G] = 0;
      }
    }
  }
}

long oracle_ls_compute_sources(const oracle_problem* p, oracle_state* s,
                               oracle_ls_state* ls, int iteration) {
  long neg = oracle_compute_sources(p, s, iteration, ls->negative_allowed);
  if (p->solve_3d) {
    ls_sources_3d(p, s, ls, iteration);
    return neg;
  }
  const long R = p->num_fsrs;
  const int G = p->num_groups;
  set_threads(p);
#pragma omp parallel for schedule(static)
  for (long r = 0; r < R; r++) {
    real buf[1024];
    const int m = p->fsr_mat[r];
    const float* ss = p->sigma_s + (long) m * G * G;
    const float* nf = p->nu_sigma_f + (long) m * G;
    const float* ch = p->chi + (long) m * G;
    const int fissile = mat_fissile(p, m);
    const double* il = ls->ilem + r * 3;
    const real* mx = ls->mom + (r * 3 + 0) * G;
    const real* my = ls->mom + (r * 3 + 1) * G;
    for (int gd = 0; gd < G; gd++) {
      double fis_x = 0.0, fis_y = 0.0;
      if (fissile) {
        for (int g = 0; g < G; g++) buf[g] = ((real) ch[gd] * (real) nf[g]) * mx[g];
        fis_x = pairwise_sum_r(buf, G) / s->keff;
        for (int g = 0; g < G; g++) buf[g] = ((real) ch[gd] * (real) nf[g]) * my[g];
        fis_y = pairwise_sum_r(buf, G) / s->keff;
      }
      for (int g = 0; g < G; g++) buf[g] = (real) ss[gd * G + g] * mx[g];
      double sca_x = pairwise_sum_r(buf, G);
      for (int g = 0; g < G; g++) buf[g] = (real) ss[gd * G + g] * my[g];
      double sca_y = pairwise_sum_r(buf, G);
      real src_x = (real) (sca_x + fis_x), src_y = (real) (sca_y + fis_y);
      if (ls->fixed_xy) {
        src_x += ls->fixed_xy[(r * 2 + 0) * G + gd];
        src_y += ls->fixed_xy[(r * 2 + 1) * G + gd];
      }
      real* rx = ls->red_xyz + (r * 3 + 0) * G + gd;
      real* ry = ls->red_xyz + (r * 3 + 1) * G + gd;
      if (ls->negative_allowed || s->reduced[r * G + gd] > 10 * FLUX_EPSILON ||
          iteration > 29) {
        *rx = (real) (ONE_OVER_FOUR_PI / 2 * (il[0] * src_x + il[2] * src_y));
        *ry = (real) (ONE_OVER_FOUR_PI / 2 * (il[2] * src_x + il[1] * src_y));
      } else {
        *rx = 0;
        *ry = 0;
      }
    }
  }
  return neg;
}

/* Linear-source attenuation along one segment, CPULSSolver::tallyLSScalarFlux
 * 2D branch (src/CPULSSolver.cpp:653-741); pos is the segment's start in the
 * direction of travel, dir the travel direction. */
static void ls_tally_segment(const oracle_problem* p, const oracle_state* s,
                             const oracle_ls_state* ls, long fsr, real length,
                             int mat, int ang, const real pos[2],
                             const real dir[2], real* buf, real* bx, real* by,
                             float* psi) {
  const int G = p->num_groups;
  const int Ph = p->num_polar_half;
  const float* st = p->sigma_t + (long) mat * G;
  const real cx = 2 * pos[0] + length * dir[0];
  const real cy = 2 * pos[1] + length * dir[1];
  const real* qx = ls->red_xyz + (fsr * 3 + 0) * G;
  const real* qy = ls->red_xyz + (fsr * 3 + 1) * G;
  for (int pp = 0; pp < Ph; pp++) {
    const real wgt = (real) p->weights[ang * Ph + pp];
    const real inv_sin = (real) p->inv_sin[ang * Ph + pp];
    for (int g = 0; g < G; g++) {
      const int pe = pp * G + g;
      const real tau = (real) st[g] * length;
      double x = (double) (tau * inv_sin);
      if (x < 1e-8) x = 1e-8;
      const double gg = exp_g(x);
      const double f1 = (1.0 - x * gg) * (double) inv_sin;
      const double gs = gg * (double) inv_sin;
      const real F1 = (real) f1, F2 = (real) (2.0 * gs - f1);
      real H = (real) (f1 - gs);
      const real src_flat = s->reduced[fsr * G + g] + qx[g] * cx + qy[g] * cy;
      const real src_lin = dir[0] * qx[g] + dir[1] * qy[g];
      H *= wgt * tau * length * (real) psi[pe];
      real delta = (tau * (real) psi[pe] - length * src_flat) * F1 -
                   length * length * src_lin * F2;
      psi[pe] = (float) ((real) psi[pe] - delta);
      delta *= wgt;
      buf[g] += delta;
      bx[g] += H * dir[0] + delta * pos[0];
      by[g] += H * dir[1] + delta * pos[1];
    }
  }
}

/* CPULSSolver::accumulateLinearFluxContribution, src/CPULSSolver.cpp:749-781 */
static void ls_flush(const oracle_problem* p, oracle_state* s,
                     oracle_ls_state* ls, long fsr, real* buf, real* bx,
                     real* by, void* locks) {
  const int G = p->num_groups;
#ifdef _OPENMP
  omp_set_lock(&((omp_lock_t*) locks)[fsr]);
#else
  (void) locks;
#endif
  for (int g = 0; g < G; g++) {
    s->phi[fsr * G + g] += buf[g];
    ls->mom[(fsr * 3 + 0) * G + g] += bx[g];
    ls->mom[(fsr * 3 + 1) * G + g] += by[g];
  }
#ifdef _OPENMP
  omp_unset_lock(&((omp_lock_t*) locks)[fsr]);
#endif
  memset(buf, 0, sizeof(real) * G);
  memset(bx, 0, sizeof(real) * G);
  memset(by, 0, sizeof(real) * G);
}

/* The 3D branch of tallyLSScalarFlux (src/CPULSSolver.cpp:555-646): the
 * segment's own optical length, no polar loop; the quadrature weight is
 * applied when the buffers are flushed. */
static void ls_tally_segment_3d(const oracle_problem* p, const oracle_state* s,
                                const oracle_ls_state* ls, long fsr,
                                real length, int mat, const real pos[3],
                                const real dir[3], real* buf, real* bx,
                                real* by, real* bz, float* psi) {
  const int G = p->num_groups;
  const float* st = p->sigma_t + (long) mat * G;
  real c2[3];
  for (int i = 0; i < 3; i++) c2[i] = 2 * pos[i] + length * dir[i];
  const real* q = ls->red_xyz + fsr * 3 * G;
  for (int g = 0; g < G; g++) {
    real src_flat = s->reduced[fsr * G + g];
    for (int i = 0; i < 3; i++) src_flat += q[i * G + g] * c2[i];
    real src_lin = q[g] * dir[0];
    src_lin += q[G + g] * dir[1];
    src_lin += q[2 * G + g] * dir[2];
    const real tau = length * (real) st[g];
    const double gg = exp_g(tau > 1e-8 ? (double) tau : 1e-8);
    const real G_ = (real) gg;
    const real F1 = 1 - tau * G_;
    const real F2 = 2 * G_ - F1;
    real H = F1 - G_;
    H *= length * (real) psi[g] * tau;
    const real delta = (tau * (real) psi[g] - length * src_flat) * F1 -
                       src_lin * length * length * F2;
    psi[g] = (float) ((real) psi[g] - delta);
    buf[g] += delta;
    bx[g] += H * dir[0] + delta * pos[0];
    by[g] += H * dir[1] + delta * pos[1];
    bz[g] += H * dir[2] + delta * pos[2];
  }
}

/* CPULSSolver::accumulateLinearFluxContribution with the 3D weight. */
static void ls_flush_3d(const oracle_problem* p, oracle_state* s,
                        oracle_ls_state* ls, long fsr, real weight, real* buf,
                        void* locks) {
  const int G = p->num_groups;
#ifdef _OPENMP
  omp_set_lock(&((omp_lock_t*) locks)[fsr]);
#else
  (void) locks;
#endif
  for (int g = 0; g < G; g++) {
    s->phi[fsr * G + g] += weight * buf[g];
    for (int i = 0; i < 3; i++)
      ls->mom[(fsr * 3 + i) * G + g] += weight * buf[(i + 1) * G + g];
  }
#ifdef _OPENMP
  omp_unset_lock(&((omp_lock_t*) locks)[fsr]);
#endif
  memset(buf, 0, sizeof(real) * 4 * G);
}

static void ls_sweep_3d(const oracle_problem* p, const oracle_ls_geometry* geo,
                        oracle_state* s, oracle_ls_state* ls) {
  const long R = p->num_fsrs;
  const int G = p->num_groups;
  const long T = p->num_tracks;
  const int F = fluxes_per_track(p);
  memset(s->phi, 0, sizeof(real) * R * G);
  memset(ls->mom, 0, sizeof(real) * R * 3 * G);
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
    real* buf = (real*) calloc(4 * (size_t) G, sizeof(real));
#pragma omp for schedule(dynamic)
    for (long t = 0; t < T; t++) {
      const long b = p->seg_off[t];
      const int n = (int) (p->seg_off[t + 1] - b);
      const int ang = p->track_ang[t];
      const real weight = (real) p->weights[ang];
      /* TransportSweep::onTrack, src/TrackTraversingAlgorithms.cpp:913-926 */
      const double sth = geo->pol_sin[ang], cth = geo->pol_cos[ang];
      real dir[3] = {(real) (geo->ang_dir[2 * ang] * sth),
                     (real) (geo->ang_dir[2 * ang + 1] * sth), (real) cth};
      float* psi = s->boundary + (t * 2) * (long) F;
      for (int k = 0; k < n; k++) {
        const long fsr = p->seg_fsr[b + k];
        const real pos[3] = {(real) geo->seg_x[b + k], (real) geo->seg_y[b + k],
                             (real) geo->seg_z[b + k]};
        ls_tally_segment_3d(p, s, ls, fsr, (real) p->seg_len[b + k],
                            p->fsr_mat[fsr], pos, dir, buf, buf + G,
                            buf + 2 * G, buf + 3 * G, psi);
        if (k < n - 1 && fsr != p->seg_fsr[b + k + 1])
          ls_flush_3d(p, s, ls, fsr, weight, buf, locks);
      }
      transfer(p, s, t, 1, psi);
      const real fdir[3] = {dir[0], dir[1], dir[2]};
      for (int i = 0; i < 3; i++) dir[i] = -dir[i];
      psi = s->boundary + (t * 2 + 1) * (long) F;
      for (int k = n - 1; k >= 0; k--) {
        const long fsr = p->seg_fsr[b + k];
        const real len = (real) p->seg_len[b + k];
        const real pos[3] = {(real) geo->seg_x[b + k] + fdir[0] * len,
                             (real) geo->seg_y[b + k] + fdir[1] * len,
                             (real) geo->seg_z[b + k] + fdir[2] * len};
        ls_tally_segment_3d(p, s, ls, fsr, len, p->fsr_mat[fsr], pos, dir,
                            buf, buf + G, buf + 2 * G, buf + 3 * G, psi);
        if (k == 0 || fsr != p->seg_fsr[b + k - 1])
          ls_flush_3d(p, s, ls, fsr, weight, buf, locks);
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

/* CPUSolver::transportSweep with the linear-source tally: as oracle_sweep,
 * the direction of a track from its angles (src/TrackTraversingAlgorithms.
 * cpp:913-926), reversed for the backward pass, which starts each segment
 * at its far end. */
void oracle_ls_sweep(const oracle_problem* p, const oracle_ls_geometry* geo,
                     oracle_state* s, oracle_ls_state* ls) {
  if (p->solve_3d) {
    ls_sweep_3d(p, geo, s, ls);
    return;
  }
  const long R = p->num_fsrs;
  const int G = p->num_groups;
  const long T = p->num_tracks;
  const int F = fluxes_per_track(p);
  memset(s->phi, 0, sizeof(real) * R * G);
  memset(ls->mom, 0, sizeof(real) * R * 3 * G);
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
    real* buf = (real*) calloc(3 * (size_t) G, sizeof(real));
    real* bx = buf + G;
    real* by = buf + 2 * G;
#pragma omp for schedule(dynamic)
    for (long t = 0; t < T; t++) {
      const long b = p->seg_off[t];
      const int n = (int) (p->seg_off[t + 1] - b);
      const int ang = p->track_ang[t];
      real dir[2] = {(real) geo->ang_dir[2 * ang], (real) geo->ang_dir[2 * ang + 1]};
      float* psi = s->boundary + (t * 2) * (long) F;
      for (int k = 0; k < n; k++) {
        const long fsr = p->seg_fsr[b + k];
        const real pos[2] = {(real) geo->seg_x[b + k], (real) geo->seg_y[b + k]};
        ls_tally_segment(p, s, ls, fsr, (real) p->seg_len[b + k],
                         p->fsr_mat[fsr], ang, pos, dir, buf, bx, by, psi);
        if (k < n - 1 && fsr != p->seg_fsr[b + k + 1])
          ls_flush(p, s, ls, fsr, buf, bx, by, locks);
      }
      transfer(p, s, t, 1, psi);
      const real fdir[2] = {dir[0], dir[1]};
      dir[0] = -dir[0];
      dir[1] = -dir[1];
      psi = s->boundary + (t * 2 + 1) * (long) F;
      for (int k = n - 1; k >= 0; k--) {
        const long fsr = p->seg_fsr[b + k];
        const real len = (real) p->seg_len[b + k];
        const real pos[2] = {(real) geo->seg_x[b + k] + fdir[0] * len,
                             (real) geo->seg_y[b + k] + fdir[1] * len};
        ls_tally_segment(p, s, ls, fsr, len, p->fsr_mat[fsr], ang, pos, dir,
                         buf, bx, by, psi);
        if (k == 0 || fsr != p->seg_fsr[b + k - 1])
          ls_flush(p, s, ls, fsr, buf, bx, by, locks);
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

/* CPULSSolver::addSourceToScalarFlux (2D), src/CPULSSolver.cpp:787-882 */
/* The 3D branch: six source constants per group (src/CPULSSolver.cpp:
 * 824-846). */
static long ls_add_source_3d(const oracle_problem* p, oracle_state* s,
                             oracle_ls_state* ls) {
  const long R = p->num_fsrs;
  const int G = p->num_groups;
  long neg = 0;
  set_threads(p);
#pragma omp parallel for schedule(static) reduction(+:neg)
  for (long r = 0; r < R; r++) {
    real vol = (real) p->fsr_vol[r];
    if (vol < (real) ZERO_VOLUME) vol = (real) 1e30;
    const float* st = p->sigma_t + (long) p->fsr_mat[r] * G;
    const real* c = ls->src_const + r * 6 * G;
    for (int e = 0; e < G; e++) {
      const real fc = (real) (FOUR_PI * 2);
      const real qx = ls->red_xyz[(r * 3 + 0) * G + e];
      const real qy = ls->red_xyz[(r * 3 + 1) * G + e];
      const real qz = ls->red_xyz[(r * 3 + 2) * G + e];
      real v = s->phi[r * G + e];
      v /= vol;
      v += (real) FOUR_PI * s->reduced[r * G + e];
      v /= (real) st[e];
      real mx = ls->mom[(r * 3 + 0) * G + e];
      mx /= vol;
      mx += fc * qx * c[e];
      mx += fc * qy * c[2 * G + e];
      real my = ls->mom[(r * 3 + 1) * G + e];
      my /= vol;
      my += fc * qx * c[2 * G + e];
      my += fc * qy * c[G + e];
      mx += fc * qz * c[3 * G + e];
      my += fc * qz * c[4 * G + e];
      real mz = ls->mom[(r * 3 + 2) * G + e];
      mz /= vol;
      mz += fc * qx * c[3 * G + e];
      mz += fc * qy * c[4 * G + e];
      mz += fc * qz * c[5 * G + e];
      mx /= (real) st[e];
      my /= (real) st[e];
      mz /= (real) st[e];
      if (v < (real) 0 && !ls->negative_allowed) {
        neg++;
        real old = s->phi_old[r * G + e];
        v = old > FLUX_EPSILON ? old : FLUX_EPSILON;
        mx = my = mz = 0;
      }
      s->phi[r * G + e] = v;
      ls->mom[(r * 3 + 0) * G + e] = mx;
      ls->mom[(r * 3 + 1) * G + e] = my;
      ls->mom[(r * 3 + 2) * G + e] = mz;
    }
  }
  return neg;
}

long oracle_ls_add_source(const oracle_problem* p, oracle_state* s,
                          oracle_ls_state* ls) {
  if (p->solve_3d) return ls_add_source_3d(p, s, ls);
  const long R = p->num_fsrs;
  const int G = p->num_groups;
  long neg = 0;
  set_threads(p);
#pragma omp parallel for schedule(static) reduction(+:neg)
  for (long r = 0; r < R; r++) {
    real vol = (real) p->fsr_vol[r];
    if (vol < (real) ZERO_VOLUME) vol = (real) 1e30;
    const float* st = p->sigma_t + (long) p->fsr_mat[r] * G;
    const real* sc = ls->src_const + r * 3 * G;
    for (int e = 0; e < G; e++) {
      const real flux_const = (real) (FOUR_PI * 2);
      const real qx = ls->red_xyz[(r * 3 + 0) * G + e];
      const real qy = ls->red_xyz[(r * 3 + 1) * G + e];
      real v = s->phi[r * G + e];
      v /= vol;
      v += (real) FOUR_PI * s->reduced[r * G + e];
      v /= (real) st[e];
      real mx = ls->mom[(r * 3 + 0) * G + e];
      mx /= vol;
      mx += flux_const * qx * sc[e];
      mx += flux_const * qy * sc[2 * G + e];
      real my = ls->mom[(r * 3 + 1) * G + e];
      my /= vol;
      my += flux_const * qx * sc[2 * G + e];
      my += flux_const * qy * sc[G + e];
      mx /= (real) st[e];
      my /= (real) st[e];
      if (v < (real) 0 && !ls->negative_allowed) {
        neg++;
        real old = s->phi_old[r * G + e];
        v = old > FLUX_EPSILON ? old : FLUX_EPSILON;
        mx = 0;
        my = 0;
      }
      s->phi[r * G + e] = v;
      ls->mom[(r * 3 + 0) * G + e] = mx;
      ls->mom[(r * 3 + 1) * G + e] = my;
    }
  }
  return neg;
}

/* CPULSSolver::computeStabilizingFlux, moment part
 * (src/CPULSSolver.cpp:886-965), after the flat part.  DIAGONAL: where the
 * in-group scattering is negative, -f sigma_s,gg / sigma_t,g times each
 * moment; GLOBAL: (1 / f - 1) times each moment.  YAMAMOTO: the reference's
 * moment branch assigns `ratio = max_ratio` where the flat branch raises
 * max_ratio, so its ratio stays 0 and the stabilizing moments are zero. */
void oracle_ls_compute_stabilizing_moments(const oracle_problem* p,
                                           const oracle_state* s,
                                           oracle_ls_state* ls) {
  const long R = p->num_fsrs;
  const int G = p->num_groups;
  if (!ls->stab_xyz) return;
  if (s->stab_type == 0) {
    for (long r = 0; r < R; r++) {
      const int m = p->fsr_mat[r];
      for (int e = 0; e < G; e++) {
        const real sigma_s = (real) p->sigma_s[((long) m * G + e) * G + e];
        const real sigma_t = (real) p->sigma_t[(long) m * G + e];
        if (sigma_s < 0.0)
          for (int i = 0; i < 3; i++)
            ls->stab_xyz[(r * 3 + i) * G + e] =
                (real) (-ls->mom[(r * 3 + i) * G + e] * s->stab_factor *
                        sigma_s / sigma_t);
      }
    }
  } else if (s->stab_type == 1) {
    const real max_ratio = 0.0;
    for (long i = 0; i < R * 3 * G; i++) ls->stab_xyz[i] = ls->mom[i] * max_ratio;
  } else {
    const real mult = (real) (1.0 / s->stab_factor - 1.0);
    for (long i = 0; i < R * 3 * G; i++) ls->stab_xyz[i] = ls->mom[i] * mult;
  }
}

/* CPULSSolver::stabilizeFlux, moment part (src/CPULSSolver.cpp:970-1049):
 * the stabilizing moments added and the sum scaled as the flat flux is
 * (DIAGONAL 1 / (1 - f sigma_s,gg / sigma_t,g) where sigma_s,gg < 0,
 * YAMAMOTO 1 / (1 + 0), GLOBAL f). */
void oracle_ls_stabilize_moments(const oracle_problem* p, const oracle_state* s,
                                 oracle_ls_state* ls) {
  const long R = p->num_fsrs;
  const int G = p->num_groups;
  if (!ls->stab_xyz) return;
  for (long r = 0; r < R; r++) {
    const int m = p->fsr_mat[r];
    for (int e = 0; e < G; e++) {
      const real sigma_s = (real) p->sigma_s[((long) m * G + e) * G + e];
      const real sigma_t = (real) p->sigma_t[(long) m * G + e];
      for (int i = 0; i < 3; i++) {
        real* x = &ls->mom[(r * 3 + i) * G + e];
        const real add = ls->stab_xyz[(r * 3 + i) * G + e];
        if (s->stab_type == 0) {
          if (sigma_s < 0.0) {
            *x += add;
            *x = (real) (*x / (1.0 - s->stab_factor * sigma_s / sigma_t));
          }
        } else if (s->stab_type == 1) {
          *x += add;
          *x = (real) (*x / (1.0 + 0.0));
        } else {
          *x += add;
          *x = (real) (*x * s->stab_factor);
        }
      }
    }
  }
}

/* Solver::computeEigenvalue with the linear-source hooks. */
int oracle_ls_compute_eigenvalue(const oracle_problem* p,
                                 const oracle_ls_geometry* geo,
                                 oracle_state* s, oracle_ls_state* ls,
                                 int max_iters, int res_type, double threshold,
                                 double* residual_out) {
  s->keff = 1.0;
  oracle_ls_constants(p, geo, ls);
  oracle_zero_track_fluxes(p, s);
  oracle_ls_flatten(p, s, ls, 1.0);
  oracle_ls_normalize(p, s, ls);
  oracle_store(p, s);
  double k_prev = s->keff;
  double residual = 0.0;
  int iters = 0;
  if (s->stab_flux)
    memset(s->stab_flux, 0, sizeof(real) * p->num_fsrs * p->num_groups);
  if (ls->stab_xyz)
    memset(ls->stab_xyz, 0, sizeof(real) * p->num_fsrs * 3 * p->num_groups);
  for (int i = 0; i < max_iters; i++) {
    if (i > 0 && s->stab_flux) {
      oracle_compute_stabilizing_flux(p, s);
      oracle_ls_compute_stabilizing_moments(p, s, ls);
    }
    oracle_ls_compute_sources(p, s, ls, i);
    oracle_ls_sweep(p, geo, s, ls);
    oracle_ls_add_source(p, s, ls);
    oracle_compute_keff(p, s);
    if (i > 0 && s->stab_flux) {
      oracle_stabilize_flux(p, s);
      oracle_ls_stabilize_moments(p, s, ls);
    }
    oracle_ls_normalize(p, s, ls);
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

/* Solver::computeSource with the linear-source hooks. */
int oracle_ls_compute_source(const oracle_problem* p,
                             const oracle_ls_geometry* geo, oracle_state* s,
                             oracle_ls_state* ls, int max_iters, double k_eff,
                             int res_type, double threshold,
                             double* residual_out) {
  s->keff = k_eff;
  oracle_ls_constants(p, geo, ls);
  oracle_zero_track_fluxes(p, s);
  oracle_ls_flatten(p, s, ls, 1.0);
  oracle_store(p, s);
  double residual = 0.0;
  for (int i = 0; i < max_iters; i++) {
    oracle_ls_compute_sources(p, s, ls, i);
    oracle_ls_sweep(p, geo, s, ls);
    oracle_ls_add_source(p, s, ls);
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

/* Solver::computeFlux (only the fixed source) with the linear-source hooks. */
int oracle_ls_compute_flux(const oracle_problem* p,
                           const oracle_ls_geometry* geo, oracle_state* s,
                           oracle_ls_state* ls, int max_iters,
                           double threshold, double* residual_out) {
  s->keff = 1.0;
  oracle_ls_constants(p, geo, ls);
  oracle_zero_track_fluxes(p, s);
  oracle_ls_flatten(p, s, ls, 0.0);
  oracle_store(p, s);
  oracle_ls_compute_sources(p, s, ls, 0);
  double residual = 0.0;
  for (int i = 0; i < max_iters; i++) {
    oracle_ls_sweep(p, geo, s, ls);
    oracle_ls_add_source(p, s, ls);
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
