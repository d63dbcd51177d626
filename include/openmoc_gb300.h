/**
 * @file openmoc_gb300.h
 * @brief C ABI of the GB300 (sm_103a) method-of-characteristics transport
 *        solver: the drop-in back end for OpenMOC's Solver hooks.
 *
 * Every entry point takes plain pointers and sizes and returns an int status
 * (MOC_OK = 0, negative on error); nothing throws across the ABI.  The text
 * of the last error on the calling thread is available from moc_last_error().
 * The OpenMOC-side subclass (openmoc_gb300/adapter/GB300Solver.h) turns a
 * non-zero status into log_printf(ERROR, ...), which throws std::logic_error
 * exactly like OpenMOC's own validation failures (src/log.cpp:588-599).
 *
 * A context owns one problem on one GPU: packed tracks, cross sections and
 * every flux array live in device memory until moc_destroy.  Host arrays
 * passed in are copied during the call and may be freed afterwards.  A
 * context is single-owner and not thread-safe.
 *
 * Array layouts (the packing done by openmoc_gb300/adapter/pack_reference.h
 * from OpenMOC's TrackGenerator, Geometry and Material objects):
 *   tracks are in UID order (src/TrackGenerator.cpp:1795-1818);
 *   seg_len[S] float, seg_fsr[S] int32, seg_off[T+1] int64;
 *   track_ang[T] int32: row of weights / inv_sin for the track;
 *   next[2T] int64: next track at the forward / backward end;
 *   flags[T] uint8: bit0 the forward exit enters its next track forward,
 *     bit1 the backward exit enters forward, bit2 / bit3 the forward /
 *     backward outgoing flux is transferred (REFLECTIVE or PERIODIC boundary);
 *   weights[A][Ph], inv_sin[A][Ph] float (2D: A = num_azim/2,
 *     Ph = num_polar/2; 3D: A = num_azim/2*num_polar, Ph = 1, inv_sin = 1);
 *   sigma_t[M][G], sigma_s[M][G][G] ([dest][orig]), nu_sigma_f[M][G],
 *     chi[M][G] float; fsr_mat[R] int32; fsr_vol[R] float;
 *   scalar fluxes / sources [R][G] float; boundary angular fluxes
 *     [T][2][F] float with F = G*Ph, polar-major within a direction
 *     (src/Solver.h:49-54).
 */
#ifndef OPENMOC_GB300_H_
#define OPENMOC_GB300_H_

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MOC_OK 0
#define MOC_ERR_ARG (-1)         /* invalid argument or inconsistent input */
#define MOC_ERR_CUDA (-2)        /* a CUDA runtime call failed */
#define MOC_ERR_STATE (-3)       /* call made in the wrong order */
#define MOC_ERR_MEMORY (-4)      /* device memory budget exceeded */
#define MOC_ERR_UNSUPPORTED (-5) /* feature not supported by this back end */
#define MOC_ERR_TIMEOUT (-6)     /* a device-side bounded wait ran out */

/* Residual types, same values as OpenMOC's residualType (src/Solver.h:82-92) */
#define MOC_SCALAR_FLUX 0
#define MOC_FISSION_SOURCE 1
#define MOC_TOTAL_SOURCE 2

/* Exponential evaluators for the attenuation factor 1 - exp(-tau/sin) */
#define MOC_EXP_TABLE 0     /* shared-memory interpolation table (default) */
#define MOC_EXP_INTRINSIC 1 /* hardware ex2 with a series below x = 1/16 */

/* Kernels of computeFSRSources (src/CPUSolver.cpp:1939-2025) */
#define MOC_SOURCES_AUTO 0   /* tensor cores (3xTF32) at >= 70 groups */
#define MOC_SOURCES_FP32 1   /* FP32 CUDA cores, one warp per FSR */
#define MOC_SOURCES_TF32X3 2 /* per-material batched contraction on the
                                tensor cores, TF32 high/low split products
                                (64 to 96 groups) */

typedef struct moc_ctx moc_ctx;

typedef struct {
  int32_t num_groups;     /* G */
  int32_t num_polar_half; /* Ph: polar values per track direction */
  int32_t num_angles;     /* A: rows of the weight tables */
  int32_t num_materials;  /* M */
  int64_t num_fsrs;       /* R */
  int64_t num_tracks;     /* T */
  int64_t num_segments;   /* S */
  int32_t solve_3d;       /* 1: explicit 3D tracks (weight per track) */
  int32_t device;         /* CUDA device ordinal */
} moc_dims;

/** Text of the last error reported on this thread ("" if none). */
const char* moc_last_error(void);

/** Library version string. */
const char* moc_version(void);

/** Creates a context; replaces GPUSolver's constructor + device setup
 *  (src/accel/cuda/GPUSolver.cu:771-796, src/accel/cuda/GPUQuery.cu). */
int moc_create(const moc_dims* dims, moc_ctx** out);

/** Frees every device buffer of the context (GPUSolver::~GPUSolver,
 *  src/accel/cuda/GPUSolver.cu:798-825). */
int moc_destroy(moc_ctx* ctx);

/** Uploads packed tracks and segments; replaces GPUSolver::initializeTracks
 *  and clone_track (src/accel/cuda/GPUSolver.cu:1312-1358,
 *  src/accel/cuda/clone.cu:86-126).  Checks every index on the host. */
int moc_upload_tracks(moc_ctx* ctx, const float* seg_len,
                      const int32_t* seg_fsr, const int64_t* seg_off,
                      const int32_t* track_ang, const int64_t* next,
                      const uint8_t* flags);

/** Uploads the quadrature tables; replaces GPUSolver::copyQuadrature
 *  (src/accel/cuda/GPUSolver.cu:1098-1148) and
 *  Quadrature::getWeightInline / getInvSinThetaInline (src/Quadrature.h:
 *  317-336). */
int moc_upload_quadrature(moc_ctx* ctx, const float* weights,
                          const float* inv_sin);

/** Uploads cross sections; replaces GPUSolver::initializeMaterials and
 *  clone_material (src/accel/cuda/GPUSolver.cu:1253-1310,
 *  src/accel/cuda/clone.cu:12-84). */
int moc_upload_materials(moc_ctx* ctx, const float* sigma_t,
                         const float* sigma_s, const float* nu_sigma_f,
                         const float* chi);

/** Optional fission cross sections sigma_f[M][G], needed only for
 *  moc_compute_fsr_fission_rates with nu = 0 (Material::getSigmaF,
 *  src/Material.h:81-103). */
int moc_upload_sigma_f(moc_ctx* ctx, const float* sigma_f);

/** Uploads FSR materials and volumes; replaces GPUSolver::initializeFSRs
 *  (src/accel/cuda/GPUSolver.cu:1170-1251). */
int moc_upload_fsrs(moc_ctx* ctx, const int32_t* fsr_mat,
                    const float* fsr_vol);

/** Sets (q != NULL) or clears (q == NULL) the [R][G] fixed sources;
 *  Solver::setFixedSourceByFSR / resetFixedSources (src/Solver.h:481-485),
 *  GPUSolver::initializeFixedSources (src/accel/cuda/GPUSolver.cu:1416). */
int moc_set_fixed_sources(moc_ctx* ctx, const float* q);

/** Solver::setConvergenceThreshold (src/Solver.cpp:461). */
int moc_set_convergence_threshold(moc_ctx* ctx, double threshold);

/** Selects the exponential evaluator (MOC_EXP_*);
 *  Solver::useExponentialInterpolation / useExponentialIntrinsic
 *  (src/Solver.cpp:575-595). */
int moc_set_exponential(moc_ctx* ctx, int kind);
int moc_get_exponential(moc_ctx* ctx, int* kind);

/** Autotuner of the sweep kernel: times every lanes-per-track-direction
 *  shape (and, unless moc_set_exponential fixed it, both exponential
 *  evaluators) on this context's problem and keeps the fastest.  Runs by
 *  itself at the first solve unless disabled with moc_set_autotune(ctx, 0)
 *  or a shape is set with moc_set_sweep_shape; results are cached per
 *  problem size for the process.  moc_autotune runs it now (and leaves zero
 *  fluxes behind); moc_get_tuning_log reports every timed candidate. */
int moc_set_autotune(moc_ctx* ctx, int on);
int moc_autotune(moc_ctx* ctx, int* lps, int* slots, int* exp_kind);
int moc_get_tuning_log(moc_ctx* ctx, int* lps, int* slots, int* exp_kind,
                       float* ms, int capacity, int* count);

/** Sweep kernel shape: lps lanes per track direction (power of two <= 32)
 *  each carrying `slots` pairs of energy groups, the fewest that cover the
 *  groups (slots = ceil(ceil(G / 2) / lps), at most the kernel's limit);
 *  lps = 0 restores the built-in choice.  Replaces
 *  GPUSolver::setNumThreadBlocks / setNumThreadsPerBlock
 *  (src/accel/cuda/GPUSolver.cu:987-1015). */
int moc_set_sweep_shape(moc_ctx* ctx, int lps, int slots);
int moc_get_sweep_shape(moc_ctx* ctx, int* lps, int* slots);

/** Iterations enqueued between two checks of the device convergence flag
 *  (default 4). */
int moc_set_iterations_per_sync(moc_ctx* ctx, int k);

/** Chooses the kernel of computeFSRSources (MOC_SOURCES_*); the group-count
 *  preconditions of MOC_SOURCES_TF32X3 are checked here.  No counterpart in
 *  the reference, which has one source kernel per back end. */
int moc_set_source_kernel(moc_ctx* ctx, int kind);
/** The kernel that computeFSRSources runs (MOC_SOURCES_FP32 or _TF32X3). */
int moc_get_source_kernel(moc_ctx* ctx, int* kind);
/** No counterpart in the reference.  How many times the tensor-core source
 *  kernel polls an mbarrier (its operand copy, its products) before it gives
 *  up: it then records the failure, waits once more with the full default
 *  limit for the work in flight, frees its tensor memory and returns, and
 *  the solve returns MOC_ERR_TIMEOUT.  polls < 0 restores the default
 *  (2^22); 0 gives up at once (a way to exercise the failure path). */
int moc_set_tensor_wait_limit(moc_ctx* ctx, int64_t polls);

/* ---- whole solves, device-resident (Solver::computeEigenvalue,
 *      computeSource, computeFlux; src/Solver.cpp:1352-1700) ------------- */
int moc_compute_eigenvalue(moc_ctx* ctx, int max_iters, int res_type);
int moc_compute_source(moc_ctx* ctx, int max_iters, double k_eff,
                       int res_type);
int moc_compute_flux(moc_ctx* ctx, int max_iters, int only_fixed_source);

/* ---- results ------------------------------------------------------------ */
int moc_get_keff(moc_ctx* ctx, double* keff);            /* Solver::getKeff */
int moc_get_num_iterations(moc_ctx* ctx, int* iters);    /* getNumIterations */
int moc_get_residual(moc_ctx* ctx, double* residual);
/** Solver::getFluxes / GPUSolver::getFluxes (src/accel/cuda/GPUSolver.cu:
 *  962-985): copies the [R][G] scalar flux to out (n = R*G). */
int moc_get_fluxes(moc_ctx* ctx, float* out, int64_t n);
/** Solver::setFluxes / GPUSolver::setFluxes (src/Solver.h:478,
 *  src/accel/cuda/GPUSolver.cu:1075-1096): sets the scalar flux (and the stored flux). */
int moc_set_fluxes(moc_ctx* ctx, const float* in, int64_t n);
/** Wall time of transport sweeps since the last solve started (ms), and
 *  the number of sweeps: Timer split "Transport Sweep"
 *  (src/CPUSolver.cpp:2365-2378). */
int moc_get_sweep_time(moc_ctx* ctx, double* ms, int64_t* num_sweeps);

/* ---- the protected Solver hooks, one call each (src/Solver.h:334-431) --- */
int moc_zero_track_fluxes(moc_ctx* ctx);
int moc_flatten_fsr_fluxes(moc_ctx* ctx, float value);
int moc_flatten_fsr_fluxes_chi(moc_ctx* ctx, int material);
int moc_store_fsr_fluxes(moc_ctx* ctx);
int moc_normalize_fluxes(moc_ctx* ctx, double* factor);
int moc_compute_fsr_sources(moc_ctx* ctx, int iteration);
int moc_transport_sweep(moc_ctx* ctx);
int moc_add_source_to_scalar_flux(moc_ctx* ctx);
int moc_compute_keff(moc_ctx* ctx);
int moc_compute_residual(moc_ctx* ctx, int res_type, double* residual);
int moc_set_keff(moc_ctx* ctx, double keff);
/** Solver::computeFSRFissionRates (src/Solver.h:539-540,
 *  src/accel/cuda/GPUSolver.cu:1970): volume-integrated
 *  (nu-)fission rate per FSR. */
int moc_compute_fsr_fission_rates(moc_ctx* ctx, double* rates, int64_t n,
                                  int nu);

/* ---- state access for tests and restart --------------------------------- */
/** Reduced sources Q/(4 pi) per FSR and group (Solver::getFSRSource*4pi). */
int moc_get_reduced_sources(moc_ctx* ctx, float* out, int64_t n);
/** Old (stored) scalar flux. */
int moc_get_old_fluxes(moc_ctx* ctx, float* out, int64_t n);
int moc_set_old_fluxes(moc_ctx* ctx, const float* in, int64_t n);
/** Track angular fluxes that the next sweep starts from ([T][2][F]), i.e.
 *  OpenMOC's _start_flux (src/Solver.h:252-253). */
int moc_get_start_flux(moc_ctx* ctx, float* out, int64_t n);
int moc_set_start_flux(moc_ctx* ctx, const float* in, int64_t n);

/** Measurement: `steps` eigenvalue iterations from the initial flux guess
 *  with the convergence exit disabled; step_ms[i] / sweep_ms[i] receive the
 *  CUDA-event time of iteration i and of its transport sweep.  With
 *  flush_l2 != 0 a buffer twice the L2 size is overwritten before each
 *  iteration, outside the timed interval.  Plays the role of the "Transport
 *  Sweep" timer split of Solver::printTimerReport (src/Solver.cpp:
 *  1802-1970). */
int moc_bench_iterations(moc_ctx* ctx, int steps, int res_type, int flush_l2,
                         double* step_ms, double* sweep_ms);

/** g = 1 - exp(-x) for n values with the sweep's evaluator `kind` (the
 *  attenuation the sweep applies; ExpEvaluator::computeExponential returns
 *  g(x)/x per unit path, src/ExpEvaluator.h:170-183).  For tests. */
int moc_eval_attenuation(moc_ctx* ctx, int kind, const float* x, float* g,
                         int64_t n);

/** No counterpart in the reference.  Contexts keep the device memory they
 *  free (up to 16 GiB), so that a context created and destroyed per request
 *  reuses it without cudaMalloc / cudaFree, and row copies to pageable host
 *  memory go through a kept page-locked bounce buffer; this returns all of
 *  it (and the page-locked scalar buffers) to the driver.  Call it with no
 *  context in use. */
int moc_release_cached_memory(void);

/** Largest num_fsrs that moc_fission_source_total_noalloc accepts. */
#define MOC_NOALLOC_MAX_FSRS (1 << 19)

/** No counterpart in the reference: an entry point that allocates nothing.
 *  Writes to *total (one device double) the total volume-integrated
 *  nu-fission source sum_r V_r sum_g nu_sigma_f[fsr_mat[r]][g] phi[r*ld+g],
 *  the sum keff and the flux normalisation are built from, for callers that
 *  own their device arrays but cannot allocate device memory: code whose
 *  GPU memory is held by another framework's pool or caching allocator, and
 *  code on a latency-critical path that cannot take cudaMalloc's implicit
 *  device synchronisation.  All pointers are device memory of the current
 *  device; stream is a cudaStream_t (NULL: the legacy default stream).
 *  nu_sigma_f holds num_materials rows of num_groups; an FSR whose
 *  fsr_mat entry is outside [0, num_materials) reads nothing and makes
 *  *total NaN.  Scratch is a fixed 4 MiB per-FSR array inside the library
 *  (held by every GPU that loads it), so num_fsrs may not exceed
 *  MOC_NOALLOC_MAX_FSRS; the first call in each CUDA context of a device
 *  (again after cudaDeviceReset) looks up that array's address (make it
 *  before any stream capture).  Calls share the array: calls that overlap
 *  on the GPU (different streams, or threads) race and must be serialised.
 *  The sum is deterministic. */
int moc_fission_source_total_noalloc(const float* phi, int64_t ld,
                                     const float* nu_sigma_f,
                                     int32_t num_materials,
                                     const int32_t* fsr_mat,
                                     const float* fsr_vol, int64_t num_fsrs,
                                     int32_t num_groups, void* stream,
                                     double* total);

/* ---- linear source (CPULSSolver, 2D and explicit 3D tracks) --------------
 * Switches the context from OpenMOC's CPUSolver to its CPULSSolver
 * semantics (src/CPULSSolver.cpp): flat plus linear (x, y; x, y, z on 3D
 * tracks) source and flux moments per FSR and group.  The arrays are what
 * pack_linear_source (openmoc_gb300/adapter/pack_reference.h) reads from
 * OpenMOC once the segments are re-centred on the FSR centroids. */
typedef struct {
  const float* seg_x;     /* [S] segment::_starting_position[0] relative to
                             its FSR centroid (src/TrackTraversingAlgorithms.
                             cpp:1320-1331) */
  const float* seg_y;     /* [S] */
  const double* ang_dir;  /* [A][2] cos(phi), sin(phi) of each angle row's
                             tracks (Track::getPhi) */
  const double* ang_wgt;  /* [A] Quadrature::getAzimSpacing * getAzimWeight */
  const double* pol_sin;  /* [A][Ph] Quadrature::getSinTheta */
  const double* pol_wgt;  /* [A][Ph] Quadrature::getPolarWeight */
  /* explicit 3D tracks (NULL for 2D); angle rows a * num_polar + p, Ph = 1,
   * pol_sin the sin of Track3D::getTheta and pol_wgt
   * getPolarSpacing * getPolarWeight of each row: */
  const float* seg_z;     /* [S] the z of the start relative to the FSR
                             centroid */
  const double* pol_cos;  /* [A] cos of Track3D::getTheta */
} moc_ls_geometry;

/** Sets the linear-source geometry (g != NULL) and computes the linear
 *  expansion matrices and source constants on the device
 *  (CPULSSolver::initializeFSRs + LinearExpansionGenerator,
 *  src/CPULSSolver.cpp:136-146, src/TrackTraversingAlgorithms.cpp:470-830);
 *  g == NULL returns to the flat source.  Needs tracks, quadrature,
 *  materials and FSRs uploaded; recomputed when materials or FSRs are
 *  uploaded again, dropped when tracks are. */
int moc_set_linear_source(moc_ctx* ctx, const moc_ls_geometry* g);
/** Whether the linear source is on, and how many FSRs have a singular
 *  expansion matrix (flat source there, as the reference warns). */
int moc_get_linear_source(moc_ctx* ctx, int* enabled, int64_t* num_flat);
/** Flux moments, reduced source moments (CPULSSolver::_scalar_flux_xyz,
 *  _reduced_sources_xyz) and fixed source moments
 *  (setFixedSourceMomentByFSR, src/CPULSSolver.cpp:280-307; NULL clears)
 *  as [R][3][G] (x, y, z; z is 0 in 2D). */
int moc_get_flux_moments(moc_ctx* ctx, float* out, int64_t n);
int moc_set_flux_moments(moc_ctx* ctx, const float* in, int64_t n);
int moc_get_source_moments(moc_ctx* ctx, float* out, int64_t n);
int moc_set_fixed_source_moments(moc_ctx* ctx, const float* in, int64_t n);
/** The inverse expansion matrices [R][NC] and the source constants
 *  [R][NC][G] (CPULSSolver::getLinearExpansionCoeffsBuffer,
 *  getSourceConstantsBuffer; either pointer may be NULL), NC = 3 (xx, yy,
 *  xy) in 2D and 6 (xx, yy, xy, xz, yz, zz) on 3D tracks. */
int moc_get_linear_expansion(moc_ctx* ctx, double* ilem, float* src_const);
/** Solver::allowNegativeFluxes (src/Solver.cpp:623): no clamping of
 *  negative sources or fluxes. */
int moc_set_negative_fluxes_allowed(moc_ctx* ctx, int allowed);

/** Transport stabilization types (stabilizationType, src/Solver.h:103-113). */
#define MOC_STABILIZE_DIAGONAL 0
#define MOC_STABILIZE_YAMAMOTO 1
#define MOC_STABILIZE_GLOBAL 2

/** Solver::stabilizeTransport(factor, type) (src/Solver.cpp:676-681):
 *  from the second eigenvalue iteration on, the flux after keff is blended
 *  with the flux at the start of the iteration
 *  (CPUSolver::computeStabilizingFlux + stabilizeFlux,
 *  src/CPUSolver.cpp:2665-2810) before the normalisation.  on = 0 turns it
 *  off.  With a linear source the flux moments take the same correction
 *  against their own start-of-iteration values (CPULSSolver::
 *  computeStabilizingFlux / stabilizeFlux, src/CPULSSolver.cpp:886-1049),
 *  except under YAMAMOTO, whose moment branch in the reference leaves them
 *  as they are. */
int moc_set_transport_stabilization(moc_ctx* ctx, int on, double factor,
                                    int type);
/** The protected hooks: CPUSolver::computeStabilizingFlux keeps the current
 *  flux (and a linear source's moments) as the base of the correction;
 *  stabilizeFlux applies it (src/CPUSolver.cpp:2665-2810,
 *  src/CPULSSolver.cpp:886-1049). */
int moc_compute_stabilizing_flux(moc_ctx* ctx);
int moc_stabilize_flux(moc_ctx* ctx);
/** CPUSolver::computeFSRFissionSources / computeFSRScatterSources
 *  (src/CPUSolver.cpp:2030-2110): the reduced source holds the fission (or
 *  the scattering) part alone, sum over g' of M[g][g'] phi[g'] / (4 pi), as
 *  the Krylov solvers of openmoc.krylov use it; read it back with
 *  moc_get_reduced_sources. */
int moc_compute_fsr_fission_sources(moc_ctx* ctx);
int moc_compute_fsr_scatter_sources(moc_ctx* ctx);

/** No counterpart in the reference: instances.  The context's problem holds
 *  num_instances cross-section sets over one track laydown, their groups
 *  side by side (wide group k * G + g; the materials' arrays of
 *  moc_upload_materials are [M][K*G] and the scattering matrix block
 *  diagonal).  moc_compute_eigenvalue then solves them together: one sweep
 *  per iteration carries every instance's groups along each track, while
 *  sources, keff and the normalisation stay per instance (the solve stops
 *  when the largest residual over the wide groups and every instance's keff
 *  change meet the criterion).  num_instances = 0 returns to one problem.
 *  Flat-source eigenvalue loop of stored segments only; the source
 *  contraction runs on the CUDA cores. */
int moc_set_instances(moc_ctx* ctx, int num_instances);
/** Each instance's keff after moc_compute_eigenvalue. */
int moc_get_instance_keffs(moc_ctx* ctx, double* keffs, int num_instances);

/** Solver::setKeffFromNeutronBalance (src/Solver.cpp:2045-2048; used by
 *  CPUSolver::computeKeff and transferBoundaryFlux, src/CPUSolver.cpp:
 *  2258-2330, 2593-2600): on = 1 computes keff = fission / (absorption +
 *  leakage), the leakage tallied by the sweep at vacuum track ends, instead
 *  of keff *= fission / num_FSRs.  For the flat-source sweep of stored
 *  segments; with CMFD the coarse solve's keff applies. */
int moc_set_keff_from_neutron_balance(moc_ctx* ctx, int on);

/* ---- on-the-fly 3D segmentation ------------------------------------------
 * For explicit 3D problems made by extruding a radial lattice
 * (moc_lattice_extrude): instead of the stored 3D segments, every 3D track
 * is cut from the radial segments under it during the sweep (the
 * OTF_TRACKS segment formation of OpenMOC's TrackGenerator3D,
 * src/TraverseSegments.cpp:151-265).  Arrays as moc_lattice_export_otf
 * (include/openmoc_gb300_lattice.h) gives them. */
typedef struct {
  int64_t num_radial_tracks;     /* T2 */
  int64_t num_radial_segments;   /* S2 */
  const int32_t* trk;      /* [T][4] radial track, first radial segment
                              crossed (in traversal order), count, 1 if the
                              traversal runs against the radial track */
  const float* trk_f;      /* [T][4] start a0 along the traversal, span,
                              height above the cut at a0, 0 */
  const float* ang;        /* [A][4] cot theta, 1 / cot theta, 1 / sin theta, 0 */
  const float* rad_len;    /* [S2] radial segment lengths */
  const int32_t* rad_fsr;  /* [S2] their FSR ids */
  const int64_t* rad_off;  /* [T2 + 1] */
  const float* rad_start;  /* [S2] start of each radial segment on its track */
  const float* rad_total;  /* [T2] radial track lengths */
  int32_t above_fsr;       /* the region above the cut plane */
} moc_otf_tracks;

/** Switches a 3D context (tracks, quadrature, materials and FSRs uploaded;
 *  the explicit segments may be empty) to on-the-fly segmentation; NULL
 *  returns to the stored segments.  Dropped when tracks are re-uploaded. */
int moc_set_otf_tracks(moc_ctx* ctx, const moc_otf_tracks* tracks);
int moc_get_otf_tracks(moc_ctx* ctx, int* enabled);

/* ---- CMFD acceleration ----------------------------------------------------
 * Coarse-mesh finite-difference acceleration of moc_compute_eigenvalue
 * (2D problems, flat or linear source; replaces the reference's Cmfd, src/Cmfd.h, as
 * Geometry::setCmfd attaches it and Solver::computeEigenvalue calls
 * Cmfd::computeKeff in place of computeKeff, src/Solver.cpp:1597-1645).
 * Every iteration the sweep also tallies the partial currents out of the
 * coarse cells; the FSR fluxes are reduced on the mesh, the coarse
 * diffusion eigenproblem (cross sections collapsed by flux, surface
 * diffusion coefficients with Larsen's correction and the nonlinear
 * correction term, relaxation, flux limiting) is solved in FP64 on the
 * host, and the FSR fluxes are scaled by the ratio of the new to the old
 * coarse flux.  The mesh must not cut an FSR: each FSR lies in one cell. */
#define MOC_BC_VACUUM 0
#define MOC_BC_REFLECTIVE 1
typedef struct {
  int32_t num_x, num_y;        /* Cmfd::setLatticeStructure */
  const double* widths_x;      /* [num_x] cm (Cmfd::setWidths) */
  const double* widths_y;      /* [num_y] cm */
  const int32_t* fsr_cell;     /* [R] cell of every FSR: iy * num_x + ix,
                                  iy counted from y-min (Cmfd::findCmfdCell,
                                  src/Cmfd.cpp:2007-2026) */
  const int8_t* track_end_face;/* [T][2] mesh boundary face crossed where the
                                  forward / backward traversal of each track
                                  leaves the geometry (0 x-min, 1 y-min,
                                  2 x-max, 3 y-max), -1 none */
  int32_t boundary[4];         /* x-min, y-min, x-max, y-max:
                                  MOC_BC_VACUUM or MOC_BC_REFLECTIVE */
  int32_t num_cmfd_groups;     /* E (Cmfd::setGroupStructure) */
  const int32_t* group_of;     /* [G] coarse group of each group, 0 for the
                                  first, rising by at most 1; NULL: E = G,
                                  one coarse group per group */
  int32_t num_edc_angles;      /* n > 0: Larsen's effective diffusion
                                  coefficient correction over these angles
                                  (azimuthal < num_azim / 2 x polar <
                                  num_polar / 2); 0: no correction */
  const double* edc_mu;        /* [n] cos theta */
  const double* edc_weight;    /* [n] azimuthal x polar weight */
  double relaxation;           /* setCMFDRelaxationFactor (reference 0.7) */
  double sor_factor;           /* setSORRelaxationFactor (reference 1.5) */
  int32_t flux_limiting;       /* useFluxLimiting (reference 1) */
  int32_t num_unbounded_iterations; /* setNumUnboundedIterations (0) */
  int32_t solve_on_host;       /* 0: the coarse solve runs on the GPU in
                                  FP32 (as the reference's single-precision
                                  build), with no host round trip; 1: on the
                                  host in FP64, tallies read back every
                                  iteration; 2: on the GPU on one block;
                                  3: on the GPU cell-parallel (one thread per
                                  coarse cell over a cluster of blocks; up to
                                  8 coarse groups).  0 takes 3 where it
                                  applies, else 2. */
  int32_t k_nearest;           /* 0: each FSR takes its cell's ratio;
                                  1..9: Cmfd::setKNearest, the ratio
                                  weighted over the nearest of the 3 x 3
                                  cells around it by centroid distance */
  const double* fsr_centroid;  /* [R][2] (x, y), needed when k_nearest > 0
                                  (TrackGenerator::generateFSRCentroids) */
  double origin_x, origin_y;   /* the mesh's x-min / y-min corner */
} moc_cmfd_mesh;

/** Attaches CMFD to the context (tracks, quadrature, materials and FSRs
 *  uploaded; not with on-the-fly segmentation); NULL detaches it.  With the
 *  linear source the flux moments are prolonged too and Larsen's factor is
 *  not applied (CPULSSolver's CMFD).  Dropped when tracks are re-uploaded.
 *  Uses the hardware exponential (MOC_ERR_UNSUPPORTED if the table was
 *  requested). */
int moc_set_cmfd(moc_ctx* ctx, const moc_cmfd_mesh* mesh);
/** Whether CMFD is attached, the last coarse eigenvalue, the coarse power
 *  iterations and SOR sweeps of the last coarse solve, its prolongation
 *  ratio farthest from 1, and whether it failed to converge (no
 *  prolongation that iteration); any pointer may be NULL. */
int moc_get_cmfd_info(moc_ctx* ctx, int* enabled, double* keff,
                      int* power_iterations, int* linear_iterations,
                      double* max_ratio, int* failed);
/** The coarse fluxes of the last coarse solve, [cells][E], before (old) and
 *  after (new) it, each normalised to unit total fission source
 *  (Cmfd::rescaleFlux); either pointer may be NULL. */
int moc_get_cmfd_fluxes(moc_ctx* ctx, double* old_flux, double* new_flux,
                        int64_t n);

/** Number of CUDA kernels this library launched on the context so far. */
int moc_get_launch_count(moc_ctx* ctx, int64_t* launches);

#ifdef __cplusplus
}
#endif

#endif /* OPENMOC_GB300_H_ */
