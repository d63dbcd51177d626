/**
 * @file GB300Solver.h
 * @brief OpenMOC Solver subclass that runs the flat-source MOC hot path on a
 *        GB300 GPU through libopenmoc_gb300.so (include/openmoc_gb300.h).
 *
 * Drop-in for OpenMOC's CPUSolver / GPUSolver (src/CPUSolver.h,
 * src/accel/cuda/GPUSolver.h): it overrides the protected hooks of the
 * abstract Solver (src/Solver.h:334-431) and the public virtuals used by
 * callers (getFlux, getFluxes, setFluxes, resetFixedSources,
 * computeFSRFissionRates), so OpenMOC's own Solver::computeEigenvalue /
 * computeSource / computeFlux drive it hook by hook.  computeEigenvalue,
 * computeSource and computeFlux are also redeclared here (hiding the base
 * versions for callers that hold a GB300Solver) to run the whole source
 * iteration device-resident, with the same initialisation sequence and
 * convergence tests as src/Solver.cpp:1352-1700.
 *
 * Errors from the library become log_printf(ERROR, ...), which throws
 * std::logic_error like every OpenMOC validation failure
 * (src/log.cpp:588-599); SWIG maps that to a Python RuntimeError.
 *
 * Compiled against OpenMOC's headers (-I <openmoc>/src, with OpenMOC's
 * FP_PRECISION / CMFD_PRECISION macros) and linked with its library and with
 * libopenmoc_gb300.so and libcudart.
 */
#ifndef OPENMOC_GB300_SOLVER_H_
#define OPENMOC_GB300_SOLVER_H_

#include <map>
#include <vector>

#include "Solver.h"

struct moc_ctx;

class GB300Solver : public Solver {
 protected:
  moc_ctx* _ctx;
  int _device;
  int _exp_kind;           /* -1: chosen by the autotuner */
  bool _uploaded;

  void check(int status, const char* what);
  virtual void upload();
  /* CMFD from the Geometry (Solver::initializeCmfd), attached to the
   * context as moc_set_cmfd wants it */
  void attachCmfd();
  double _cmfd_relaxation, _cmfd_sor;
  bool _cmfd_flux_limiting, _cmfd_on_host;
  int _cmfd_unbounded, _cmfd_k_nearest;
  int materialIndex(Material* m);

  /* Solver hooks (src/Solver.h:334-431) */
  void initializeFluxArrays();
  void initializeSourceArrays();
  void initializeFSRs();
  void zeroTrackFluxes();
  void flattenFSRFluxes(FP_PRECISION value);
  void flattenFSRFluxesChiSpectrum();
  void storeFSRFluxes();
  double normalizeFluxes();
  void computeStabilizingFlux();
  void stabilizeFlux();
  void computeFSRSources(int iteration);
  void computeFSRFissionSources();
  void computeFSRScatterSources();
  double computeResidual(residualType res_type);
  void computeKeff();
  void addSourceToScalarFlux();
  void transportSweep();

 public:
  GB300Solver(TrackGenerator* track_generator = NULL, int device = 0);
  virtual ~GB300Solver();

  void setTrackGenerator(TrackGenerator* track_generator);
  double getFlux(long fsr_id, int group);
  void getFluxes(FP_PRECISION* out_fluxes, int num_fluxes);
  void setFluxes(FP_PRECISION* in_fluxes, int num_fluxes);
  void resetFixedSources();
  void computeFSRFissionRates(double* fission_rates, long num_FSRs,
                              bool nu = false);

  /** Shared-memory table (0) or hardware ex2 (1) for 1 - exp(-x); the
   *  default lets the autotuner pick the faster. */
  void setExponentialEvaluator(int kind);
  /** The factors of the Geometry's Cmfd, which OpenMOC keeps private:
   *  relaxation (Cmfd::setCMFDRelaxationFactor, default 0.7), SOR factor
   *  (setSORRelaxationFactor, 1.5), flux limiting (useFluxLimiting, on),
   *  unbounded iterations (setNumUnboundedIterations, 0), k of
   *  setKNearest (used when the Cmfd's centroid update is on, default 1);
   *  on_host runs the coarse solve on the host in FP64 instead of on the
   *  GPU in FP32. */
  void setCmfdFactors(double relaxation, double sor, bool flux_limiting,
                      int unbounded_iterations, bool on_host = false,
                      int k_nearest = 1);

  /* device-resident source iteration */
  void computeEigenvalue(int max_iters = 1000,
                         residualType res_type = FISSION_SOURCE);
  void computeSource(int max_iters = 1000, double k_eff = 1.0,
                     residualType res_type = TOTAL_SOURCE);
  void computeFlux(int max_iters = 1000, bool only_fixed_source = true);
};

/**
 * The linear-source counterpart (OpenMOC's CPULSSolver, src/CPULSSolver.h)
 * for 2D tracks: the same hooks with flat plus x/y source and flux moments.
 * upload() also packs the segments' start positions relative to the FSR
 * centroids (re-centred by Solver::initializeFSRs) and the angle data
 * (pack_linear_source) and hands them to moc_set_linear_source, which
 * computes the linear expansion matrices and source constants on the GPU.
 */
class GB300LSSolver : public GB300Solver {
 protected:
  std::map<std::pair<long, int>, std::vector<double> > _fix_src_xyz_FSR_map;
  void upload();
  void initializeSourceArrays();

 public:
  GB300LSSolver(TrackGenerator* track_generator = NULL, int device = 0);

  /** CPULSSolver::setFixedSourceMomentByFSR (src/CPULSSolver.cpp:280-307);
   *  group is 1-based, src_z is ignored for 2D tracks. */
  void setFixedSourceMomentByFSR(long fsr_id, int group, double src_x,
                                 double src_y, double src_z);
  void resetFixedSources();
  /** Flux moments [R][3][G] (x, y, z), CPULSSolver::_scalar_flux_xyz. */
  void getFluxMoments(FP_PRECISION* out, long n);
  /** Flux at (x, y) relative to the FSR's centroid
   *  (CPULSSolver::getFluxByCoords, src/CPULSSolver.cpp:1082-1133). */
  double getFluxByOffset(long fsr_id, double dx, double dy, int group);
};

#endif
