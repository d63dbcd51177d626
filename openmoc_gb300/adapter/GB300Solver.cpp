/**
 * @file GB300Solver.cpp
 * @brief OpenMOC Solver hooks forwarded to the GB300 C ABI.
 *
 * Hook-by-hook correspondence (reference -> this file -> C ABI):
 *   initializeFluxArrays   CPUSolver.cpp:281   upload()  moc_create + uploads
 *   zeroTrackFluxes        CPUSolver.cpp:463   moc_zero_track_fluxes
 *   flattenFSRFluxes       CPUSolver.cpp:1816  moc_flatten_fsr_fluxes
 *   storeFSRFluxes         CPUSolver.cpp:1846  moc_store_fsr_fluxes
 *   normalizeFluxes        CPUSolver.cpp:1860  moc_normalize_fluxes
 *   computeFSRSources      CPUSolver.cpp:1939  moc_compute_fsr_sources
 *   computeResidual        CPUSolver.cpp:2113  moc_compute_residual
 *   computeKeff            CPUSolver.cpp:2258  moc_compute_keff
 *   transportSweep         CPUSolver.cpp:2338  moc_transport_sweep
 *   addSourceToScalarFlux  CPUSolver.cpp:2608  moc_add_source_to_scalar_flux
 * The host keeps no flux arrays: getFlux / getFluxes read the device.
 */
#include "GB300Solver.h"

#include <cstring>
#include <map>
#include <vector>

#include "../../include/openmoc_gb300.h"
#include "pack_reference.h"

GB300Solver::GB300Solver(TrackGenerator* track_generator, int device)
    : Solver(NULL), _ctx(NULL), _device(device), _exp_kind(-1),
      _uploaded(false) {
  _gpu_solver = true;
  if (track_generator != NULL) setTrackGenerator(track_generator);
}

GB300Solver::~GB300Solver() {
  if (_ctx) moc_destroy(_ctx);
  _ctx = NULL;
}

void GB300Solver::check(int status, const char* what) {
  if (status != MOC_OK)
    log_printf(ERROR, "GB300Solver %s failed (%d): %s", what, status,
               moc_last_error());
}

void GB300Solver::setTrackGenerator(TrackGenerator* track_generator) {
  Solver::setTrackGenerator(track_generator);
  _uploaded = false;
}

void GB300Solver::setExponentialEvaluator(int kind) {
  _exp_kind = kind;
  if (_ctx) check(moc_set_exponential(_ctx, kind), "setExponentialEvaluator");
}

int GB300Solver::materialIndex(Material* m) {
  std::map<int, Material*> mats = _geometry->getAllMaterials();
  int i = 0;
  for (std::map<int, Material*>::iterator it = mats.begin(); it != mats.end();
       ++it, ++i)
    if (it->second == m) return i;
  log_printf(ERROR, "Material %d is not in the geometry", m->getId());
  return -1;
}

void GB300Solver::initializeFSRs() {
  Solver::initializeFSRs();
}

/* Packs tracks (after initializeExpEvaluators may have split segments),
 * quadrature, materials and FSRs and hands them to the device. */
void GB300Solver::upload() {
  openmoc_gb300::PackedProblem p;
  openmoc_gb300::pack_tracks(_track_generator, p);
  openmoc_gb300::pack_materials(_geometry, _FSR_volumes, p);
  if (_ctx) moc_destroy(_ctx);
  _ctx = NULL;
  moc_dims d;
  d.num_groups = p.num_groups;
  d.num_polar_half = p.num_polar_half;
  d.num_angles = p.num_angles;
  d.num_materials = p.num_materials;
  d.num_fsrs = p.num_fsrs;
  d.num_tracks = p.num_tracks;
  d.num_segments = p.num_segments;
  d.solve_3d = p.solve_3d;
  d.device = _device;
  check(moc_create(&d, &_ctx), "moc_create");
  check(moc_upload_tracks(_ctx, p.seg_len.data(), p.seg_fsr.data(),
                          p.seg_off.data(), p.track_ang.data(), p.next.data(),
                          p.flags.data()),
        "moc_upload_tracks");
  check(moc_upload_quadrature(_ctx, p.weights.data(), p.inv_sin.data()),
        "moc_upload_quadrature");
  check(moc_upload_materials(_ctx, p.sigma_t.data(), p.sigma_s.data(),
                             p.nu_sigma_f.data(), p.chi.data()),
        "moc_upload_materials");
  check(moc_upload_fsrs(_ctx, p.fsr_mat.data(), p.fsr_vol.data()),
        "moc_upload_fsrs");
  check(moc_set_convergence_threshold(_ctx, _converge_thresh),
        "moc_set_convergence_threshold");
  if (_exp_kind >= 0)
    check(moc_set_exponential(_ctx, _exp_kind), "moc_set_exponential");
  _uploaded = true;
}

void GB300Solver::initializeFluxArrays() {
  upload();
  check(moc_set_negative_fluxes_allowed(_ctx, _negative_fluxes_allowed ? 1 : 0),
        "allowNegativeFluxes");
  check(moc_zero_track_fluxes(_ctx), "zeroTrackFluxes");
}

void GB300Solver::initializeSourceArrays() {
  if (!_ctx) return;
  if (_fixed_sources_on) {
    Solver::initializeFixedSources();
    std::vector<float> q((size_t) _num_FSRs * _num_groups, 0.f);
    for (std::map<std::pair<int, int>, FP_PRECISION>::iterator it =
             _fix_src_FSR_map.begin();
         it != _fix_src_FSR_map.end(); ++it) {
      long r = it->first.first;
      int g = it->first.second;
      if (g <= 0 || g > _num_groups || r < 0 || r >= _num_FSRs)
        log_printf(ERROR, "Unable to use fixed source for FSR %ld group %d",
                   r, g);
      q[(size_t) r * _num_groups + g - 1] = (float) it->second;
    }
    check(moc_set_fixed_sources(_ctx, q.data()), "setFixedSources");
  } else {
    check(moc_set_fixed_sources(_ctx, NULL), "resetFixedSources");
  }
}

void GB300Solver::zeroTrackFluxes() {
  check(moc_zero_track_fluxes(_ctx), "zeroTrackFluxes");
}

void GB300Solver::flattenFSRFluxes(FP_PRECISION value) {
  check(moc_flatten_fsr_fluxes(_ctx, (float) value), "flattenFSRFluxes");
}

void GB300Solver::flattenFSRFluxesChiSpectrum() {
  if (_chi_spectrum_material == NULL)
    log_printf(ERROR, "A flattening of the FSR fluxes for a chi spectrum was "
               "requested but no chi spectrum material was set.");
  check(moc_flatten_fsr_fluxes_chi(_ctx, materialIndex(_chi_spectrum_material)),
        "flattenFSRFluxesChiSpectrum");
}

void GB300Solver::storeFSRFluxes() {
  check(moc_store_fsr_fluxes(_ctx), "storeFSRFluxes");
}

double GB300Solver::normalizeFluxes() {
  double f = 1.0;
  check(moc_normalize_fluxes(_ctx, &f), "normalizeFluxes");
  return f;
}

void GB300Solver::computeStabilizingFlux() {
  log_printf(ERROR, "GB300Solver does not implement transport stabilization");
}

void GB300Solver::stabilizeFlux() {
  log_printf(ERROR, "GB300Solver does not implement transport stabilization");
}

void GB300Solver::computeFSRSources(int iteration) {
  check(moc_set_keff(_ctx, _k_eff), "setKeff");
  check(moc_compute_fsr_sources(_ctx, iteration), "computeFSRSources");
}

void GB300Solver::computeFSRFissionSources() {
  log_printf(ERROR, "GB300Solver does not implement the fission-only source "
             "(openmoc.krylov helper)");
}

void GB300Solver::computeFSRScatterSources() {
  log_printf(ERROR, "GB300Solver does not implement the scatter-only source "
             "(openmoc.krylov helper)");
}

double GB300Solver::computeResidual(residualType res_type) {
  double r = 0.0;
  check(moc_set_keff(_ctx, _k_eff), "setKeff");
  check(moc_compute_residual(_ctx, (int) res_type, &r), "computeResidual");
  return r;
}

void GB300Solver::computeKeff() {
  check(moc_set_keff(_ctx, _k_eff), "setKeff");
  check(moc_compute_keff(_ctx), "computeKeff");
  check(moc_get_keff(_ctx, &_k_eff), "getKeff");
}

void GB300Solver::addSourceToScalarFlux() {
  check(moc_add_source_to_scalar_flux(_ctx), "addSourceToScalarFlux");
}

void GB300Solver::transportSweep() {
  _timer->startTimer();
  check(moc_transport_sweep(_ctx), "transportSweep");
  _timer->stopTimer();
  _timer->recordSplit("Transport Sweep");
}

double GB300Solver::getFlux(long fsr_id, int group) {
  if (fsr_id < 0 || fsr_id >= _num_FSRs)
    log_printf(ERROR, "Unable to return a scalar flux for FSR ID = %ld "
               "since the max FSR ID = %ld", fsr_id, _num_FSRs - 1);
  if (group <= 0 || group > _num_groups)
    log_printf(ERROR, "Unable to return a scalar flux in group %d "
               "since there are only %d groups", group, _num_groups);
  if (!_ctx)
    log_printf(ERROR, "Unable to return a scalar flux since it has not yet "
               "been computed");
  std::vector<float> f((size_t) _num_FSRs * _num_groups);
  check(moc_get_fluxes(_ctx, f.data(), (int64_t) f.size()), "getFluxes");
  return f[(size_t) fsr_id * _num_groups + group - 1];
}

void GB300Solver::getFluxes(FP_PRECISION* out_fluxes, int num_fluxes) {
  if (num_fluxes != _num_FSRs * _num_groups)
    log_printf(ERROR, "Unable to get FSR scalar fluxes since there are "
               "%d groups and %ld FSRs", _num_groups, _num_FSRs);
  std::vector<float> f((size_t) num_fluxes);
  check(moc_get_fluxes(_ctx, f.data(), num_fluxes), "getFluxes");
  for (int i = 0; i < num_fluxes; i++) out_fluxes[i] = f[i];
}

void GB300Solver::setFluxes(FP_PRECISION* in_fluxes, int num_fluxes) {
  if (!_ctx) upload();
  std::vector<float> f(in_fluxes, in_fluxes + num_fluxes);
  check(moc_set_fluxes(_ctx, f.data(), num_fluxes), "setFluxes");
  _user_fluxes = true;
}

void GB300Solver::resetFixedSources() {
  _fix_src_FSR_map.clear();
  _fix_src_cell_map.clear();
  _fix_src_material_map.clear();
  _fixed_sources_on = false;
  _fixed_sources_initialized = false;
  if (_ctx) check(moc_set_fixed_sources(_ctx, NULL), "resetFixedSources");
}

void GB300Solver::computeFSRFissionRates(double* fission_rates,
                                         long num_FSRs, bool nu) {
  if (num_FSRs != _num_FSRs)
    log_printf(ERROR, "The number of FSRs passed in (%ld) does not match the "
               "solver's (%ld)", num_FSRs, _num_FSRs);
  if (!nu) {
    std::map<int, Material*> mats = _geometry->getAllMaterials();
    std::vector<float> sf((size_t) mats.size() * _num_groups, 0.f);
    int m = 0;
    for (std::map<int, Material*>::iterator it = mats.begin();
         it != mats.end(); ++it, ++m) {
      FP_PRECISION* s = it->second->getSigmaF();
      for (int g = 0; s && g < _num_groups; g++)
        sf[(size_t) m * _num_groups + g] = (float) s[g];
    }
    check(moc_upload_sigma_f(_ctx, sf.data()), "uploadSigmaF");
  }
  check(moc_compute_fsr_fission_rates(_ctx, fission_rates, num_FSRs, nu),
        "computeFSRFissionRates");
}

/* Solver::computeEigenvalue's initialisation (src/Solver.cpp:1542-1600),
 * then the whole loop on the device. */
void GB300Solver::computeEigenvalue(int max_iters, residualType res_type) {
  if (_track_generator == NULL)
    log_printf(ERROR, "The Solver is unable to compute the eigenvalue "
               "since it does not contain a TrackGenerator");
  clearTimerSplits();
  _timer->startTimer();
  _k_eff = 1.;
  initializeMaterials(_solver_mode);
  initializeFSRs();
  countFissionableFSRs();
  initializeExpEvaluators();
  initializeFluxArrays();
  initializeSourceArrays();
  check(moc_compute_eigenvalue(_ctx, max_iters, (int) res_type),
        "computeEigenvalue");
  check(moc_get_keff(_ctx, &_k_eff), "getKeff");
  check(moc_get_num_iterations(_ctx, &_num_iterations), "getNumIterations");
  if (_num_iterations == max_iters)
    log_printf(WARNING, "Unable to converge the source distribution");
  _timer->stopTimer();
  _timer->recordSplit("Total time");
}

void GB300Solver::computeSource(int max_iters, double k_eff,
                                residualType res_type) {
  if (_track_generator == NULL)
    log_printf(ERROR, "The Solver is unable to compute the source "
               "since it does not contain a TrackGenerator");
  else if (k_eff <= 0.)
    log_printf(ERROR, "The Solver is unable to compute the source with "
               "keff = %f since it is not a positive value", k_eff);
  clearTimerSplits();
  _timer->startTimer();
  _k_eff = k_eff;
  initializeMaterials(_solver_mode);
  initializeFSRs();
  initializeExpEvaluators();
  initializeFluxArrays();
  initializeSourceArrays();
  check(moc_compute_source(_ctx, max_iters, k_eff, (int) res_type),
        "computeSource");
  check(moc_get_num_iterations(_ctx, &_num_iterations), "getNumIterations");
  _timer->stopTimer();
  _timer->recordSplit("Total time");
}

void GB300Solver::computeFlux(int max_iters, bool only_fixed_source) {
  if (_track_generator == NULL)
    log_printf(ERROR, "The Solver is unable to compute the flux "
               "since it does not contain a TrackGenerator");
  clearTimerSplits();
  _timer->startTimer();
  _k_eff = 1.;
  initializeMaterials(_solver_mode);
  initializeFSRs();
  countFissionableFSRs();
  initializeSourceArrays();
  initializeExpEvaluators();
  initializeFluxArrays();
  initializeSourceArrays();
  check(moc_compute_flux(_ctx, max_iters, only_fixed_source ? 1 : 0),
        "computeFlux");
  check(moc_get_num_iterations(_ctx, &_num_iterations), "getNumIterations");
  _timer->stopTimer();
  _timer->recordSplit("Total time");
}

/* ---------------------------------------------------------- linear source */
GB300LSSolver::GB300LSSolver(TrackGenerator* track_generator, int device)
    : GB300Solver(track_generator, device) {}

void GB300LSSolver::upload() {
  GB300Solver::upload();
  openmoc_gb300::PackedProblem p;
  openmoc_gb300::pack_tracks(_track_generator, p);
  try {
    openmoc_gb300::pack_linear_source(_track_generator, p);
  } catch (std::exception& e) {
    log_printf(ERROR, "GB300LSSolver: %s", e.what());
  }
  moc_ls_geometry g;
  g.seg_x = p.seg_x.data();
  g.seg_y = p.seg_y.data();
  g.ang_dir = p.ang_dir.data();
  g.ang_wgt = p.ang_wgt.data();
  g.pol_sin = p.pol_sin.data();
  g.pol_wgt = p.pol_wgt.data();
  check(moc_set_linear_source(_ctx, &g), "moc_set_linear_source");
}

void GB300LSSolver::initializeSourceArrays() {
  GB300Solver::initializeSourceArrays();
  if (!_ctx) return;
  if (_fix_src_xyz_FSR_map.empty()) {
    check(moc_set_fixed_source_moments(_ctx, NULL, 0), "resetFixedSources");
    return;
  }
  std::vector<float> m((size_t) _num_FSRs * 3 * _num_groups, 0.f);
  for (std::map<std::pair<long, int>, std::vector<double> >::iterator it =
           _fix_src_xyz_FSR_map.begin();
       it != _fix_src_xyz_FSR_map.end(); ++it) {
    const long r = it->first.first;
    const int g = it->first.second;
    for (int i = 0; i < 3; i++)
      m[((size_t) r * 3 + i) * _num_groups + g - 1] = (float) it->second[i];
  }
  check(moc_set_fixed_source_moments(_ctx, m.data(), (int64_t) m.size()),
        "setFixedSourceMoments");
}

void GB300LSSolver::setFixedSourceMomentByFSR(long fsr_id, int group,
                                              double src_x, double src_y,
                                              double src_z) {
  if (group <= 0 || group > _num_groups)
    log_printf(ERROR, "Unable to set fixed source for group %d in "
               "in a %d energy group problem", group, _num_groups);
  if (fsr_id < 0 || fsr_id >= _num_FSRs)
    log_printf(ERROR, "Unable to set fixed source for FSR %ld with only "
               "%ld FSRs in the geometry", fsr_id, _num_FSRs);
  std::vector<double>& v = _fix_src_xyz_FSR_map[std::make_pair(fsr_id, group)];
  v.assign(3, 0.0);
  v[0] = src_x;
  v[1] = src_y;
  v[2] = src_z;
}

void GB300LSSolver::resetFixedSources() {
  GB300Solver::resetFixedSources();
  _fix_src_xyz_FSR_map.clear();
  if (_ctx) check(moc_set_fixed_source_moments(_ctx, NULL, 0), "resetFixedSources");
}

void GB300LSSolver::getFluxMoments(FP_PRECISION* out, long n) {
  if (!_ctx) log_printf(ERROR, "no flux moments computed yet");
  std::vector<float> f((size_t) n);
  check(moc_get_flux_moments(_ctx, f.data(), n), "getFluxMoments");
  for (long i = 0; i < n; i++) out[i] = f[i];
}

double GB300LSSolver::getFluxByOffset(long fsr_id, double dx, double dy,
                                      int group) {
  const double flat = getFlux(fsr_id, group);
  std::vector<double> il((size_t) _num_FSRs * 3);
  check(moc_get_linear_expansion(_ctx, il.data(), NULL), "getLinearExpansion");
  std::vector<float> m((size_t) _num_FSRs * 3 * _num_groups);
  check(moc_get_flux_moments(_ctx, m.data(), (int64_t) m.size()),
        "getFluxMoments");
  const double mx = m[((size_t) fsr_id * 3 + 0) * _num_groups + group - 1];
  const double my = m[((size_t) fsr_id * 3 + 1) * _num_groups + group - 1];
  const double* c = &il[(size_t) fsr_id * 3];
  return flat + dx * (c[0] * mx + c[2] * my) + dy * (c[2] * mx + c[1] * my);
}
