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
 *   computeStabilizingFlux CPUSolver.cpp:2665  moc_compute_stabilizing_flux
 *   stabilizeFlux          CPUSolver.cpp:2736  moc_stabilize_flux
 *   computeFSRFissionSources CPUSolver.cpp:2030 moc_compute_fsr_fission_sources
 *   computeFSRScatterSources CPUSolver.cpp:2074 moc_compute_fsr_scatter_sources
 * Solver::stabilizeTransport and setKeffFromNeutronBalance reach the device
 * at initializeFluxArrays (moc_set_transport_stabilization,
 * moc_set_keff_from_neutron_balance).
 * The host keeps no flux arrays: getFlux / getFluxes read the device.
 */
#include "GB300Solver.h"

#include <cmath>
#include <cstring>
#include <map>
#include <vector>

#include "../../include/openmoc_gb300.h"
#include "Cmfd.h"
#include "pack_reference.h"

GB300Solver::GB300Solver(TrackGenerator* track_generator, int device)
    : Solver(NULL), _ctx(NULL), _device(device), _exp_kind(-1),
      _uploaded(false), _cmfd_relaxation(0.7), _cmfd_sor(1.5),
      _cmfd_flux_limiting(true), _cmfd_on_host(false), _cmfd_unbounded(0),
      _cmfd_k_nearest(1) {
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

void GB300Solver::setCmfdFactors(double relaxation, double sor,
                                 bool flux_limiting, int unbounded_iterations,
                                 bool on_host, int k_nearest) {
  _cmfd_k_nearest = k_nearest;
  _cmfd_relaxation = relaxation;
  _cmfd_sor = sor;
  _cmfd_flux_limiting = flux_limiting;
  _cmfd_unbounded = unbounded_iterations;
  _cmfd_on_host = on_host;
}

/* The Geometry's Cmfd (Solver::initializeCmfd, src/Solver.cpp:1145-1185)
 * as a moc_cmfd_mesh: OpenMOC's own FSR-to-cell map, lattice widths,
 * boundaries and group structure, the boundary face at each track end, and
 * the quadrature of Cmfd::computeLarsensEDCFactor. */
void GB300Solver::attachCmfd() {
  initializeCmfd();
  if (_cmfd == NULL || !_cmfd->isFluxUpdateOn()) {
    check(moc_set_cmfd(_ctx, NULL), "moc_set_cmfd");
    return;
  }
  if (_SOLVE_3D || _cmfd->getNumZ() > 1)
    log_printf(ERROR, "GB300Solver supports CMFD on 2D meshes only");
  const int nx = _cmfd->getNumX(), ny = _cmfd->getNumY();
  Lattice* lat = _cmfd->getLattice();
  std::vector<double> wx(lat->getWidthsX()), wy(lat->getWidthsY());
  if ((int) wx.size() != nx || (int) wy.size() != ny)
    log_printf(ERROR, "GB300Solver: unexpected CMFD lattice widths");
  std::vector<int32_t> cell(_num_FSRs);
  for (long r = 0; r < _num_FSRs; r++)
    cell[r] = _cmfd->convertFSRIdToCmfdCell(r);
  const double x0 = _geometry->getMinX(), x1 = _geometry->getMaxX();
  const double y0 = _geometry->getMinY(), y1 = _geometry->getMaxY();
  const double tol = 1e-9 * std::max(x1 - x0, y1 - y0);
  Track** tracks = _track_generator->get2DTracksArray();
  const long T = _track_generator->getNum2DTracks();
  std::vector<int8_t> ends(2 * T);
  for (long t = 0; t < T; t++) {
    Point* q[2] = {tracks[t]->getEnd(), tracks[t]->getStart()};
    for (int d = 0; d < 2; d++) {
      int8_t f = -1;
      if (std::fabs(q[d]->getX() - x0) <= tol) f = 0;
      else if (std::fabs(q[d]->getX() - x1) <= tol) f = 2;
      else if (std::fabs(q[d]->getY() - y0) <= tol) f = 1;
      else if (std::fabs(q[d]->getY() - y1) <= tol) f = 3;
      ends[2 * t + d] = f;
    }
  }
  const int sides[4] = {SURFACE_X_MIN, SURFACE_Y_MIN, SURFACE_X_MAX,
                        SURFACE_Y_MAX};
  moc_cmfd_mesh m;
  std::memset(&m, 0, sizeof(m));
  for (int f = 0; f < 4; f++) {
    const int b = _cmfd->getBoundary(sides[f]);
    if (b != VACUUM && b != REFLECTIVE)
      log_printf(ERROR, "GB300Solver supports vacuum and reflective CMFD "
                 "boundaries only");
    m.boundary[f] = (b == VACUUM) ? MOC_BC_VACUUM : MOC_BC_REFLECTIVE;
  }
  std::vector<int32_t> group_of(_num_groups);
  for (int g = 0; g < _num_groups; g++) group_of[g] = _cmfd->getCmfdGroup(g);
  std::vector<double> mu, w;
  for (size_t a = 0; a < _quad->getNumAzimAngles() / 2; a++)
    for (size_t p = 0; p < _quad->getNumPolarAngles() / 2; p++) {
      const double sn = _quad->getSinTheta(a, p);
      mu.push_back(std::sqrt(1.0 - sn * sn));
      w.push_back(_quad->getAzimWeight(a) * _quad->getPolarWeight(a, p));
    }
  m.num_x = nx;
  m.num_y = ny;
  m.widths_x = wx.data();
  m.widths_y = wy.data();
  m.fsr_cell = cell.data();
  m.track_end_face = ends.data();
  m.num_cmfd_groups = _cmfd->getNumCmfdGroups();
  m.group_of = group_of.data();
  m.num_edc_angles = (int32_t) mu.size();
  m.edc_mu = mu.data();
  m.edc_weight = w.data();
  m.relaxation = _cmfd_relaxation;
  m.sor_factor = _cmfd_sor;
  m.flux_limiting = _cmfd_flux_limiting ? 1 : 0;
  m.num_unbounded_iterations = _cmfd_unbounded;
  m.solve_on_host = _cmfd_on_host ? 1 : 0;
  // the k-nearest update from the FSR centroids OpenMOC generated
  // (Solver::initializeFSRs, src/Solver.cpp:865)
  std::vector<double> cen;
  if (_cmfd->isCentroidUpdateOn()) {
    cen.resize(2 * _num_FSRs);
    for (long r = 0; r < _num_FSRs; r++) {
      Point* q = _geometry->getFSRCentroid(r);
      cen[2 * r] = q->getX();
      cen[2 * r + 1] = q->getY();
    }
    m.k_nearest = _cmfd_k_nearest;
    m.fsr_centroid = cen.data();
    m.origin_x = lat->getMinX();
    m.origin_y = lat->getMinY();
  }
  check(moc_set_cmfd(_ctx, &m), "moc_set_cmfd");
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
  check(moc_set_keff_from_neutron_balance(_ctx, _keff_from_fission_rates ? 0 : 1),
        "setKeffFromNeutronBalance");
  check(moc_set_transport_stabilization(_ctx, _stabilize_transport ? 1 : 0,
                                        _stabilization_factor,
                                        (int) _stabilization_type),
        "stabilizeTransport");
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
  check(moc_compute_stabilizing_flux(_ctx), "computeStabilizingFlux");
}

void GB300Solver::stabilizeFlux() {
  check(moc_stabilize_flux(_ctx), "stabilizeFlux");
}

void GB300Solver::computeFSRSources(int iteration) {
  check(moc_set_keff(_ctx, _k_eff), "setKeff");
  check(moc_compute_fsr_sources(_ctx, iteration), "computeFSRSources");
}

void GB300Solver::computeFSRFissionSources() {
  check(moc_compute_fsr_fission_sources(_ctx), "computeFSRFissionSources");
}

void GB300Solver::computeFSRScatterSources() {
  check(moc_compute_fsr_scatter_sources(_ctx), "computeFSRScatterSources");
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
  attachCmfd();
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
