/*
 * Generates the golden fixtures under tests/golden/ by running OpenMOC's own
 * C++ library (compiled from the reference sources by oracle/ref.mk) on small
 * problems.  Built twice, against the FP_PRECISION=float and =double builds,
 * by tests/golden/make_fixtures.sh.
 *
 * For every case it writes <case>_<prec>.bin + <case>_<prec>.json:
 *   - the packed tracks / quadrature / cross sections exactly as the GB300
 *     adapter hands them to the C ABI (openmoc_gb300/adapter/pack_reference.h);
 *   - the converged solve (iterations, keff, FSR scalar fluxes);
 *   - (float build) a hook-by-hook probe from the converged state: the
 *     reduced sources of computeFSRSources, the raw sweep tallies and the
 *     outgoing boundary fluxes of one transportSweep, the flux after
 *     addSourceToScalarFlux, keff after computeKeff, the normalisation factor
 *     and the residual (src/CPUSolver.cpp:1860-2660);
 *   - linear-source cases (CPULSSolver): the re-centred segment start
 *     positions and angle data of pack_linear_source, OpenMOC's linear
 *     expansion matrix inverse and source constants
 *     (src/TrackTraversingAlgorithms.cpp:470-830), the converged flux moments,
 *     and (float build, eigenvalue cases) the same hook-by-hook probe with the
 *     moments of every step (src/CPULSSolver.cpp:343-886).
 * Track generation runs on one thread so FSR numbering is reproducible, as
 * the reference test harness does (tests/testing_harness.py).
 */
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "CPULSSolver.h"
#include "Cmfd.h"
#include "CPUSolver.h"
#include "Geometry.h"
#include "TrackGenerator.h"
#include "TrackGenerator3D.h"
#include "log.h"

#include "../../openmoc_gb300/adapter/pack_reference.h"
#include "../../openmoc_gb300/csrc/synthetic_xs.h"

using openmoc_gb300::MaterialXS;
using openmoc_gb300::PackedProblem;

#ifdef SINGLE
static const char* PREC = "f32";
#else
static const char* PREC = "f64";
#endif

/* ------------------------------------------------------------------ output */
struct Writer {
  std::string bin_path, json_path;
  std::ofstream bin;
  std::stringstream arrays, scalars;
  long offset = 0;
  bool first_arr = true, first_sc = true;

  Writer(const std::string& base) {
    bin_path = base + ".bin";
    json_path = base + ".json";
    bin.open(bin_path.c_str(), std::ios::binary);
  }
  template <typename T>
  void arr(const char* name, const char* dtype, const T* data, long n,
           long rows = -1) {
    while (offset % 16) { char z = 0; bin.write(&z, 1); offset++; }
    bin.write((const char*) data, n * sizeof(T));
    if (!first_arr) arrays << ",\n";
    first_arr = false;
    arrays << "    \"" << name << "\": {\"dtype\": \"" << dtype
           << "\", \"offset\": " << offset << ", \"count\": " << n;
    if (rows > 0) arrays << ", \"rows\": " << rows;
    arrays << "}";
    offset += n * sizeof(T);
  }
  void sc(const char* name, double v) {
    if (!first_sc) scalars << ",\n";
    first_sc = false;
    char buf[64];
    snprintf(buf, sizeof(buf), "%.17g", v);
    scalars << "    \"" << name << "\": " << buf;
  }
  void close() {
    bin.close();
    std::ofstream js(json_path.c_str());
    js << "{\n  \"precision\": \"" << PREC << "\",\n  \"arrays\": {\n"
       << arrays.str() << "\n  },\n  \"scalars\": {\n" << scalars.str()
       << "\n  }\n}\n";
  }
};

static void write_problem(Writer& w, const PackedProblem& p) {
  w.sc("num_groups", p.num_groups);
  w.sc("num_polar_half", p.num_polar_half);
  w.sc("num_angles", p.num_angles);
  w.sc("num_materials", p.num_materials);
  w.sc("solve_3d", p.solve_3d);
  w.sc("num_fsrs", p.num_fsrs);
  w.sc("num_tracks", p.num_tracks);
  w.sc("num_segments", p.num_segments);
  w.arr("seg_len", "f4", p.seg_len.data(), p.seg_len.size());
  w.arr("seg_fsr", "i4", p.seg_fsr.data(), p.seg_fsr.size());
  w.arr("seg_off", "i8", p.seg_off.data(), p.seg_off.size());
  w.arr("track_ang", "i4", p.track_ang.data(), p.track_ang.size());
  w.arr("next", "i8", p.next.data(), p.next.size());
  w.arr("flags", "u1", p.flags.data(), p.flags.size());
  w.arr("weights", "f4", p.weights.data(), p.weights.size());
  w.arr("inv_sin", "f4", p.inv_sin.data(), p.inv_sin.size());
  w.arr("sigma_t", "f4", p.sigma_t.data(), p.sigma_t.size());
  w.arr("sigma_s", "f4", p.sigma_s.data(), p.sigma_s.size());
  w.arr("nu_sigma_f", "f4", p.nu_sigma_f.data(), p.nu_sigma_f.size());
  w.arr("chi", "f4", p.chi.data(), p.chi.size());
  w.arr("fsr_mat", "i4", p.fsr_mat.data(), p.fsr_mat.size());
  w.arr("fsr_vol", "f4", p.fsr_vol.data(), p.fsr_vol.size());
}

/* ---------------------------------------------- solver with hook access */
class ProbeSolver : public CPUSolver {
 public:
  explicit ProbeSolver(TrackGenerator* tg) : CPUSolver(tg) {}

  template <typename T>
  static std::vector<float> tof(const T* a, long n) {
    std::vector<float> v(n);
    for (long i = 0; i < n; i++) v[i] = (float) a[i];
    return v;
  }
  long nflux() const { return _num_FSRs * _num_groups; }
  long nbound() const { return 2 * _tot_num_tracks * _fluxes_per_track; }

  /* One pass of every hook from the converged state; with partial, then
   * the fission and the scattering parts of the source alone from the
   * normalised flux (computeFSRFissionSources / computeFSRScatterSources). */
  void probe(Writer& w, bool partial = false) {
    w.sc("probe_keff_in", _k_eff);
    std::vector<float> v = tof(_scalar_flux, nflux());
    w.arr("probe_phi_in", "f4", v.data(), v.size());
    std::vector<float> so = tof(_old_scalar_flux, nflux());
    w.arr("probe_phi_old", "f4", so.data(), so.size());
    computeFSRSources(100);
    v = tof(_reduced_sources, nflux());
    w.arr("probe_reduced_sources", "f4", v.data(), v.size());
    w.arr("probe_start_flux_in", "f4", _start_flux, nbound());
    transportSweep();
    v = tof(_scalar_flux, nflux());
    w.arr("probe_phi_sweep", "f4", v.data(), v.size());
    w.arr("probe_start_flux_out", "f4", _start_flux, nbound());
    addSourceToScalarFlux();
    v = tof(_scalar_flux, nflux());
    w.arr("probe_phi_addsrc", "f4", v.data(), v.size());
    computeKeff();
    w.sc("probe_keff_out", _k_eff);
    double f = normalizeFluxes();
    w.sc("probe_norm_factor", f);
    v = tof(_scalar_flux, nflux());
    w.arr("probe_phi_norm", "f4", v.data(), v.size());
    w.sc("probe_residual_fission", computeResidual(FISSION_SOURCE));
    w.sc("probe_residual_flux", computeResidual(SCALAR_FLUX));
    w.sc("probe_residual_total", computeResidual(TOTAL_SOURCE));
    if (partial) {
      computeFSRFissionSources();
      v = tof(_reduced_sources, nflux());
      w.arr("probe_fission_sources", "f4", v.data(), v.size());
      computeFSRScatterSources();
      v = tof(_reduced_sources, nflux());
      w.arr("probe_scatter_sources", "f4", v.data(), v.size());
    }
  }
};

/* ----------------------------- linear-source solver with hook access */
class ProbeLSSolver : public CPULSSolver {
 public:
  explicit ProbeLSSolver(TrackGenerator* tg) : CPULSSolver(tg) {}

  long nflux() const { return _num_FSRs * _num_groups; }
  long nbound() const { return 2 * _tot_num_tracks * _fluxes_per_track; }
  /* flux moments [R][3][G] (x, y, z), src/CPULSSolver.h:20 */
  std::vector<float> moments() const {
    return ProbeSolver::tof(_scalar_flux_xyz, 3 * nflux());
  }
  /* expansion coefficients per FSR: 3 in 2D, 6 in 3D */
  int ncoeffs() const { return _SOLVE_3D ? 6 : 3; }
  std::vector<double> lin_exp() const {
    std::vector<double> v(_FSR_lin_exp_matrix,
                          _FSR_lin_exp_matrix + ncoeffs() * _num_FSRs);
    return v;
  }
  std::vector<double> src_constants() const {
    std::vector<double> v(ncoeffs() * nflux());
    for (long i = 0; i < ncoeffs() * nflux(); i++)
      v[i] = _FSR_source_constants[i];
    return v;
  }

  void probe(Writer& w) {
    w.sc("probe_keff_in", _k_eff);
    std::vector<float> v = ProbeSolver::tof(_scalar_flux, nflux());
    w.arr("probe_phi_in", "f4", v.data(), v.size());
    v = moments();
    w.arr("probe_mom_in", "f4", v.data(), v.size());
    std::vector<float> so = ProbeSolver::tof(_old_scalar_flux, nflux());
    w.arr("probe_phi_old", "f4", so.data(), so.size());
    computeFSRSources(100);
    v = ProbeSolver::tof(_reduced_sources, nflux());
    w.arr("probe_reduced_sources", "f4", v.data(), v.size());
    v = ProbeSolver::tof(_reduced_sources_xyz, 3 * nflux());
    w.arr("probe_reduced_xyz", "f4", v.data(), v.size());
    w.arr("probe_start_flux_in", "f4", _start_flux, nbound());
    transportSweep();
    v = ProbeSolver::tof(_scalar_flux, nflux());
    w.arr("probe_phi_sweep", "f4", v.data(), v.size());
    v = moments();
    w.arr("probe_mom_sweep", "f4", v.data(), v.size());
    w.arr("probe_start_flux_out", "f4", _start_flux, nbound());
    addSourceToScalarFlux();
    v = ProbeSolver::tof(_scalar_flux, nflux());
    w.arr("probe_phi_addsrc", "f4", v.data(), v.size());
    v = moments();
    w.arr("probe_mom_addsrc", "f4", v.data(), v.size());
    computeKeff();
    w.sc("probe_keff_out", _k_eff);
    double f = normalizeFluxes();
    w.sc("probe_norm_factor", f);
    v = ProbeSolver::tof(_scalar_flux, nflux());
    w.arr("probe_phi_norm", "f4", v.data(), v.size());
    v = moments();
    w.arr("probe_mom_norm", "f4", v.data(), v.size());
    w.sc("probe_residual_fission", computeResidual(FISSION_SOURCE));
  }
};

/* ---------------------------------------------------------- model pieces */
static Material* make_material(int id, const char* name, const MaterialXS& x) {
  Material* m = new Material(id, name);
  const int G = x.num_groups;
  m->setNumEnergyGroups(G);
  std::vector<double> t = x.sigma_t, s = x.sigma_s, nf = x.nu_sigma_f,
                      f = x.sigma_f, c = x.chi;
  m->setSigmaT(t.data(), G);
  m->setSigmaS(s.data(), G * G);
  m->setSigmaF(f.data(), G);
  m->setNuSigmaF(nf.data(), G);
  m->setChi(c.data(), G);
  return m;
}

/* C5G7 UO2 and water 7-group data as listed in the reference's pin-cell
 * driver (profile/models/pin-cell/pin-cell-3d.cpp:36-95); the published
 * C5G7 benchmark data. */
static MaterialXS c5g7(bool uo2) {
  MaterialXS x;
  x.num_groups = 7;
  if (uo2) {
    x.sigma_t = {0.177949, 0.329805, 0.480388, 0.554367, 0.311801, 0.395168,
                 0.564406};
    x.nu_sigma_f = {0.02005998, 0.002027303, 0.01570599, 0.04518301,
                    0.04334208, 0.2020901, 0.5257105};
    x.sigma_f = {0.00721206, 8.19301E-4, 0.0064532, 0.0185648, 0.0178084,
                 0.0830348, 0.216004};
    x.chi = {0.58791, 0.41176, 3.3906E-4, 1.1761E-7, 0.0, 0.0, 0.0};
    x.sigma_s = {0.127537, 0.042378, 9.4374E-6, 5.5163E-9, 0, 0, 0,
                 0, 0.324456, 0.0016314, 3.1427E-9, 0, 0, 0,
                 0, 0, 0.45094, 0.0026792, 0, 0, 0,
                 0, 0, 0, 0.452565, 0.0055664, 0, 0,
                 0, 0, 0, 1.2525E-4, 0.271401, 0.010255, 1.0021E-8,
                 0, 0, 0, 0, 0.0012968, 0.265802, 0.016809,
                 0, 0, 0, 0, 0, 0.0085458, 0.27308};
  } else {
    x.sigma_t = {0.159206, 0.41297, 0.59031, 0.58435, 0.718, 1.25445,
                 2.65038};
    x.nu_sigma_f.assign(7, 0.0);
    x.sigma_f.assign(7, 0.0);
    x.chi.assign(7, 0.0);
    x.sigma_s = {0.0444777, 0.1134, 7.2347E-4, 3.7499E-6, 5.3184E-8, 0, 0,
                 0, 0.282334, 0.12994, 6.234E-4, 4.8002E-5, 7.4486E-6,
                 1.0455E-6,
                 0, 0, 0.345256, 0.22457, 0.016999, 0.0026443, 5.0344E-4,
                 0, 0, 0, 0.0910284, 0.41551, 0.063732, 0.012139,
                 0, 0, 0, 7.1437E-5, 0.139138, 0.51182, 0.061229,
                 0, 0, 0, 0, 0.0022157, 0.699913, 0.53732,
                 0, 0, 0, 0, 0, 0.13244, 2.4807};
  }
  return x;
}

static std::vector<double> linspace(double a, double b, int n) {
  std::vector<double> v(n);
  for (int i = 0; i < n; i++) v[i] = (n == 1) ? a : a + (b - a) * i / (n - 1);
  return v;
}

/* The 70-group linspace data of tests/test_forward_pin_cell_70g. */
static MaterialXS lin70(bool fuel) {
  MaterialXS x;
  x.num_groups = 70;
  if (fuel) {
    x.nu_sigma_f = linspace(0, 1, 70);
    for (double& v : x.nu_sigma_f) v *= 7;
    x.sigma_s = linspace(0, 1, 4900);
    for (double& v : x.sigma_s) v /= 1000;
    x.chi.assign(70, 1 / 70.);
    x.sigma_t = linspace(2, 3, 70);
  } else {
    x.nu_sigma_f.assign(70, 0.0);
    x.sigma_s = linspace(1, 2, 4900);
    for (double& v : x.sigma_s) v /= 1000;
    x.chi.assign(70, 0.0);
    x.sigma_t = linspace(3, 4, 70);
  }
  x.sigma_f = x.nu_sigma_f;
  return x;
}

struct PinSpec {
  double radius, pitch;
  int fuel_rings, fuel_sectors, mod_sectors;
};

/* A pin universe: fuel (-cylinder) and moderator (+cylinder). */
static Universe* make_pin(Material* fuel, Material* mod, const PinSpec& ps) {
  ZCylinder* cyl = new ZCylinder(0.0, 0.0, ps.radius);
  Cell* f = new Cell();
  f->setFill(fuel);
  f->addSurface(-1, cyl);
  if (ps.fuel_rings) f->setNumRings(ps.fuel_rings);
  if (ps.fuel_sectors) f->setNumSectors(ps.fuel_sectors);
  Cell* m = new Cell();
  m->setFill(mod);
  m->addSurface(+1, cyl);
  if (ps.mod_sectors) m->setNumSectors(ps.mod_sectors);
  Universe* u = new Universe();
  u->addCell(f);
  u->addCell(m);
  return u;
}

/* Root universe: a box of half-width hw around a lattice or a single pin. */
static Geometry* make_box_geometry(Universe* fill_or_null, Lattice* lat,
                                   double hw, boundaryType bxmin,
                                   boundaryType bxmax, boundaryType bymin,
                                   boundaryType bymax) {
  XPlane* xmin = new XPlane(-hw);
  XPlane* xmax = new XPlane(hw);
  YPlane* ymin = new YPlane(-hw);
  YPlane* ymax = new YPlane(hw);
  xmin->setBoundaryType(bxmin);
  xmax->setBoundaryType(bxmax);
  ymin->setBoundaryType(bymin);
  ymax->setBoundaryType(bymax);
  Cell* root = new Cell();
  root->addSurface(+1, xmin);
  root->addSurface(-1, xmax);
  root->addSurface(+1, ymin);
  root->addSurface(-1, ymax);
  if (lat) root->setFill(lat);
  else root->setFill(fill_or_null);
  Universe* ru = new Universe();
  ru->addCell(root);
  Geometry* g = new Geometry();
  g->setRootUniverse(ru);
  return g;
}

/* The reference PinCellInput geometry (tests/input_set.py:95-137): r=1 pin
 * in a +-2 cm reflective box, no rings or sectors. */
static Geometry* pincell_input(Material* fuel, Material* water) {
  ZCylinder* cyl = new ZCylinder(0.0, 0.0, 1.0);
  XPlane* xmin = new XPlane(-2.0);
  XPlane* xmax = new XPlane(2.0);
  YPlane* ymin = new YPlane(-2.0);
  YPlane* ymax = new YPlane(2.0);
  xmin->setBoundaryType(REFLECTIVE);
  xmax->setBoundaryType(REFLECTIVE);
  ymin->setBoundaryType(REFLECTIVE);
  ymax->setBoundaryType(REFLECTIVE);
  Cell* f = new Cell();
  f->setFill(fuel);
  f->addSurface(-1, cyl);
  Cell* m = new Cell();
  m->setFill(water);
  m->addSurface(+1, cyl);
  m->addSurface(+1, xmin);
  m->addSurface(-1, xmax);
  m->addSurface(+1, ymin);
  m->addSurface(-1, ymax);
  Universe* ru = new Universe();
  ru->addCell(f);
  ru->addCell(m);
  Geometry* g = new Geometry();
  g->setRootUniverse(ru);
  return g;
}

/* n x n lattice of pins; positions listed in water_pins hold a pin whose
 * inner circle is filled with the moderator. */
static Geometry* lattice_geometry(int n, Material* fuel, Material* mod,
                                  const PinSpec& ps,
                                  const std::vector<int>& water_pins,
                                  boundaryType bxmin, boundaryType bxmax,
                                  boundaryType bymin, boundaryType bymax) {
  Universe* pin = make_pin(fuel, mod, ps);
  Universe* wpin = make_pin(mod, mod, ps);
  std::vector<Universe*> u(n * n, pin);
  for (int k : water_pins) u[k] = wpin;
  Lattice* lat = new Lattice();
  lat->setWidth(ps.pitch, ps.pitch);
  lat->setUniverses(1, n, n, u.data());
  return make_box_geometry(NULL, lat, 0.5 * n * ps.pitch, bxmin, bxmax, bymin,
                           bymax);
}

/* The HomInfMedInput geometry of tests/input_set.py:52-92: a 10 x 10
 * lattice of 0.25 cm cells in a 2.5 cm box, every cell a universe holding
 * one cell filled with `mat`.  If src_pos >= 0 that lattice position
 * ([row from the top][column], as Lattice::setUniverses takes it) holds a
 * universe of its own whose cell is returned in *src_cell. */
static Geometry* hom_lattice_geometry(Material* mat, Cell** src_cell,
                                      int src_pos, boundaryType bxmin,
                                      boundaryType bxmax, boundaryType bymin,
                                      boundaryType bymax) {
  Cell* fill = new Cell();
  fill->setFill(mat);
  Universe* fu = new Universe();
  fu->addCell(fill);
  std::vector<Universe*> u(100, fu);
  if (src_pos >= 0) {
    Cell* sc = new Cell();
    sc->setFill(mat);
    Universe* su = new Universe();
    su->addCell(sc);
    u[src_pos] = su;
    *src_cell = sc;
  }
  Lattice* lat = new Lattice();
  lat->setWidth(0.25, 0.25);
  lat->setUniverses(1, 10, 10, u.data());
  return make_box_geometry(NULL, lat, 1.25, bxmin, bxmax, bymin, bymax);
}

/* ------------------------------------------------------------------ runs */
enum RunKind { EIGEN, SOURCE, FLUX };

struct CaseSpec {
  const char* name;
  Geometry* geo;
  int num_azim;
  double spacing;
  int max_iters;
  double tol;
  residualType res;
  RunKind kind;
  double k_source;
  bool probe;
  Material* src_material;  /* fixed source in every group of this material */
  double src_value;
  int num_polar;           /* 3D cases: polar angles and axial spacing; */
  double z_spacing;        /* 0 for 2D cases (omitted initialisers) */
  bool linear_source;      /* CPULSSolver instead of CPUSolver */
  bool allow_negative;     /* Solver::allowNegativeFluxes(true) */
  Cell* src_cell;          /* fixed source by cell: flat value per group */
  std::vector<double> src_cell_flat;     /* [G] */
  std::vector<double> src_cell_moments;  /* [G][3], empty: none */
  Cmfd* cmfd;              /* attached to geo before the FSRs are made */
  int k_nearest;           /* the Cmfd's setKNearest (0: not set) */
  bool keff_balance;       /* Solver::setKeffFromNeutronBalance */
  int stab_type;           /* stabilizeTransport type + 1 (0: off) */
  double stab_factor;
  bool probe_partial;      /* probe the fission / scatter source hooks */
};

/* What the CMFD mesh of a case is laid over, in the arrays
 * Problem.cmfd_geometry reads (prefix cm_): the reference's own FSR-to-cell
 * map (Cmfd::convertFSRIdToCmfdCell) on its uniform mesh, the boundary face
 * at each track end, the Larsen-EDC quadrature (Cmfd::computeLarsensEDCFactor
 * reads getSinTheta, getAzimWeight, getPolarWeight for azim < num_azim / 2,
 * polar < num_polar / 2), the geometry's bounds and boundary types. */
static void write_cmfd(Writer& w, const CaseSpec& c, TrackGenerator& tg,
                       const PackedProblem& p) {
  Cmfd* cm = c.cmfd;
  Geometry* geo = c.geo;
  const int nx = cm->getNumX(), ny = cm->getNumY();
  const double x0 = geo->getMinX(), x1 = geo->getMaxX();
  const double y0 = geo->getMinY(), y1 = geo->getMaxY();
  const double wx = (x1 - x0) / nx, wy = (y1 - y0) / ny;
  std::vector<int32_t> cell(p.num_fsrs);
  for (long r = 0; r < p.num_fsrs; r++) {
    cell[r] = cm->convertFSRIdToCmfdCell(r);
    /* the cell numbering (y from y-min) checked on a point of the FSR */
    Point* pt = geo->getFSRPoint(r);
    const int ix = (int) std::floor((pt->getX() - x0) / wx);
    const int iy = (int) std::floor((pt->getY() - y0) / wy);
    if (ix >= 0 && ix < nx && iy >= 0 && iy < ny && cell[r] != iy * nx + ix)
      throw std::runtime_error("unexpected CMFD cell numbering");
  }
  w.arr("cm_fsr_cell", "i4", cell.data(), cell.size());
  std::vector<double> wxs(nx, wx), wys(ny, wy);
  w.arr("cm_widths_x", "f8", wxs.data(), wxs.size());
  w.arr("cm_widths_y", "f8", wys.data(), wys.size());
  Track** tracks = tg.get2DTracksArray();
  const long T = tg.getNum2DTracks();
  const double tol = 1e-9 * std::max(x1 - x0, y1 - y0);
  auto face = [&](Point* q) -> int8_t {
    if (std::fabs(q->getX() - x0) <= tol) return 0;
    if (std::fabs(q->getX() - x1) <= tol) return 2;
    if (std::fabs(q->getY() - y0) <= tol) return 1;
    if (std::fabs(q->getY() - y1) <= tol) return 3;
    return -1;
  };
  std::vector<int8_t> ends(2 * T);
  for (long t = 0; t < T; t++) {
    ends[2 * t] = face(tracks[t]->getEnd());
    ends[2 * t + 1] = face(tracks[t]->getStart());
  }
  w.arr("cm_end_face", "i1", ends.data(), ends.size());
  Quadrature* q = tg.getQuadrature();
  std::vector<double> mu, wt;
  for (int a = 0; a < q->getNumAzimAngles() / 2; a++)
    for (int pp = 0; pp < q->getNumPolarAngles() / 2; pp++) {
      const double sn = q->getSinTheta(a, pp);
      mu.push_back(std::sqrt(1.0 - sn * sn));
      wt.push_back(q->getAzimWeight(a) * q->getPolarWeight(a, pp));
    }
  w.arr("cm_edc_mu", "f8", mu.data(), mu.size());
  w.arr("cm_edc_w", "f8", wt.data(), wt.size());
  double bounds[4] = {x0, x1, y0, y1};
  w.arr("cm_bounds", "f8", bounds, 4);
  auto code = [](boundaryType b) -> int32_t {
    return b == VACUUM ? 0 : b == REFLECTIVE ? 1 : 2;
  };
  int32_t bc[4] = {code(geo->getMinXBoundaryType()),
                   code(geo->getMinYBoundaryType()),
                   code(geo->getMaxXBoundaryType()),
                   code(geo->getMaxYBoundaryType())};
  w.arr("cm_bc", "i4", bc, 4);
  if (cm->isCentroidUpdateOn()) {
    /* the centroids the k-nearest stencils were built from */
    std::vector<double> cen(2 * p.num_fsrs);
    for (long r = 0; r < p.num_fsrs; r++) {
      Point* q = geo->getFSRCentroid(r);
      cen[2 * r] = q->getX();
      cen[2 * r + 1] = q->getY();
    }
    w.arr("cm_fsr_centroid", "f8", cen.data(), cen.size());
    int32_t k = c.k_nearest;
    w.arr("cm_k_nearest", "i4", &k, 1);
  }
}

static void run_case(const CaseSpec& c, const std::string& outdir) {
  c.geo->initializeFlatSourceRegions();
  TrackGenerator* tgp;
  if (c.z_spacing > 0) {
    /* explicit 3D segments (TrackGenerator3D, src/TrackGenerator3D.h) */
    TrackGenerator3D* t3 = new TrackGenerator3D(c.geo, c.num_azim,
                                                c.num_polar, c.spacing,
                                                c.z_spacing);
    t3->setSegmentFormation(EXPLICIT_3D);
    tgp = t3;
  } else {
    tgp = new TrackGenerator(c.geo, c.num_azim, c.spacing);
  }
  TrackGenerator& tg = *tgp;
  tg.setNumThreads(1);
  tg.generateTracks();

  /* Linear-source cases: re-centre the segments on the FSR centroids now
   * (Solver::initializeFSRs does it again without moving them,
   * src/TrackGenerator.cpp:1681-1710) and pack the start positions before
   * the sweeps move them in place (src/CPULSSolver.cpp:738-740). */
  PackedProblem p;
  if (c.linear_source) {
    tg.initializeFSRVolumesBuffer();
    tg.generateFSRCentroids(tg.getFSRVolumes());
    openmoc_gb300::pack_tracks(&tg, p);
    openmoc_gb300::pack_linear_source(&tg, p);
  }

  ProbeSolver* flat = NULL;
  ProbeLSSolver* ls = NULL;
  CPUSolver* sp;
  if (c.linear_source) sp = ls = new ProbeLSSolver(&tg);
  else sp = flat = new ProbeSolver(&tg);
  CPUSolver& solver = *sp;
  solver.setNumThreads(1);
  solver.setConvergenceThreshold(c.tol);
  if (c.allow_negative) solver.allowNegativeFluxes(true);
  if (c.keff_balance) solver.setKeffFromNeutronBalance();
  if (c.stab_type > 0)
    solver.stabilizeTransport(c.stab_factor,
                              (stabilizationType) (c.stab_type - 1));
  const int G0 = c.geo->getNumEnergyGroups();
  if (c.src_material)
    for (int g = 1; g <= G0; g++)
      solver.setFixedSourceByMaterial(c.src_material, g, c.src_value);
  if (c.src_cell) {
    for (int g = 1; g <= G0; g++)
      if (c.src_cell_flat[g - 1] != 0.0)
        solver.setFixedSourceByCell(c.src_cell, g, c.src_cell_flat[g - 1]);
    for (int g = 1; ls && g <= G0 && !c.src_cell_moments.empty(); g++) {
      const double* m = &c.src_cell_moments[3 * (g - 1)];
      if (m[0] != 0.0 || m[1] != 0.0 || m[2] != 0.0)
        ls->setFixedSourceMomentsByCell(c.src_cell, g, m[0], m[1], m[2]);
    }
  }
  if (c.kind == EIGEN)
    solver.computeEigenvalue(c.max_iters, c.res);
  else if (c.kind == SOURCE)
    solver.computeSource(c.max_iters, c.k_source, c.res);
  else
    solver.computeFlux(c.max_iters, true);

  if (!c.linear_source) {
    openmoc_gb300::pack_tracks(&tg, p);
  } else {
    /* the solve must not have split segments after the packing above */
    PackedProblem q2;
    openmoc_gb300::pack_tracks(&tg, q2);
    if (q2.seg_len != p.seg_len || q2.seg_fsr != p.seg_fsr)
      throw std::runtime_error("segments changed during the solve");
  }
  openmoc_gb300::pack_materials(c.geo, tg.getFSRVolumes(), p);

  Writer w(outdir + "/" + c.name + "_" + PREC);
  write_problem(w, p);
  w.sc("num_azim", c.num_azim);
  w.sc("spacing", c.spacing);
  w.sc("max_iters", c.max_iters);
  w.sc("tolerance", c.tol);
  w.sc("res_type", (int) c.res);
  w.sc("run_kind", (int) c.kind);
  w.sc("k_source", c.k_source);
  w.sc("linear_source", c.linear_source ? 1 : 0);
  w.sc("allow_negative", c.allow_negative ? 1 : 0);
  w.sc("keff_balance", c.keff_balance ? 1 : 0);
  w.sc("stab_type", c.stab_type - 1);
  w.sc("stab_factor", c.stab_factor);
  w.sc("iterations", solver.getNumIterations());
  w.sc("keff", solver.getKeff());
  const long R = p.num_fsrs;
  const int G = p.num_groups;
  std::vector<float> flux((size_t) R * G);
  for (long r = 0; r < R; r++)
    for (int g = 0; g < G; g++)
      flux[(size_t) r * G + g] = (float) solver.getFlux(r, g + 1);
  w.arr("flux", "f4", flux.data(), flux.size());
  std::vector<float> q((size_t) R * G, 0.0f);
  bool any_fixed = false;
  if (c.src_material) {
    /* the fixed source per FSR and group, as setFixedSourceByMaterial
     * spreads it (Solver::initializeFixedSources, src/Solver.cpp:1100-1135) */
    for (long r = 0; r < R; r++)
      if (c.geo->findFSRMaterial(r) == c.src_material)
        for (int g = 0; g < G; g++) q[(size_t) r * G + g] = (float) c.src_value;
    any_fixed = true;
  }
  if (c.src_cell) {
    /* setFixedSourceByCell: every FSR of the cell (its id in the FSR key) */
    std::vector<float> mom((size_t) R * 2 * G, 0.0f);
    for (long r = 0; r < R; r++) {
      if (c.geo->findCellContainingFSR(r) != c.src_cell) continue;
      for (int g = 0; g < G; g++) {
        q[(size_t) r * G + g] = (float) c.src_cell_flat[g];
        if (!c.src_cell_moments.empty()) {
          mom[((size_t) r * 2 + 0) * G + g] = (float) c.src_cell_moments[3 * g];
          mom[((size_t) r * 2 + 1) * G + g] =
              (float) c.src_cell_moments[3 * g + 1];
        }
      }
    }
    any_fixed = true;
    if (!c.src_cell_moments.empty())
      w.arr("fixed_source_xy", "f4", mom.data(), mom.size());
  }
  if (any_fixed) w.arr("fixed_source", "f4", q.data(), q.size());
  if (ls) {
    w.arr("ls_seg_x", "f4", p.seg_x.data(), p.seg_x.size());
    w.arr("ls_seg_y", "f4", p.seg_y.data(), p.seg_y.size());
    w.arr("ls_ang_dir", "f8", p.ang_dir.data(), p.ang_dir.size());
    w.arr("ls_ang_wgt", "f8", p.ang_wgt.data(), p.ang_wgt.size());
    w.arr("ls_pol_sin", "f8", p.pol_sin.data(), p.pol_sin.size());
    w.arr("ls_pol_wgt", "f8", p.pol_wgt.data(), p.pol_wgt.size());
    w.arr("ls_centroid", "f8", p.centroid.data(), p.centroid.size());
    if (p.solve_3d) {
      w.arr("ls_seg_z", "f4", p.seg_z.data(), p.seg_z.size());
      w.arr("ls_pol_cos", "f8", p.pol_cos.data(), p.pol_cos.size());
    }
    std::vector<double> ilem = ls->lin_exp();
    w.arr("ls_ilem", "f8", ilem.data(), ilem.size());
    std::vector<double> sc = ls->src_constants();
    w.arr("ls_src_constants", "f8", sc.data(), sc.size());
    std::vector<float> mom = ls->moments();
    w.arr("ls_moments", "f4", mom.data(), mom.size());
  }
  if (c.cmfd) write_cmfd(w, c, tg, p);
  if (c.probe && c.kind == EIGEN) {
#ifdef SINGLE
    if (flat) flat->probe(w, c.probe_partial);
    else ls->probe(w);
#endif
  }
  w.close();
  printf("%s [%s]: R=%ld T=%ld S=%ld iters=%d keff=%.8f\n", c.name, PREC,
         p.num_fsrs, p.num_tracks, p.num_segments, solver.getNumIterations(),
         solver.getKeff());
  delete sp;
}

/* An axially extruded pin cell: fuel pin and moderator for z < zf,
 * homogeneous moderator above up to zt; reflective radially, vacuum at the
 * bottom and top (the construction of the 3D benchmark, on one pin). */
static Geometry* pin3d_geometry(Material* fuel, Material* mod, const PinSpec& ps,
                                double zf, double zt) {
  const double hw = 0.5 * ps.pitch;
  ZCylinder* cyl = new ZCylinder(0.0, 0.0, ps.radius);
  XPlane* xmin = new XPlane(-hw);
  XPlane* xmax = new XPlane(hw);
  YPlane* ymin = new YPlane(-hw);
  YPlane* ymax = new YPlane(hw);
  ZPlane* zmin = new ZPlane(0.0);
  ZPlane* zmid = new ZPlane(zf);
  ZPlane* zmax = new ZPlane(zt);
  xmin->setBoundaryType(REFLECTIVE);
  xmax->setBoundaryType(REFLECTIVE);
  ymin->setBoundaryType(REFLECTIVE);
  ymax->setBoundaryType(REFLECTIVE);
  zmin->setBoundaryType(VACUUM);
  zmax->setBoundaryType(VACUUM);
  Cell* f = new Cell();
  f->setFill(fuel);
  f->addSurface(-1, cyl);
  f->addSurface(+1, zmin);
  f->addSurface(-1, zmid);
  if (ps.fuel_rings) f->setNumRings(ps.fuel_rings);
  if (ps.fuel_sectors) f->setNumSectors(ps.fuel_sectors);
  Cell* m = new Cell();
  m->setFill(mod);
  m->addSurface(+1, cyl);
  m->addSurface(+1, xmin);
  m->addSurface(-1, xmax);
  m->addSurface(+1, ymin);
  m->addSurface(-1, ymax);
  m->addSurface(+1, zmin);
  m->addSurface(-1, zmid);
  if (ps.mod_sectors) m->setNumSectors(ps.mod_sectors);
  Cell* top = new Cell();
  top->setFill(mod);
  top->addSurface(+1, xmin);
  top->addSurface(-1, xmax);
  top->addSurface(+1, ymin);
  top->addSurface(-1, ymax);
  top->addSurface(+1, zmid);
  top->addSurface(-1, zmax);
  Universe* ru = new Universe();
  ru->addCell(f);
  ru->addCell(m);
  ru->addCell(top);
  Geometry* g = new Geometry();
  g->setRootUniverse(ru);
  return g;
}

int main(int argc, char** argv) {
  std::string outdir = argc > 1 ? argv[1] : "tests/golden";
  std::string only = argc > 2 ? argv[2] : "";
  set_log_level("ERROR");
  const boundaryType REF = REFLECTIVE, VAC = VACUUM;

  std::vector<CaseSpec> cases;

  /* 1. tests/test_forward_pin_cell: C5G7, 4 azimuthal, 0.1 cm, 1e-5 */
  {
    Material* fuel = make_material(1, "UO2", c5g7(true));
    Material* water = make_material(2, "Water", c5g7(false));
    cases.push_back({"pin_c5g7", pincell_input(fuel, water), 4, 0.1, 500,
                     1e-5, FISSION_SOURCE, EIGEN, 1.0, true, NULL, 0.0});
  }
  /* 2. tests/test_forward_pin_cell_70g: linspace 70-group data */
  {
    Material* fuel = make_material(3, "UO2-70", lin70(true));
    Material* water = make_material(4, "Water-70", lin70(false));
    cases.push_back({"pin_70g", pincell_input(fuel, water), 4, 0.1, 1000,
                     1e-5, SCALAR_FLUX, EIGEN, 1.0, true, NULL, 0.0});
  }
  /* 3. the 7-group synthetic pin cell: r=0.54 in 1.26 cm, 3 rings x 8
   *    sectors in fuel, 8 moderator sectors, 32 azimuthal, 0.05 cm */
  PinSpec pin = {0.54, 1.26, 3, 8, 8};
  {
    Material* fuel = make_material(5, "fuel7",
        openmoc_gb300::make_synthetic_xs(0xC0FFEEULL, 7, true));
    Material* mod = make_material(6, "mod7",
        openmoc_gb300::make_synthetic_xs(0xC0FFEEULL + 1000, 7, false));
    Lattice* lat = NULL;
    Universe* u = make_pin(fuel, mod, pin);
    cases.push_back({"pin7_synth", make_box_geometry(u, lat, 0.63, REF, REF,
                     REF, REF), 32, 0.05, 1000, 1e-5, FISSION_SOURCE, EIGEN,
                     1.0, true, NULL, 0.0});
  }
  /* 4. 3x3 lattice, 2 groups, vacuum on +x and +y, centre pin water */
  {
    Material* fuel = make_material(7, "fuel2",
        openmoc_gb300::make_synthetic_xs(0xC0FFEEULL + 2, 2, true));
    Material* mod = make_material(8, "mod2",
        openmoc_gb300::make_synthetic_xs(0xC0FFEEULL + 1002, 2, false));
    cases.push_back({"lat3_g2_vac", lattice_geometry(3, fuel, mod, pin, {4},
                     REF, VAC, REF, VAC), 16, 0.1, 1000, 1e-5,
                     FISSION_SOURCE, EIGEN, 1.0, true, NULL, 0.0});
  }
  /* 5. 2x2 lattice, 16 groups, reflective */
  {
    Material* fuel = make_material(9, "fuel16",
        openmoc_gb300::make_synthetic_xs(0xC0FFEEULL + 3, 16, true));
    Material* mod = make_material(10, "mod16",
        openmoc_gb300::make_synthetic_xs(0xC0FFEEULL + 1003, 16, false));
    cases.push_back({"lat2_g16", lattice_geometry(2, fuel, mod, pin, {3},
                     REF, REF, REF, REF), 8, 0.1, 1000, 1e-5,
                     FISSION_SOURCE, EIGEN, 1.0, true, NULL, 0.0});
  }
  /* 6-7. fixed-source problems (tests/test_compute_source and
   *      test_compute_flux run Solver::computeSource / computeFlux): a 3x3
   *      lattice, 7 groups, vacuum on +x and +y, unit source in the fuel.
   *      computeSource with keff 1 (the lattice's own keff is 0.3, so the
   *      source iteration converges); computeFlux with the fixed source
   *      alone. */
  {
    Material* fuel = make_material(11, "fuel7s",
        openmoc_gb300::make_synthetic_xs(0xC0FFEEULL + 4, 7, true));
    Material* mod = make_material(12, "mod7s",
        openmoc_gb300::make_synthetic_xs(0xC0FFEEULL + 1004, 7, false));
    cases.push_back({"src3_g7", lattice_geometry(3, fuel, mod, pin, {4},
                     REF, VAC, REF, VAC), 16, 0.1, 1000, 1e-5,
                     TOTAL_SOURCE, SOURCE, 1.0, false, fuel, 1.0});
    Material* fuel2 = make_material(13, "fuel7f",
        openmoc_gb300::make_synthetic_xs(0xC0FFEEULL + 4, 7, true));
    Material* mod2 = make_material(14, "mod7f",
        openmoc_gb300::make_synthetic_xs(0xC0FFEEULL + 1004, 7, false));
    cases.push_back({"flux3_g7", lattice_geometry(3, fuel2, mod2, pin, {4},
                     REF, VAC, REF, VAC), 16, 0.1, 1000, 1e-5,
                     SCALAR_FLUX, FLUX, 1.0, false, fuel2, 1.0});
  }

  /* 8. explicit 3D: the pin extruded 2 cm, fuel below 1.6 cm, vacuum top
   *    and bottom; 4 azimuthal, 4 polar, 0.1 cm radial, 0.4 cm axial */
  {
    Material* fuel = make_material(15, "fuel7z",
        openmoc_gb300::make_synthetic_xs(0xC0FFEEULL + 5, 7, true));
    Material* mod = make_material(16, "mod7z",
        openmoc_gb300::make_synthetic_xs(0xC0FFEEULL + 1005, 7, false));
    PinSpec p3 = {0.54, 1.26, 2, 4, 4};
    cases.push_back({"pin3d_g7", pin3d_geometry(fuel, mod, p3, 1.6, 2.0), 4,
                     0.1, 1000, 1e-5, FISSION_SOURCE, EIGEN, 1.0, false, NULL,
                     0.0, 4, 0.4});
  }

  /* 8b. the 3D pin of case 8 with the linear source (CPULSSolver on
   *     explicit 3D segments: x, y and z moments) */
  {
    Material* fuel = make_material(39, "fuel7zl",
        openmoc_gb300::make_synthetic_xs(0xC0FFEEULL + 5, 7, true));
    Material* mod = make_material(40, "mod7zl",
        openmoc_gb300::make_synthetic_xs(0xC0FFEEULL + 1005, 7, false));
    PinSpec p3 = {0.54, 1.26, 2, 4, 4};
    cases.push_back({"pin3d_ls", pin3d_geometry(fuel, mod, p3, 1.6, 2.0), 4,
                     0.1, 1000, 1e-5, FISSION_SOURCE, EIGEN, 1.0, false, NULL,
                     0.0, 4, 0.4, true, false, NULL});
  }

  /* 9. tests/test_2d_gradient_linear_source: the 2-group homogeneous
   *    medium of tests/input_set.py (HomInfMedInput, a 10 x 10 lattice of
   *    one-cell universes in a 2.5 cm box) with vacuum on xmin and ymax,
   *    CPULSSolver, 4 azimuthal, 0.1 cm, FISSION_SOURCE, 1e-5 */
  {
    MaterialXS x;
    x.num_groups = 2;
    x.sigma_f = {0.000625, 0.135416667};
    x.nu_sigma_f = {0.0015, 0.325};
    x.sigma_s = {0.1, 0.117, 0.0, 1.42};
    x.chi = {1.0, 0.0};
    x.sigma_t = {0.2208, 1.604};
    Material* med = make_material(17, "2-group infinite medium", x);
    cases.push_back({"grad2d_ls", hom_lattice_geometry(med, NULL, -1, VAC,
                     REF, REF, VAC), 4, 0.1, 500, 1e-5, FISSION_SOURCE, EIGEN,
                     1.0, true, NULL, 0.0, 0, 0.0, true, false, NULL});
  }
  /* 10. tests/test_fixed_linear_source: the same lattice, all vacuum, filled
   *     with C5G7 water, one lattice cell holding a fixed source with flat
   *     values and first moments; computeFlux with negative fluxes allowed */
  {
    Material* water = make_material(18, "Water", c5g7(false));
    Cell* src = NULL;
    Geometry* geo = hom_lattice_geometry(water, &src, 3 * 10 + 3, VAC, VAC,
                                         VAC, VAC);
    CaseSpec cs = {"fixls_c5g7", geo, 4, 0.1, 500, 1e-5, SCALAR_FLUX, FLUX,
                   1.0, false, NULL, 0.0, 0, 0.0, true, true, src};
    cs.src_cell_flat = {1.0, 0.5, 0.25, 1.0, 0.5, 0.25, 1.0};
    cs.src_cell_moments = {0.01, 0.1, 0.2,  -0.1, 0.0, -0.04,  0.02, 0.0, 0.0,
                           0, 0, 0,  0, 0, 0,  0, 0, 0,  0, 0, 0};
    cases.push_back(cs);
  }
  /* 11. the 7-group synthetic pin cell of case 3 with the linear source */
  {
    Material* fuel = make_material(19, "fuel7ls",
        openmoc_gb300::make_synthetic_xs(0xC0FFEEULL, 7, true));
    Material* mod = make_material(20, "mod7ls",
        openmoc_gb300::make_synthetic_xs(0xC0FFEEULL + 1000, 7, false));
    Universe* u = make_pin(fuel, mod, pin);
    cases.push_back({"pin7_ls", make_box_geometry(u, NULL, 0.63, REF, REF,
                     REF, REF), 32, 0.05, 1000, 1e-5, FISSION_SOURCE, EIGEN,
                     1.0, true, NULL, 0.0, 0, 0.0, true, false, NULL});
  }
  /* 12. the fixed-source 3x3 lattice of case 6 (computeSource, keff 1)
   *     with the linear source */
  {
    Material* fuel = make_material(21, "fuel7sl",
        openmoc_gb300::make_synthetic_xs(0xC0FFEEULL + 4, 7, true));
    Material* mod = make_material(22, "mod7sl",
        openmoc_gb300::make_synthetic_xs(0xC0FFEEULL + 1004, 7, false));
    cases.push_back({"src3_ls", lattice_geometry(3, fuel, mod, pin, {4},
                     REF, VAC, REF, VAC), 16, 0.1, 1000, 1e-5,
                     TOTAL_SOURCE, SOURCE, 1.0, false, fuel, 1.0, 0, 0.0,
                     true, false, NULL});
  }

  /* 13-14. CMFD acceleration (tests/test_cmfd_* set Cmfd up the same way:
   *        setLatticeStructure, setGroupStructure, relaxation factors).
   *        A 3x3 lattice, 7 groups, reflective, centre pin water, on a 3x3
   *        mesh with two coarse groups; a 5x5 lattice, 7 groups, vacuum on
   *        +x and +y, on a 5x5 mesh with a coarse group per group. */
  {
    Material* fuel = make_material(23, "fuel7c",
        openmoc_gb300::make_synthetic_xs(0xC0FFEEULL + 5, 7, true));
    Material* mod = make_material(24, "mod7c",
        openmoc_gb300::make_synthetic_xs(0xC0FFEEULL + 1005, 7, false));
    Geometry* geo = lattice_geometry(3, fuel, mod, pin, {4}, REF, REF, REF,
                                     REF);
    Cmfd* cm = new Cmfd();
    cm->setLatticeStructure(3, 3);
    cm->setGroupStructure({{1, 2, 3}, {4, 5, 6, 7}});
    cm->setCMFDRelaxationFactor(0.7);
    cm->setSORRelaxationFactor(1.5);
    geo->setCmfd(cm);
    CaseSpec cs = {"cmfd_lat3", geo, 16, 0.1, 1000, 1e-5, FISSION_SOURCE,
                   EIGEN, 1.0, false, NULL, 0.0};
    cs.cmfd = cm;
    cases.push_back(cs);
  }
  {
    Material* fuel = make_material(25, "fuel7v",
        openmoc_gb300::make_synthetic_xs(0xC0FFEEULL + 6, 7, true));
    Material* mod = make_material(26, "mod7v",
        openmoc_gb300::make_synthetic_xs(0xC0FFEEULL + 1006, 7, false));
    Geometry* geo = lattice_geometry(5, fuel, mod, pin, {6, 12, 18}, REF,
                                     VAC, REF, VAC);
    Cmfd* cm = new Cmfd();
    cm->setLatticeStructure(5, 5);
    cm->setSORRelaxationFactor(1.5);
    geo->setCmfd(cm);
    CaseSpec cs = {"cmfd_lat5_vac", geo, 16, 0.1, 1000, 1e-5, FISSION_SOURCE,
                   EIGEN, 1.0, false, NULL, 0.0};
    cs.cmfd = cm;
    cases.push_back(cs);
  }

  /* 15. the reflective 3x3 lattice of case 13 with the linear source
   *     (CPULSSolver with CMFD: no Larsen factor, moments prolonged); SOR
   *     factor 1.0 as tests/test_cmfd_linear_source sets it (at 1.5
   *     OpenMOC's FP32 coarse solve fails on this case) */
  {
    Material* fuel = make_material(27, "fuel7cl",
        openmoc_gb300::make_synthetic_xs(0xC0FFEEULL + 5, 7, true));
    Material* mod = make_material(28, "mod7cl",
        openmoc_gb300::make_synthetic_xs(0xC0FFEEULL + 1005, 7, false));
    Geometry* geo = lattice_geometry(3, fuel, mod, pin, {4}, REF, REF, REF,
                                     REF);
    Cmfd* cm = new Cmfd();
    cm->setLatticeStructure(3, 3);
    cm->setGroupStructure({{1, 2, 3}, {4, 5, 6, 7}});
    cm->setCMFDRelaxationFactor(0.7);
    cm->setSORRelaxationFactor(1.0);
    geo->setCmfd(cm);
    CaseSpec cs = {"cmfd_lat3_ls", geo, 16, 0.1, 1000, 1e-5, FISSION_SOURCE,
                   EIGEN, 1.0, false, NULL, 0.0, 0, 0.0, true, false, NULL};
    cs.cmfd = cm;
    cases.push_back(cs);
  }

  /* 16. case 13 with the k-nearest update (Cmfd::setKNearest(3), as
   *     tests/test_cmfd_pwr_assembly sets it) */
  {
    Material* fuel = make_material(29, "fuel7ck",
        openmoc_gb300::make_synthetic_xs(0xC0FFEEULL + 5, 7, true));
    Material* mod = make_material(30, "mod7ck",
        openmoc_gb300::make_synthetic_xs(0xC0FFEEULL + 1005, 7, false));
    Geometry* geo = lattice_geometry(3, fuel, mod, pin, {4}, REF, REF, REF,
                                     REF);
    Cmfd* cm = new Cmfd();
    cm->setLatticeStructure(3, 3);
    cm->setGroupStructure({{1, 2, 3}, {4, 5, 6, 7}});
    cm->setCMFDRelaxationFactor(0.7);
    cm->setSORRelaxationFactor(1.5);
    cm->setKNearest(3);
    geo->setCmfd(cm);
    CaseSpec cs = {"cmfd_lat3_k3", geo, 16, 0.1, 1000, 1e-5, FISSION_SOURCE,
                   EIGEN, 1.0, false, NULL, 0.0};
    cs.cmfd = cm;
    cs.k_nearest = 3;
    cases.push_back(cs);
  }

  /* 17. case 4 (3x3, 2 groups, vacuum on +x and +y) with keff from the
   *     neutron balance (Solver::setKeffFromNeutronBalance); the probe also
   *     takes the fission and scattering source hooks */
  {
    Material* fuel = make_material(31, "fuel2b",
        openmoc_gb300::make_synthetic_xs(0xC0FFEEULL + 2, 2, true));
    Material* mod = make_material(32, "mod2b",
        openmoc_gb300::make_synthetic_xs(0xC0FFEEULL + 1002, 2, false));
    CaseSpec cs = {"lat3_bal", lattice_geometry(3, fuel, mod, pin, {4}, REF,
                   VAC, REF, VAC), 16, 0.1, 1000, 1e-5, FISSION_SOURCE, EIGEN,
                   1.0, true, NULL, 0.0};
    cs.keff_balance = true;
    cs.probe_partial = true;
    cases.push_back(cs);
  }
  /* 18-20. transport stabilization (Solver::stabilizeTransport): the
   *     7-group pin cell of case 3 with YAMAMOTO (factor 0.5) and GLOBAL
   *     (0.5); DIAGONAL on a 3x3 lattice, 7 groups, vacuum on +x and +y,
   *     whose moderator has negative within-group scattering in its last two
   *     groups (as transport-corrected data can), factor 1 */
  for (int k = 0; k < 2; k++) {
    Material* fuel = make_material(33 + 2 * k, "fuel7st",
        openmoc_gb300::make_synthetic_xs(0xC0FFEEULL, 7, true));
    Material* mod = make_material(34 + 2 * k, "mod7st",
        openmoc_gb300::make_synthetic_xs(0xC0FFEEULL + 1000, 7, false));
    Universe* u = make_pin(fuel, mod, pin);
    CaseSpec cs = {k == 0 ? "pin7_stab_y" : "pin7_stab_g",
                   make_box_geometry(u, NULL, 0.63, REF, REF, REF, REF), 32,
                   0.05, 1000, 1e-5, FISSION_SOURCE, EIGEN, 1.0, false, NULL,
                   0.0};
    cs.stab_type = (k == 0 ? (int) YAMAMOTO : (int) GLOBAL) + 1;
    cs.stab_factor = 0.5;
    cases.push_back(cs);
  }
  {
    Material* fuel = make_material(37, "fuel7sd",
        openmoc_gb300::make_synthetic_xs(0xC0FFEEULL + 4, 7, true));
    MaterialXS mx = openmoc_gb300::make_synthetic_xs(0xC0FFEEULL + 1004, 7,
                                                     false);
    for (int g = 5; g < 7; g++) mx.sigma_s[g * 7 + g] = -0.05 * mx.sigma_t[g];
    Material* mod = make_material(38, "mod7sd", mx);
    CaseSpec cs = {"lat3_stab_d", lattice_geometry(3, fuel, mod, pin, {4},
                   REF, VAC, REF, VAC), 16, 0.1, 1000, 1e-5, FISSION_SOURCE,
                   EIGEN, 1.0, false, NULL, 0.0};
    cs.stab_type = (int) DIAGONAL + 1;
    cs.stab_factor = 1.0;
    cases.push_back(cs);
  }

  for (const CaseSpec& c : cases) {
    if (!only.empty() && only != c.name) continue;
    run_case(c, outdir);
  }
  return 0;
}
