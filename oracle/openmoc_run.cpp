/*
 * OpenMOC itself on the benchmark configurations.  TEST INFRASTRUCTURE ONLY:
 * the generator of the benchmark-size golden files and the timed OpenMOC CPU
 * baseline.  Linked against OpenMOC's library, compiled from its own sources
 * by oracle/ref.mk (an FP_PRECISION=float and an FP_PRECISION=double build);
 * nothing in the product library uses it.
 *
 *   openmoc_run_<f32|f64> <config> golden <iterations> <out.json>
 *   openmoc_run_<f32|f64> <config> time <warmup> <iterations> <threads>
 *   openmoc_run_<f32|f64> <config3d> laydown3d <out dir> <threads>
 *
 * Configurations (the same geometry, quadrature and seeded cross sections as
 * openmoc_gb300/lattice.py builds them):
 *   pin7        one pin cell, 7 groups, 32 azimuthal, 0.05 cm, reflective
 *   assembly70  17 x 17 pins with 25 water-filled guide tubes, 70 groups,
 *               64 azimuthal, 0.05 cm, reflective
 *   core51      3 x 3 such assemblies, three fuel sets in a checkerboard of
 *               assemblies, 7 groups, 128 azimuthal, 0.03 cm, vacuum on +x
 *               and +y, reflective on -x and -y
 * All with the default Tabuchi-Yamamoto quadrature of 6 polar angles
 * (TrackGenerator's default) and single-threaded track generation, so FSR
 * numbering is reproducible (as the reference's test harness does).
 * 3D configurations (TrackGenerator3D, explicit 3D segments, its default
 * Gauss-Legendre polar quadrature; the lattice below the fuel height, one
 * homogeneous moderator cell above, reflective radially, vacuum at the
 * bottom and top):
 *   assembly3d  the 17 x 17 assembly, 20 cm tall, fuel below 16 cm, 7
 *               groups, 16 azimuthal, 6 polar, 0.1 cm radial, 0.5 cm axial
 *   lattice3d   a 3 x 3 lattice (one water pin), 2 cm tall, fuel below
 *               1.6 cm, 7 groups, 8 azimuthal, 4 polar, 0.1 cm, 0.4 cm
 *
 * laydown3d: the 3D tracks and their explicit segments, written to <out dir>
 *   as raw little-endian arrays (<name>.bin, listed with dtype and length in
 *   meta.json), in track UID order: azimuthal, xy, polar and stack index;
 *   start and end points; segment count, total length and the length above
 *   the fuel height (segments starting there); the forward / backward
 *   connecting tracks and flags as the packer forms them; per (azimuthal,
 *   polar) row the corrected polar angle, polar spacing and weight, the
 *   azimuthal spacing and weight, the total weight and the l / z counts;
 *   and the FSR volumes.
 *
 * golden: CPUSolver::computeEigenvalue for exactly <iterations> source
 *   iterations (a convergence threshold of 1e-30 never stops it earlier),
 *   FISSION_SOURCE residual; writes checksums of the integer track data
 *   (FSR ids, offsets, angles, links, flags, materials), quantised sums of
 *   the float data (segment lengths on a 2^-24 cm grid, FSR volumes on a
 *   2^-20 cm^2 grid: the plain and the index-weighted sum of the rounded
 *   values, exact in integers, so a value that differs by one unit in the
 *   last place moves them by at most one grid step, and rarely at all),
 *   keff, every group's flux summed over FSRs and a fixed sample of 4096
 *   FSR fluxes.
 * time: CPUSolver with setNumThreads(<threads>), computeEigenvalue(<warmup>)
 *   then computeEigenvalue(<iterations>) with the same solver; prints the
 *   second run's Timer splits (src/Solver.cpp:1552-1700: "Total time",
 *   "Solver initialization"; src/CPUSolver.cpp:2365-2378: "Transport
 *   Sweep") and the integration count 2 * F * S per iteration
 *   (src/Solver.cpp:1901) as one JSON line.
 */
#include <omp.h>

#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "CPUSolver.h"
#include "Geometry.h"
#include "TrackGenerator.h"
#include "TrackGenerator3D.h"
#include "log.h"

#include "../openmoc_gb300/adapter/pack_reference.h"
#include "../openmoc_gb300/csrc/synthetic_xs.h"

using openmoc_gb300::MaterialXS;
using openmoc_gb300::PackedProblem;

#ifdef SINGLE
static const char* PREC = "f32";
#else
static const char* PREC = "f64";
#endif

static const uint64_t SEED = 0xC0FFEEULL;

/* A CPUSolver whose Timer splits can be read. */
class TimedSolver : public CPUSolver {
 public:
  explicit TimedSolver(TrackGenerator* tg) : CPUSolver(tg) {}
  double split(const char* name) { return _timer->getSplit(name); }
};

static Material* make_material(int id, const MaterialXS& x) {
  Material* m = new Material(id);
  const int G = x.num_groups;
  std::vector<double> t = x.sigma_t, s = x.sigma_s, nf = x.nu_sigma_f,
                      f = x.sigma_f, c = x.chi;
  m->setNumEnergyGroups(G);
  m->setSigmaT(t.data(), G);
  m->setSigmaS(s.data(), G * G);
  m->setSigmaF(f.data(), G);
  m->setNuSigmaF(nf.data(), G);
  m->setChi(c.data(), G);
  return m;
}

/* The pin: fuel inside r = 0.54 cm in 3 equal-area rings x 8 sectors,
 * moderator outside in 8 sectors. */
static Universe* make_pin(Material* inner, Material* outer) {
  ZCylinder* cyl = new ZCylinder(0.0, 0.0, 0.54);
  Cell* f = new Cell();
  f->setFill(inner);
  f->addSurface(-1, cyl);
  f->setNumRings(3);
  f->setNumSectors(8);
  Cell* m = new Cell();
  m->setFill(outer);
  m->addSurface(+1, cyl);
  m->setNumSectors(8);
  Universe* u = new Universe();
  u->addCell(f);
  u->addCell(m);
  return u;
}

/* n x n lattice at 1.26 cm in a box; u[row from the top * n + column]. */
static Geometry* lattice_box(int n, std::vector<Universe*> u,
                             boundaryType bxmin, boundaryType bxmax,
                             boundaryType bymin, boundaryType bymax) {
  const double pitch = 1.26, hw = 0.5 * n * pitch;
  Lattice* lat = new Lattice();
  lat->setWidth(pitch, pitch);
  lat->setUniverses(1, n, n, u.data());
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
  root->setFill(lat);
  Universe* ru = new Universe();
  ru->addCell(root);
  Geometry* g = new Geometry();
  g->setRootUniverse(ru);
  return g;
}

/* Guide-tube positions of a 17 x 17 PWR assembly, (row, column) from the
 * top left (24 guide tubes and the instrument tube). */
static const int GUIDE_TUBES[25][2] = {
    {2, 5}, {2, 8}, {2, 11}, {3, 3}, {3, 13}, {5, 2}, {5, 5}, {5, 8},
    {5, 11}, {5, 14}, {8, 2}, {8, 5}, {8, 8}, {8, 11}, {8, 14}, {11, 2},
    {11, 5}, {11, 8}, {11, 11}, {11, 14}, {13, 3}, {13, 13}, {14, 5},
    {14, 8}, {14, 11}};

struct Config {
  Geometry* geo;
  int num_azim;
  double spacing;
};

/* Fuel materials get ids 1..n_fuel and the moderator id 100, so the packed
 * material index (OpenMOC's material map order) is fuel 0..n_fuel-1 and then
 * the moderator, as the library's lattice builder numbers them. */
static Config make_config(const std::string& name) {
  const boundaryType REF = REFLECTIVE, VAC = VACUUM;
  if (name == "pin7") {
    Material* fuel = make_material(1, openmoc_gb300::make_synthetic_xs(
                                          SEED + 0, 7, true));
    Material* mod = make_material(100, openmoc_gb300::make_synthetic_xs(
                                           SEED + 1000, 7, false));
    return {lattice_box(1, {make_pin(fuel, mod)}, REF, REF, REF, REF), 32,
            0.05};
  }
  if (name == "assembly70") {
    Material* fuel = make_material(1, openmoc_gb300::make_synthetic_xs(
                                          SEED + 1, 70, true));
    Material* mod = make_material(100, openmoc_gb300::make_synthetic_xs(
                                           SEED + 1001, 70, false));
    Universe* pin = make_pin(fuel, mod);
    Universe* water = make_pin(mod, mod);
    std::vector<Universe*> u(17 * 17, pin);
    for (const auto& rc : GUIDE_TUBES) u[rc[0] * 17 + rc[1]] = water;
    return {lattice_box(17, u, REF, REF, REF, REF), 64, 0.05};
  }
  if (name == "core51") {
    Universe* pins[3];
    Material* mod = make_material(100, openmoc_gb300::make_synthetic_xs(
                                           SEED + 3 + 1000, 7, false));
    for (int k = 0; k < 3; k++)
      pins[k] = make_pin(make_material(1 + k, openmoc_gb300::make_synthetic_xs(
                                                   SEED + 3 + k, 7, true)),
                         mod);
    Universe* water = make_pin(mod, mod);
    std::vector<Universe*> u(51 * 51, NULL);
    for (int ar = 0; ar < 3; ar++)
      for (int ac = 0; ac < 3; ac++) {
        Universe* fuel = pins[(ar + ac) % 3];
        for (int r = 0; r < 17; r++)
          for (int c = 0; c < 17; c++)
            u[(17 * ar + r) * 51 + 17 * ac + c] = fuel;
        for (const auto& rc : GUIDE_TUBES)
          u[(17 * ar + rc[0]) * 51 + 17 * ac + rc[1]] = water;
      }
    return {lattice_box(51, u, REF, VAC, REF, VAC), 128, 0.03};
  }
  fprintf(stderr, "unknown configuration %s\n", name.c_str());
  exit(2);
}

struct Config3D {
  Geometry* geo;
  int num_azim, num_polar;
  double spacing, z_spacing, fuel_height;
};

/* The n x n lattice for 0 < z < zf and a moderator cell above up to zt. */
static Geometry* lattice_box_3d(int n, std::vector<Universe*> u, Material* mod,
                                double zf, double zt) {
  const double pitch = 1.26, hw = 0.5 * n * pitch;
  Lattice* lat = new Lattice();
  lat->setWidth(pitch, pitch);
  lat->setUniverses(1, n, n, u.data());
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
  Cell* low = new Cell();
  low->addSurface(+1, xmin);
  low->addSurface(-1, xmax);
  low->addSurface(+1, ymin);
  low->addSurface(-1, ymax);
  low->addSurface(+1, zmin);
  low->addSurface(-1, zmid);
  low->setFill(lat);
  Cell* top = new Cell();
  top->addSurface(+1, xmin);
  top->addSurface(-1, xmax);
  top->addSurface(+1, ymin);
  top->addSurface(-1, ymax);
  top->addSurface(+1, zmid);
  top->addSurface(-1, zmax);
  top->setFill(mod);
  Universe* ru = new Universe();
  ru->addCell(low);
  ru->addCell(top);
  Geometry* g = new Geometry();
  g->setRootUniverse(ru);
  return g;
}

static Config3D make_config_3d(const std::string& name) {
  if (name == "assembly3d") {
    Material* fuel = make_material(1, openmoc_gb300::make_synthetic_xs(
                                          SEED + 4, 7, true));
    Material* mod = make_material(100, openmoc_gb300::make_synthetic_xs(
                                           SEED + 1004, 7, false));
    Universe* pin = make_pin(fuel, mod);
    Universe* water = make_pin(mod, mod);
    std::vector<Universe*> u(17 * 17, pin);
    for (const auto& rc : GUIDE_TUBES) u[rc[0] * 17 + rc[1]] = water;
    return {lattice_box_3d(17, u, mod, 16.0, 20.0), 16, 6, 0.1, 0.5, 16.0};
  }
  if (name == "lattice3d") {
    Material* fuel = make_material(1, openmoc_gb300::make_synthetic_xs(
                                          SEED + 0, 7, true));
    Material* mod = make_material(100, openmoc_gb300::make_synthetic_xs(
                                           SEED + 1000, 7, false));
    Universe* pin = make_pin(fuel, mod);
    Universe* water = make_pin(mod, mod);
    std::vector<Universe*> u(9, pin);
    u[4] = water;
    return {lattice_box_3d(3, u, mod, 1.6, 2.0), 8, 4, 0.1, 0.4, 1.6};
  }
  fprintf(stderr, "unknown 3D configuration %s\n", name.c_str());
  exit(2);
}

template <typename T>
static void dump(const std::string& dir, const char* name, const char* dtype,
                 const std::vector<T>& a, FILE* meta, bool& first) {
  FILE* f = fopen((dir + "/" + name + ".bin").c_str(), "wb");
  if (!f) {
    perror(name);
    exit(1);
  }
  fwrite(a.data(), sizeof(T), a.size(), f);
  fclose(f);
  fprintf(meta, "%s\n  \"%s\": [\"%s\", %zu]", first ? "" : ",", name, dtype,
          a.size());
  first = false;
}

static int laydown3d(const std::string& name, const std::string& dir,
                     int threads) {
  Config3D c = make_config_3d(name);
  c.geo->initializeFlatSourceRegions();
  TrackGenerator3D tg(c.geo, c.num_azim, c.num_polar, c.spacing, c.z_spacing);
  tg.setSegmentFormation(EXPLICIT_3D);
  tg.setNumThreads(threads);
  tg.generateTracks();
  PackedProblem p;
  openmoc_gb300::pack_tracks(&tg, p);
  const long T = tg.getNum3DTracks();
  const int A = c.num_azim / 2, P = c.num_polar;
  std::vector<int32_t> ta(T), txy(T), tp(T), tz(T), nseg(T);
  std::vector<double> start(3 * T), end(3 * T), lsum(T), ltop(T);
  Track3D**** t3d = tg.get3DTracks();
  int*** tps = tg.getTracksPerStack();
  Track** t2 = tg.get2DTracksArray();
  long n2 = tg.getNum2DTracks();
  for (long i = 0; i < n2; i++) {
    const int a = t2[i]->getAzimIndex(), xy = t2[i]->getXYIndex();
    for (int pp = 0; pp < P; pp++)
      for (int z = 0; z < tps[a][xy][pp]; z++) {
        Track3D* t = &t3d[a][xy][pp][z];
        const long u = t->getUid();
        ta[u] = a;
        txy[u] = xy;
        tp[u] = pp;
        tz[u] = z;
        start[3 * u] = t->getStart()->getX();
        start[3 * u + 1] = t->getStart()->getY();
        start[3 * u + 2] = t->getStart()->getZ();
        end[3 * u] = t->getEnd()->getX();
        end[3 * u + 1] = t->getEnd()->getY();
        end[3 * u + 2] = t->getEnd()->getZ();
        nseg[u] = t->getNumSegments();
        double s = 0, top = 0;
        for (int k = 0; k < t->getNumSegments(); k++) {
          segment* sg = t->getSegment(k);
          s += sg->_length;
          if (sg->_starting_position[2] >= c.fuel_height - 1e-9)
            top += sg->_length;
        }
        lsum[u] = s;
        ltop[u] = top;
      }
  }
  Quadrature* q = tg.getQuadrature();
  std::vector<double> theta(A * P), pspace(A * P), pwgt(A * P), aspace(A * P),
      awgt(A * P), wtot(A * P);
  std::vector<int32_t> numl(A * P), numz(A * P);
  for (int a = 0; a < A; a++)
    for (int pp = 0; pp < P; pp++) {
      const int r = a * P + pp;
      theta[r] = q->getTheta(a, pp);
      pspace[r] = q->getPolarSpacing(a, pp);
      pwgt[r] = q->getPolarWeight(a, pp);
      aspace[r] = q->getAzimSpacing(a);
      awgt[r] = q->getAzimWeight(a);
      wtot[r] = q->getWeightInline(a, pp);
      numl[r] = tg.getNumL(a, pp);
      numz[r] = tg.getNumZ(a, pp);
    }
  const long R = c.geo->getNumFSRs();
  tg.initializeFSRVolumesBuffer();
  FP_PRECISION* vols = tg.getFSRVolumes();
  std::vector<double> vol(vols, vols + R);
  FILE* meta = fopen((dir + "/meta.json").c_str(), "w");
  if (!meta) {
    perror("meta.json");
    return 1;
  }
  fprintf(meta, "{\n  \"config\": [\"%s\", 0]", name.c_str());
  bool first = false;
  dump(dir, "azim", "i4", ta, meta, first);
  dump(dir, "xy", "i4", txy, meta, first);
  dump(dir, "polar", "i4", tp, meta, first);
  dump(dir, "stack", "i4", tz, meta, first);
  dump(dir, "start", "f8", start, meta, first);
  dump(dir, "end", "f8", end, meta, first);
  dump(dir, "nseg", "i4", nseg, meta, first);
  dump(dir, "len_sum", "f8", lsum, meta, first);
  dump(dir, "len_top", "f8", ltop, meta, first);
  dump(dir, "next", "i8", p.next, meta, first);
  dump(dir, "flags", "u1", p.flags, meta, first);
  dump(dir, "theta", "f8", theta, meta, first);
  dump(dir, "polar_spacing", "f8", pspace, meta, first);
  dump(dir, "polar_weight", "f8", pwgt, meta, first);
  dump(dir, "azim_spacing", "f8", aspace, meta, first);
  dump(dir, "azim_weight", "f8", awgt, meta, first);
  dump(dir, "weight", "f8", wtot, meta, first);
  dump(dir, "num_l", "i4", numl, meta, first);
  dump(dir, "num_z", "i4", numz, meta, first);
  dump(dir, "fsr_vol", "f8", vol, meta, first);
  if (p.num_segments < 10000000) {
    /* small cases: every segment (length, start height, FSR id), UID order */
    std::vector<double> sl, sz;
    std::vector<int32_t> sfsr;
    std::vector<Track3D*> by_uid(T);
    for (long i = 0; i < n2; i++) {
      const int a = t2[i]->getAzimIndex(), xy = t2[i]->getXYIndex();
      for (int pp = 0; pp < P; pp++)
        for (int z = 0; z < tps[a][xy][pp]; z++)
          by_uid[t3d[a][xy][pp][z].getUid()] = &t3d[a][xy][pp][z];
    }
    for (long u = 0; u < T; u++)
      for (int k = 0; k < by_uid[u]->getNumSegments(); k++) {
        segment* sg = by_uid[u]->getSegment(k);
        sl.push_back(sg->_length);
        sz.push_back(sg->_starting_position[2]);
        sfsr.push_back((int32_t) sg->_region_id);
      }
    dump(dir, "seg_len", "f8", sl, meta, first);
    dump(dir, "seg_z0", "f8", sz, meta, first);
    dump(dir, "seg_fsr", "i4", sfsr, meta, first);
  }
  fprintf(meta, "\n}\n");
  fclose(meta);
  printf("%s: R=%ld T=%ld S=%ld\n", name.c_str(), R, T, p.num_segments);
  return 0;
}

/* Order-sensitive checksum of an array's bytes taken as little-endian words
 * of the element size: sum over i of (word_i + 1) * (2 i + 1) mod 2^64.
 * tests/test_benchmark_configs.py computes the same with numpy. */
template <typename T>
static uint64_t checksum(const std::vector<T>& a) {
  static_assert(sizeof(T) <= 8, "word size");
  uint64_t s = 0;
  for (size_t i = 0; i < a.size(); i++) {
    uint64_t w = 0;
    std::memcpy(&w, &a[i], sizeof(T));
    s += (w + 1) * (2 * (uint64_t) i + 1);
  }
  return s;
}

/* The sum and the sum of (i mod 1009 + 1) * q_i (mod 2^64) of
 * q_i = floor(v_i * 2^bits + 1/2), both exact (the same as tests/conftest.py's
 * quantised_sums). */
static std::vector<uint64_t> quantised_sums(const std::vector<float>& a,
                                           int bits) {
  std::vector<uint64_t> m(2, 0);
  const double scale = std::ldexp(1.0, bits);
  for (size_t i = 0; i < a.size(); i++) {
    const uint64_t q = (uint64_t) (int64_t) std::floor((double) a[i] * scale + 0.5);
    m[0] += q;
    m[1] += (uint64_t) (i % 1009 + 1) * q;
  }
  return m;
}

static double seconds_since(std::chrono::steady_clock::time_point t0) {
  return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0)
      .count();
}

int main(int argc, char** argv) {
  if (argc < 4) {
    fprintf(stderr,
            "usage: %s <pin7|assembly70|core51> golden <iterations> <out.json>\n"
            "       %s <pin7|assembly70|core51> time <warmup> <iterations> "
            "<threads>\n",
            argv[0], argv[0]);
    return 2;
  }
  set_log_level("ERROR");
  const std::string name = argv[1], mode = argv[2];
  if (mode == "laydown3d")
    return laydown3d(name, argv[3], argc > 4 ? atoi(argv[4]) : 1);
  const bool golden = mode == "golden";
  if (!golden && (mode != "time" || argc < 6)) {
    fprintf(stderr, "unknown mode or missing arguments\n");
    return 2;
  }
  Config cfg = make_config(name);
  auto t0 = std::chrono::steady_clock::now();
  cfg.geo->initializeFlatSourceRegions();
  TrackGenerator tg(cfg.geo, cfg.num_azim, cfg.spacing);
  tg.setNumThreads(1);
  tg.generateTracks();
  const double t_tracks = seconds_since(t0);

  TimedSolver solver(&tg);
  solver.setConvergenceThreshold(1e-30);
  if (golden) {
    const int iters = atoi(argv[3]);
    solver.setNumThreads(omp_get_num_procs());
    solver.computeEigenvalue(iters, FISSION_SOURCE);
    PackedProblem p;
    openmoc_gb300::pack_tracks(&tg, p);
    openmoc_gb300::pack_materials(cfg.geo, tg.getFSRVolumes(), p);
    const long R = p.num_fsrs;
    const int G = p.num_groups;
    FILE* f = fopen(argv[4], "w");
    if (!f) {
      perror(argv[4]);
      return 1;
    }
    fprintf(f, "{\n  \"config\": \"%s\",\n  \"precision\": \"%s\",\n", name.c_str(),
            PREC);
    fprintf(f, "  \"iterations\": %d,\n  \"keff\": %.17g,\n",
            solver.getNumIterations(), solver.getKeff());
    fprintf(f, "  \"num_fsrs\": %ld,\n  \"num_tracks\": %ld,\n"
               "  \"num_segments\": %ld,\n  \"num_groups\": %d,\n",
            R, p.num_tracks, p.num_segments, G);
    fprintf(f, "  \"checksums\": {\"seg_fsr\": \"%llu\", "
               "\"seg_off\": \"%llu\", \"track_ang\": \"%llu\", \"next\": "
               "\"%llu\", \"flags\": \"%llu\", \"fsr_mat\": \"%llu\"},\n",
            (unsigned long long) checksum(p.seg_fsr),
            (unsigned long long) checksum(p.seg_off),
            (unsigned long long) checksum(p.track_ang),
            (unsigned long long) checksum(p.next),
            (unsigned long long) checksum(p.flags),
            (unsigned long long) checksum(p.fsr_mat));
    const std::vector<uint64_t> ql = quantised_sums(p.seg_len, 24),
                                qv = quantised_sums(p.fsr_vol, 20);
    fprintf(f, "  \"seg_len_q24\": [\"%llu\", \"%llu\"],\n",
            (unsigned long long) ql[0], (unsigned long long) ql[1]);
    fprintf(f, "  \"fsr_vol_q20\": [\"%llu\", \"%llu\"],\n",
            (unsigned long long) qv[0], (unsigned long long) qv[1]);
    fprintf(f, "  \"group_flux_sums\": [");
    for (int g = 0; g < G; g++) {
      double s = 0;
      for (long r = 0; r < R; r++) s += solver.getFlux(r, g + 1);
      fprintf(f, "%s%.17g", g ? ", " : "", s);
    }
    fprintf(f, "],\n");
    /* a fixed sample of (FSR, group) fluxes: index k*2654435761 mod R*G */
    const int K = 4096;
    const uint64_t n = (uint64_t) R * G;
    fprintf(f, "  \"flux_sample_index\": [");
    for (int k = 0; k < K; k++)
      fprintf(f, "%s%llu", k ? ", " : "",
              (unsigned long long) (((uint64_t) k * 2654435761ULL) % n));
    fprintf(f, "],\n  \"flux_sample\": [");
    for (int k = 0; k < K; k++) {
      uint64_t i = ((uint64_t) k * 2654435761ULL) % n;
      fprintf(f, "%s%.17g", k ? ", " : "",
              solver.getFlux((long) (i / G), (int) (i % G) + 1));
    }
    fprintf(f, "]\n}\n");
    fclose(f);
    printf("%s [%s]: R=%ld T=%ld S=%ld, %d iterations, keff %.10f, "
           "tracks %.1f s\n",
           name.c_str(), PREC, R, p.num_tracks, p.num_segments,
           solver.getNumIterations(), solver.getKeff(), t_tracks);
    return 0;
  }

  const int warmup = atoi(argv[3]), iters = atoi(argv[4]);
  const int threads = atoi(argv[5]);
  solver.setNumThreads(threads);
  if (warmup > 0) solver.computeEigenvalue(warmup, FISSION_SOURCE);
  solver.computeEigenvalue(iters, FISSION_SOURCE);
  const double total = solver.split("Total time");
  const double init = solver.split("Solver initialization");
  const double sweep = solver.split("Transport Sweep");
  long S = 0;
  Track** tracks = tg.get2DTracksArray();
  for (long t = 0; t < tg.getNum2DTracks(); t++)
    S += tracks[t]->getNumSegments();
  const int G = cfg.geo->getNumEnergyGroups();
  const int Ph = tg.getQuadrature()->getNumPolarAngles() / 2;
  const double ints = 2.0 * G * Ph * (double) S;
  printf("{\"config\": \"%s\", \"precision\": \"%s\", \"threads\": %d, "
         "\"iterations\": %d, \"fsrs\": %ld, \"tracks\": %ld, \"segments\": %ld, "
         "\"groups\": %d, \"integrations_per_iteration\": %.0f, "
         "\"track_generation_s\": %.6f, \"total_s\": %.6f, \"init_s\": %.6f, "
         "\"transport_sweep_s\": %.6f, \"keff\": %.10f}\n",
         name.c_str(), PREC, threads, solver.getNumIterations(),
         (long) cfg.geo->getNumFSRs(), (long) tg.getNum2DTracks(), S, G, ints,
         t_tracks, total, init, sweep, solver.getKeff());
  return 0;
}
