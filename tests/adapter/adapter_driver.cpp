// Drives GB300Solver (openmoc_gb300/adapter) through OpenMOC's own API on
// the reference pin cell: geometry, TrackGenerator, then the solver.  With
// a GPU it prints keff and the iteration count; without one, the error the
// adapter raises through log_printf(ERROR) (a std::logic_error).
#include <cstdio>
#include <stdexcept>

#include "CPUSolver.h"
#include "GB300Solver.h"
#include "log.h"

int main() {
  set_log_level("ERROR");
  const int G = 2;
  double st[G] = {0.2208, 1.604};
  double ss[G * G] = {0.1, 0.117, 0.0, 1.42};
  double nf[G] = {0.0015, 0.325};
  double sf[G] = {0.000625, 0.135416667};
  double chi[G] = {1.0, 0.0};
  Material* mat = new Material(1, "hom");
  mat->setNumEnergyGroups(G);
  mat->setSigmaT(st, G);
  mat->setSigmaS(ss, G * G);
  mat->setNuSigmaF(nf, G);
  mat->setSigmaF(sf, G);
  mat->setChi(chi, G);
  Material* mod = new Material(2, "mod");
  mod->setNumEnergyGroups(G);
  double st2[G] = {0.3, 1.2};
  double ss2[G * G] = {0.2, 0.09, 0.0, 1.1};
  double z[G] = {0.0, 0.0};
  mod->setSigmaT(st2, G);
  mod->setSigmaS(ss2, G * G);
  mod->setNuSigmaF(z, G);
  mod->setSigmaF(z, G);
  mod->setChi(z, G);
  ZCylinder cyl(0.0, 0.0, 0.5);
  XPlane xmin(-1.0), xmax(1.0);
  YPlane ymin(-1.0), ymax(1.0);
  xmin.setBoundaryType(REFLECTIVE);
  xmax.setBoundaryType(REFLECTIVE);
  ymin.setBoundaryType(REFLECTIVE);
  ymax.setBoundaryType(REFLECTIVE);
  Cell* fuel = new Cell();
  fuel->setFill(mat);
  fuel->addSurface(-1, &cyl);
  Cell* water = new Cell();
  water->setFill(mod);
  water->addSurface(+1, &cyl);
  water->addSurface(+1, &xmin);
  water->addSurface(-1, &xmax);
  water->addSurface(+1, &ymin);
  water->addSurface(-1, &ymax);
  Universe* root = new Universe();
  root->addCell(fuel);
  root->addCell(water);
  Geometry geo;
  geo.setRootUniverse(root);
  geo.initializeFlatSourceRegions();
  TrackGenerator tg(&geo, 8, 0.1);
  tg.setNumThreads(1);
  tg.generateTracks();

  CPUSolver cpu(&tg);
  cpu.setNumThreads(1);
  cpu.computeEigenvalue(1000);
  printf("cpu keff %.8f iterations %d\n", cpu.getKeff(),
         cpu.getNumIterations());
  try {
    GB300Solver gpu(&tg);
    gpu.computeEigenvalue(1000);
    printf("gb300 keff %.8f iterations %d\n", gpu.getKeff(),
           gpu.getNumIterations());
    printf("gb300 flux(0,1) %.8e cpu %.8e\n", gpu.getFlux(0, 1),
           cpu.getFlux(0, 1));
  } catch (std::exception& e) {
    printf("gb300 error: %s\n", e.what());
  }
  try {
    GB300LSSolver gpu_ls(&tg);
    gpu_ls.computeEigenvalue(1000);
    printf("gb300 ls keff %.8f iterations %d\n", gpu_ls.getKeff(),
           gpu_ls.getNumIterations());
  } catch (std::exception& e) {
    printf("gb300 ls error: %s\n", e.what());
  }
  return 0;
}
