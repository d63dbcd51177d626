// Test shim: a C interface over the host coarse solve of the CMFD
// accelerator (openmoc_gb300/csrc/cmfd_solve.cpp), so that the CPU tests can
// drive it step by step next to the oracle without a GPU.
#include <cstdint>
#include <cstring>

#include "../../openmoc_gb300/csrc/cmfd_internal.h"

extern "C" {

void* shim_create(int nx, int ny, const double* wx, const double* wy, int G,
                  int E, const int32_t* group_of, const int32_t* bc,
                  int n_edc, const double* edc_mu, const double* edc_w,
                  double relaxation, double sor, int flux_limiting,
                  int unbounded) {
  auto* s = new moc_cmfd::Solver();
  moc_cmfd::Config& c = s->cfg;
  c.nx = nx;
  c.ny = ny;
  c.G = G;
  c.E = E;
  c.wx.assign(wx, wx + nx);
  c.wy.assign(wy, wy + ny);
  c.group_of.assign(group_of, group_of + G);
  c.gstart.assign(E + 1, G);
  for (int g = G - 1; g >= 0; g--) c.gstart[group_of[g]] = g;
  for (int f = 0; f < 4; f++) c.bc[f] = bc[f];
  c.edc_mu.assign(edc_mu, edc_mu + n_edc);
  c.edc_w.assign(edc_w, edc_w + n_edc);
  c.relaxation = relaxation;
  c.sor = sor;
  c.flux_limiting = flux_limiting != 0;
  c.unbounded = unbounded;
  return s;
}

void shim_set_fine(void* h, int M, const double* st, const double* nf,
                   const double* chi, const double* ss, int P,
                   const int32_t* pair_cell, const int32_t* pair_mat,
                   const double* cell_vol) {
  auto* s = static_cast<moc_cmfd::Solver*>(h);
  const int G = s->cfg.G, C = s->cfg.cells();
  moc_cmfd::Fine& f = s->fine;
  f.M = M;
  f.st.assign(st, st + (size_t) M * G);
  f.nf.assign(nf, nf + (size_t) M * G);
  f.chi.assign(chi, chi + (size_t) M * G);
  f.ss.assign(ss, ss + (size_t) M * G * G);
  f.pair_cell.assign(pair_cell, pair_cell + P);
  f.pair_mat.assign(pair_mat, pair_mat + P);
  f.cell_vol.assign(cell_vol, cell_vol + C);
}

void shim_reset(void* h, double threshold) {
  auto* s = static_cast<moc_cmfd::Solver*>(h);
  s->reset();
  s->source_threshold = 0.1 * threshold;
}

void shim_set_source_threshold(void* h, double t) {
  static_cast<moc_cmfd::Solver*>(h)->source_threshold = t;
}

double shim_step(void* h, int moc_iter, const double* S, const float* cur,
                 int ld, double* ratio_out, int* power_iterations) {
  auto* s = static_cast<moc_cmfd::Solver*>(h);
  const double k = s->step(moc_iter, S, cur, ld);
  std::memcpy(ratio_out, s->ratio.data(), sizeof(double) * s->ratio.size());
  *power_iterations = s->stats.power_iterations;
  return k;
}

void shim_destroy(void* h) { delete static_cast<moc_cmfd::Solver*>(h); }

}  // extern "C"
