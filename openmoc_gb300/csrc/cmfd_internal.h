// Host side of the CMFD accelerator: the coarse-mesh diffusion problem built
// from the sweep's tallies and solved in FP64 on the host (the reference's
// Cmfd::computeKeff, src/Cmfd.cpp:1192-1302, and linalg.cpp's power
// iteration with red-black SOR).  The device side (partial-current tallies in
// the sweep, flux reductions and the prolongation) is in cmfd.cu.
#pragma once

#include <cstdint>
#include <vector>

namespace moc_cmfd {

// Mesh faces: 0 x-min, 1 y-min, 2 x-max, 3 y-max (opposite face f ^ 2).
constexpr int kFaces = 4;

struct Config {
  int nx = 0, ny = 0;
  int G = 0, E = 0;                 // transport groups, coarse groups
  std::vector<double> wx, wy;       // cell widths
  std::vector<int> group_of;        // [G] coarse group of each group
  std::vector<int> gstart;          // [E + 1] first group of each coarse group
  std::vector<double> edc_mu, edc_w;  // Larsen EDC quadrature (empty: off)
  int bc[kFaces] = {1, 1, 1, 1};    // 0 vacuum, 1 reflective
  double relaxation = 0.7;
  double sor = 1.5;
  bool flux_limiting = true;
  int unbounded = 0;                // setNumUnboundedIterations
  int cells() const { return nx * ny; }
};

// The transport problem as the coarse solve sees it: cross sections by
// material and the (coarse cell, material) pairs the FSRs fall into.
struct Fine {
  int M = 0;
  std::vector<double> st, nf, chi;  // [M][G]
  std::vector<double> ss;           // [M][dest][orig]
  std::vector<int> pair_cell, pair_mat;
  std::vector<double> cell_vol;     // [cells]
  int pairs() const { return (int) pair_cell.size(); }
};

struct Stats {
  int power_iterations = 0;
  int linear_iterations = 0;        // total SOR sweeps of the last solve
  double max_ratio = 1.0;           // prolongation ratio farthest from 1
  bool failed = false;              // the last coarse solve did not converge
};

// The k-nearest prolongation of Cmfd::getUpdateRatio (src/Cmfd.cpp:
// 3178-3220) with the stencils of Cmfd::generateKNearestStencils
// (src/Cmfd.cpp:2887-2960) as per-FSR coefficients: the update ratio of FSR
// r is sum over j in [off[r], off[r+1]) of coef[j] * ratio[cell[j]].
void knearest_coefficients(const Config& cfg, int k, double origin_x,
                           double origin_y, const double* centroid,
                           const int32_t* fsr_cell, int64_t R,
                           std::vector<int32_t>& off,
                           std::vector<int32_t>& cell,
                           std::vector<float>& coef);

class Solver {
 public:
  Config cfg;
  Fine fine;
  double keff = 1.0;
  double source_threshold = 1e-5;   // setSourceConvergenceThreshold
  Stats stats;
  std::vector<double> phi_old, phi_new;  // [cells][E] of the last solve
  std::vector<double> ratio;              // [cells][E] prolongation factors

  // Starts a new eigenvalue solve: relaxation history and keff reset.
  void reset();
  // One acceleration step after the sweep of MOC iteration `moc_iter`.
  // S = [pairs][G] sums of phi * volume, cur = [cells][4][ld] outgoing
  // partial currents.  Fills `ratio` (all ones when the coarse solve fails,
  // keff then unchanged) and returns keff.
  double step(int moc_iter, const double* S, const float* cur, int ld);

 private:
  // collapsed cross sections and diffusion data of the current step
  std::vector<double> sig_t, nu_f, chi_c, dif, vol;   // [cells][E]
  std::vector<double> sig_s;                          // [cells][E][E] e -> g
  std::vector<double> dcorr_old;                      // [cells][4][E]
  bool dcorr_valid = false;
  // A: per row the in-cell block [cells][E][E] (row e, column g) and the
  // neighbour couplings [cells][4][E]; M: [cells][E][E]
  std::vector<double> a_blk, a_nb, m_blk;

  void collapse(const double* S, const float* cur, int ld,
                std::vector<double>& J);
  double larsen(double d, double delta) const;
  void build(int moc_iter, const std::vector<double>& J);
  void fission(const std::vector<double>& x, std::vector<double>& out) const;
  bool linear_solve(std::vector<double>& x, const std::vector<double>& b,
                    double tol);
  bool dd_linear_solve(std::vector<double>& x, const std::vector<double>& b,
                       double tol);
  double eigen_solve(std::vector<double>& x, double k, double tol);
  int neighbour(int cell, int face) const;
};

}  // namespace moc_cmfd
