// CMFD coarse-mesh solve on the host, FP64 (see cmfd_internal.h).
//
// Follows the reference's formulation step by step (the equations have to be
// the reference's for the accelerated iteration to behave like it):
//   * cross-section collapse, Cmfd::collapseXS (src/Cmfd.cpp:720-1000);
//   * surface diffusion coefficients, Cmfd::getSurfaceDiffusionCoefficient
//     (src/Cmfd.cpp:1048-1170) with Larsen's effective diffusion coefficient
//     factor, Cmfd::computeLarsensEDCFactor (src/Cmfd.cpp:1625-1650);
//   * loss and fission matrices, Cmfd::constructMatrices
//     (src/Cmfd.cpp:1353-1500);
//   * power iteration over red-black SOR, eigenvalueSolve and linearSolve
//     (src/linalg.cpp:25-176, 179-385) with computeRMSE's integrated form
//     (src/linalg.cpp:595-680);
//   * flux rescaling and prolongation ratios, Cmfd::rescaleFlux,
//     Cmfd::updateMOCFlux and Cmfd::getFluxRatio (src/Cmfd.cpp:1304-1350,
//     1509-1580, 3222-3300), ratios bounded to [0.05, 20] after the
//     unbounded iterations.
#include "cmfd_internal.h"

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <limits>

namespace moc_cmfd {

namespace {
constexpr double kZeroSigmaT = 1e-6;       // src/constants.h:34
constexpr double kFluxEpsilon = 1e-25;     // src/constants.h:15
constexpr double kLinalgTol = 1e-7;        // LINALG_TOL of the FP32 build
constexpr int kMinPowerIters = 25;         // src/constants.h:74-81
constexpr int kMaxPowerIters = 25000;
constexpr int kMinLinearIters = 25;
constexpr int kMaxLinearIters = 10000;
}  // namespace

void Solver::reset() {
  keff = 1.0;
  source_threshold = 1e-5;
  dcorr_valid = false;
  const int C = cfg.cells(), E = cfg.E;
  dcorr_old.assign((size_t) C * kFaces * E, 0.0);
  ratio.assign((size_t) C * E, 1.0);
  phi_old.assign((size_t) C * E, 0.0);
  phi_new.assign((size_t) C * E, 0.0);
  stats = Stats{};
}

int Solver::neighbour(int cell, int face) const {
  const int ix = cell % cfg.nx, iy = cell / cfg.nx;
  switch (face) {
    case 0: return ix > 0 ? cell - 1 : -1;
    case 1: return iy > 0 ? cell - cfg.nx : -1;
    case 2: return ix + 1 < cfg.nx ? cell + 1 : -1;
    default: return iy + 1 < cfg.ny ? cell + cfg.nx : -1;
  }
}

// Larsen's correction for a diffusion coefficient d over a cell of width
// delta: 1 + delta rho / (2 d), rho = sum 2 mu w alpha(mu),
// alpha = (1 + e) / (1 - e) - 2 (3 d mu) / delta, e = exp(-delta / (3 d mu)).
double Solver::larsen(double d, double delta) const {
  double rho = 0.0;
  for (size_t i = 0; i < cfg.edc_mu.size(); i++) {
    const double mu = cfg.edc_mu[i];
    const double e = std::exp(-delta / (3.0 * d * mu));
    const double alpha = (1.0 + e) / (1.0 - e) - 2.0 * (3.0 * d * mu) / delta;
    rho += 2.0 * mu * cfg.edc_w[i] * alpha;
  }
  return 1.0 + delta * rho / (2.0 * d);
}

// Coarse cross sections, diffusion coefficients and fluxes from the pair
// sums, and the coarse-group currents J [cells][4][E].
void Solver::collapse(const double* S, const float* cur, int ld,
                      std::vector<double>& J) {
  const int C = cfg.cells(), E = cfg.E, G = cfg.G, P = fine.pairs();
  sig_t.assign((size_t) C * E, 0.0);
  nu_f.assign((size_t) C * E, 0.0);
  chi_c.assign((size_t) C * E, 0.0);
  dif.assign((size_t) C * E, 0.0);
  vol.assign((size_t) C * E, 0.0);
  sig_s.assign((size_t) C * E * E, 0.0);
  phi_old.assign((size_t) C * E, 0.0);
  // pairs of each cell
  std::vector<std::vector<int>> of_cell(C);
  for (int p = 0; p < P; p++) of_cell[fine.pair_cell[p]].push_back(p);
  std::vector<double> chi_t(E), scat(E);
  for (int c = 0; c < C; c++) {
    const std::vector<int>& ps = of_cell[c];
    // fission spectrum weighted by each pair's neutron production
    double prod_total = 0.0;
    std::fill(chi_t.begin(), chi_t.end(), 0.0);
    for (int p : ps) {
      const int m = fine.pair_mat[p];
      const double* s = S + (size_t) p * G;
      double prod = 0.0;
      for (int h = 0; h < G; h++) prod += fine.nf[(size_t) m * G + h] * s[h];
      for (int e = 0; e < E; e++) {
        double ch = 0.0;
        for (int h = cfg.gstart[e]; h < cfg.gstart[e + 1]; h++)
          ch += fine.chi[(size_t) m * G + h];
        chi_t[e] += ch * prod;
      }
      prod_total += prod;
    }
    for (int e = 0; e < E; e++)
      chi_c[(size_t) c * E + e] =
          std::fabs(prod_total) > 0.0 ? chi_t[e] / prod_total : 0.0;
    for (int e = 0; e < E; e++) {
      double total = 0.0, nuf = 0.0, rxn = 0.0, dsum = 0.0;
      std::fill(scat.begin(), scat.end(), 0.0);
      for (int h = cfg.gstart[e]; h < cfg.gstart[e + 1]; h++) {
        double r = 0.0, t = 0.0;
        for (int p : ps) {
          const int m = fine.pair_mat[p];
          const double s = S[(size_t) p * G + h];
          r += s;
          t += fine.st[(size_t) m * G + h] * s;
          nuf += fine.nf[(size_t) m * G + h] * s;
          const double* col = fine.ss.data() + (size_t) m * G * G + h;
          for (int g = 0; g < G; g++)
            scat[cfg.group_of[g]] += col[(size_t) g * G] * s;
        }
        total += t;
        rxn += r;
        // D of the group from its flux-averaged total cross section
        if (std::fabs(t) > std::fabs(r) * FLT_EPSILON) dsum += r / (3.0 * (t / r));
      }
      if (rxn <= 0.0) {
        rxn = kZeroSigmaT;
        dsum = kZeroSigmaT;
        total = kZeroSigmaT;
        if (nuf != 0.0) nuf = kZeroSigmaT;
        std::fill(scat.begin(), scat.end(), 0.0);
      }
      const size_t ce = (size_t) c * E + e;
      sig_t[ce] = total / rxn;
      nu_f[ce] = nuf / rxn;
      for (int g = 0; g < E; g++) sig_s[ce * E + g] = scat[g] / rxn;
      dif[ce] = dsum / rxn;
      vol[ce] = fine.cell_vol[c];
      phi_old[ce] = rxn / fine.cell_vol[c];
    }
  }
  J.assign((size_t) C * kFaces * E, 0.0);
  for (int c = 0; c < C; c++)
    for (int f = 0; f < kFaces; f++) {
      const float* src = cur + ((size_t) c * kFaces + f) * ld;
      double* dst = J.data() + ((size_t) c * kFaces + f) * E;
      for (int h = 0; h < G; h++) dst[cfg.group_of[h]] += (double) src[h];
    }
}

// Surface diffusion coefficients and the loss / fission matrices.
void Solver::build(int moc_iter, const std::vector<double>& J) {
  const int C = cfg.cells(), E = cfg.E;
  a_blk.assign((size_t) C * E * E, 0.0);
  a_nb.assign((size_t) C * kFaces * E, 0.0);
  m_blk.assign((size_t) C * E * E, 0.0);
  const bool edc = !cfg.edc_mu.empty();
  for (int c = 0; c < C; c++) {
    const int ix = c % cfg.nx, iy = c / cfg.nx;
    for (int e = 0; e < E; e++) {
      const size_t ce = (size_t) c * E + e;
      const double V = vol[ce];
      double* row = a_blk.data() + ce * E;
      row[e] += sig_t[ce] * V;
      // in-scattering from every coarse group g
      for (int g = 0; g < E; g++) {
        const double v = -sig_s[((size_t) c * E + g) * E + e] * V;
        if (std::fabs(v) > FLT_EPSILON) row[g] += v;
      }
      for (int f = 0; f < kFaces; f++) {
        const bool xf = (f == 0 || f == 2);
        const double width = xf ? cfg.wy[iy] : cfg.wx[ix];   // face area (2D)
        const double delta = xf ? cfg.wx[ix] : cfg.wy[iy];   // across the cell
        const int n = neighbour(c, f);
        const double flux = phi_old[ce];
        double d = dif[ce];
        if (edc) d *= larsen(d, delta);
        double dh = 0.0, dt = 0.0;
        const double j_out = J[((size_t) c * kFaces + f) * E + e];
        if (n < 0) {
          if (cfg.bc[f] == 0) {   // vacuum
            const double cur_out = j_out / width;
            dh = 2.0 * d / delta / (1.0 + 4.0 * d / delta);
            dt = (dh * flux - cur_out) / flux;
          }
        } else {
          const int nix = n % cfg.nx, niy = n / cfg.nx;
          const double delta_n = xf ? cfg.wx[nix] : cfg.wy[niy];
          const size_t ne = (size_t) n * E + e;
          double dn = dif[ne];
          if (edc) dn *= larsen(dn, delta_n);
          const double flux_n = phi_old[ne];
          const double j_in = J[((size_t) n * kFaces + (f ^ 2)) * E + e];
          dh = 2.0 * d * dn / (delta_n * d + delta * dn);
          const double current = (j_out - j_in) / width;
          dt = -(dh * (flux_n - flux) + current) / (flux_n + flux);
          if (cfg.flux_limiting && moc_iter > 0 && std::fabs(dt / dh) > 1.0) {
            dh = current > 0.0 ? std::fabs(current / (2.0 * flux))
                               : std::fabs(current / (2.0 * flux_n));
            dt = -(dh * (flux_n - flux) + current) / (flux_n + flux);
            dh = std::max(dh, std::fabs(dt));
          }
        }
        double& old = dcorr_old[((size_t) c * kFaces + f) * E + e];
        if (dcorr_valid)
          dt = cfg.relaxation * dt + (1.0 - cfg.relaxation) * old;
        // the first iteration solves the plain diffusion problem
        if (moc_iter == 0) dt = 0.0;
        old = dt;
        row[e] += (dh - dt) * width;
        if (n >= 0) a_nb[((size_t) c * kFaces + f) * E + e] = -(dh + dt) * width;
      }
      double* mrow = m_blk.data() + ce * E;
      for (int g = 0; g < E; g++) {
        const double v = chi_c[ce] * nu_f[(size_t) c * E + g] * V;
        if (std::fabs(v) > FLT_EPSILON) mrow[g] += v;
      }
    }
  }
  dcorr_valid = true;
}

// out = M x
void Solver::fission(const std::vector<double>& x,
                     std::vector<double>& out) const {
  const int C = cfg.cells(), E = cfg.E;
  out.assign((size_t) C * E, 0.0);
  for (int c = 0; c < C; c++)
    for (int e = 0; e < E; e++) {
      const double* mrow = m_blk.data() + ((size_t) c * E + e) * E;
      const double* xc = x.data() + (size_t) c * E;
      double s = 0.0;
      for (int g = 0; g < E; g++) s += mrow[g] * xc[g];
      out[(size_t) c * E + e] = s;
    }
}

namespace {
// computeRMSE(integrated): per cell the relative change of the group sum
double rmse_integrated(const std::vector<double>& x,
                       const std::vector<double>& y, int C, int E) {
  double sum = 0.0;
  for (int c = 0; c < C; c++) {
    double a = 0.0, b = 0.0;
    for (int e = 0; e < E; e++) {
      a += x[(size_t) c * E + e];
      b += y[(size_t) c * E + e];
    }
    if (std::fabs(b) > kFluxEpsilon) sum += ((a - b) / b) * ((a - b) / b);
  }
  return std::sqrt(sum / std::max(C, 1));
}
}  // namespace

// Red-black SOR on A x = b; false when it diverges or does not converge.
bool Solver::linear_solve(std::vector<double>& x, const std::vector<double>& b,
                          double tol) {
  const int C = cfg.cells(), E = cfg.E;
  const double w = cfg.sor;
  tol = std::max(kLinalgTol, tol);
  std::vector<double> old_src, new_src;
  fission(x, old_src);
  double residual = 0.0, initial = 0.0, min_res = 1e6;
  int iter = 0;
  bool ok = true;
  while (iter < kMaxLinearIters) {
    for (int color = 0; color < 2; color++) {
      for (int iy = 0; iy < cfg.ny; iy++) {
        for (int ix = (iy + color) % 2; ix < cfg.nx; ix += 2) {
          const int c = iy * cfg.nx + ix;
          int nb[kFaces];
          for (int f = 0; f < kFaces; f++) nb[f] = neighbour(c, f);
          for (int e = 0; e < E; e++) {
            const size_t r = (size_t) c * E + e;
            const double* row = a_blk.data() + r * E;
            const double diag = row[e];
            double v = (1.0 - w) * x[r] * (diag / w);
            for (int g = 0; g < E; g++)
              if (g != e) v -= row[g] * x[(size_t) c * E + g];
            for (int f = 0; f < kFaces; f++)
              if (nb[f] >= 0)
                v -= a_nb[((size_t) c * kFaces + f) * E + e] *
                     x[(size_t) nb[f] * E + e];
            v += b[r];
            x[r] = v * (w / diag);
          }
        }
      }
    }
    fission(x, new_src);
    if (iter == 0) {
      residual = rmse_integrated(new_src, old_src, C, E);
      initial = residual;
    }
    iter++;
    if (iter > kMinLinearIters) {
      residual = rmse_integrated(new_src, old_src, C, E);
      min_res = std::min(min_res, residual);
      if ((residual > 1e3 * min_res && min_res > 1e-10) ||
          !std::isfinite(residual)) {
        ok = false;
        break;
      }
      if (residual / initial < 0.1 || residual < tol) break;
    }
    if (iter > kMinLinearIters - 1 && iter < kMaxLinearIters) old_src = new_src;
  }
  stats.linear_iterations += iter;
  if (iter == kMaxLinearIters) ok = false;
  return ok;
}

// ddLinearSolve (src/linalg.cpp:717-900): A made diagonally dominant by
// dd = max(0, sum |off-diagonal| - diagonal) on each diagonal, the
// difference moved to the right side (b + dd x), linear solves repeated
// until the fission source settles; A restored on success.
bool Solver::dd_linear_solve(std::vector<double>& x,
                             const std::vector<double>& b, double tol) {
  const int C = cfg.cells(), E = cfg.E;
  std::vector<double> dd((size_t) C * E, 0.0), rhs((size_t) C * E);
  for (int c = 0; c < C; c++)
    for (int e = 0; e < E; e++) {
      const size_t r = (size_t) c * E + e;
      double* row = a_blk.data() + r * E;
      double sum = 0.0;
      for (int g = 0; g < E; g++)
        if (g != e) sum += std::fabs(row[g]);
      for (int f = 0; f < kFaces; f++)
        sum += std::fabs(a_nb[((size_t) c * kFaces + f) * E + e]);
      if (sum > row[e]) dd[r] = sum - row[e];
      row[e] += dd[r];
    }
  std::vector<double> old_src, new_src;
  fission(x, new_src);
  double initial = 0.0, min_res = 1e6;
  for (int it = 0; it < kMaxLinearIters; it++) {
    old_src = new_src;
    for (size_t r = 0; r < rhs.size(); r++) rhs[r] = b[r] + dd[r] * x[r];
    linear_solve(x, rhs, tol);      // a failure is only noted
    fission(x, new_src);
    const double res = rmse_integrated(new_src, old_src, C, E);
    if (it == 0) initial = res < 1e-14 ? 1e-10 : res;
    min_res = std::min(min_res, res);
    if ((res > 1e3 * min_res && min_res > 1e-10) || !std::isfinite(res))
      return false;
    if (res / initial < 0.1 || res < tol) break;
  }
  for (int c = 0; c < C; c++)
    for (int e = 0; e < E; e++)
      a_blk[((size_t) c * E + e) * E + e] -= dd[(size_t) c * E + e];
  return true;
}

// Power iteration; returns keff, or -1 when a linear solve fails.
double Solver::eigen_solve(std::vector<double>& x, double k, double tol) {
  const int C = cfg.cells(), E = cfg.E;
  tol = std::max(kLinalgTol, tol);
  std::vector<double> old_src, new_src;
  fission(x, old_src);
  const double rows = (double) C * E;
  double s = 0.0;
  for (double v : old_src) s += v;
  if (!(s > 0.0) || !std::isfinite(s)) return -1.0;
  for (double& v : old_src) v *= rows / s;
  for (double& v : x) v *= rows * k / s;
  double initial = 0.0;
  int iter;
  bool dd_mode = false;
  for (iter = 0; iter < kMaxPowerIters; iter++) {
    // plain linear solves, diagonally dominated from the first failure on
    bool ok = !dd_mode && linear_solve(x, old_src, tol * 1e-1);
    if (!ok) {
      dd_mode = true;
      ok = dd_linear_solve(x, old_src, tol * 1e-1);
    }
    if (!ok) {
      stats.power_iterations = iter + 1;
      return -1.0;
    }
    fission(x, new_src);
    double ns = 0.0;
    for (double v : new_src) ns += v;
    k = ns / rows;
    for (double& v : new_src) v /= k;
    const double residual = rmse_integrated(new_src, old_src, C, E);
    if (iter == 0) {
      initial = residual;
      if (initial < 1e-14) initial = 1e-10;
    }
    old_src.swap(new_src);
    if ((residual / initial < 0.03 || residual < kLinalgTol) &&
        iter > kMinPowerIters)
      break;
  }
  stats.power_iterations = iter + 1;
  return k;
}

double Solver::step(int moc_iter, const double* S, const float* cur, int ld) {
  const int C = cfg.cells(), E = cfg.E;
  std::vector<double> J;
  collapse(S, cur, ld, J);
  build(moc_iter, J);
  stats.linear_iterations = 0;
  // the collapsed flux is the starting guess
  phi_new = phi_old;
  const double k = eigen_solve(phi_new, keff, source_threshold);
  ratio.assign((size_t) C * E, 1.0);
  stats.max_ratio = 1.0;
  if (!(std::fabs(k + 1.0) > FLT_EPSILON) || !std::isfinite(k)) {
    // no prolongation; the previous coarse eigenvalue stands
    stats.failed = true;
    return keff;
  }
  stats.failed = false;
  keff = k;
  // both fluxes to unit average fission source
  std::vector<double> src;
  fission(phi_new, src);
  double sn = 0.0;
  for (double v : src) sn += v;
  fission(phi_old, src);
  double so = 0.0;
  for (double v : src) so += v;
  for (double& v : phi_new) v /= sn;
  for (double& v : phi_old) v /= so;
  for (size_t i = 0; i < ratio.size(); i++) {
    // bounded to [0.05, 20] by the prolongation, after any k-nearest
    // weighting (Cmfd::updateMOCFlux, src/Cmfd.cpp:1530-1540)
    const double r = std::fabs(phi_old[i]) > kFluxEpsilon
                         ? phi_new[i] / phi_old[i] : 0.0;
    ratio[i] = r;
    if (r > 0.0 && std::fabs(std::log(r)) > std::fabs(std::log(stats.max_ratio)))
      stats.max_ratio = r;
  }
  return keff;
}

void knearest_coefficients(const Config& cfg, int k, double origin_x,
                           double origin_y, const double* centroid,
                           const int32_t* fsr_cell, int64_t R,
                           std::vector<int32_t>& off,
                           std::vector<int32_t>& cell,
                           std::vector<float>& coef) {
  // cell centres from the accumulated widths
  std::vector<double> cx(cfg.nx), cy(cfg.ny);
  double acc = 0.0;
  for (int i = 0; i < cfg.nx; i++) {
    cx[i] = acc + cfg.wx[i] / 2;
    acc += cfg.wx[i];
  }
  acc = 0.0;
  for (int i = 0; i < cfg.ny; i++) {
    cy[i] = acc + cfg.wy[i] / 2;
    acc += cfg.wy[i];
  }
  constexpr double kFar = 1.0e300;   // FLT_INFINITY, src/constants.h:18
  off.assign(R + 1, 0);
  cell.clear();
  coef.clear();
  std::vector<std::pair<int, double>> st;
  for (int64_t r = 0; r < R; r++) {
    const int c = fsr_cell[r], ix = c % cfg.nx, iy = c / cfg.nx;
    const double dx = centroid[2 * r] - origin_x;
    const double dy = centroid[2 * r + 1] - origin_y;
    // distances to the 3 x 3 cells around (stencil 0..8, row by row from
    // y-min; 4 is the FSR's own cell), the missing ones infinitely far
    st.clear();
    for (int j = 0; j < 9; j++) {
      const int sx = ix + j % 3 - 1, sy = iy + j / 3 - 1;
      double d = std::numeric_limits<double>::max();
      if (sx >= 0 && sx < cfg.nx && sy >= 0 && sy < cfg.ny)
        d = std::pow(std::pow(dx - cx[sx], 2.0) + std::pow(dy - cy[sy], 2.0),
                     0.5);
      st.push_back(std::make_pair(j, d));
    }
    std::sort(st.begin(), st.end(),
              [](const std::pair<int, double>& a,
                 const std::pair<int, double>& b) {
                return a.second < b.second;
              });
    st.erase(std::remove_if(st.begin(), st.end(),
                            [&](const std::pair<int, double>& e) {
                              return e.second > kFar;
                            }),
             st.end());
    st.resize(std::min<size_t>((size_t) k, st.size()));
    double total = 1.e-10;
    for (const auto& e : st) total += e.second;
    for (auto& e : st) e.second = 1.0 - e.second / total;
    // Cmfd::getUpdateRatio: the stencil cells other than the FSR's own,
    // then the own cell with the first entry's weight, all over (n - 1);
    // a one-entry stencil adds the own cell's ratio undivided
    const size_t n = st.size();
    const double div = n == 1 ? 1.0 : (double) (n - 1);
    for (const auto& e : st) {
      if (e.first == 4) continue;
      const int j = e.first;
      cell.push_back((iy + j / 3 - 1) * cfg.nx + (ix + j % 3 - 1));
      coef.push_back((float) (e.second / div));
    }
    cell.push_back(c);
    coef.push_back(n == 1 ? 1.0f : (float) (st[0].second / div));
    off[r + 1] = (int32_t) cell.size();
  }
}

}  // namespace moc_cmfd
