// Track laydown and ray tracing for square lattices of pin cells: the
// producer of the benchmark workloads on hosts that do not have OpenMOC.
//
// It restates, for this one geometry family, what OpenMOC's 2D
// TrackGenerator and Geometry produce:
//   - cyclic track laydown with corrected angles and spacings
//     (TrackGenerator::initializeTracks, src/TrackGenerator.cpp:950-1083);
//   - track connections and boundary conditions
//     (TrackGenerator::initializeTrackReflections, :1086-1222);
//   - UIDs in azimuth-major order (initializeTracksArray, :1795-1818);
//   - segments between successive surface crossings
//     (Geometry::segmentize2D, src/Geometry.cpp:2085-2230), with FSR ids in
//     order of first touch over tracks in UID order (the single-thread
//     numbering the reference test harness uses);
//   - pin cells split into equal-area fuel rings (Cell::ringify,
//     src/Cell.cpp:1397-1590) and sectors bounded by planes at
//     pi/4 + i*2*pi/n (Cell::sectorize, src/Cell.cpp:1325-1390);
//   - FSR volumes from segment lengths times the azimuthal weight and
//     spacing (VolumeKernel, src/MOCKernel.cpp:86-170);
//   - azimuthal weights and the Tabuchi-Yamamoto polar quadrature
//     (Quadrature::precomputeWeights, src/Quadrature.cpp:674-745;
//     TYPolarQuad, :797-895).
// Segments are found analytically (circle, sector-line and lattice-line
// crossings sorted along the ray, each sub-interval classified at its
// midpoint), not by nudging a point across surfaces.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <string>
#include <unordered_map>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "lattice_internal.h"

namespace moc_lat {
namespace {
thread_local std::string g_lat_error;
}  // namespace

int lat_fail(const std::string& m) {
  g_lat_error = m;
  return -1;
}



namespace {


// Region of a point relative to its pin-cell centre: ring index (0 =
// outermost fuel ring, fuel_rings-1 = innermost; fuel_rings = moderator)
// and sector index.
struct Classifier {
  int rings;
  int fuel_sectors, mod_sectors;
  std::vector<double> r2;   // squared ring radii, outer to inner

  int sector_of(double ang, int n) const {
    // sector boundaries at k*2pi/n - pi/4 (Cell::sectorize planes at
    // pi/4 + k*2pi/n, sector k between planes k and k+1)
    if (n <= 1) return 0;
    const double d = 2.0 * kPi / n;
    double x = ang + kPi / 4.0;
    x = std::fmod(x, 2.0 * kPi);
    if (x < 0) x += 2.0 * kPi;
    int s = (int) std::floor(x / d);
    if (s >= n) s = n - 1;
    return s;
  }
  // returns (ring, sector) packed
  uint32_t classify(double dx, double dy) const {
    const double rr = dx * dx + dy * dy;
    int ring = rings;  // moderator
    if (rr < r2[0]) {
      ring = 0;
      for (int k = 1; k < rings; k++)
        if (rr < r2[k]) ring = k;
    }
    const double ang = std::atan2(dy, dx);
    const int sec = sector_of(ang, ring < rings ? fuel_sectors : mod_sectors);
    return (uint32_t) ring << 16 | (uint32_t) sec;
  }
};

void add_sector_lines(std::vector<double>& dirs, int n) {
  if (n <= 1) return;
  const double d = 2.0 * kPi / n;
  for (int k = 0; k < n; k++) dirs.push_back(k * d - kPi / 4.0);
}

}  // namespace

int lat_validate(const moc_lattice_spec& s) {
  if (s.nx < 1 || s.ny < 1 || !(s.pitch > 0) || !(s.pin_radius > 0) ||
      s.pin_radius >= 0.5 * s.pitch)
    return lat_fail("bad lattice or pin dimensions");
  if (s.num_azim < 4 || s.num_azim % 4)
    return lat_fail("num_azim must be a positive multiple of 4");
  if (!(s.spacing > 0)) return lat_fail("spacing must be positive");
  if (s.num_polar != 2 && s.num_polar != 4 && s.num_polar != 6)
    return lat_fail("num_polar must be 2, 4 or 6 (Tabuchi-Yamamoto)");
  if (s.fuel_rings < 1 || s.fuel_sectors < 0 || s.mod_sectors < 0)
    return lat_fail("bad ring / sector counts");
  if (!s.pin_material) return lat_fail("pin_material is required");
  for (int b = 0; b < 4; b++)
    if (s.bc[b] != 0 && s.bc[b] != 1)
      return lat_fail("boundary conditions are 0 (vacuum) or 1 (reflective)");
  return 0;
}

void lat_laydown(const moc_lattice_spec& s, moc_lattice* L, LatGeo& X) {
  const int A = s.num_azim;
  const double W = s.nx * s.pitch, H = s.ny * s.pitch;
  const double xmin = -0.5 * W, ymin = -0.5 * H;

  // ---- angles, spacings, counts (TrackGenerator::initializeTracks) ----
  std::vector<int> num_x(A / 2), num_y(A / 2);
  std::vector<double> phis(A / 2), dx_eff(A / 2), dy_eff(A / 2), spac(A / 2);
  for (int a = 0; a < A / 4; a++) {
    const double phi_d = 2.0 * kPi / A * (0.5 + a);
    num_x[a] = (int) (std::fabs(W / s.spacing * std::sin(phi_d))) + 1;
    num_y[a] = (int) (std::fabs(H / s.spacing * std::cos(phi_d))) + 1;
    num_x[A / 2 - a - 1] = num_x[a];
    num_y[A / 2 - a - 1] = num_y[a];
    const double phi = std::atan((H * num_x[a]) / (W * num_y[a]));
    phis[a] = phi;
    phis[A / 2 - a - 1] = kPi - phi;
    dx_eff[a] = dx_eff[A / 2 - a - 1] = W / num_x[a];
    dy_eff[a] = dy_eff[A / 2 - a - 1] = H / num_y[a];
    spac[a] = spac[A / 2 - a - 1] = dx_eff[a] * std::sin(phi);
  }
  // azimuthal weights (Quadrature::precomputeWeights)
  std::vector<double> wa(A / 2);
  for (int a = 0; a < A / 4; a++) {
    double x1 = (a < A / 4 - 1) ? 0.5 * (phis[a + 1] - phis[a])
                                : 0.5 * kPi - phis[a];
    double x2 = (a >= 1) ? 0.5 * (phis[a] - phis[a - 1]) : phis[a];
    wa[a] = wa[A / 2 - a - 1] = (x1 + x2) / kPi;
  }
  // Tabuchi-Yamamoto polar sets: sin(theta) and weight per half space
  std::vector<double> sin_t, w_p;
  if (s.num_polar == 2) {
    sin_t = {0.798184};
    w_p = {0.5};
  } else if (s.num_polar == 4) {
    sin_t = {0.363900, 0.899900};
    w_p = {0.212854 / 2.0, 0.787146 / 2.0};
  } else {
    sin_t = {0.166648, 0.537707, 0.932954};
    w_p = {0.046233 / 2.0, 0.283619 / 2.0, 0.670148 / 2.0};
  }
  const int Ph = s.num_polar / 2;
  L->A = A / 2;
  L->Ph = Ph;
  L->weights.resize((size_t) (A / 2) * Ph);
  L->inv_sin.resize((size_t) (A / 2) * Ph);
  for (int a = 0; a < A / 2; a++)
    for (int p = 0; p < Ph; p++) {
      const double st = std::sin(std::asin(sin_t[p]));
      const double w = 2.0 * kPi * wa[a] * spac[a] * w_p[p] * 2.0 * st;
      L->weights[a * Ph + p] = (float) w;
      L->inv_sin[a * Ph + p] = (float) (1.f / st);
    }

  // ---- tracks ----
  std::vector<int64_t> first(A / 2 + 1, 0);
  for (int a = 0; a < A / 2; a++) first[a + 1] = first[a] + num_x[a] + num_y[a];
  const int64_t T = first[A / 2];
  L->T = T;
  std::vector<Track> tracks(T);
  for (int a = 0; a < A / 2; a++) {
    const int nx = num_x[a], ny = num_y[a];
    const double dx = dx_eff[a], dy = dy_eff[a];
    for (int i = 0; i < nx + ny; i++) {
      Track& t = tracks[first[a] + i];
      t.a = a;
      t.phi = phis[a];
      if (a < A / 4) {
        if (i < nx) { t.x0 = xmin + W - dx * (i + 0.5); t.y0 = ymin; }
        else { t.x0 = xmin; t.y0 = ymin + dy * (i - nx + 0.5); }
        if (i < ny) { t.x1 = xmin + W; t.y1 = ymin + dy * (i + 0.5); }
        else { t.x1 = xmin + W - dx * ((i - ny) + 0.5); t.y1 = ymin + H; }
      } else {
        if (i < nx) { t.x0 = xmin + dx * (i + 0.5); t.y0 = ymin; }
        else { t.x0 = xmin + W; t.y0 = ymin + dy * (i - nx + 0.5); }
        if (i < ny) { t.x1 = xmin; t.y1 = ymin + dy * (i + 0.5); }
        else { t.x1 = xmin + dx * (i - ny + 0.5); t.y1 = ymin + H; }
      }
    }
  }
  // ---- connections (TrackGenerator::initializeTrackReflections) ----
  L->next.assign(2 * T, 0);
  L->flags.assign(T, 0);
  L->track_ang.assign(T, 0);
  const int BXMIN = s.bc[0], BXMAX = s.bc[1], BYMIN = s.bc[2], BYMAX = s.bc[3];
  for (int a = 0; a < A / 2; a++) {
    const int ac = A / 2 - a - 1;
    const int nx = num_x[a], ny = num_y[a];
    for (int i = 0; i < nx + ny; i++) {
      const int64_t id = first[a] + i;
      int bc_fwd, bc_bwd;
      if (a < A / 4) {
        bc_fwd = (i < ny) ? BXMAX : BYMAX;
        bc_bwd = (i < nx) ? BYMIN : BXMIN;
      } else {
        bc_fwd = (i < ny) ? BXMIN : BYMAX;
        bc_bwd = (i < nx) ? BYMIN : BXMAX;
      }
      bool fwd_fwd, bwd_fwd;
      int64_t nf, nb;
      if (i < ny) {
        fwd_fwd = true;
        nf = first[ac] + i + nx;
      } else {
        fwd_fwd = false;
        nf = first[ac] + (nx + ny) - (i - ny) - 1;
      }
      if (i < nx) {
        nb = first[ac] + nx - i - 1;
        bwd_fwd = true;
      } else {
        bwd_fwd = false;
        nb = first[ac] + i - nx;
      }
      L->next[2 * id] = nf;
      L->next[2 * id + 1] = nb;
      uint8_t f = 0;
      if (fwd_fwd) f |= 1;
      if (bwd_fwd) f |= 2;
      if (bc_fwd == 1) f |= 4;
      if (bc_bwd == 1) f |= 8;
      L->flags[id] = f;
      L->track_ang[id] = a;
    }
  }
  X.A = A / 2;
  X.Ph = Ph;
  X.T = T;
  X.W = W;
  X.H = H;
  X.xmin = xmin;
  X.ymin = ymin;
  X.tracks = tracks;
  X.spac = spac;
  X.wa = wa;
  X.sin_t = sin_t;
  X.w_p = w_p;
}

void lat_cells(const moc_lattice_spec& s, LatCells& c) {
  c.rings = s.fuel_rings;
  c.fuel_sectors = s.fuel_sectors;
  c.mod_sectors = s.mod_sectors;
  for (int k = 0; k < s.fuel_rings; k++) {
    // equal-area rings: r_k = r * sqrt(1 - k/n)
    const double r = s.pin_radius * std::sqrt(1.0 - (double) k / s.fuel_rings);
    c.r2.push_back(r * r);
  }
  for (double v : c.r2) c.radii.push_back(std::sqrt(v));
  add_sector_lines(c.line_dirs, s.fuel_sectors);
  add_sector_lines(c.line_dirs, s.mod_sectors);
  std::sort(c.line_dirs.begin(), c.line_dirs.end());
}

void lat_finish(const moc_lattice_spec& s, moc_lattice* L, const LatGeo& X,
                const std::vector<uint64_t>& keys, bool volumes) {
  const std::vector<Track>& tracks = X.tracks;
  const std::vector<double>& spac = X.spac;
  const std::vector<double>& wa = X.wa;
  const std::vector<double>& sin_t = X.sin_t;
  const std::vector<double>& w_p = X.w_p;
  const int Ph = X.Ph;
  const int64_t T = X.T;
  const int64_t R = (int64_t) keys.size();
  L->R = R;
  L->fsr_mat.resize(R);
  if (volumes) L->fsr_vol.assign(R, 0.0f);
  int32_t maxmat = s.moderator_material;
  for (int64_t r = 0; r < R; r++) {
    const uint64_t key = keys[r];
    const int64_t cell = (int64_t) (key >> 32);
    const int ring = (int) ((key >> 16) & 0xFFFF);
    const int m = (ring < s.fuel_rings) ? s.pin_material[cell]
                                        : s.moderator_material;
    L->fsr_mat[r] = m;
    maxmat = std::max(maxmat, m);
  }
  L->M = maxmat + 1;
  // volumes: sum of segment lengths times azimuthal weight x spacing
  if (volumes) {
    std::vector<double> vol(R, 0.0);
    for (int64_t t = 0; t < T; t++) {
      const double w = spac[tracks[t].a] * wa[tracks[t].a];
      for (int64_t k = L->seg_off[t]; k < L->seg_off[t + 1]; k++)
        vol[L->seg_fsr[k]] += w * (double) L->seg_len[k];
    }
    for (int64_t r = 0; r < R; r++) L->fsr_vol[r] = (float) vol[r];
  }
  L->az_spacing.assign(spac.begin(), spac.end());
  L->az_weight.assign(wa.begin(), wa.end());
  L->tracks = tracks;
  for (int p = 0; p < Ph; p++) {
    L->pol_sin.push_back(std::sin(std::asin(sin_t[p])));
    L->pol_wgt.push_back(w_p[p]);
  }
  L->moderator = s.moderator_material;
  L->fsr_pin.resize(R);
  for (int64_t r = 0; r < R; r++) L->fsr_pin[r] = (int32_t) (keys[r] >> 32);
  L->nx = s.nx;
  L->ny = s.ny;
  L->pitch = s.pitch;
  L->xmin = X.xmin;
  L->ymin = X.ymin;
}

}  // namespace moc_lat

using namespace moc_lat;

extern "C" const char* moc_lattice_last_error(void) {
  return g_lat_error.c_str();
}

extern "C" int moc_lattice_generate(const moc_lattice_spec* sp,
                                    moc_lattice** out) {
  if (!sp || !out) return lat_fail("null argument");
  *out = nullptr;
  const moc_lattice_spec& s = *sp;
  if (lat_validate(s)) return -1;
  moc_lattice* L = new moc_lattice();
  LatGeo X;
  lat_laydown(s, L, X);
  const std::vector<Track>& tracks = X.tracks;
  const double xmin = X.xmin, ymin = X.ymin;
  const int64_t T = X.T;
  LatCells cells;
  lat_cells(s, cells);
  Classifier cls;
  cls.rings = cells.rings;
  cls.fuel_sectors = cells.fuel_sectors;
  cls.mod_sectors = cells.mod_sectors;
  cls.r2 = cells.r2;
  const std::vector<double>& radii = cells.radii;
  const std::vector<double>& line_dirs = cells.line_dirs;

  std::vector<std::vector<float>> seg_len_t(T);
  std::vector<std::vector<uint64_t>> seg_key_t(T);
#ifdef _OPENMP
  if (s.num_threads > 0) omp_set_num_threads(s.num_threads);
#pragma omp parallel for schedule(dynamic, 16)
#endif
  for (int64_t t = 0; t < T; t++) {
    const Track& tr = tracks[t];
    const double ux = std::cos(tr.phi), uy = std::sin(tr.phi);
    const double len =
        std::sqrt((tr.x1 - tr.x0) * (tr.x1 - tr.x0) + (tr.y1 - tr.y0) * (tr.y1 - tr.y0));
    std::vector<double> cuts;
    cuts.push_back(0.0);
    // lattice lines
    for (int k = 1; k < s.nx; k++) {
      if (std::fabs(ux) < 1e-300) break;
      const double tt = (xmin + k * s.pitch - tr.x0) / ux;
      if (tt > 0 && tt < len) cuts.push_back(tt);
    }
    for (int k = 1; k < s.ny; k++) {
      if (std::fabs(uy) < 1e-300) break;
      const double tt = (ymin + k * s.pitch - tr.y0) / uy;
      if (tt > 0 && tt < len) cuts.push_back(tt);
    }
    cuts.push_back(len);
    std::sort(cuts.begin(), cuts.end());
    std::vector<double> pts;
    std::vector<float>& out_len = seg_len_t[t];
    std::vector<uint64_t>& out_key = seg_key_t[t];
    for (size_t c = 0; c + 1 < cuts.size(); c++) {
      const double ta = cuts[c], tb = cuts[c + 1];
      if (tb - ta <= 0) continue;
      const double tm = 0.5 * (ta + tb);
      const double mx = tr.x0 + tm * ux, my = tr.y0 + tm * uy;
      int ci = (int) std::floor((mx - xmin) / s.pitch);
      int cj = (int) std::floor((my - ymin) / s.pitch);
      ci = std::min(std::max(ci, 0), s.nx - 1);
      cj = std::min(std::max(cj, 0), s.ny - 1);
      const double cx = xmin + (ci + 0.5) * s.pitch;
      const double cy = ymin + (cj + 0.5) * s.pitch;
      pts.clear();
      pts.push_back(ta);
      const double px = tr.x0 - cx, py = tr.y0 - cy;
      const double b = px * ux + py * uy;
      const double pp = px * px + py * py;
      for (double r : radii) {
        const double disc = b * b - (pp - r * r);
        if (disc <= 0) continue;
        const double sq = std::sqrt(disc);
        const double t1 = -b - sq, t2 = -b + sq;
        if (t1 > ta && t1 < tb) pts.push_back(t1);
        if (t2 > ta && t2 < tb) pts.push_back(t2);
      }
      for (double beta : line_dirs) {
        const double vx = std::cos(beta), vy = std::sin(beta);
        const double den = ux * vy - uy * vx;
        if (std::fabs(den) < 1e-14) continue;
        // P0 + t u = c + s v  ->  t = ((c - P0) x v) / (u x v)
        const double qx = cx - tr.x0, qy = cy - tr.y0;
        const double tt = (qx * vy - qy * vx) / den;
        const double ss = (qx * uy - qy * ux) / den;
        // ss >= 0: a ray through the pin centre is cut there, where every
        // sector plane meets
        if (ss > -1e-12 && tt > ta && tt < tb) pts.push_back(tt);
      }
      pts.push_back(tb);
      std::sort(pts.begin(), pts.end());
      const uint64_t cell = (uint64_t) ((int64_t) (s.ny - 1 - cj) * s.nx + ci);
      for (size_t k = 0; k + 1 < pts.size(); k++) {
        const double l = pts[k + 1] - pts[k];
        // sub-intervals below the reference's surface nudge do not form
        // segments of their own
        if (l <= kTinyMove) continue;
        const double mm = 0.5 * (pts[k] + pts[k + 1]);
        const uint32_t rs =
            cls.classify(tr.x0 + mm * ux - cx, tr.y0 + mm * uy - cy);
        const uint64_t key = cell << 32 | rs;
        if (!out_key.empty() && out_key.back() == key) {
          out_len.back() = (float) ((double) out_len.back() + l);
        } else {
          out_key.push_back(key);
          out_len.push_back((float) l);
        }
      }
    }
  }
  // ---- FSR ids by first touch, UID order ----
  std::unordered_map<uint64_t, int32_t> ids;
  ids.reserve((size_t) s.nx * s.ny * 64);
  std::vector<uint64_t> keys;
  L->seg_off.assign(T + 1, 0);
  for (int64_t t = 0; t < T; t++)
    L->seg_off[t + 1] = L->seg_off[t] + (int64_t) seg_len_t[t].size();
  const int64_t S = L->seg_off[T];
  L->S = S;
  L->seg_len.resize(S);
  L->seg_fsr.resize(S);
  for (int64_t t = 0; t < T; t++) {
    const int64_t base = L->seg_off[t];
    for (size_t k = 0; k < seg_len_t[t].size(); k++) {
      const uint64_t key = seg_key_t[t][k];
      auto it = ids.find(key);
      int32_t id;
      if (it == ids.end()) {
        id = (int32_t) keys.size();
        ids.emplace(key, id);
        keys.push_back(key);
      } else {
        id = it->second;
      }
      L->seg_fsr[base + k] = id;
      L->seg_len[base + k] = seg_len_t[t][k];
    }
    std::vector<float>().swap(seg_len_t[t]);
    std::vector<uint64_t>().swap(seg_key_t[t]);
  }
  lat_finish(s, L, X, keys, true);
  *out = L;
  return 0;
}

extern "C" int moc_lattice_sizes(moc_lattice* L, int64_t* R, int64_t* T,
                                 int64_t* S, int32_t* A, int32_t* Ph,
                                 int32_t* M) {
  if (!L) return lat_fail("null lattice");
  *R = L->R;
  *T = L->T;
  *S = L->S;
  *A = L->A;
  *Ph = L->Ph;
  *M = L->M;
  return 0;
}

extern "C" int moc_lattice_export(moc_lattice* L, float* seg_len,
                                  int32_t* seg_fsr, int64_t* seg_off,
                                  int32_t* track_ang, int64_t* next,
                                  uint8_t* flags, float* weights,
                                  float* inv_sin, int32_t* fsr_mat,
                                  float* fsr_vol) {
  if (!L) return lat_fail("null lattice");
  std::memcpy(seg_len, L->seg_len.data(), 4 * L->S);
  std::memcpy(seg_fsr, L->seg_fsr.data(), 4 * L->S);
  std::memcpy(seg_off, L->seg_off.data(), 8 * (L->T + 1));
  std::memcpy(track_ang, L->track_ang.data(), 4 * L->T);
  std::memcpy(next, L->next.data(), 8 * 2 * L->T);
  std::memcpy(flags, L->flags.data(), L->T);
  std::memcpy(weights, L->weights.data(), 4 * L->weights.size());
  std::memcpy(inv_sin, L->inv_sin.data(), 4 * L->inv_sin.size());
  std::memcpy(fsr_mat, L->fsr_mat.data(), 4 * L->R);
  std::memcpy(fsr_vol, L->fsr_vol.data(), 4 * L->R);
  return 0;
}

// Linear-source geometry of a 2D lattice: FSR centroids by
// CentroidGenerator's formula (length- and azimuthal-weight-averaged segment
// midpoints, src/TrackTraversingAlgorithms.cpp:377-460) and each segment's
// start relative to its FSR's centroid (RecenterSegments, :1320-1331), with
// starts walked along the track from its first point as the reference
// walks them; per angle row cos / sin phi and spacing x azimuthal weight;
// the polar set repeated per angle row.
extern "C" int moc_lattice_export_ls(moc_lattice* L, float* seg_x,
                                     float* seg_y, double* centroid,
                                     double* ang_dir, double* ang_wgt,
                                     double* pol_sin, double* pol_wgt) {
  if (!L) return lat_fail("null lattice");
  if (L->tracks.empty() || (int64_t) L->tracks.size() != L->T)
    return lat_fail("the linear-source geometry needs a 2D lattice");
  if (!seg_x || !seg_y || !centroid || !ang_dir || !ang_wgt || !pol_sin ||
      !pol_wgt)
    return lat_fail("null output array");
  const int64_t T = L->T, R = L->R;
  std::vector<double> cx(R, 0.0), cy(R, 0.0);
  for (int pass = 0; pass < 2; pass++) {
    for (int64_t t = 0; t < T; t++) {
      const Track& tr = L->tracks[t];
      const double c = std::cos(tr.phi), sn = std::sin(tr.phi);
      const double w = L->az_spacing[tr.a] * L->az_weight[tr.a];
      double x = tr.x0, y = tr.y0;
      for (int64_t k = L->seg_off[t]; k < L->seg_off[t + 1]; k++) {
        const int32_t r = L->seg_fsr[k];
        const double l = (double) L->seg_len[k];
        if (pass == 0) {
          const double v = (double) L->fsr_vol[r];
          cx[r] += w * (x + 0.5 * c * l) * l / v;
          cy[r] += w * (y + 0.5 * sn * l) * l / v;
        } else {
          seg_x[k] = (float) (x - cx[r]);
          seg_y[k] = (float) (y - cy[r]);
        }
        x += c * l;
        y += sn * l;
      }
    }
  }
  for (int64_t r = 0; r < R; r++) {
    centroid[2 * r] = cx[r];
    centroid[2 * r + 1] = cy[r];
  }
  for (int a = 0; a < L->A; a++) {
    ang_dir[2 * a] = ang_dir[2 * a + 1] = 0.0;
    ang_wgt[a] = L->az_spacing[a] * L->az_weight[a];
    for (int p = 0; p < L->Ph; p++) {
      pol_sin[a * L->Ph + p] = L->pol_sin[p];
      pol_wgt[a * L->Ph + p] = L->pol_wgt[p];
    }
  }
  for (int64_t t = 0; t < T; t++) {
    const Track& tr = L->tracks[t];
    ang_dir[2 * tr.a] = std::cos(tr.phi);
    ang_dir[2 * tr.a + 1] = std::sin(tr.phi);
  }
  return 0;
}

extern "C" int moc_lattice_otf_sizes(moc_lattice* L, int64_t* num_radial_tracks,
                                     int64_t* num_radial_segments,
                                     int32_t* above_fsr) {
  if (!L || L->rad_off.empty())
    return lat_fail("not an extruded 3D lattice");
  *num_radial_tracks = (int64_t) L->rad_total.size();
  *num_radial_segments = (int64_t) L->rad_len.size();
  *above_fsr = L->above_fsr;
  return 0;
}

extern "C" int moc_lattice_export_otf(moc_lattice* L, int32_t* trk,
                                      float* trk_f, float* ang,
                                      float* rad_len, int32_t* rad_fsr,
                                      int64_t* rad_off, float* rad_start,
                                      float* rad_total) {
  if (!L || L->rad_off.empty())
    return lat_fail("not an extruded 3D lattice");
  std::memcpy(trk, L->otf_trk.data(), 4 * L->otf_trk.size());
  std::memcpy(trk_f, L->otf_trk_f.data(), 4 * L->otf_trk_f.size());
  std::memcpy(ang, L->otf_ang.data(), 4 * L->otf_ang.size());
  std::memcpy(rad_len, L->rad_len.data(), 4 * L->rad_len.size());
  std::memcpy(rad_fsr, L->rad_fsr.data(), 4 * L->rad_fsr.size());
  std::memcpy(rad_off, L->rad_off.data(), 8 * L->rad_off.size());
  std::memcpy(rad_start, L->rad_start.data(), 4 * L->rad_start.size());
  std::memcpy(rad_total, L->rad_total.data(), 4 * L->rad_total.size());
  return 0;
}

extern "C" int moc_lattice_destroy(moc_lattice* L) {
  delete L;
  return 0;
}

// ---- seeded synthetic cross sections (openmoc_gb300/csrc/synthetic_xs.h) --
#include "synthetic_xs.h"

extern "C" int moc_synthetic_xs(uint64_t seed, int32_t num_groups,
                                int32_t fissile, uint64_t perturb_seed,
                                double perturb_sigma, double* sigma_t,
                                double* sigma_s, double* nu_sigma_f,
                                double* sigma_f, double* chi) {
  if (num_groups < 1 || !sigma_t || !sigma_s || !nu_sigma_f || !sigma_f || !chi)
    return lat_fail("bad synthetic cross-section request");
  openmoc_gb300::MaterialXS m =
      openmoc_gb300::make_synthetic_xs(seed, num_groups, fissile != 0);
  if (perturb_sigma > 0.0)
    m = openmoc_gb300::perturb_xs(m, perturb_seed, perturb_sigma);
  const int G = num_groups;
  std::memcpy(sigma_t, m.sigma_t.data(), 8 * G);
  std::memcpy(sigma_s, m.sigma_s.data(), 8 * (size_t) G * G);
  std::memcpy(nu_sigma_f, m.nu_sigma_f.data(), 8 * G);
  std::memcpy(sigma_f, m.sigma_f.data(), 8 * G);
  std::memcpy(chi, m.chi.data(), 8 * G);
  return 0;
}

// ---- axial extrusion into explicit 3D tracks ------------------------------
// A lattice of height `height`, its pins for z < fuel_height and one
// homogeneous moderator region above, reflective radially and vacuum at the
// bottom and top: the shape of an axially extruded 3D benchmark with explicit
// 3D segments (OpenMOC's TrackGenerator3D with EXPLICIT_3D,
// src/TrackGenerator3D.cpp).  This is not OpenMOC's 3D laydown: it is a
// laydown of its own on the same radial tracks, built so that every 3D link
// is exact.
//   - Radial tracks with reflective ends form closed cycles of directed 2D
//     tracks; each cycle is unrolled into one periodic line coordinate s.
//   - For each polar angle of a Gauss-Legendre set (mu = cos theta, half the
//     angles upward), lines z = z0 + s cot(theta) start at the bottom (or
//     top) at s_j = (j + 1/2) ds, with ds = L_cycle / n and
//     n = round(L_cycle |cot theta| / dz): equally spaced along the cycle,
//     vertical spacing dz' = ds |cot theta| close to dz.
//   - A line is cut where it passes from one radial track to the next; each
//     piece is a 3D track whose forward neighbour is the next piece (entered
//     forward) and backward neighbour the previous one; the first and last
//     pieces end on the vacuum bottom / top.
//   - Segments: the radial segments under the piece, cut at z = fuel_height;
//     above it the single moderator region (id R2); length = radial length /
//     sin(theta).
//   - Weights: one row per (cycle, polar angle): 2 pi w_a w_p d_a dz' sin(theta),
//     w_a and d_a the azimuthal weight and spacing of the cycle's tracks, w_p
//     the polar weight normalised to 1 over all polar angles (each 3D track is
//     swept in both directions); FSR volumes are sum(w / 2 pi * length), as
//     the radial laydown's volumes are sum(w_a d_a length).
extern "C" int moc_lattice_extrude(const moc_lattice* L2, double height,
                                   double fuel_height, double z_spacing,
                                   int32_t num_polar, int32_t num_threads,
                                   moc_lattice** out) {
  if (!L2 || !out) return lat_fail("null argument");
  *out = nullptr;
  if (!(height > 0) || !(fuel_height > 0) || fuel_height > height ||
      !(z_spacing > 0))
    return lat_fail("bad axial dimensions");
  if (num_polar != 2 && num_polar != 4 && num_polar != 6)
    return lat_fail("num_polar must be 2, 4 or 6 (Gauss-Legendre)");
  const int64_t T2 = L2->T;
  for (int64_t t = 0; t < T2; t++)
    if ((L2->flags[t] & 12) != 12)
      return lat_fail("the extrusion needs reflective radial boundaries");
  if (L2->az_spacing.empty()) return lat_fail("radial lattice has no spacings");

  // Gauss-Legendre nodes and weights on [-1, 1] (sum of weights 2)
  static const double gl_mu[3][3] = {{0.5773502691896258, 0, 0},
                                     {0.3399810435848563, 0.8611363115940526, 0},
                                     {0.2386191860831969, 0.6612093864662645,
                                      0.9324695142031521}};
  static const double gl_w[3][3] = {{1.0, 0, 0},
                                    {0.6521451548625461, 0.3478548451374538, 0},
                                    {0.4679139345726910, 0.3607615730481386,
                                     0.1713244923791704}};
  const int P = num_polar, half = P / 2, row = half - 1;
  std::vector<double> mu(P), wp(P);
  for (int k = 0; k < half; k++) {
    mu[half - 1 - k] = -gl_mu[row][k];   // downward, steepest last
    mu[half + k] = gl_mu[row][k];
    wp[half - 1 - k] = wp[half + k] = 0.5 * gl_w[row][k];
  }

  // radial segment boundaries per track
  std::vector<int64_t> off(L2->seg_off.begin(), L2->seg_off.end());
  std::vector<double> cum((size_t) L2->S + T2);
  std::vector<double> len2(T2);
  for (int64_t t = 0; t < T2; t++) {
    double c = 0;
    cum[off[t] + t] = 0;
    for (int64_t k = off[t]; k < off[t + 1]; k++) {
      c += (double) L2->seg_len[k];
      cum[k + 1 + t] = c;
    }
    len2[t] = c;
  }
  // cum of track t: cum[off[t] + t + i], i = 0..n_t

  // cycles of directed tracks (t, d); the reverse cycle is left out
  struct Cycle {
    std::vector<int64_t> tr;
    std::vector<int> dir;
    std::vector<double> s0;
    double len = 0;
  };
  std::vector<Cycle> cycles;
  std::vector<uint8_t> seen(2 * T2, 0);
  for (int64_t t0 = 0; t0 < T2; t0++)
    for (int d0 = 0; d0 < 2; d0++) {
      if (seen[2 * t0 + d0]) continue;
      Cycle c;
      int64_t t = t0;
      int d = d0;
      for (int64_t guard = 0;; guard++) {
        if (guard > 2 * T2) return lat_fail("radial track links do not close");
        c.tr.push_back(t);
        c.dir.push_back(d);
        c.s0.push_back(c.len);
        c.len += len2[t];
        seen[2 * t + d] = 1;
        seen[2 * t + (1 - d)] = 1;
        const int64_t nt = L2->next[2 * t + d];
        const bool fwd = (L2->flags[t] & (d ? 2 : 1)) != 0;
        t = nt;
        d = fwd ? 0 : 1;
        if (t == t0 && d == d0) break;
      }
      cycles.push_back(std::move(c));
    }
  const int64_t R2 = L2->R;
  const int64_t nitems = (int64_t) cycles.size() * P;

  // one work item per (cycle, polar angle): its tracks and segments
  struct Item {
    std::vector<float> seg_len;
    std::vector<int32_t> seg_fsr;
    std::vector<int32_t> nseg;
    std::vector<uint8_t> first, last;   // first / last piece of its line
    std::vector<int32_t> otf;           // per 3D track: t, first, count, rev
    std::vector<float> otf_f;           // per 3D track: a0, span, w0, 0
    double weight = 0;
    float cot = 0, sin_t = 0;
  };
  std::vector<Item> items(nitems);
#ifdef _OPENMP
  if (num_threads > 0) omp_set_num_threads(num_threads);
#pragma omp parallel for schedule(dynamic, 1)
#endif
  for (int64_t it = 0; it < nitems; it++) {
    const Cycle& c = cycles[it / P];
    const int p = (int) (it % P);
    Item& out_item = items[it];
    const double sin_t = std::sqrt(1.0 - mu[p] * mu[p]);
    const double cot = mu[p] / sin_t;          // dz / ds, signed
    const double run = height / std::fabs(cot);
    const int64_t n = std::max<int64_t>(
        1, (int64_t) std::llround(c.len * std::fabs(cot) / z_spacing));
    const double ds = c.len / (double) n;
    const double dz_eff = ds * std::fabs(cot);
    const int a = L2->track_ang[c.tr[0]];
    out_item.weight = 2.0 * kPi * L2->az_weight[a] * wp[p] *
                      L2->az_spacing[a] * dz_eff * sin_t;
    out_item.cot = (float) cot;
    out_item.sin_t = (float) sin_t;
    const size_t ncyc = c.tr.size();
    for (int64_t j = 0; j < n; j++) {
      double s = (j + 0.5) * ds;
      double z = (cot > 0) ? 0.0 : height;
      double remaining = run;
      size_t k = (size_t) (std::upper_bound(c.s0.begin(), c.s0.end(), s) -
                           c.s0.begin()) - 1;
      bool first_piece = true;
      while (remaining > 1e-12) {
        const int64_t t = c.tr[k];
        const int d = c.dir[k];
        const double L = len2[t];
        const double a0 = std::max(0.0, s - c.s0[k]);
        const double take = std::min(L - a0, remaining);
        const double a1 = a0 + take;
        // radial segments under [a0, a1] in traversal order, cut at the
        // top of the fuel
        const double* cb = cum.data() + off[t] + t;
        const int64_t nsg = off[t + 1] - off[t];
        const size_t seg_start = out_item.seg_len.size();
        int32_t last_fsr = -1;
        auto emit = [&](int32_t fsr, double l3) {
          if (l3 <= 1e-10) return;
          if (fsr == last_fsr && out_item.seg_len.size() > seg_start) {
            out_item.seg_len.back() = (float) ((double) out_item.seg_len.back() + l3);
          } else {
            out_item.seg_fsr.push_back(fsr);
            out_item.seg_len.push_back((float) l3);
            last_fsr = fsr;
          }
        };
        auto piece = [&](int32_t fsr2, double u0, double u1) {
          // traversal interval [u0, u1] of one radial segment
          const double z0 = z + (u0 - a0) * cot, z1 = z + (u1 - a0) * cot;
          const double lo = std::min(z0, z1), hi = std::max(z0, z1);
          if (hi <= fuel_height) {
            emit(fsr2, (u1 - u0) / sin_t);
          } else if (lo >= fuel_height) {
            emit((int32_t) R2, (u1 - u0) / sin_t);
          } else {
            const double uc = u0 + (fuel_height - z0) / cot;
            const bool below_first = z0 < fuel_height;
            emit(below_first ? fsr2 : (int32_t) R2, (uc - u0) / sin_t);
            emit(below_first ? (int32_t) R2 : fsr2, (u1 - uc) / sin_t);
          }
        };
        // the radial segments crossed, for the on-the-fly description
        int64_t i_first = 0, n_crossed = 0;
        if (d == 0) {
          int64_t i = (int64_t) (std::upper_bound(cb, cb + nsg + 1, a0) - cb) - 1;
          i_first = i;
          for (; i < nsg && cb[i] < a1; i++) {
            const double u0 = std::max(a0, cb[i]), u1 = std::min(a1, cb[i + 1]);
            if (u1 > u0) piece(L2->seg_fsr[off[t] + i], u0, u1);
            n_crossed++;
          }
        } else {
          // natural coordinate x = L - u
          const double x0 = L - a1, x1 = L - a0;
          int64_t i = (int64_t) (std::upper_bound(cb, cb + nsg + 1, x1) - cb) - 1;
          if (i >= nsg) i = nsg - 1;
          i_first = i;
          for (; i >= 0 && cb[i + 1] > x0; i--) {
            const double v0 = std::max(x0, cb[i]), v1 = std::min(x1, cb[i + 1]);
            if (v1 > v0) piece(L2->seg_fsr[off[t] + i], L - v1, L - v0);
            n_crossed++;
          }
        }
        out_item.otf.insert(out_item.otf.end(),
                            {(int32_t) t, (int32_t) i_first,
                             (int32_t) n_crossed, (int32_t) d});
        out_item.otf_f.insert(out_item.otf_f.end(),
                              {(float) a0, (float) take,
                               (float) (z - fuel_height), 0.0f});
        out_item.nseg.push_back(
            (int32_t) (out_item.seg_len.size() - seg_start));
        remaining -= take;
        z += take * cot;
        out_item.first.push_back(first_piece ? 1 : 0);
        out_item.last.push_back(remaining > 1e-12 ? 0 : 1);
        first_piece = false;
        k = (k + 1) % ncyc;
        s = c.s0[k];
      }
    }
  }

  // concatenate in item order
  moc_lattice* L = new moc_lattice();
  int64_t T = 0, S = 0;
  for (const Item& m : items) {
    T += (int64_t) m.nseg.size();
    S += (int64_t) m.seg_len.size();
  }
  if (T >= (1LL << 31) || S >= (1LL << 40)) {
    delete L;
    return lat_fail("extruded problem too large");
  }
  L->R = R2 + 1;
  L->T = T;
  L->S = S;
  L->A = (int32_t) nitems;
  L->Ph = 1;
  L->M = L2->M;
  L->seg_len.resize(S);
  L->seg_fsr.resize(S);
  L->seg_off.assign(T + 1, 0);
  L->track_ang.resize(T);
  L->next.resize(2 * T);
  L->flags.resize(T);
  L->weights.resize(nitems);
  L->inv_sin.assign(nitems, 1.0f);
  L->otf_trk.resize(4 * (size_t) T);
  L->otf_trk_f.resize(4 * (size_t) T);
  L->otf_ang.resize(4 * (size_t) nitems);
  std::vector<double> vol(R2 + 1, 0.0);
  int64_t tb = 0, sb = 0;
  for (int64_t it = 0; it < nitems; it++) {
    const Item& m = items[it];
    L->weights[it] = (float) m.weight;
    L->otf_ang[4 * it + 0] = m.cot;
    L->otf_ang[4 * it + 1] = 1.0f / m.cot;
    L->otf_ang[4 * it + 2] = 1.0f / m.sin_t;
    L->otf_ang[4 * it + 3] = 0.0f;
    std::memcpy(L->otf_trk.data() + 4 * tb, m.otf.data(), 4 * m.otf.size());
    std::memcpy(L->otf_trk_f.data() + 4 * tb, m.otf_f.data(),
                4 * m.otf_f.size());
    const double wv = m.weight / (2.0 * kPi);
    std::memcpy(L->seg_len.data() + sb, m.seg_len.data(), 4 * m.seg_len.size());
    std::memcpy(L->seg_fsr.data() + sb, m.seg_fsr.data(), 4 * m.seg_fsr.size());
    for (size_t q = 0; q < m.seg_len.size(); q++)
      vol[m.seg_fsr[q]] += wv * (double) m.seg_len[q];
    for (size_t q = 0; q < m.nseg.size(); q++) {
      const int64_t t = tb + (int64_t) q;
      L->seg_off[t + 1] = L->seg_off[t] + m.nseg[q];
      L->track_ang[t] = (int32_t) it;
      uint8_t f = 1;                       // forward exit enters forward
      if (!m.last[q]) f |= 4;              // transfer forward
      if (!m.first[q]) f |= 8;             // transfer backward
      L->flags[t] = f;                     // backward exit enters backward
      L->next[2 * t] = m.last[q] ? t : t + 1;
      L->next[2 * t + 1] = m.first[q] ? t : t - 1;
    }
    tb += (int64_t) m.nseg.size();
    sb += (int64_t) m.seg_len.size();
  }
  L->fsr_mat.assign(L2->fsr_mat.begin(), L2->fsr_mat.end());
  L->fsr_mat.push_back(L2->moderator);
  // the radial segments the on-the-fly tracks are cut from
  L->rad_len = L2->seg_len;
  L->rad_fsr = L2->seg_fsr;
  L->rad_off = L2->seg_off;
  L->rad_start.resize(L2->S);
  L->rad_total.resize(T2);
  for (int64_t t = 0; t < T2; t++) {
    for (int64_t k = off[t]; k < off[t + 1]; k++)
      L->rad_start[k] = (float) cum[k + t];
    L->rad_total[t] = (float) len2[t];
  }
  L->above_fsr = (int32_t) R2;
  L->fsr_vol.resize(R2 + 1);
  for (int64_t r = 0; r <= R2; r++) L->fsr_vol[r] = (float) vol[r];
  *out = L;
  return 0;
}

extern "C" int moc_lattice_export_cmfd(moc_lattice* L, double* fsr_box,
                                       int8_t* end_face, double* edc_mu,
                                       double* edc_w, double* bounds,
                                       double* centroid) {
  if (!L) return lat_fail("null lattice");
  if (L->tracks.empty() || (int64_t) L->tracks.size() != L->T ||
      (int64_t) L->fsr_pin.size() != L->R)
    return lat_fail("the CMFD geometry needs a 2D lattice");
  if (!fsr_box || !end_face || !edc_mu || !edc_w || !bounds)
    return lat_fail("null output array");
  const double W = L->nx * L->pitch, H = L->ny * L->pitch;
  const double x0 = L->xmin, y0 = L->ymin;
  for (int64_t r = 0; r < L->R; r++) {
    const int pin = L->fsr_pin[r];
    const int ci = pin % L->nx, row = pin / L->nx;
    const int cj = L->ny - 1 - row;
    fsr_box[4 * r] = x0 + ci * L->pitch;
    fsr_box[4 * r + 1] = x0 + (ci + 1) * L->pitch;
    fsr_box[4 * r + 2] = y0 + cj * L->pitch;
    fsr_box[4 * r + 3] = y0 + (cj + 1) * L->pitch;
  }
  // the boundary face a track end lies on (x faces first at a corner)
  const double tol = 1e-9 * std::max(W, H);
  auto face = [&](double x, double y) -> int8_t {
    if (std::fabs(x - x0) <= tol) return 0;
    if (std::fabs(x - (x0 + W)) <= tol) return 2;
    if (std::fabs(y - y0) <= tol) return 1;
    if (std::fabs(y - (y0 + H)) <= tol) return 3;
    return -1;
  };
  for (int64_t t = 0; t < L->T; t++) {
    const Track& tr = L->tracks[t];
    end_face[2 * t] = face(tr.x1, tr.y1);
    end_face[2 * t + 1] = face(tr.x0, tr.y0);
  }
  for (int a = 0; a < L->A; a++)
    for (int p = 0; p < L->Ph; p++) {
      const double sn = L->pol_sin[p];
      edc_mu[a * L->Ph + p] = std::sqrt(1.0 - sn * sn);
      edc_w[a * L->Ph + p] = L->az_weight[a] * L->pol_wgt[p];
    }
  bounds[0] = x0;
  bounds[1] = x0 + W;
  bounds[2] = y0;
  bounds[3] = y0 + H;
  // FSR centroids (TrackGenerator::generateFSRCentroids,
  // src/TrackGenerator.cpp:1681-1710): segment midpoints weighted by length,
  // azimuthal spacing and weight, over the FSR volume
  if (centroid) {
    std::vector<double> cx(L->R, 0.0), cy(L->R, 0.0);
    for (int64_t t = 0; t < L->T; t++) {
      const Track& tr = L->tracks[t];
      const double c = std::cos(tr.phi), sn = std::sin(tr.phi);
      const double w = L->az_spacing[tr.a] * L->az_weight[tr.a];
      double x = tr.x0, y = tr.y0;
      for (int64_t k = L->seg_off[t]; k < L->seg_off[t + 1]; k++) {
        const int32_t r = L->seg_fsr[k];
        const double l = (double) L->seg_len[k];
        const double v = (double) L->fsr_vol[r];
        cx[r] += w * (x + 0.5 * c * l) * l / v;
        cy[r] += w * (y + 0.5 * sn * l) * l / v;
        x += c * l;
        y += sn * l;
      }
    }
    for (int64_t r = 0; r < L->R; r++) {
      centroid[2 * r] = cx[r];
      centroid[2 * r + 1] = cy[r];
    }
  }
  return 0;
}
