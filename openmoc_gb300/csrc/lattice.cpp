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
  std::vector<std::vector<double>> seg_pos_t(T);
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
    std::vector<double>& out_pos = seg_pos_t[t];
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
          out_pos.push_back(pts[k]);
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
  L->seg_pos.resize(S);
  for (int64_t t = 0; t < T; t++) {
    const int64_t base = L->seg_off[t];
    std::memcpy(L->seg_pos.data() + base, seg_pos_t[t].data(),
                sizeof(double) * seg_pos_t[t].size());
    std::vector<double>().swap(seg_pos_t[t]);
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
// bottom and top, with OpenMOC's own 3D laydown (TrackGenerator3D with
// EXPLICIT_3D segments, src/TrackGenerator3D.cpp) over the radial tracks:
//   - Gauss-Legendre polar angles (TrackGenerator3D's default GLPolarQuad,
//     src/Quadrature.cpp:1014-1073: theta_p = acos of the Legendre roots in
//     ascending order for the upper half, pi - theta for the lower half,
//     weights half the Gauss-Legendre weights).
//   - Per azimuthal angle and polar pair, the l / z counts and effective
//     spacings, and the polar angle corrected to atan(dl / dz)
//     (TrackGenerator3D::initializeTracks, src/TrackGenerator3D.cpp:683-800).
//   - Chains of radial tracks linked periodically from the y-min boundary to
//     the y-max boundary (initialize2DTrackChains, :886-925); along each
//     chain, for every polar angle, nl + nz lines laid at the effective
//     spacings (getFirst2DTrackLinkIndex, :975-1097) and cut where they
//     reach an x / y boundary of a radial track or the bottom / top: each
//     piece is a 3D track of the stack (azimuthal angle, radial track, polar
//     angle) it lies over, stacked in the order laid (set3DTrackData,
//     :1099-1251).  Tracks are numbered azimuthal, radial track, polar
//     angle, stack index, as get3DTrackID numbers them.
//   - Segments: the radial segments under the piece, cut at z = fuel_height;
//     above it the single moderator region (id R2); length = radial length /
//     sin(theta).
//   - Connections: a track leaving through a reflective x / y boundary
//     continues in the stack of the radial track's reflected neighbour
//     (forward keeps the polar angle, an entry from the end takes the
//     complementary one), in the track that starts (ends) at the exit point;
//     the bottom and top are vacuum.
//   - Weights per (azimuthal, polar) row: 2 pi w_a d_a w_p d_p with d_p the
//     polar spacing dz sin(theta) (Quadrature::precomputeWeights,
//     src/Quadrature.cpp:728-743); FSR volumes sum(w / 2 pi * length)
//     (VolumeKernel, src/MOCKernel.cpp:86-160).
namespace {

struct Piece {
  int32_t t2;                 // radial track
  double x0, y0, z0, x1, y1, z1;
};

}  // namespace

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
  if (L2->az_spacing.empty() || (int64_t) L2->tracks.size() != T2 ||
      !(L2->pitch > 0))
    return lat_fail("the extrusion needs a radial lattice with its tracks");

  const double W = L2->nx * L2->pitch, H = L2->ny * L2->pitch;
  const double xmin = L2->xmin, xmax = L2->xmin + W;
  const double ymin = L2->ymin, ymax = L2->ymin + H;
  const double zmin = 0.0, zmax = height;
  const int A = L2->A;                       // azimuthal angles in (0, pi)
  const int P = num_polar, half = P / 2;
  // radial tracks per azimuthal angle, and those starting on y = ymin
  std::vector<int64_t> first(A + 1, 0);
  std::vector<int> num_x(A, 0);
  for (int64_t t = 0; t < T2; t++) {
    const moc_lat::Track& tr = L2->tracks[t];
    if (tr.a < 0 || tr.a >= A) return lat_fail("radial track angle out of range");
    first[tr.a + 1]++;
    if (tr.y0 == ymin) num_x[tr.a]++;
  }
  for (int a = 0; a < A; a++) first[a + 1] += first[a];
  std::vector<int> num_y(A);
  for (int a = 0; a < A; a++) num_y[a] = (int) (first[a + 1] - first[a]) - num_x[a];

  // Gauss-Legendre nodes (ascending, upper half) and weights on [-1, 1]
  static const double gl_mu[3][3] = {{0.5773502691896258, 0, 0},
                                     {0.3399810435848563, 0.8611363115940526, 0},
                                     {0.2386191860831969, 0.6612093864662645,
                                      0.9324695142031521}};
  static const double gl_w[3][3] = {{1.0, 0, 0},
                                    {0.6521451548625461, 0.3478548451374538, 0},
                                    {0.4679139345726910, 0.3607615730481386,
                                     0.1713244923791704}};
  const int row = half - 1;
  // per (azimuthal, polar): corrected theta, l / z counts and spacings
  std::vector<double> theta((size_t) A * P), dl_eff((size_t) A * P),
      dz_eff((size_t) A * P), wpol((size_t) A * P);
  std::vector<int> nl((size_t) A * P), nz((size_t) A * P);
  for (int a = 0; a < A / 2; a++) {
    const double phi = L2->tracks[first[a]].phi;
    for (int j = 0; j < half; j++) {
      const double th = std::acos(gl_mu[row][j]);
      const double length = H / std::sin(phi);
      const int l = (int) std::ceil(length * std::tan(0.5 * kPi - th) / z_spacing);
      const int z = (int) std::ceil(height * l * std::tan(th) / length);
      const double dl = H / (std::sin(phi) * l);
      const double dz = height / z;
      const double th_new = std::atan(dl / dz);
      const int sa = A - a - 1, cp = P - j - 1;
      for (int aa : {a, sa})
        for (int pp : {j, cp}) {
          const size_t r = (size_t) aa * P + pp;
          nl[r] = l;
          nz[r] = z;
          dl_eff[r] = dl;
          dz_eff[r] = dz;
          theta[r] = (pp == j) ? th_new : kPi - th_new;
          wpol[r] = 0.5 * gl_w[row][j];
        }
    }
  }

  // chains: radial tracks linked periodically from y = ymin up to y = ymax
  // (the periodic forward neighbour of xy < num_y is xy + num_x)
  struct Chain {
    int a;
    std::vector<int32_t> xy;
  };
  std::vector<Chain> chains;
  for (int a = 0; a < A; a++)
    for (int x = 0; x < num_x[a]; x++) {
      Chain c;
      c.a = a;
      int xy = x;
      c.xy.push_back(xy);
      while (xy < num_y[a]) {
        xy += num_x[a];
        c.xy.push_back(xy);
      }
      chains.push_back(std::move(c));
    }

  // the pieces of every (chain, polar angle), in the order laid
  const int64_t nitems = (int64_t) chains.size() * P;
  std::vector<std::vector<Piece>> laid(nitems);
#ifdef _OPENMP
  if (num_threads > 0) omp_set_num_threads(num_threads);
#pragma omp parallel for schedule(dynamic, 1)
#endif
  for (int64_t it = 0; it < nitems; it++) {
    const Chain& ch = chains[it / P];
    const int p = (int) (it % P);
    const int a = ch.a;
    const size_t r = (size_t) a * P + p;
    const int NL = nl[r], NZ = nz[r];
    const double dz = dz_eff[r], dl = dl_eff[r], th = theta[r];
    const moc_lat::Track& c0 = L2->tracks[first[a] + ch.xy[0]];
    const double phi = c0.phi, cphi = std::cos(phi), sphi = std::sin(phi);
    std::vector<Piece>& outp = laid[it];
    for (int lz = 0; lz < NL + NZ; lz++) {
      // start point and link (getFirst2DTrackLinkIndex)
      double l_start = 0.0;
      if (p < half && lz < NL)
        l_start = H / sphi - (lz + 0.5) * dl;
      else if (p >= half && lz >= NZ)
        l_start = dl * (lz - NZ + 0.5);
      double x_ext = c0.x0 - xmin + l_start * cphi;
      double y_ext = c0.y0 - ymin + l_start * sphi;
      bool nudged = false;
      if (std::fabs(l_start) > 1e-12) {
        if (std::fabs(std::round(x_ext / W) * W - x_ext) < kTinyMove ||
            std::fabs(std::round(y_ext / H) * H - y_ext) < kTinyMove) {
          l_start += 10 * kTinyMove;
          x_ext = c0.x0 - xmin + l_start * cphi;
          y_ext = c0.y0 - ymin + l_start * sphi;
          nudged = true;
        }
      }
      int link = std::abs((int) std::floor(x_ext / W));
      double x1 = (x_ext < 0.0) ? std::fmod(x_ext, W) + xmax : std::fmod(x_ext, W) + xmin;
      double y1 = std::fmod(y_ext, H) + ymin;
      double z1, zend;
      if (p < half) {
        z1 = zmin + std::max(0., (lz - NL + 0.5)) * dz;
        zend = zmax + std::min(0., (lz - NZ + 0.5)) * dz;
      } else {
        z1 = zmax + std::min(0., (lz - NZ + 0.5)) * dz;
        zend = zmin + std::max(0., (lz - NL + 0.5)) * dz;
      }
      if (nudged) {
        x1 -= 10 * kTinyMove * cphi;
        y1 -= 10 * kTinyMove * sphi;
      }
      // walk the chain (set3DTrackData)
      const int first_link = link;
      double x2 = x1, y2 = y1, z2 = z1;
      bool end_of_chain = false;
      while (!end_of_chain) {
        if (link >= (int) ch.xy.size()) break;
        const int xy = ch.xy[link];
        const moc_lat::Track& t2 = L2->tracks[first[a] + xy];
        x1 = x2;
        y1 = y2;
        z1 = z2;
        double dl_xy;
        if (link == first_link) {
          const double ddx = t2.x1 - x1, ddy = t2.y1 - y1;
          dl_xy = std::sqrt(ddx * ddx + ddy * ddy);
        } else {
          const double ddx = t2.x1 - t2.x0, ddy = t2.y1 - t2.y0;
          dl_xy = std::sqrt(ddx * ddx + ddy * ddy);
        }
        double dl_z;
        if (p < half)
          dl_z = (zend - z1) * std::tan(th);
        else
          dl_z = (z1 - zend) / std::tan(th - 0.5 * kPi);
        const double d = std::min(dl_z, dl_xy);
        x2 = x1 + d * std::cos(t2.phi);
        y2 = y1 + d * std::sin(t2.phi);
        if (p < half)
          z2 = z1 + d / std::tan(th);
        else
          z2 = z1 - d * std::tan(th - 0.5 * kPi);
        if (std::fabs(x2 - x1) < kTinyMove || std::fabs(y2 - y1) < kTinyMove ||
            std::fabs(z2 - z1) < kTinyMove)
          break;
        if (dl_z < dl_xy || xy >= num_y[a]) end_of_chain = true;
        Piece pc;
        pc.t2 = (int32_t) (first[a] + xy);
        pc.x0 = std::max(xmin, std::min(xmax, x1));
        pc.y0 = std::max(ymin, std::min(ymax, y1));
        pc.z0 = std::max(zmin, std::min(zmax, z1));
        pc.x1 = std::max(xmin, std::min(xmax, x2));
        pc.y1 = std::max(ymin, std::min(ymax, y2));
        pc.z1 = std::max(zmin, std::min(zmax, z2));
        outp.push_back(pc);
        link++;
        if (!end_of_chain) x2 = (a < A / 2) ? xmin : xmax;
      }
    }
  }

  // stacks (azimuthal angle, radial track, polar angle): the pieces in the
  // order laid; each stack is filled by one chain
  std::vector<int64_t> stack_n((size_t) T2 * P, 0);
  for (int64_t it = 0; it < nitems; it++) {
    const int p = (int) (it % P);
    for (const Piece& pc : laid[it]) stack_n[(size_t) pc.t2 * P + p]++;
  }
  std::vector<int64_t> stack_first((size_t) T2 * P + 1, 0);
  for (size_t k = 0; k < (size_t) T2 * P; k++) stack_first[k + 1] = stack_first[k] + stack_n[k];
  const int64_t T = stack_first[(size_t) T2 * P];
  if (T >= (1LL << 31)) return lat_fail("extruded problem too large");
  std::vector<Piece> pieces(T);
  std::vector<int32_t> prow(T);
  {
    std::vector<int64_t> fill(stack_first.begin(), stack_first.end() - 1);
    for (int64_t it = 0; it < nitems; it++) {
      const int p = (int) (it % P);
      for (const Piece& pc : laid[it]) {
        const size_t k = (size_t) pc.t2 * P + p;
        pieces[fill[k]] = pc;
        prow[fill[k]] = (int32_t) L2->tracks[pc.t2].a * P + p;
        fill[k]++;
      }
    }
  }
  laid.clear();
  laid.shrink_to_fit();

  // radial segment boundaries per track: the tracer's double-precision
  // crossings where it kept them, else the summed lengths
  std::vector<int64_t> off(L2->seg_off.begin(), L2->seg_off.end());
  std::vector<double> cum((size_t) L2->S + T2);
  std::vector<double> len2(T2);
  const bool exact = (int64_t) L2->seg_pos.size() == L2->S;
  for (int64_t t = 0; t < T2; t++) {
    double c = 0;
    cum[off[t] + t] = 0;
    for (int64_t k = off[t]; k < off[t + 1]; k++) {
      c += (double) L2->seg_len[k];
      if (exact && k > off[t]) cum[k + t] = L2->seg_pos[k];
      cum[k + 1 + t] = c;
    }
    if (exact) {
      const moc_lat::Track& tr = L2->tracks[t];
      c = std::hypot(tr.x1 - tr.x0, tr.y1 - tr.y0);
      if (off[t + 1] > off[t]) cum[off[t + 1] + t] = c;
    }
    len2[t] = c;
  }
  const int64_t R2 = L2->R;
  // A piece shorter (in 3D) than the reference tracer's step past a surface
  // forms no segment; with summed lengths, the boundaries are only good to
  // their float rounding
  const double kSliver = exact ? kTinyMove : 1e-6;

  // segments of every 3D track (in parallel, then concatenated)
  std::vector<std::vector<float>> sl(T);
  std::vector<std::vector<int32_t>> sf(T);
  std::vector<int32_t> otf_i((size_t) 4 * T);
  std::vector<float> otf_f((size_t) 4 * T);
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 256)
#endif
  for (int64_t t = 0; t < T; t++) {
    const Piece& pc = pieces[t];
    const int64_t t2 = pc.t2;
    const moc_lat::Track& tr = L2->tracks[t2];
    const double th = theta[prow[t]];
    const double sin_t = std::sin(th), cot = std::cos(th) / sin_t;
    // the piece's span along the radial track, from its start point
    const double a0 = std::hypot(pc.x0 - tr.x0, pc.y0 - tr.y0);
    const double a1 = std::hypot(pc.x1 - tr.x0, pc.y1 - tr.y0);
    const double* cb = cum.data() + off[t2] + t2;
    const int64_t nsg = off[t2 + 1] - off[t2];
    int32_t last_fsr = -1;
    auto emit = [&](int32_t fsr, double l3) {
      if (l3 <= 1e-10) return;
      if (fsr == last_fsr && !sl[t].empty()) {
        sl[t].back() = (float) ((double) sl[t].back() + l3);
      } else {
        sf[t].push_back(fsr);
        sl[t].push_back((float) l3);
        last_fsr = fsr;
      }
    };
    // A track that starts or ends on a radial boundary leaves a sliver of
    // the neighbouring region at that end; the reference's tracing forms no
    // such segment, so the radial pieces crossed start after a sliver at a0
    // and stop before one at a1.
    int64_t i = (int64_t) (std::upper_bound(cb, cb + nsg + 1, a0) - cb) - 1;
    if (i < 0) i = 0;
    if (i + 1 < nsg && cb[i + 1] - a0 < kSliver * sin_t) i++;
    const int64_t i_first = i;
    int64_t i_end = i;
    while (i_end < nsg && cb[i_end] < a1) i_end++;
    if (i_end - 1 > i_first && a1 - cb[i_end - 1] < kSliver * sin_t) i_end--;
    const int64_t n_crossed = i_end - i_first;
    for (; i < i_end; i++) {
      const double u0 = std::max(a0, cb[i]), u1 = std::min(a1, cb[i + 1]);
      if (!(u1 > u0)) continue;
      const int32_t fsr2 = L2->seg_fsr[off[t2] + i];
      const double z0 = pc.z0 + (u0 - a0) * cot, z1 = pc.z0 + (u1 - a0) * cot;
      const double lo = std::min(z0, z1), hi = std::max(z0, z1);
      if (hi <= fuel_height) {
        emit(fsr2, (u1 - u0) / sin_t);
      } else if (lo >= fuel_height) {
        emit((int32_t) R2, (u1 - u0) / sin_t);
      } else {
        // cut at the fuel top (a sliver on either side of the cut, where the
        // track crosses it on a radial boundary, joins the other side)
        const double uc = u0 + (fuel_height - z0) / cot;
        const bool below_first = z0 < fuel_height;
        const int32_t f0 = below_first ? fsr2 : (int32_t) R2;
        const int32_t f1 = below_first ? (int32_t) R2 : fsr2;
        if (uc - u0 < kSliver * sin_t) {
          emit(f1, (u1 - u0) / sin_t);
        } else if (u1 - uc < kSliver * sin_t) {
          emit(f0, (u1 - u0) / sin_t);
        } else {
          emit(f0, (uc - u0) / sin_t);
          emit(f1, (u1 - uc) / sin_t);
        }
      }
    }
    otf_i[4 * t + 0] = (int32_t) t2;
    otf_i[4 * t + 1] = (int32_t) i_first;
    otf_i[4 * t + 2] = (int32_t) n_crossed;
    otf_i[4 * t + 3] = 0;
    otf_f[4 * t + 0] = (float) a0;
    otf_f[4 * t + 1] = (float) (a1 - a0);
    otf_f[4 * t + 2] = (float) (pc.z0 - fuel_height);
    otf_f[4 * t + 3] = 0.0f;
  }

  // connections: the track of the reflected stack that starts (forward
  // entry) or ends (backward entry) at the exit point
  const double ztol = 1e-9, ptol = 1e-6;
  auto find_in_stack = [&](int64_t t2n, int pn, bool at_start, double x,
                           double y, double z) -> int64_t {
    const size_t k = (size_t) t2n * P + pn;
    int64_t best = -1;
    double bd = ptol;
    for (int64_t u = stack_first[k]; u < stack_first[k + 1]; u++) {
      const Piece& q = pieces[u];
      const double qx = at_start ? q.x0 : q.x1, qy = at_start ? q.y0 : q.y1,
                   qz = at_start ? q.z0 : q.z1;
      const double dd = std::fabs(qx - x) + std::fabs(qy - y) + std::fabs(qz - z);
      if (dd < bd) {
        bd = dd;
        best = u;
      }
    }
    return best;
  };
  moc_lattice* L = new moc_lattice();
  L->next.assign(2 * T, 0);
  L->flags.assign(T, 0);
  int bad = 0;
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 1024) reduction(+ : bad)
#endif
  for (int64_t t = 0; t < T; t++) {
    const Piece& pc = pieces[t];
    const int p = prow[t] % P, pcomp = P - p - 1;
    const int64_t t2 = pc.t2;
    uint8_t f = 0;
    int64_t nf = t, nb = t;
    // forward end
    if (std::fabs(pc.z1 - zmin) > ztol && std::fabs(pc.z1 - zmax) > ztol) {
      const bool ff = (L2->flags[t2] & 1) != 0;
      nf = find_in_stack(L2->next[2 * t2], ff ? p : pcomp, ff, pc.x1, pc.y1, pc.z1);
      if (nf < 0) {
        bad++;
        nf = t;
      } else {
        f |= 4;
        if (ff) f |= 1;
      }
    }
    // backward end
    if (std::fabs(pc.z0 - zmin) > ztol && std::fabs(pc.z0 - zmax) > ztol) {
      const bool bf = (L2->flags[t2] & 2) != 0;
      nb = find_in_stack(L2->next[2 * t2 + 1], bf ? pcomp : p, bf, pc.x0, pc.y0, pc.z0);
      if (nb < 0) {
        bad++;
        nb = t;
      } else {
        f |= 8;
        if (bf) f |= 2;
      }
    }
    L->next[2 * t] = nf;
    L->next[2 * t + 1] = nb;
    L->flags[t] = f;
  }
  if (bad) {
    delete L;
    return lat_fail("3D tracks whose exit point starts no track of the "
                    "reflected stack: " + std::to_string(bad));
  }

  // concatenate the segments; weights, volumes, on-the-fly description
  int64_t S = 0;
  for (int64_t t = 0; t < T; t++) S += (int64_t) sl[t].size();
  const int nrows = A * P;
  L->R = R2 + 1;
  L->T = T;
  L->S = S;
  L->A = nrows;
  L->Ph = 1;
  L->M = L2->M;
  L->seg_len.resize(S);
  L->seg_fsr.resize(S);
  L->seg_off.assign(T + 1, 0);
  L->track_ang.assign(prow.begin(), prow.end());
  L->weights.resize(nrows);
  L->inv_sin.assign(nrows, 1.0f);
  L->otf_ang.resize(4 * (size_t) nrows);
  std::vector<double> wrow(nrows);
  L->row_phi.resize(nrows);
  L->row_theta.resize(nrows);
  L->row_azw.resize(nrows);
  L->row_polw.resize(nrows);
  for (int rr = 0; rr < nrows; rr++) {
    const int a = rr / P;
    const double th = theta[rr];
    const double dp = dz_eff[rr] * std::sin(th);   // polar spacing
    wrow[rr] = 2.0 * kPi * L2->az_weight[a] * L2->az_spacing[a] * wpol[rr] * dp;
    L->weights[rr] = (float) wrow[rr];
    L->row_phi[rr] = L2->tracks[first[a]].phi;
    L->row_theta[rr] = th;
    L->row_azw[rr] = L2->az_spacing[a] * L2->az_weight[a];
    L->row_polw[rr] = dp * wpol[rr];
    const double c = std::cos(th) / std::sin(th);
    L->otf_ang[4 * rr + 0] = (float) c;
    L->otf_ang[4 * rr + 1] = (float) (1.0 / c);
    L->otf_ang[4 * rr + 2] = (float) (1.0 / std::sin(th));
    L->otf_ang[4 * rr + 3] = 0.0f;
  }
  std::vector<double> vol(R2 + 1, 0.0);
  int64_t sb = 0;
  for (int64_t t = 0; t < T; t++) {
    const double wv = wrow[prow[t]] / (2.0 * kPi);
    const size_t n = sl[t].size();
    std::memcpy(L->seg_len.data() + sb, sl[t].data(), 4 * n);
    std::memcpy(L->seg_fsr.data() + sb, sf[t].data(), 4 * n);
    for (size_t q = 0; q < n; q++) vol[sf[t][q]] += wv * (double) sl[t][q];
    sb += (int64_t) n;
    L->seg_off[t + 1] = sb;
  }
  L->otf_trk = std::move(otf_i);
  L->otf_trk_f = std::move(otf_f);
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
  // the 3D track ends, for comparisons with the reference laydown
  L->tracks3d.resize(6 * (size_t) T);
  for (int64_t t = 0; t < T; t++) {
    const Piece& pc = pieces[t];
    double* e = L->tracks3d.data() + 6 * t;
    e[0] = pc.x0; e[1] = pc.y0; e[2] = pc.z0;
    e[3] = pc.x1; e[4] = pc.y1; e[5] = pc.z1;
  }
  *out = L;
  return 0;
}

// Linear-source geometry of an extruded 3D lattice (the explicit 3D
// branches of CentroidGenerator::onTrack and RecenterSegments,
// src/TrackTraversingAlgorithms.cpp:377-460, :1320-1331): FSR centroids as
// the segment midpoints weighted by length and w_a d_a w_p d_p over the FSR
// volume, each segment's start walked from its 3D track's start along
// (cos phi sin theta, sin phi sin theta, cos theta) and taken relative to
// its FSR's centroid; per angle row cos / sin phi, w_a d_a, sin / cos theta
// and w_p d_p.
extern "C" int moc_lattice_export_ls3d(moc_lattice* L, float* seg_x,
                                       float* seg_y, float* seg_z,
                                       double* centroid, double* ang_dir,
                                       double* ang_wgt, double* pol_sin,
                                       double* pol_cos, double* pol_wgt) {
  if (!L) return lat_fail("null lattice");
  if ((int64_t) L->tracks3d.size() != 6 * L->T ||
      (int64_t) L->row_theta.size() != L->A)
    return lat_fail("not an extruded 3D lattice");
  if (!seg_x || !seg_y || !seg_z || !centroid || !ang_dir || !ang_wgt ||
      !pol_sin || !pol_cos || !pol_wgt)
    return lat_fail("null output array");
  const int64_t T = L->T, R = L->R;
  std::vector<double> dx(L->A), dy(L->A), dz(L->A), w(L->A);
  for (int rr = 0; rr < L->A; rr++) {
    const double sth = std::sin(L->row_theta[rr]);
    dx[rr] = std::cos(L->row_phi[rr]) * sth;
    dy[rr] = std::sin(L->row_phi[rr]) * sth;
    dz[rr] = std::cos(L->row_theta[rr]);
    w[rr] = L->row_azw[rr] * L->row_polw[rr];
    ang_dir[2 * rr] = std::cos(L->row_phi[rr]);
    ang_dir[2 * rr + 1] = std::sin(L->row_phi[rr]);
    ang_wgt[rr] = L->row_azw[rr];
    pol_sin[rr] = sth;
    pol_cos[rr] = dz[rr];
    pol_wgt[rr] = L->row_polw[rr];
  }
  std::vector<double> cx(R, 0.0), cy(R, 0.0), cz(R, 0.0);
  for (int pass = 0; pass < 2; pass++) {
    for (int64_t t = 0; t < T; t++) {
      const int rr = L->track_ang[t];
      const double* e = L->tracks3d.data() + 6 * t;
      double x = e[0], y = e[1], z = e[2];
      for (int64_t k = L->seg_off[t]; k < L->seg_off[t + 1]; k++) {
        const int32_t r = L->seg_fsr[k];
        const double l = (double) L->seg_len[k];
        if (pass == 0) {
          const double v = (double) L->fsr_vol[r];
          cx[r] += w[rr] * (x + dx[rr] * l / 2.0) * l / v;
          cy[r] += w[rr] * (y + dy[rr] * l / 2.0) * l / v;
          cz[r] += w[rr] * (z + dz[rr] * l / 2.0) * l / v;
        } else {
          seg_x[k] = (float) (x - cx[r]);
          seg_y[k] = (float) (y - cy[r]);
          seg_z[k] = (float) (z - cz[r]);
        }
        x += dx[rr] * l;
        y += dy[rr] * l;
        z += dz[rr] * l;
      }
    }
  }
  for (int64_t r = 0; r < R; r++) {
    centroid[3 * r] = cx[r];
    centroid[3 * r + 1] = cy[r];
    centroid[3 * r + 2] = cz[r];
  }
  return 0;
}

extern "C" int moc_lattice_export_ends3d(moc_lattice* L, double* ends) {
  if (!L || !ends) return lat_fail("null argument");
  if ((int64_t) L->tracks3d.size() != 6 * L->T)
    return lat_fail("not an extruded 3D lattice");
  std::memcpy(ends, L->tracks3d.data(), sizeof(double) * L->tracks3d.size());
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
