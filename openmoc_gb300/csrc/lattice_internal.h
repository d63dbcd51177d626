// Internal declarations shared by the host lattice generator (lattice.cpp)
// and its device ray tracer (lattice_gpu.cu).  Not part of the public ABI
// (include/openmoc_gb300_lattice.h).
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "openmoc_gb300_lattice.h"

namespace moc_lat {

struct Track {
  double x0, y0, x1, y1, phi;
  int a;
};

constexpr double kPi = 3.14159265358979323846;
constexpr double kTinyMove = 1e-8;   // src/constants.h:41

// The laydown's products besides those stored in moc_lattice.
struct LatGeo {
  int A = 0, Ph = 0;            // azimuthal angles in (0, pi), polar per half
  int64_t T = 0;
  double W = 0, H = 0, xmin = 0, ymin = 0;
  std::vector<Track> tracks;
  std::vector<double> spac, wa, sin_t, w_p;
};

// Ring / sector layout of a pin cell: squared ring radii (outer to inner),
// radii, and the sector-line directions (fuel and moderator, sorted).
struct LatCells {
  int rings = 0, fuel_sectors = 0, mod_sectors = 0;
  std::vector<double> r2, radii, line_dirs;
};

int lat_fail(const std::string& m);
int lat_validate(const moc_lattice_spec& s);
void lat_laydown(const moc_lattice_spec& s, moc_lattice* L, LatGeo& X);
void lat_cells(const moc_lattice_spec& s, LatCells& c);
// FSR materials (from each FSR's key: cell << 32 | ring << 16 | sector),
// counts, and -- with volumes -- FSR volumes summed over segments in track
// order; stores the per-angle and polar data and the tracks in L.
void lat_finish(const moc_lattice_spec& s, moc_lattice* L, const LatGeo& X,
                const std::vector<uint64_t>& keys, bool volumes);

}  // namespace moc_lat

struct moc_lattice {
  int64_t R = 0, T = 0, S = 0;
  int32_t A = 0, Ph = 0, M = 0;
  std::vector<float> seg_len;
  std::vector<int32_t> seg_fsr;
  // 2D lattices traced on the host: each segment's start along its track in
  // double precision (the axial extrusion cuts its 3D tracks there)
  std::vector<double> seg_pos;
  std::vector<int64_t> seg_off;
  std::vector<int32_t> track_ang;
  std::vector<int64_t> next;
  std::vector<uint8_t> flags;
  std::vector<float> weights, inv_sin;
  std::vector<int32_t> fsr_mat;
  std::vector<float> fsr_vol;
  // per azimuthal index: effective spacing and azimuthal weight (used by the
  // axial extrusion); moderator material
  std::vector<double> az_spacing, az_weight;
  int32_t moderator = 0;
  // 2D lattices: the tracks (start, angle) and the polar set, for the
  // linear-source geometry (empty for extruded 3D lattices)
  std::vector<moc_lat::Track> tracks;
  std::vector<double> pol_sin, pol_wgt;
  // Extruded 3D lattices: the on-the-fly description of every 3D track
  // (radial track, first radial segment in traversal order, count, 1 if
  // reversed; a0, span, height above the cut at a0), per angle row cot,
  // 1/cot, 1/sin, and the radial segments they are cut from.
  std::vector<int32_t> otf_trk;     // [T][4]
  std::vector<float> otf_trk_f;     // [T][4]
  std::vector<float> otf_ang;       // [A][4]
  std::vector<float> rad_len, rad_start, rad_total;
  std::vector<int32_t> rad_fsr;
  std::vector<int64_t> rad_off;
  int32_t above_fsr = -1;
  // Extruded 3D lattices: each 3D track's start and end points [T][6], and
  // per angle row phi, theta, azimuthal spacing x weight and polar spacing
  // x weight (for the linear-source geometry)
  std::vector<double> tracks3d;
  std::vector<double> row_phi, row_theta, row_azw, row_polw;
  // 2D lattices: the lattice cell of every FSR (row 0 at the top, as the
  // FSR keys number them) and the lattice's placement, for CMFD meshes
  std::vector<int32_t> fsr_pin;
  int32_t nx = 0, ny = 0;
  double pitch = 0.0, xmin = 0.0, ymin = 0.0;
};
