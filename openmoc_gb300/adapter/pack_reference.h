/**
 * @file pack_reference.h
 * @brief Packs the tracks, segments, quadrature and cross sections that
 *        OpenMOC's own TrackGenerator / Geometry / Material objects hold into
 *        the flat structure-of-arrays layout that the GB300 C ABI
 *        (include/openmoc_gb300.h) consumes.
 *
 * This header is compiled only against OpenMOC's headers (it is the part of
 * the drop-in adapter that reads OpenMOC objects).  It replaces the
 * per-track cudaMalloc/cudaMemcpy cloning of the reference GPU back end
 * (src/accel/cuda/clone.cu:12-126) with one host-side pass that produces a
 * handful of contiguous arrays, uploaded with one copy each.
 *
 * Layout produced (all little-endian, host order):
 *   seg_len[S]   float   segment length, (float) of segment::_length
 *                        (src/Track.h:27-58; the sweep casts it the same way,
 *                        src/CPUSolver.cpp:2407)
 *   seg_fsr[S]   int32   segment::_region_id
 *   seg_off[T+1] int64   prefix sum of Track::getNumSegments() in UID order
 *   track_ang[T] int32   row of the angle tables used by this track:
 *                        2D: azimuthal index a; 3D: a*num_polar + p
 *   next[2T]     int64   [t][0] = getTrackNextFwd, [t][1] = getTrackNextBwd
 *   flags[T]     uint8   bit0 getNextFwdFwd, bit1 getNextBwdFwd,
 *                        bit2 forward flux is transferred (bc_fwd REFLECTIVE
 *                        or PERIODIC), bit3 backward flux is transferred
 *                        (src/CPUSolver.cpp:2560-2600)
 *   weights[A][Ph], inv_sin[A][Ph]  float  Quadrature::getWeightInline /
 *                        getInvSinThetaInline (src/Quadrature.h:317-336);
 *                        3D: Ph = 1, inv_sin = 1, weights[a*P+p] = w(a,p)
 *   sigma_t[M][G], sigma_s[M][G][G] (destination-major, [dest*G+orig],
 *   src/Material.cpp:721-735), nu_sigma_f[M][G], chi[M][G]   float
 *   fsr_mat[R] int32 (dense material index), fsr_vol[R] float
 */
#ifndef OPENMOC_GB300_PACK_REFERENCE_H_
#define OPENMOC_GB300_PACK_REFERENCE_H_

#include <cmath>
#include <cstdint>
#include <map>
#include <stdexcept>
#include <vector>

#include "TrackGenerator.h"
#include "TrackGenerator3D.h"
#include "Geometry.h"
#include "Material.h"
#include "Quadrature.h"

namespace openmoc_gb300 {

struct PackedProblem {
  int num_groups = 0;
  int num_polar_half = 0;     /* polar values carried per track direction */
  int num_angles = 0;         /* rows of weights / inv_sin */
  int num_materials = 0;
  int solve_3d = 0;
  long num_fsrs = 0;
  long num_tracks = 0;
  long num_segments = 0;

  std::vector<float> seg_len;
  std::vector<int32_t> seg_fsr;
  std::vector<int64_t> seg_off;
  std::vector<int32_t> track_ang;
  std::vector<int64_t> next;
  std::vector<uint8_t> flags;

  std::vector<float> weights;
  std::vector<float> inv_sin;

  std::vector<float> sigma_t;
  std::vector<float> sigma_s;
  std::vector<float> nu_sigma_f;
  std::vector<float> chi;
  std::vector<int32_t> fsr_mat;
  std::vector<float> fsr_vol;

  /* Dense index of every Material, keyed by the Material pointer. */
  std::map<Material*, int> material_index;

  /* Linear-source geometry (pack_linear_source):
   *   seg_x[S], seg_y[S]  float   segment::_starting_position relative to
   *                               the FSR centroid (RecenterSegments,
   *                               src/TrackTraversingAlgorithms.cpp:1320-1331)
   *   ang_dir[A][2]       double  cos(phi), sin(phi) of the tracks of each
   *                               angle row (Track::getPhi)
   *   ang_wgt[A]          double  Quadrature::getAzimSpacing * getAzimWeight
   *   pol_sin[A][Ph], pol_wgt[A][Ph]  double  getSinTheta, getPolarWeight
   *   centroid[R][2]      double  Geometry::getFSRCentroid (for reporting)
   * and for explicit 3D tracks (angle rows a * num_polar + p, Ph = 1):
   *   seg_z[S]            float   the z of the start, relative likewise
   *   pol_sin[A], pol_cos[A]  double  sin, cos of Track3D::getTheta
   *   pol_wgt[A]          double  getPolarSpacing * getPolarWeight
   *   centroid[R][3]      double */
  std::vector<float> seg_x, seg_y, seg_z;
  std::vector<double> ang_dir, ang_wgt, pol_sin, pol_wgt, pol_cos, centroid;
};

inline bool transfers_flux(boundaryType bc) {
  return bc == REFLECTIVE || bc == PERIODIC;
}

/**
 * Packs the explicit 2D or 3D segments of a TrackGenerator whose tracks have
 * been generated and (if needed) split by Solver::initializeExpEvaluators
 * (src/Solver.cpp:716-785).  FSR volumes come from the TrackGenerator
 * (src/TrackGenerator.cpp:368) and materials from Geometry::findFSRMaterial
 * (src/Geometry.cpp:1125).
 */
inline void pack_tracks(TrackGenerator* tg, PackedProblem& out) {
  TrackGenerator3D* tg3 = dynamic_cast<TrackGenerator3D*>(tg);
  Quadrature* quad = tg->getQuadrature();
  const int num_azim = tg->getNumAzim();
  const int num_polar = quad->getNumPolarAngles();

  Track** tracks = NULL;
  long T = 0;
  std::vector<Track*> uid_order;
  if (tg3 != NULL && tg3->getSegmentFormation() == EXPLICIT_3D) {
    /* 3D tracks live in a [azim][xy][polar][z] ragged array; order them by
     * UID, the index of their boundary fluxes (src/Solver.h:49-54). */
    out.solve_3d = 1;
    T = tg3->getNum3DTracks();
    uid_order.assign(T, (Track*) NULL);
    Track3D**** t3d = tg3->get3DTracks();
    int*** per_stack = tg3->getTracksPerStack();
    long num_2d = tg->getNum2DTracks();
    Track** tracks_2d = tg->get2DTracksArray();
    for (long i2 = 0; i2 < num_2d; i2++) {
      int a = tracks_2d[i2]->getAzimIndex();
      int xy = tracks_2d[i2]->getXYIndex();
      for (int p = 0; p < num_polar; p++)
        for (int z = 0; z < per_stack[a][xy][p]; z++) {
          Track3D* t3 = &t3d[a][xy][p][z];
          long uid = t3->getUid();
          if (uid < 0 || uid >= T)
            throw std::runtime_error("3D track UID out of range");
          uid_order[uid] = t3;
        }
    }
    for (long t = 0; t < T; t++)
      if (uid_order[t] == NULL)
        throw std::runtime_error("3D track UIDs are not a permutation");
    tracks = uid_order.data();
  } else if (tg3 == NULL) {
    out.solve_3d = 0;
    T = tg->getNum2DTracks();
    tracks = tg->get2DTracksArray();
  } else {
    throw std::runtime_error("only explicit 2D or explicit 3D segments can "
                             "be packed");
  }

  out.num_tracks = T;
  out.seg_off.assign(T + 1, 0);
  out.track_ang.assign(T, 0);
  out.next.assign(2 * T, 0);
  out.flags.assign(T, 0);

  for (long t = 0; t < T; t++) {
    Track* track = tracks[t];
    if ((long) track->getUid() != t)
      throw std::runtime_error("tracks array is not ordered by UID");
    out.seg_off[t + 1] = out.seg_off[t] + track->getNumSegments();
    int a = track->getAzimIndex();
    if (out.solve_3d) {
      Track3D* t3 = static_cast<Track3D*>(track);
      out.track_ang[t] = a * num_polar + t3->getPolarIndex();
    } else {
      out.track_ang[t] = a;
    }
    out.next[2 * t] = track->getTrackNextFwd();
    out.next[2 * t + 1] = track->getTrackNextBwd();
    uint8_t f = 0;
    if (track->getNextFwdFwd()) f |= 1;
    if (track->getNextBwdFwd()) f |= 2;
    if (transfers_flux(track->getBCFwd())) f |= 4;
    if (transfers_flux(track->getBCBwd())) f |= 8;
    out.flags[t] = f;
  }

  long S = out.seg_off[T];
  out.num_segments = S;
  out.seg_len.resize(S);
  out.seg_fsr.resize(S);
  for (long t = 0; t < T; t++) {
    segment* segs = tracks[t]->getSegments();
    long base = out.seg_off[t];
    int n = tracks[t]->getNumSegments();
    for (int s = 0; s < n; s++) {
      out.seg_len[base + s] = (float) (FP_PRECISION) segs[s]._length;
      out.seg_fsr[base + s] = segs[s]._region_id;
    }
  }

  if (out.solve_3d) {
    out.num_polar_half = 1;
    out.num_angles = (num_azim / 2) * num_polar;
    out.weights.resize(out.num_angles);
    out.inv_sin.assign(out.num_angles, 1.0f);
    for (int a = 0; a < num_azim / 2; a++)
      for (int p = 0; p < num_polar; p++)
        out.weights[a * num_polar + p] = (float) quad->getWeightInline(a, p);
  } else {
    out.num_polar_half = num_polar / 2;
    out.num_angles = num_azim / 2;
    out.weights.resize(out.num_angles * out.num_polar_half);
    out.inv_sin.resize(out.num_angles * out.num_polar_half);
    for (int a = 0; a < num_azim / 2; a++)
      for (int p = 0; p < num_polar / 2; p++) {
        out.weights[a * out.num_polar_half + p] =
            (float) quad->getWeightInline(a, p);
        out.inv_sin[a * out.num_polar_half + p] =
            (float) quad->getInvSinThetaInline(a, p);
      }
  }
}

/**
 * Packs what the linear-source sweep reads beyond the flat-source arrays
 * (CPULSSolver::tallyLSScalarFlux, src/CPULSSolver.cpp:542-741, and the
 * LinearExpansionGenerator, src/TrackTraversingAlgorithms.cpp:470-830).
 * Call after pack_tracks, once the segments have been re-centred on the FSR
 * centroids (TrackGenerator::generateFSRCentroids, which
 * Solver::initializeFSRs runs, src/Solver.cpp:865).  2D tracks only.
 */
inline void pack_linear_source_3d(TrackGenerator* tg, PackedProblem& out);

inline void pack_linear_source(TrackGenerator* tg, PackedProblem& out) {
  if (out.solve_3d) {
    pack_linear_source_3d(tg, out);
    return;
  }
  Geometry* geo = tg->getGeometry();
  if (!geo->containsFSRCentroids())
    throw std::runtime_error("FSR centroids have not been generated");
  Quadrature* quad = tg->getQuadrature();
  const int A = out.num_angles, Ph = out.num_polar_half;
  const long T = out.num_tracks, R = geo->getNumFSRs();
  Track** tracks = tg->get2DTracksArray();
  out.seg_x.resize(out.num_segments);
  out.seg_y.resize(out.num_segments);
  out.ang_dir.assign(2 * (size_t) A, 0.0);
  std::vector<char> seen(A, 0);
  for (long t = 0; t < T; t++) {
    segment* segs = tracks[t]->getSegments();
    const long base = out.seg_off[t];
    const int n = tracks[t]->getNumSegments();
    for (int k = 0; k < n; k++) {
      out.seg_x[base + k] = (float) segs[k]._starting_position[0];
      out.seg_y[base + k] = (float) segs[k]._starting_position[1];
    }
    const int a = out.track_ang[t];
    const double phi = tracks[t]->getPhi();
    if (!seen[a]) {
      seen[a] = 1;
      out.ang_dir[2 * a] = std::cos(phi);
      out.ang_dir[2 * a + 1] = std::sin(phi);
    } else if (out.ang_dir[2 * a] != std::cos(phi) ||
               out.ang_dir[2 * a + 1] != std::sin(phi)) {
      throw std::runtime_error("tracks of one azimuthal index differ in phi");
    }
  }
  out.ang_wgt.resize(A);
  out.pol_sin.resize((size_t) A * Ph);
  out.pol_wgt.resize((size_t) A * Ph);
  for (int a = 0; a < A; a++) {
    out.ang_wgt[a] = quad->getAzimSpacing(a) * quad->getAzimWeight(a);
    for (int p = 0; p < Ph; p++) {
      out.pol_sin[(size_t) a * Ph + p] = quad->getSinTheta(a, p);
      out.pol_wgt[(size_t) a * Ph + p] = quad->getPolarWeight(a, p);
    }
  }
  out.centroid.resize(2 * (size_t) R);
  for (long r = 0; r < R; r++) {
    Point* c = geo->getFSRCentroid(r);
    out.centroid[2 * r] = c->getX();
    out.centroid[2 * r + 1] = c->getY();
  }
}

/** The explicit 3D tracks' linear-source geometry, in UID order as
 *  pack_tracks leaves them (the 3D branches of
 *  LinearExpansionGenerator::onTrack and TransportSweep::onTrack,
 *  src/TrackTraversingAlgorithms.cpp:680-700, :913-926). */
inline void pack_linear_source_3d(TrackGenerator* tg, PackedProblem& out) {
  TrackGenerator3D* tg3 = dynamic_cast<TrackGenerator3D*>(tg);
  Geometry* geo = tg->getGeometry();
  if (!tg3 || !geo->containsFSRCentroids())
    throw std::runtime_error("3D tracks with FSR centroids are needed");
  Quadrature* quad = tg->getQuadrature();
  const int num_polar = quad->getNumPolarAngles();
  const int A = out.num_angles;
  const long T = out.num_tracks, R = geo->getNumFSRs();
  out.seg_x.resize(out.num_segments);
  out.seg_y.resize(out.num_segments);
  out.seg_z.resize(out.num_segments);
  out.ang_dir.assign(2 * (size_t) A, 0.0);
  out.ang_wgt.assign(A, 0.0);
  out.pol_sin.assign(A, 0.0);
  out.pol_cos.assign(A, 0.0);
  out.pol_wgt.assign(A, 0.0);
  std::vector<char> seen(A, 0);
  Track3D**** t3d = tg3->get3DTracks();
  int*** per_stack = tg3->getTracksPerStack();
  Track** tracks_2d = tg->get2DTracksArray();
  for (long i2 = 0; i2 < tg->getNum2DTracks(); i2++) {
    const int a = tracks_2d[i2]->getAzimIndex();
    const int xy = tracks_2d[i2]->getXYIndex();
    for (int p = 0; p < num_polar; p++)
      for (int z = 0; z < per_stack[a][xy][p]; z++) {
        Track3D* t = &t3d[a][xy][p][z];
        const long uid = t->getUid();
        if (uid < 0 || uid >= T)
          throw std::runtime_error("3D track UID out of range");
        segment* segs = t->getSegments();
        const long base = out.seg_off[uid];
        for (int k = 0; k < t->getNumSegments(); k++) {
          out.seg_x[base + k] = (float) segs[k]._starting_position[0];
          out.seg_y[base + k] = (float) segs[k]._starting_position[1];
          out.seg_z[base + k] = (float) segs[k]._starting_position[2];
        }
        const int row = out.track_ang[uid];
        const double phi = t->getPhi(), theta = t->getTheta();
        if (!seen[row]) {
          seen[row] = 1;
          out.ang_dir[2 * row] = std::cos(phi);
          out.ang_dir[2 * row + 1] = std::sin(phi);
          out.pol_sin[row] = std::sin(theta);
          out.pol_cos[row] = std::cos(theta);
          out.ang_wgt[row] = quad->getAzimSpacing(a) * quad->getAzimWeight(a);
          out.pol_wgt[row] = quad->getPolarSpacing(a, p) *
                             quad->getPolarWeight(a, p);
        } else if (out.ang_dir[2 * row] != std::cos(phi) ||
                   out.pol_cos[row] != std::cos(theta)) {
          throw std::runtime_error("tracks of one angle row differ in angle");
        }
      }
  }
  out.centroid.resize(3 * (size_t) R);
  for (long r = 0; r < R; r++) {
    Point* c = geo->getFSRCentroid(r);
    out.centroid[3 * r] = c->getX();
    out.centroid[3 * r + 1] = c->getY();
    out.centroid[3 * r + 2] = c->getZ();
  }
}

/** Packs materials, FSR materials and FSR volumes. */
inline void pack_materials(Geometry* geo, FP_PRECISION* fsr_volumes,
                           PackedProblem& out) {
  std::map<int, Material*> mats = geo->getAllMaterials();
  const int G = geo->getNumEnergyGroups();
  out.num_groups = G;
  out.num_materials = (int) mats.size();
  out.sigma_t.assign((size_t) out.num_materials * G, 0.f);
  out.sigma_s.assign((size_t) out.num_materials * G * G, 0.f);
  out.nu_sigma_f.assign((size_t) out.num_materials * G, 0.f);
  out.chi.assign((size_t) out.num_materials * G, 0.f);
  int m = 0;
  for (std::map<int, Material*>::iterator it = mats.begin();
       it != mats.end(); ++it, ++m) {
    Material* mat = it->second;
    out.material_index[mat] = m;
    FP_PRECISION* st = mat->getSigmaT();
    FP_PRECISION* ss = mat->getSigmaS();
    FP_PRECISION* nf = mat->getNuSigmaF();
    FP_PRECISION* ch = mat->getChi();
    for (int g = 0; g < G; g++) {
      out.sigma_t[(size_t) m * G + g] = (float) st[g];
      out.nu_sigma_f[(size_t) m * G + g] = nf ? (float) nf[g] : 0.f;
      out.chi[(size_t) m * G + g] = ch ? (float) ch[g] : 0.f;
      for (int h = 0; h < G; h++)
        out.sigma_s[((size_t) m * G + g) * G + h] = (float) ss[g * G + h];
    }
  }
  long R = geo->getNumFSRs();
  out.num_fsrs = R;
  out.fsr_mat.resize(R);
  out.fsr_vol.resize(R);
  for (long r = 0; r < R; r++) {
    Material* mat = geo->findFSRMaterial(r);
    std::map<Material*, int>::iterator it = out.material_index.find(mat);
    if (it == out.material_index.end())
      throw std::runtime_error("FSR material missing from the geometry map");
    out.fsr_mat[r] = it->second;
    out.fsr_vol[r] = (float) fsr_volumes[r];
  }
}

}  // namespace openmoc_gb300

#endif
