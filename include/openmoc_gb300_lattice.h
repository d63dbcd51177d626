/**
 * @file openmoc_gb300_lattice.h
 * @brief Workload producer for hosts without OpenMOC: 2D tracks and
 *        segments of square pin-cell lattices, laid down and ray-traced the
 *        way OpenMOC's TrackGenerator and Geometry do for that geometry
 *        family (src/TrackGenerator.cpp:950-1222, src/Geometry.cpp:
 *        2085-2230, src/Cell.cpp:1325-1590), plus seeded synthetic
 *        cross sections.  Output arrays use the layout of openmoc_gb300.h.
 *        Every function returns 0 on success, -1 on error
 *        (moc_lattice_last_error gives the text).
 */
#ifndef OPENMOC_GB300_LATTICE_H_
#define OPENMOC_GB300_LATTICE_H_

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct moc_lattice moc_lattice;

typedef struct {
  int32_t nx, ny;          /* pin cells along x and y */
  double pitch;            /* cm */
  double pin_radius;       /* cm */
  int32_t fuel_rings;      /* equal-area rings inside the pin */
  int32_t fuel_sectors;    /* sectors inside the pin (0: none) */
  int32_t mod_sectors;     /* sectors of the moderator around the pin */
  int32_t bc[4];           /* xmin, xmax, ymin, ymax: 0 vacuum, 1 reflective */
  int32_t num_azim;        /* multiple of 4 */
  double spacing;          /* cm */
  int32_t num_polar;       /* 2, 4 or 6 (Tabuchi-Yamamoto) */
  int32_t moderator_material;
  int32_t num_threads;     /* 0: OpenMP default */
  const int32_t* pin_material; /* [ny*nx] material inside each pin; row 0 is
                                  the top row, as Lattice::setUniverses
                                  takes it (src/Universe.cpp:1604-1616) */
} moc_lattice_spec;

const char* moc_lattice_last_error(void);
/** TrackGenerator::generateTracks for a pin lattice (2D, explicit). */
int moc_lattice_generate(const moc_lattice_spec* spec, moc_lattice** out);
int moc_lattice_sizes(moc_lattice* lat, int64_t* num_fsrs,
                      int64_t* num_tracks, int64_t* num_segments,
                      int32_t* num_angles, int32_t* num_polar_half,
                      int32_t* num_materials);
int moc_lattice_export(moc_lattice* lat, float* seg_len, int32_t* seg_fsr,
                       int64_t* seg_off, int32_t* track_ang, int64_t* next,
                       uint8_t* flags, float* weights, float* inv_sin,
                       int32_t* fsr_mat, float* fsr_vol);
/** What a CMFD mesh (moc_cmfd_mesh, openmoc_gb300.h) is laid over, for a
 *  2D lattice: per FSR the box of its lattice cell [R][4] (xmin, xmax,
 *  ymin, ymax), per track the boundary face at the end of its forward and
 *  backward traversal [T][2] (0 x-min, 1 y-min, 2 x-max, 3 y-max; -1 none),
 *  the Larsen-EDC quadrature [A][Ph] (cos theta; azimuthal x polar weight),
 *  the geometry's bounds [4] (xmin, xmax, ymin, ymax) and, when centroid is
 *  not NULL, the FSR centroids [R][2] for the k-nearest update. */
int moc_lattice_export_cmfd(moc_lattice* lat, double* fsr_box,
                            int8_t* end_face, double* edc_mu, double* edc_w,
                            double* bounds, double* centroid);
int moc_lattice_destroy(moc_lattice* lat);

/** moc_lattice_generate with the ray tracing on CUDA device `device`: the
 *  laydown on the host, segmentation (one thread per track), FSR numbering
 *  by first touch and FSR volumes on the GPU.  Segment lengths, FSR ids,
 *  links and flags are bit-identical to moc_lattice_generate's; volumes are
 *  summed in a different order (FP64 atomics).  At most 16 fuel rings and
 *  64 sector lines per pin cell. */
int moc_lattice_generate_device(const moc_lattice_spec* spec, int32_t device,
                                moc_lattice** out);

/** Linear-source geometry of a 2D lattice (the arrays of moc_ls_geometry in
 *  openmoc_gb300.h): each segment's start relative to its FSR centroid
 *  (seg_x, seg_y [S]), the centroids [R][2] (CentroidGenerator's formula,
 *  src/TrackTraversingAlgorithms.cpp:377-460), per angle row cos / sin phi
 *  [A][2] and spacing x azimuthal weight [A], sin theta and polar weight
 *  [A][Ph].  Fails for extruded 3D lattices. */
int moc_lattice_export_ls(moc_lattice* lat, float* seg_x, float* seg_y,
                          double* centroid, double* ang_dir, double* ang_wgt,
                          double* pol_sin, double* pol_wgt);

/** Explicit 3D tracks of the lattice extruded to `height` (cm): its pins
 *  below fuel_height, one homogeneous moderator region above; reflective
 *  radially (required of the radial lattice), vacuum at bottom and top;
 *  Gauss-Legendre polar angles (2, 4 or 6) and axial spacing z_spacing.
 *  OpenMOC's own 3D laydown (TrackGenerator3D with EXPLICIT_3D segments,
 *  src/TrackGenerator3D.cpp: corrected polar angles, chains of radial
 *  tracks, z-stacks, track numbering) over the radial tracks.  The result
 *  has one polar value per track (3D layout of include/openmoc_gb300.h; an
 *  angle row per azimuthal and polar angle, a * num_polar + p) and is read
 *  with moc_lattice_sizes/export. */
int moc_lattice_extrude(const moc_lattice* radial, double height,
                        double fuel_height, double z_spacing,
                        int32_t num_polar, int32_t num_threads,
                        moc_lattice** out);
/** Start and end point of every 3D track of an extruded lattice, [T][6]
 *  (x0, y0, z0, x1, y1, z1). */
int moc_lattice_export_ends3d(moc_lattice* lat, double* ends);
/** Linear-source geometry of an extruded 3D lattice (moc_ls_geometry's 3D
 *  arrays): each segment's start relative to its FSR centroid (seg_x,
 *  seg_y, seg_z [S]), the centroids [R][3] (CentroidGenerator's 3D
 *  branch), per angle row cos / sin phi [A][2], azimuthal spacing x weight
 *  [A], sin / cos theta [A] and polar spacing x weight [A]. */
int moc_lattice_export_ls3d(moc_lattice* lat, float* seg_x, float* seg_y,
                            float* seg_z, double* centroid, double* ang_dir,
                            double* ang_wgt, double* pol_sin, double* pol_cos,
                            double* pol_wgt);

/** On-the-fly description of an extruded lattice's 3D tracks (the arrays
 *  of moc_otf_tracks in openmoc_gb300.h): per 3D track [T][4] (radial
 *  track, first radial segment crossed in traversal order, count, 1 if the
 *  traversal runs against the radial track) and [T][4] floats (start a0
 *  along the radial traversal, span, height above the fuel top at a0, 0);
 *  per angle row [A][4] (cot theta, 1/cot theta, 1/sin theta, 0); the
 *  radial segments (lengths, FSR ids, offsets, start of each segment on its
 *  track, track lengths); above_fsr = the region above the fuel.
 *  moc_lattice_otf_sizes gives T2 and S2 of the radial arrays. */
int moc_lattice_otf_sizes(moc_lattice* lat, int64_t* num_radial_tracks,
                          int64_t* num_radial_segments, int32_t* above_fsr);
int moc_lattice_export_otf(moc_lattice* lat, int32_t* trk, float* trk_f,
                           float* ang, float* rad_len, int32_t* rad_fsr,
                           int64_t* rad_off, float* rad_start,
                           float* rad_total);

/** Seeded synthetic multigroup data (sigma_s origin-major [orig*G+dest]),
 *  optionally multiplied by lognormal(0, perturb_sigma) factors per group. */
int moc_synthetic_xs(uint64_t seed, int32_t num_groups, int32_t fissile,
                     uint64_t perturb_seed, double perturb_sigma,
                     double* sigma_t, double* sigma_s, double* nu_sigma_f,
                     double* sigma_f, double* chi);

#ifdef __cplusplus
}
#endif

#endif
