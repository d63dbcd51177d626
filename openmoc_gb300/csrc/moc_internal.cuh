// Internal declarations shared by the CUDA translation units of
// libopenmoc_gb300.so.  Not part of the public ABI (include/openmoc_gb300.h).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <vector>

namespace moc {

// Exponential table for the attenuation factor g(x) = 1 - exp(-x): nodes at
// x_i = i / kExpTableInvH, i < kExpTableSize.  Beyond the last node g = 1 in
// float (exp(-20) = 2.1e-9).
constexpr int kExpTableSize = 321;
constexpr float kExpTableInvH = 16.0f;
constexpr float kExpTableH = 1.0f / 16.0f;

// Largest number of group pairs handled per lane and largest polar count.
constexpr int kMaxSlots = 6;
constexpr int kMaxPolarHalf = 5;
constexpr int kSweepThreads = 128;

enum ExpKind { kExpTable = 0, kExpIntrinsic = 1 };

// Device-resident solver scalars: the iteration state machine that lets a
// whole block of iterations run without host round trips.
struct DevScalars {
  double keff;            // current eigenvalue estimate
  double k_prev;          // eigenvalue of the previous iteration
  double factor;          // last normalisation factor
  double residual;        // last residual
  double accum_rate;      // fission-rate accumulator (reset by the last block)
  double accum_res;       // residual accumulator (reset by the last block)
  double threshold;       // convergence threshold
  float scale[2];         // pending multiplier of each angular-flux buffer
  unsigned int ticket_rate;
  unsigned int ticket_res;
  unsigned int ticket_sweep;
  int cur;                // angular-flux buffer the next sweep reads
  int iteration;          // iterations completed in this solve
  int max_iters;
  int done;               // 1: converged or out of iterations
  int converged;
  int dk;                 // 1e5 * (k - k_prev), truncated
  int mode;               // SolveMode
  int res_type;
  unsigned long long neg_sources;
  unsigned long long neg_fluxes;
  long long num_fissionable;
  // batched pools: this solve's FSR rows are [row0, row0 + nrows) of the
  // pool's arrays; unused by single-problem contexts
  long long row0;
  long long nrows;
  int tc_error;           // a tensor-core source launch gave up waiting
  int negative_ok;        // pools: this solve allows negative fluxes
  // keff from the neutron balance (Solver::setKeffFromNeutronBalance):
  // absorption-rate accumulator and the leakage the last sweep tallied at
  // vacuum track ends
  double accum_abs;
  double leakage;
};

enum SolveMode { kModeEigen = 0, kModeSource = 1, kModeFlux = 2, kModeHook = 3 };

// Instances: K cross-section sets solved together over one track laydown.
// The problem's groups are the K instances' groups side by side (wide group
// k * G + g); the sweep treats them as one wide group set, while sources,
// keff and the normalisation stay per instance.
constexpr int kMaxInstances = 16;
struct InstState {
  double keff[kMaxInstances];
  double k_prev[kMaxInstances];
  double factor[kMaxInstances];
  double accum[kMaxInstances];       // fission-rate accumulators
  float scale[2][kMaxInstances];     // pending angular-flux scale per buffer
  unsigned int ticket;
  int dk;                            // largest |1e5 (k - k_prev)| this iteration
};

// One track as the single-problem sweeps visit it, stored in visiting
// order (longest first) so that the streams of a warp read theirs in one
// coalesced access: first segment, track id, segment count, angle row,
// flags and the two connecting tracks.
struct alignas(16) TrackRec {
  int64_t off;
  int32_t t, n, ang, flags, next[2];
};

struct SweepArgs {
  // [T] tracks in visiting order, read by the single-problem one-polar
  // instances (null, and elsewhere: order / seg_off / track_ang / flags /
  // next are read per track)
  const TrackRec* rec;
  const int2* segs;          // [S] {float length bits, fsr}
  const int64_t* seg_off;    // [T+1]
  const int32_t* order;      // [T] tracks by decreasing segment count
  const int32_t* track_ang;  // [T]
  const int32_t* next;       // [2T]
  const uint8_t* flags;      // [T]
  const float* weights;      // [A][Ph]
  const float* inv_sin;      // [A][Ph]
  const float* sigma_t;      // [M][G]
  const int32_t* fsr_mat;    // [R]
  const float* qt;           // [R][ld] reduced source / sigma_t
  const float* exp_table;    // [2][kExpTableSize]: 1 - exp(-x_i), exp(-x_i)
  float* phi;                // [R][ld] accumulated tallies
  float* psi[2];             // [T][2][F] angular-flux buffers
  DevScalars* sc;
  int64_t num_tracks;
  int num_groups;
  int ld;                    // row stride of phi / qt: G rounded up to even
  int num_materials;
  int lps;                   // lanes per track direction (1..32, power of 2)
  int check_done;            // return at once if sc->done is set
  int mat_packed;            // segs[].y = fsr | material << 24
  // Batched pools (null for a single problem): the solve each track belongs
  // to, whose state supplies the pending angular-flux scale and the done
  // flag; sc then only carries the pool's buffer index and ticket.
  const int32_t* track_slot; // [T]
  DevScalars* slots;         // [num_slots]
  int num_slots;
  // FSRs [hot_base, hot_base + hot_count) take a large share of all
  // segments (one region crossed by most tracks); each block tallies them in
  // shared memory and adds its totals once at its end.  Used by the
  // one-polar-value (3D) instances; hot_count = 0 elsewhere.
  int hot_base;
  int hot_count;             // 0 .. kMaxHotFsrs
  // Linear source (2D; null for the flat-source sweep): per segment
  // {length bits, fsr | material << 24, x bits, y bits} with (x, y) the
  // segment's forward start relative to its FSR centroid; per angle row
  // the forward direction (cos phi, sin phi); the reduced source moments
  // divided by sigma_t and the flux moment tallies, both [R][ld][2] with x
  // and y adjacent per group.
  const int4* segs_ls;       // [S]
  const float2* ang_dir;     // [A]
  const float* qxy;          // [R][ld][2]
  float* mom;                // [R][ld][2]
  // ... on explicit 3D tracks (null in 2D): each segment's z start, the
  // angle rows' 3D directions (cos phi sin theta, sin phi sin theta,
  // cos theta; ang_dir is then unused), the z source moment / sigma_t and
  // the z moment tallies
  const float* seg_z;        // [S]
  const float4* ang_dir3;    // [A]
  const float* qz;           // [R][ld]
  float* momz;               // [R][ld]
  // CMFD (null: none): coarse cell of every FSR (iy * cm_nx + ix), outgoing
  // partial currents [cells][4 faces][ld], and per track the boundary face
  // crossed at its forward / backward end where the flux is not
  // transferred (vacuum), else -1
  const int32_t* cm_cell;    // [R]
  float* cm_cur;             // [cells][4][ld]
  const int8_t* cm_end;      // [T][2]
  int cm_nx;
  // keff from the neutron balance: the leakage tally (null: not tallied)
  double* leakage;
  // instances (null: one problem): each wide group's angular flux takes the
  // pending scale of its instance, group / inst_groups
  InstState* inst;
  int inst_groups;
};

constexpr int kMaxHotFsrs = 8;

// Kernels that may take more than 48 KB of dynamic shared memory (the
// sweeps, whose tables grow with the materials, and the source kernels)
// have their limit raised once per device to the device's opt-in maximum,
// when a context or a server is created: never at launch, since the server
// launches them inside CUDA-graph captures, where changing a function
// attribute is not captured and fails the launch.
template <class K>
void raise_smem_limit(K* kern, int optin) {
  cudaFuncAttributes fa;
  if (cudaFuncGetAttributes(&fa, kern) != cudaSuccess) return;
  cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       optin - (int) fa.sharedSizeBytes);
}
void configure_sweeps(int optin);      // sweep.cu
void configure_ls_sweeps(int optin);   // ls_sweep_p*.cu via sweep.cu
void configure_otf_sweeps(int optin);  // otf_sweep.cu
void configure_sources(int optin);     // solver_kernels.cu
// Once per device (the current one): the above with its opt-in maximum.
void configure_kernels();

struct SolverArgs {
  const float* sigma_t;      // [M][G]
  const float* sigma_s;      // [M][G][G] dest-major
  const float* sigma_s_T;    // [M][G][G] origin-major (transposed)
  const float* nu_sigma_f;   // [M][G]
  const float* chi;          // [M][G]
  const uint8_t* fissile;    // [M]
  const int32_t* fsr_mat;    // [R]
  const float* fsr_vol;      // [R]
  const float* fixed;        // [R][ld] or null
  const float* scat_out;     // [M][G] total scattering out of each group
  const float* sigma_f;      // [M][G] or null
  float* phi;                // [R][ld]
  float* phi_old;            // [R][ld]
  float* qt;                 // [R][ld]
  float* psi[2];
  DevScalars* sc;
  int64_t num_fsrs;
  int64_t num_psi;           // 2*T*F
  int num_groups;
  int ld;                    // row stride of the [R][*] arrays (even, >= G)
  int num_materials;
  int check_done;
  // Batched pools (null for a single problem): the solve owning each FSR row
  // (-1: unused row), the per-solve states, and one FP64 partial per row for
  // the per-solve reductions.
  const int32_t* row_slot;   // [R]
  DevScalars* slots;         // [num_slots]
  double* row_val;           // [R]
  int num_slots;
  // 3xTF32 tensor-core source contraction (null / 0: CUDA-core kernel):
  // FSR ids grouped by material in tiles of kTcRows (-1 pads a tile), the
  // material of each tile, and per material the scattering matrix split
  // into TF32 high and low parts in the MMA's operand layout.
  const int32_t* tc_rows;    // [tc_tiles * kTcRows]
  const int32_t* tc_tile_mat;// [tc_tiles]
  const float* tc_b;         // [M][2][tc_n][tc_k]
  int tc_tiles;
  int tc_n, tc_k;            // padded destination / origin group counts
  // polls of an mbarrier before the tensor-core source kernel gives up on
  // its first wait (its drain waits use the full default limit)
  unsigned tc_wait_limit;
  // Linear source (null: flat source): flux moments and reduced source
  // moments / sigma_t ([R][ld][2], x and y adjacent per group), the inverse
  // expansion matrix per FSR (xx, yy, xy), the source constants [R][3][ld]
  // and the fixed source moments [R][ld][2] (or null).  On explicit 3D
  // tracks (momz set) also the z moments ([R][ld] each) and six
  // coefficients (xx, yy, xy, xz, yz, zz) per FSR: ls_ilem [R][6],
  // ls_const [R][6][ld].
  float* mom;
  float* qxy;
  const float* ls_ilem;      // [R][3] or [R][6]
  const float* ls_const;     // [R][3][ld] or [R][6][ld]
  const float* fixed_xy;
  float* momz;               // [R][ld] or null
  float* qz;                 // [R][ld] or null
  const float* fixed_z;      // [R][ld] or null
  int negative_ok;           // Solver::allowNegativeFluxes
  // keff = fission / (absorption + leakage) instead of keff *= fission / R
  // (Solver::setKeffFromNeutronBalance); absorption = sigma_t - scat_out
  int keff_balance;
  // transport stabilization (null: off): per material and group the pair
  // (c1, c2) of phi = (phi + c1 * phi_start) * c2, phi_start the flux at
  // the start of the iteration
  const float2* stab;        // [M][ld]
  // instances (null: one problem): per-instance keff, normalisation and
  // angular-flux scales; inst_groups groups per instance
  InstState* inst;
  int inst_groups;
  int num_instances;
};

// Rows (FSRs) per tile of the tensor-core source kernel: the MMA's M.
constexpr int kTcRows = 128;
// mbarrier polls before a wait of the tensor-core source kernel gives up
constexpr unsigned kTcDefaultWaitLimit = 1u << 22;

// Records the text returned by moc_last_error on this thread; returns code.
int set_error(int code, const char* msg);

// ---- launchers (sweep.cu) ------------------------------------------------
// Chooses the kernel instance for (Ph, slots, exp kind).  Returns false if
// no instance exists.
bool launch_sweep(const SweepArgs& a, int polar_half, int slots, int exp_kind,
                  cudaStream_t stream);
int sweep_max_slots(int polar_half);
bool sweep_lps_supported(int lps);
void launch_attenuation(int kind, const float* x, float* g, int64_t n,
                        const float* exp_table, cudaStream_t s);
// Writes each segment's material into the top 8 bits of its FSR word
// (valid when num_fsrs < 2^24 and num_materials <= 256); idempotent.
void launch_pack_materials(int2* segs, int64_t num_segments,
                           const int32_t* fsr_mat, cudaStream_t stream);
// Packs and checks uploaded segments on the device (*bad = the first bad
// index, or left as it was) and counts the segments of the last
// kMaxHotFsrs FSR ids into tail[kMaxHotFsrs] (tail[i]: FSR R - kMaxHotFsrs + i).
void launch_pack_segments(const float* len, const int32_t* fsr, int2* out,
                          int64_t S, int64_t R, unsigned long long* bad,
                          unsigned long long* tail, cudaStream_t stream);

// ---- launchers (solver_kernels.cu) ---------------------------------------
// iteration < 0 reads the device iteration counter; fused also zeroes phi
// after reading it (the tallies of the sweep that follows)
void launch_compute_sources(const SolverArgs& a, int iteration, int fused,
                            cudaStream_t s);
// add-source + fission-rate reduction; update: 0 none, 1 eigen update of
// keff / factor / buffer scale, 2 keff only (the factor follows the
// stabilization)
void launch_add_source(const SolverArgs& a, int update, cudaStream_t s);
// normalise by sc->factor (if normalise), residual of res_type vs phi_old,
// store phi into phi_old (if store), finish the iteration (if finish)
void launch_residual(const SolverArgs& a, int res_type, int normalise,
                     int store, int finish, cudaStream_t s);
// fission-rate reduction of phi; what: 0 keff update, 1 normalise hook
void launch_fission_rate(const SolverArgs& a, int what, cudaStream_t s);
// transport stabilization of phi from `base` (the flux at the start of the
// iteration); in_loop: only from the second iteration on, and the
// normalisation factor of the stabilized flux is computed as
// launch_fission_rate(what = 1) does; base_mom / base_momz: the flux
// moments at the start of the iteration, stabilized alongside (null: the
// moments are left as they are)
void launch_stabilize(const SolverArgs& a, const float* base, int in_loop,
                      cudaStream_t s, const float* base_mom = nullptr,
                      const float* base_momz = nullptr);
// the fission (which = 0) or scattering (which = 1) part of the reduced
// source alone into qt (CPUSolver::computeFSRFissionSources /
// computeFSRScatterSources)
void launch_partial_sources(const SolverArgs& a, int which, cudaStream_t s);
// instances: each instance's fission-rate total; what = 0: the eigenvalue
// update (keff, normalisation factor, angular-flux scale, largest dk);
// what = 1: the normalisation of the starting flux (phi scaled in place)
void launch_instance_rates(const SolverArgs& a, int what, cudaStream_t s);
void launch_scale_phi(const SolverArgs& a, cudaStream_t s);
void launch_zero_phi(const SolverArgs& a, cudaStream_t s);
void launch_fill(float* p, int64_t n, float v, cudaStream_t s);
void launch_fill_chi(float* phi, const float* chi, int64_t R, int G, int ld,
                     cudaStream_t s);
void launch_fsr_rates(const SolverArgs& a, double* out, int nu,
                      cudaStream_t s);

// ---- tensor-core sources (sources_tc.cu) -----------------------------------
// Group counts the 3xTF32 kernel takes, and its operand sizes.
bool tc_sources_supported(int num_groups);
int tc_pad_n(int num_groups);   // destination groups padded for the MMA's N
int tc_pad_k(int num_groups);   // origin groups padded to the MMA's K step
// Splits every material's [dest][orig] scattering matrix into TF32 high and
// low parts laid out as the MMA's B operand (host side): out[M][2][n][k].
void tc_pack_scattering(const float* sigma_s, int M, int G,
                        std::vector<float>& out);
void launch_sources_tc(const SolverArgs& a, int iteration, int zero_phi,
                       cudaStream_t s);

// ---- on-the-fly 3D segmentation (otf_sweep.cu) ----------------------------
// Extruded 3D tracks cut from their radial segments during the sweep.
struct OtfArgs {
  const int4* trk;          // [T] radial track, first radial segment (index
                            //     within it, in traversal order), count,
                            //     1 if the traversal runs against it
  const float4* trk_f;      // [T] start a0 along the radial traversal, span
                            //     A, height above the cut at a0, unused
  const float4* ang;        // [A] cot(theta), 1 / cot(theta), 1 / sin(theta)
  const int2* rad_segs;     // [S2] {length bits, fsr | material << 24}
  const float* rad_start;   // [S2] start of each radial segment on its track
  const int64_t* rad_off;   // [T2 + 1]
  const float* rad_total;   // [T2] radial track lengths
  int above;                // fsr | material << 24 of the region above the cut
  int above_fsr;
};
bool launch_otf_sweep(const SweepArgs& a, const OtfArgs& o, int slots,
                      cudaStream_t stream);
constexpr int kMaxOtfSlots = 4;

// ---- linear source (linear_source.cu, solver_kernels.cu, ls_sweep_*.cu) ----
// Largest group pairs per lane of the linear-source sweep instances.
constexpr int kMaxLsSlots = 5;
// LinearExpansionGenerator (2D): volume moments and source constants per
// FSR summed in FP64 over the FSR's segments, then inverted; outputs
// ilem[R][3] and cst[R][3][ld] (float) and through *num_flat the FSRs whose
// matrix is singular (flat source there); with seg_z and pol_cos (explicit
// 3D tracks: pol_sin, pol_cos and pol_wgt per angle row, Ph = 1) the six
// 3D coefficients, ilem[R][6] and cst[R][6][ld].  Allocates and frees its own
// scratch (segment buckets by FSR); returns 0 or the cudaError_t.
int launch_ls_constants(const int4* segs_ls, const int64_t* seg_off,
                        const int32_t* track_ang, int64_t T, int64_t S,
                        const double* ang_dir, const double* ang_wgt,
                        const double* pol_sin, const double* pol_wgt, int Ph,
                        const float* sigma_t, const float* fsr_vol,
                        const int32_t* fsr_mat, int64_t R, int G, int ld,
                        float* ilem, float* cst, unsigned int* num_flat,
                        cudaStream_t s, const float* seg_z = nullptr,
                        const double* pol_cos = nullptr);
// The track of every segment from the segment offsets (seg_off[0] = 0).
void launch_ls_seg_track(const int64_t* seg_off, int64_t T, int32_t* seg_track,
                         cudaStream_t s);
// The same constants from segment buckets the caller built (segment ids
// sorted by FSR, and the track of every segment) and FP64 scratch of
// ls_constants_scratch(R, ld, 3D) doubles: asynchronous, nothing
// allocated.
int64_t ls_constants_scratch(int64_t R, int ld, bool d3);
void launch_ls_constants_bucketed(const int4* segs_ls, const int32_t* list,
                                  int64_t S, const int32_t* seg_track,
                                  const int32_t* track_ang,
                                  const double* ang_dir, const double* ang_wgt,
                                  const double* pol_sin, const double* pol_wgt,
                                  int Ph, const float* sigma_t,
                                  const float* fsr_vol, const int32_t* fsr_mat,
                                  int64_t R, int G, int ld, float* ilem,
                                  float* cst, unsigned int* num_flat,
                                  double* scratch, cudaStream_t s,
                                  const float* seg_z = nullptr,
                                  const double* pol_cos = nullptr);
// Builds segs_ls from the packed segments and the start positions.
void launch_ls_pack_segments(const int2* segs, const float* x, const float* y,
                             int4* out, int64_t S, cudaStream_t s);
// Copies the FSR / material words of segs into segs_ls (after new FSR
// materials were packed into segs).
void launch_ls_refresh_ids(const int2* segs, int4* out, int64_t S,
                           cudaStream_t s);
// Flat + linear sources in one pass (CPULSSolver::computeFSRSources);
// fused zeroes phi and the moments for the sweep that follows.
void launch_ls_sources(const SolverArgs& a, int iteration, int fused,
                       cudaStream_t s);
// CPULSSolver::addSourceToScalarFlux; update as launch_add_source.
void launch_ls_add_source(const SolverArgs& a, int update, cudaStream_t s);
// Moments *= sc->factor (the normalisation of the eigenvalue loop).
void launch_ls_scale_moments(const SolverArgs& a, cudaStream_t s);
bool launch_ls_sweep(const SweepArgs& a, int polar_half, int slots,
                     cudaStream_t stream);

// ---- batched pools (solver_kernels.cu) -------------------------------------
// The loop body of every live solve of a pool; a.num_fsrs is the end of the
// highest row in use.  Sources take each row's keff and iteration from its
// solve; add-source leaves each eigenvalue row's nu-fission rate in row_val;
// rate_finish (one block per solve) updates keff, the normalisation factor
// and the pending angular-flux scale; residual normalises, leaves each row's
// residual term in row_val and stores phi_old; residual_finish ends the
// iteration of every live solve (convergence, counters, done).  In a pool
// of linear-source solves (a.mom set) the sources and add-source are
// launch_ls_sources / launch_ls_add_source, which take the same per-row
// states, and residual also normalises the flux moments.
void launch_batch_sources(const SolverArgs& a, cudaStream_t s);
void launch_batch_add_source(const SolverArgs& a, cudaStream_t s);
void launch_batch_rate_finish(const SolverArgs& a, cudaStream_t s);
void launch_batch_residual(const SolverArgs& a, cudaStream_t s);
void launch_batch_residual_finish(const SolverArgs& a, cudaStream_t s);
// Initial state of one admitted solve: rows [r0, r0 + n) of phi and phi_old
// set to value, qt (and with a linear source the flux and source moments)
// zeroed.
void launch_batch_init_rows(const SolverArgs& a, int64_t r0, int64_t n,
                            float value, cudaStream_t s);
// Rebases one admitted solve's track data from its own numbering to the
// pool's: FSR ids (+r0) with the pool material of the FSR (fsr_mat, already
// in pool numbering) packed into the top 8 bits, next-track links (+t0),
// angle rows (+a0), segment offsets (+s0, T + 1 of them); track_slot of the
// T + 1 track entries is set to slot.
void launch_batch_rebase(int2* segs, int64_t S, const int32_t* fsr_mat,
                         int32_t r0, int64_t* seg_off, int32_t* next,
                         int32_t* track_ang, int32_t* track_slot, int64_t T,
                         int64_t s0, int32_t t0, int32_t a0, int32_t slot,
                         cudaStream_t s);

// CMFD coarse solve on the device (cmfd.cu): state kept between
// iterations of a solve, and the inputs of the single-block solver.
struct CmfdDevState {
  double keff;          // coarse eigenvalue of the previous solve (1 at start)
  int valid;            // the relaxation history holds a previous step
  int power_iters;      // power iterations of the last coarse solve
  int linear_iters;     // SOR sweeps of the last coarse solve
  int failed;           // the last coarse solve did not converge
  float max_ratio;      // prolongation ratio farthest from 1
  int pad;
};

struct CmfdArgs {
  int nx, ny, C, E, G, P, n_edc, ld;
  int bc[4];                    // faces x-min, y-min, x-max, y-max: 0 vacuum
  float relax, sor;
  int flux_limiting, unbounded;
  const float* wx;              // [nx]
  const float* wy;              // [ny]
  const int32_t* gstart;        // [E + 1] first group of each coarse group
  const int32_t* cell_pair;     // [C + 1] pairs of each cell (cell-major)
  const int32_t* color_cells;   // [C] red cells ((ix + iy) even), then black
  const int32_t* cell_pos;      // [C] position of each cell in color_cells
  const int32_t* nbr_j;         // [4][C] neighbours by face, colour order
  int n_color0;
  const int32_t* pair_mat;      // [P]
  const float* st;              // [M][G] total cross sections
  const float* nf;              // [M][G] nu-fission
  const float* chi_m;           // [M][E] chi summed over each coarse group
  const float* ss_m;            // [M][G][E] scattering from h into coarse g
  const float* cell_vol;        // [C]
  const float* edc_mu;          // [n_edc]
  const float* edc_w;           // [n_edc]
  const double* S;              // [P][G] sums of phi * V
  const float* cur;             // [C][4][ld] partial currents
  float* work;                  // scratch (cmfd_work_floats)
  float* dcorr_old;             // [C][4][E] relaxation history
  float* ratio;                 // [C][E] prolongation factors
  float* flux_old;              // [C][E] coarse fluxes, unit fission source
  float* flux_new;              // [C][E]
  CmfdDevState* cm;
  DevScalars* sc;
  // The cell-parallel coarse solve (one thread per cell over a cluster of
  // map_nb blocks of map_threads threads; map_nb = 0: not available):
  // thread gid = block * map_threads + t holds the cell at colour position
  // map_j[gid] (-1: none); map_nslot[f][gid] is the slot of its face-f
  // neighbour's iterate in the block's shared memory (its own cell's slot t
  // when there is none), slots past map_threads holding copies of cells of
  // other blocks; map_push[k][gid] (k < 2) = block << 24 | slot of a copy
  // of this cell in another block (-1: none).
  const int32_t* map_j;
  const int32_t* map_nslot;
  const int32_t* map_push;
  int map_nb, map_threads, map_slots;
  int solve_kind;               // 0 cell-parallel when mapped, 2 one block
};

// Threads a block of the cell-parallel coarse solve may hold for E coarse
// groups (one cell each, its coefficients in registers), and the blocks of
// a cluster at most.
#ifndef MOC_CMFD_CELLS_THREADS_HI
#define MOC_CMFD_CELLS_THREADS_HI 320
#endif
constexpr int cmfd_cells_threads(int E) {
  return E <= 2 ? 768 : E <= 4 ? 512 : E <= 6 ? 384 : MOC_CMFD_CELLS_THREADS_HI;
}
constexpr int kCmfdMaxClusterBlocks = 8;
constexpr int kCmfdMaxCellGroups = 8;
// Dynamic shared memory (bytes) of a block of the cell-parallel solve.
int64_t cmfd_cells_smem(int E, int threads, int slots);

// Scratch floats the device coarse solve needs for C cells, E groups.
int64_t cmfd_work_floats(int C, int E);
// One coarse solve (Cmfd::computeKeff): collapse and matrices over the GPU,
// then the power iteration with red-black SOR and the ratios, cell-parallel
// over a cluster when the map is set and solve_kind is 0, else on one
// block; sets sc->keff.  Returns at once when the solve is done.  Returns
// false when the cell-parallel kernel could not be launched (the one-block
// solve ran instead).
bool launch_cmfd_solve(const CmfdArgs& a, cudaStream_t s);

// CMFD (cmfd.cu): per (coarse cell, material) pair the sums of phi * volume
// over its FSRs, [P][G] FP64, from the CSR list pair_off [P + 1] /
// pair_fsr [R]; and the prolongation phi[r][g] *= ratio[cell(r)][group(g)]
// ([cells][E] FP64), which also sets sc->keff to the coarse eigenvalue.
// Both return at once when sc->done is set.
void launch_cmfd_pair_sums(const float* phi, const float* vol,
                           const int32_t* pair_off, const int32_t* pair_fsr,
                           int P, int G, int ld, double* out, DevScalars* sc,
                           cudaStream_t s);
// k-nearest prolongation stencils (CSR per FSR; off null: none).
struct CmfdStencil {
  const int32_t* off;    // [R + 1]
  const int32_t* cell;   // coarse cells
  const float* coef;     // their weights
};
// mom (linear source, [R][ld][2]) is scaled with phi when not null; ratios
// are bounded to [0.05, 20] from MOC iteration unbounded + 1 on.
void launch_cmfd_prolong(float* phi, float* mom, const int32_t* fsr_cell,
                         const int32_t* group_of, const float* ratio,
                         const CmfdStencil& st, int64_t R, int G, int ld,
                         int E, int unbounded, DevScalars* sc,
                         cudaStream_t s);

}  // namespace moc
