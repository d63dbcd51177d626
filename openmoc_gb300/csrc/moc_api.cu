// Host side of libopenmoc_gb300.so: the solver context, uploads, the
// device-resident iteration drivers and the C ABI of include/openmoc_gb300.h.
//
// The iteration drivers restate Solver::computeEigenvalue, computeSource and
// computeFlux (src/Solver.cpp:1352-1700) with every per-iteration scalar kept
// on the device (moc::DevScalars).  A block of iterations is enqueued
// without host synchronisation; kernels of iterations after convergence
// return at once (DevScalars::done), and the host checks the state once per
// block, the only device-to-host traffic of a solve besides the result.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <numeric>
#include <string>
#include <map>
#include <mutex>
#include <tuple>
#include <vector>

#include "../../include/openmoc_gb300.h"
#include "cmfd_internal.h"
#include "moc_internal.cuh"

namespace {

thread_local std::string g_error;

int fail(int code, const std::string& msg) {
  g_error = msg;
  return code;
}

#define MOC_CUDA(call)                                                    \
  do {                                                                    \
    cudaError_t e_ = (call);                                              \
    if (e_ != cudaSuccess)                                                \
      return fail(MOC_ERR_CUDA, std::string(#call) + ": " +               \
                                    cudaGetErrorString(e_));              \
  } while (0)

#define MOC_CHECK(cond, code, msg) \
  do {                             \
    if (!(cond)) return fail(code, msg); \
  } while (0)

#define MOC_TRY(expr)        \
  do {                       \
    int s_ = (expr);         \
    if (s_ != MOC_OK) return s_; \
  } while (0)

// Device memory of the contexts is kept for reuse.  A context created,
// solved and destroyed per request (the end-to-end path) gets its buffers
// back from this cache instead of from cudaMalloc / cudaFree, whose driver
// work and implicit device synchronisation cost about a millisecond per
// context.  A block goes back to the cache only when no work can still use
// it: dfree synchronises the device first, as cudaFree would, unless the
// caller has (moc_destroy, after its stream).  At most kMaxIdleBytes stay
// cached; moc_release_cached_memory returns them to the driver.
struct DeviceBlockCache {
  std::mutex mu;
  std::map<void*, std::pair<int, size_t>> live;       // block -> device, bytes
  std::multimap<std::pair<int, size_t>, void*> idle;  // (device, bytes) -> block
  size_t idle_bytes = 0;
};
DeviceBlockCache g_blocks;
constexpr size_t kMaxIdleBytes = size_t(16) << 30;
thread_local bool g_device_idle = false;   // set while moc_destroy frees
// pinned host copies of the device scalars, kept likewise
std::mutex g_pinned_mu;
std::vector<void*> g_pinned_scalars;
// a page-locked bounce buffer for row copies to pageable host memory (a
// device-to-pageable copy that also changes the row pitch runs at a
// fraction of the link's rate); grown on demand, guarded by its mutex
std::mutex g_bounce_mu;
void* g_bounce = nullptr;
size_t g_bounce_bytes = 0;

// Frees every idle block of `device` (all devices: -1).
void release_idle(int device) {
  std::lock_guard<std::mutex> lk(g_blocks.mu);
  for (auto it = g_blocks.idle.begin(); it != g_blocks.idle.end();) {
    if (device >= 0 && it->first.first != device) {
      ++it;
      continue;
    }
    int cur = 0;
    cudaGetDevice(&cur);
    cudaSetDevice(it->first.first);
    cudaFree(it->second);
    cudaSetDevice(cur);
    g_blocks.idle_bytes -= it->first.second;
    it = g_blocks.idle.erase(it);
  }
}

size_t idle_bytes_on(int device) {
  std::lock_guard<std::mutex> lk(g_blocks.mu);
  size_t n = 0;
  for (const auto& kv : g_blocks.idle)
    if (kv.first.first == device) n += kv.first.second;
  return n;
}

template <typename T>
int dalloc(T** p, size_t n) {
  *p = nullptr;
  if (n == 0) n = 1;
  const size_t bytes = (n * sizeof(T) + 255) & ~(size_t) 255;
  int dev = 0;
  MOC_CUDA(cudaGetDevice(&dev));
  {
    // an idle block of this device at most twice the size
    std::lock_guard<std::mutex> lk(g_blocks.mu);
    auto it = g_blocks.idle.lower_bound({dev, bytes});
    if (it != g_blocks.idle.end() && it->first.first == dev &&
        it->first.second <= 2 * bytes) {
      *p = static_cast<T*>(it->second);
      g_blocks.live[it->second] = it->first;
      g_blocks.idle_bytes -= it->first.second;
      g_blocks.idle.erase(it);
      return MOC_OK;
    }
  }
  cudaError_t e = cudaMalloc((void**) p, bytes);
  if (e == cudaErrorMemoryAllocation) {
    cudaGetLastError();
    release_idle(dev);
    e = cudaMalloc((void**) p, bytes);
  }
  if (e == cudaErrorMemoryAllocation) {
    cudaGetLastError();
    *p = nullptr;
    return fail(MOC_ERR_MEMORY, "device memory exhausted allocating " +
                                    std::to_string(n * sizeof(T)) + " bytes");
  }
  MOC_CUDA(e);
  std::lock_guard<std::mutex> lk(g_blocks.mu);
  g_blocks.live[(void*) *p] = {dev, bytes};
  return MOC_OK;
}

template <typename T>
void dfree(T*& p) {
  if (!p) return;
  void* v = (void*) p;
  p = nullptr;
  std::pair<int, size_t> blk{-1, 0};
  {
    std::lock_guard<std::mutex> lk(g_blocks.mu);
    auto it = g_blocks.live.find(v);
    if (it != g_blocks.live.end()) {
      blk = it->second;
      g_blocks.live.erase(it);
    }
  }
  if (blk.first < 0 || blk.second > kMaxIdleBytes) {
    cudaFree(v);
    return;
  }
  if (!g_device_idle) cudaDeviceSynchronize();
  std::lock_guard<std::mutex> lk(g_blocks.mu);
  if (g_blocks.idle_bytes + blk.second > kMaxIdleBytes) {
    cudaFree(v);
    return;
  }
  g_blocks.idle.insert({blk, v});
  g_blocks.idle_bytes += blk.second;
}

}  // namespace

namespace moc {
int set_error(int code, const char* msg) { return fail(code, msg); }
}  // namespace moc

// One timed sweep-kernel configuration of the autotuner.
struct moc_tune_entry {
  int lps, slots, exp_kind;
  float ms;
};

struct moc_ctx {
  moc_dims d{};
  cudaStream_t stream = nullptr;

  // tracks
  int2* segs = nullptr;
  int64_t* seg_off = nullptr;
  int32_t* order = nullptr;
  int32_t* track_ang = nullptr;
  int32_t* next = nullptr;
  uint8_t* flags = nullptr;
  moc::TrackRec* trec = nullptr;   // [T] in visiting order
  // quadrature
  float* weights = nullptr;
  float* inv_sin = nullptr;
  // materials
  float* sigma_t = nullptr;
  float* sigma_s = nullptr;
  float* sigma_s_T = nullptr;         // [M][orig][dest]
  float* nu_sigma_f = nullptr;
  float* chi = nullptr;
  float* scat_out = nullptr;
  float* sigma_f = nullptr;
  uint8_t* fissile = nullptr;
  std::vector<uint8_t> h_fissile;
  std::vector<float> h_chi;
  // FSRs
  int32_t* fsr_mat = nullptr;
  float* fsr_vol = nullptr;
  float* fixed = nullptr;
  // state
  float* phi = nullptr;
  float* phi_old = nullptr;
  float* qt = nullptr;
  float* psi[2] = {nullptr, nullptr};
  float* exp_table = nullptr;
  double* rates = nullptr;
  float* flush = nullptr;             // L2 flush buffer (measurement only)
  int64_t flush_n = 0;
  moc::DevScalars* sc = nullptr;      // device
  moc::DevScalars* hsc = nullptr;     // pinned host mirror

  int mat_packed = 0;
  bool have_tracks = false, have_quad = false, have_mats = false,
       have_fsrs = false;
  double threshold = 1e-5;
  int exp_kind = MOC_EXP_TABLE;
  int exp_user_set = 0;      // evaluator fixed by the caller
  int shape_user_set = 0;    // kernel shape fixed by the caller
  int autotune = 1;          // time shapes / evaluators at the first solve
  bool tuned = false;
  std::vector<moc_tune_entry> tune_log;
  int lps = 0, slots = 0;
  int num_iterations = 0;
  double keff = 1.0;
  double residual = 0.0;
  long long num_fissionable = 0;
  int64_t launches = 0;
  double sweep_ms = 0.0;
  int64_t num_sweeps = 0;
  int iters_per_sync = 4;
  std::vector<cudaEvent_t> ev;   // event pairs around sweeps
  // 3xTF32 tensor-core sources: FSR ids by material in tiles, the material
  // of each tile, the split scattering operands
  int source_kind = MOC_SOURCES_AUTO;
  int32_t* tc_rows = nullptr;
  int32_t* tc_tile_mat = nullptr;
  float* tc_b = nullptr;
  int tc_tiles = 0;
  int64_t tc_wait_limit = -1;  // < 0: the kernel's default
  // FSRs with the last ids that take a large share of the segments (the
  // moderator above an extruded lattice): tallied in shared memory by the
  // 3D sweep instances
  int hot_base = 0, hot_count = 0;
  // Linear source (moc_set_linear_source): 16-byte segment words with the
  // start positions, per-angle FP64 data for the expansion constants (dir
  // [A][2], azimuthal weight [A], sin theta [A][Ph], polar weight [A][Ph],
  // in 3D cos theta [A]; one buffer), float directions, flux / source
  // moments [R][ld][2], inverse expansion matrices [R][3], constants
  // [R][3][ld] and fixed source moments [R][ld][2].  On explicit 3D tracks
  // (ls3d) also the segments' z starts, 3D directions, the z moments
  // [R][ld] and six coefficients: [R][6], [R][6][ld].
  bool ls = false;
  bool ls3d = false;
  int4* segs_ls = nullptr;
  double* ls_ang = nullptr;
  float2* ls_dir = nullptr;
  float* mom = nullptr;
  float* qxy = nullptr;
  float* ls_ilem = nullptr;
  float* ls_const = nullptr;
  float* fixed_xy = nullptr;
  float* ls_segz = nullptr;
  float4* ls_dir3 = nullptr;
  float* momz = nullptr;
  float* qz = nullptr;
  float* fixed_z = nullptr;
  int64_t ls_num_flat = 0;
  int negative_ok = 0;       // Solver::allowNegativeFluxes
  int keff_balance = 0;      // Solver::setKeffFromNeutronBalance
  // transport stabilization (Solver::stabilizeTransport): type DIAGONAL 0,
  // YAMAMOTO 1, GLOBAL 2; per material and group the pair (c1, c2), made
  // from the host copies of sigma_t and the scattering diagonal and the
  // materials the FSRs use; the flux saved by the computeStabilizingFlux
  // hook
  // instances (moc_set_instances): K cross-section sets over one laydown,
  // inst_groups groups each; 0: one problem
  int num_instances = 0;
  int inst_groups = 0;
  moc::InstState* inst = nullptr;
  int stab_on = 0;
  int stab_type = 0;
  double stab_factor = 0.0;
  bool stab_dirty = true;
  float2* stab = nullptr;
  float* stab_base = nullptr;
  // the linear source's flux moments (xy, z) at the start of the iteration,
  // the base of their stabilization
  float* stab_mom = nullptr;
  float* stab_momz = nullptr;
  std::vector<float> h_sigma_t, h_scat_diag;
  std::vector<uint8_t> h_mat_used;
  // On-the-fly 3D segmentation (moc_set_otf_tracks): 3D track descriptors,
  // per-angle cot / 1/cot / 1/sin, the radial segments, and the track order
  // by radial segments crossed
  bool otf = false;
  int4* otf_trk = nullptr;
  float4* otf_trk_f = nullptr;
  float4* otf_ang = nullptr;
  int2* otf_rad = nullptr;
  float* otf_rad_start = nullptr;
  int64_t* otf_rad_off = nullptr;
  float* otf_rad_total = nullptr;
  int32_t* otf_order = nullptr;
  int64_t otf_S2 = 0;
  int otf_above_fsr = 0;
  int otf_above_word = 0;    // above_fsr | material << 24
  // CMFD (moc_set_cmfd): the coarse cell of every FSR, the boundary face at
  // each track end, outgoing partial currents [cells][4][ld], coarse group
  // of each group, FSRs by (cell, material) pair (CSR), their FP64 flux
  // sums [P][G] and the prolongation ratios [cells][E]; pinned host copies
  // of the sums and currents; the host coarse solver
  moc_cmfd::Solver* cmfd = nullptr;
  std::vector<int32_t> h_cm_cell;
  std::vector<double> cm_edc_mu_h, cm_edc_w_h;   // as given (flat source)
  int32_t* cm_pro_off = nullptr;     // k-nearest stencils (null: none)
  int32_t* cm_pro_cell = nullptr;
  float* cm_pro_coef = nullptr;
  int32_t* cm_cell = nullptr;
  int8_t* cm_end = nullptr;
  float* cm_cur = nullptr;
  int32_t* cm_group = nullptr;
  int32_t* cm_pair_off = nullptr;
  int32_t* cm_pair_fsr = nullptr;
  double* cm_sums = nullptr;
  float* cm_ratio = nullptr;
  double* h_cm_sums = nullptr;
  float* h_cm_cur = nullptr;
  std::vector<float> h_cm_ratio;
  int64_t cm_sums_n = 0;
  // the device coarse solve (default; cm_host: the FP64 host solve): its
  // state, scratch, relaxation history, coarse fluxes, and the collapse
  // inputs (pairs of each cell, pair materials, chi per coarse group and
  // scattering into each coarse group by material, cell volumes, widths,
  // coarse group starts, Larsen quadrature)
  bool cm_host = false;
  moc::CmfdDevState* cm_state = nullptr;
  float* cm_work = nullptr;
  float* cm_dcorr = nullptr;
  float* cm_flux_old = nullptr;
  float* cm_flux_new = nullptr;
  int32_t* cm_cell_pair = nullptr;
  int32_t* cm_color_cells = nullptr;
  int32_t* cm_cell_pos = nullptr;
  int32_t* cm_nbr_j = nullptr;
  int cm_n_color0 = 0;
  // the cell-parallel coarse solve's map (moc::CmfdArgs::map_*; nb 0: the
  // mesh is solved on one block) and the solve asked for (0 automatic,
  // 2 one block, 3 cell-parallel)
  int32_t* cm_map_j = nullptr;
  int32_t* cm_map_nslot = nullptr;
  int32_t* cm_map_push = nullptr;
  int cm_map_nb = 0, cm_map_threads = 0, cm_map_slots = 0;
  int cm_solve_kind = 0;
  int32_t* cm_pair_mat = nullptr;
  float* cm_chi_m = nullptr;
  float* cm_ss_m = nullptr;
  float* cm_cell_vol = nullptr;
  float* cm_wx = nullptr;
  float* cm_wy = nullptr;
  int32_t* cm_gstart = nullptr;
  float* cm_edc_mu = nullptr;
  float* cm_edc_w = nullptr;
};

namespace {

int64_t fluxes_per_track(const moc_ctx* c) {
  return (int64_t) c->d.num_groups * c->d.num_polar_half;
}

int64_t num_psi(const moc_ctx* c) {
  return 2 * c->d.num_tracks * fluxes_per_track(c);
}

// Row stride of the device [R][*] arrays: G rounded up to even, so that a
// group pair is one aligned 8-byte access.
int row_stride(const moc_ctx* c) {
  return c->d.num_groups + (c->d.num_groups & 1);
}

// Elements of a device [R][ld] array.
int64_t num_flux(const moc_ctx* c) {
  return c->d.num_fsrs * row_stride(c);
}

// Elements of the host-side [R][G] view.
int64_t num_host_flux(const moc_ctx* c) {
  return c->d.num_fsrs * c->d.num_groups;
}

// keff from the neutron balance: the flat-source sweeps of stored
// segments tally the leakage; CMFD supplies its own keff
bool balance_keff(const moc_ctx* c) {
  return c->keff_balance && !c->ls && !c->otf && !c->cmfd;
}

// Instances: keff 1, no pending scale, empty accumulators.
int reset_instances(moc_ctx* c) {
  moc::InstState h{};
  for (int k = 0; k < moc::kMaxInstances; k++) {
    h.keff[k] = h.k_prev[k] = h.factor[k] = 1.0;
    h.scale[0][k] = h.scale[1][k] = 1.0f;
  }
  MOC_CUDA(cudaMemcpyAsync(c->inst, &h, sizeof(h), cudaMemcpyHostToDevice,
                           c->stream));
  MOC_CUDA(cudaStreamSynchronize(c->stream));
  return MOC_OK;
}

// The transport-stabilization coefficients (c1, c2) per material and group
// (CPUSolver::computeStabilizingFlux / stabilizeFlux, src/CPUSolver.cpp:
// 2665-2810), rebuilt after a material or FSR upload.
int ensure_stab(moc_ctx* c) {
  if (!c->stab_on || (!c->stab_dirty && c->stab)) return MOC_OK;
  const int M = c->d.num_materials, G = c->d.num_groups, ld = row_stride(c);
  MOC_CHECK((int) c->h_sigma_t.size() == M * G &&
                (int) c->h_mat_used.size() == M,
            MOC_ERR_STATE, "upload materials and FSRs before stabilizing");
  const double f = c->stab_factor;
  std::vector<float2> cf((size_t) M * ld, make_float2(0.0f, 1.0f));
  if (c->stab_type == MOC_STABILIZE_YAMAMOTO) {
    for (int g = 0; g < G; g++) {
      float max_ratio = 0.0f;
      for (int m = 0; m < M; m++) {
        if (!c->h_mat_used[m]) continue;
        const float ratio = std::abs(c->h_scat_diag[(int64_t) m * G + g] /
                                     c->h_sigma_t[(int64_t) m * G + g]);
        if (ratio > max_ratio) max_ratio = ratio;
      }
      const float mr = (float) (max_ratio * f);
      for (int m = 0; m < M; m++)
        cf[(int64_t) m * ld + g] = make_float2(mr, 1.0f / (1.0f + mr));
    }
  } else {
    for (int m = 0; m < M; m++)
      for (int g = 0; g < G; g++) {
        const int64_t i = (int64_t) m * G + g;
        if (c->stab_type == MOC_STABILIZE_GLOBAL) {
          cf[(int64_t) m * ld + g] =
              make_float2((float) (1.0 / f - 1.0), (float) f);
        } else if (c->h_scat_diag[i] < 0.0f) {
          const double r = f * c->h_scat_diag[i] / c->h_sigma_t[i];
          cf[(int64_t) m * ld + g] =
              make_float2((float) -r, (float) (1.0 / (1.0 - r)));
        }
      }
  }
  if (!c->stab) MOC_TRY(dalloc(&c->stab, (int64_t) M * ld));
  MOC_CUDA(cudaMemcpy(c->stab, cf.data(), sizeof(float2) * cf.size(),
                      cudaMemcpyHostToDevice));
  c->stab_dirty = false;
  return MOC_OK;
}

}  // namespace (file helpers)

namespace moc {

void configure_kernels() {
  static std::mutex mu;
  static std::vector<int> done;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return;
  std::lock_guard<std::mutex> lk(mu);
  if (std::find(done.begin(), done.end(), dev) != done.end()) return;
  int optin = 0;
  if (cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin,
                             dev) != cudaSuccess || optin <= 0)
    return;
  configure_sweeps(optin);
  configure_ls_sweeps(optin);
  configure_otf_sweeps(optin);
  configure_sources(optin);
  cudaGetLastError();   // an instance the device cannot run is left as is
  done.push_back(dev);
}

}  // namespace moc

namespace {

moc::SweepArgs sweep_args(moc_ctx* c, int check_done) {
  moc::SweepArgs a{};
  a.rec = c->trec;
  a.segs = c->segs;
  a.seg_off = c->seg_off;
  a.order = c->order;
  a.track_ang = c->track_ang;
  a.next = c->next;
  a.flags = c->flags;
  a.weights = c->weights;
  a.inv_sin = c->inv_sin;
  a.sigma_t = c->sigma_t;
  a.fsr_mat = c->fsr_mat;
  a.qt = c->qt;
  a.exp_table = c->exp_table;
  a.phi = c->phi;
  a.psi[0] = c->psi[0];
  a.psi[1] = c->psi[1];
  a.sc = c->sc;
  a.num_tracks = c->d.num_tracks;
  a.num_groups = c->d.num_groups;
  a.ld = row_stride(c);
  a.num_materials = c->d.num_materials;
  a.lps = c->lps;
  a.mat_packed = c->mat_packed;
  a.check_done = check_done;
  a.hot_count = (c->d.num_polar_half == 1) ? c->hot_count : 0;
  a.hot_base = a.hot_count ? c->hot_base : (int) c->d.num_fsrs;
  if (c->ls) {
    a.segs_ls = c->segs_ls;
    a.ang_dir = c->ls_dir;
    a.qxy = c->qxy;
    a.mom = c->mom;
    if (c->ls3d) {
      a.seg_z = c->ls_segz;
      a.ang_dir3 = c->ls_dir3;
      a.qz = c->qz;
      a.momz = c->momz;
    }
  }
  if (c->cmfd && !c->otf) {
    a.cm_cell = c->cm_cell;
    a.cm_cur = c->cm_cur;
    a.cm_end = c->cm_end;
    a.cm_nx = c->cmfd->cfg.nx;
  }
  if (balance_keff(c)) a.leakage = &c->sc->leakage;
  if (c->num_instances) {
    a.inst = c->inst;
    a.inst_groups = c->inst_groups;
  }
  return a;
}

// Whether computeFSRSources runs on the tensor cores.
bool use_tc_sources(const moc_ctx* c) {
  if (!c->tc_b || !c->tc_rows || c->tc_tiles == 0) return false;
  if (c->num_instances) return false;   // the per-instance fission is FP32
  if (c->source_kind == MOC_SOURCES_TF32X3) return true;
  return c->source_kind == MOC_SOURCES_AUTO && c->d.num_groups >= 70;
}

moc::SolverArgs solver_args(moc_ctx* c, int check_done) {
  moc::SolverArgs a{};
  if (use_tc_sources(c)) {
    a.tc_rows = c->tc_rows;
    a.tc_tile_mat = c->tc_tile_mat;
    a.tc_b = c->tc_b;
    a.tc_tiles = c->tc_tiles;
    a.tc_n = moc::tc_pad_n(c->d.num_groups);
    a.tc_k = moc::tc_pad_k(c->d.num_groups);
    a.tc_wait_limit = c->tc_wait_limit < 0 ? moc::kTcDefaultWaitLimit
                                           : (unsigned) c->tc_wait_limit;
  }
  a.sigma_t = c->sigma_t;
  a.sigma_s = c->sigma_s;
  a.sigma_s_T = c->sigma_s_T;
  a.nu_sigma_f = c->nu_sigma_f;
  a.chi = c->chi;
  a.fissile = c->fissile;
  a.fsr_mat = c->fsr_mat;
  a.fsr_vol = c->fsr_vol;
  a.fixed = c->fixed;
  a.scat_out = c->scat_out;
  a.sigma_f = c->sigma_f;
  a.phi = c->phi;
  a.phi_old = c->phi_old;
  a.qt = c->qt;
  a.psi[0] = c->psi[0];
  a.psi[1] = c->psi[1];
  a.sc = c->sc;
  a.num_fsrs = c->d.num_fsrs;
  a.num_psi = num_psi(c);
  a.num_groups = c->d.num_groups;
  a.ld = row_stride(c);
  a.num_materials = c->d.num_materials;
  a.check_done = check_done;
  a.negative_ok = c->negative_ok;
  a.keff_balance = balance_keff(c) ? 1 : 0;
  a.stab = c->stab_on ? c->stab : nullptr;
  if (c->num_instances) {
    a.inst = c->inst;
    a.inst_groups = c->inst_groups;
    a.num_instances = c->num_instances;
  }
  if (c->ls) {
    a.mom = c->mom;
    a.qxy = c->qxy;
    a.ls_ilem = c->ls_ilem;
    a.ls_const = c->ls_const;
    a.fixed_xy = c->fixed_xy;
    if (c->ls3d) {
      a.momz = c->momz;
      a.qz = c->qz;
      a.fixed_z = c->fixed_z;
    }
  }
  return a;
}

int ready(moc_ctx* c) {
  MOC_CHECK(c != nullptr, MOC_ERR_ARG, "null context");
  MOC_CHECK(c->have_tracks && c->have_quad && c->have_mats && c->have_fsrs,
            MOC_ERR_STATE,
            "tracks, quadrature, materials and FSRs must be uploaded first");
  MOC_CUDA(cudaSetDevice(c->d.device));
  return MOC_OK;
}

int pull(moc_ctx* c) {
  MOC_CUDA(cudaMemcpyAsync(c->hsc, c->sc, sizeof(moc::DevScalars),
                           cudaMemcpyDeviceToHost, c->stream));
  MOC_CUDA(cudaStreamSynchronize(c->stream));
  return MOC_OK;
}

int push(moc_ctx* c) {
  MOC_CUDA(cudaMemcpyAsync(c->sc, c->hsc, sizeof(moc::DevScalars),
                           cudaMemcpyHostToDevice, c->stream));
  MOC_CUDA(cudaStreamSynchronize(c->stream));
  return MOC_OK;
}

// Utilisation of lanes for G groups split over lps lanes.
double lane_use(int G, int lps, int slots) {
  return (double) G / (double) (2 * lps * slots);
}

// Group pairs per lane for G groups over lps lanes.
int pair_slots(int G, int lps) {
  const int pairs = (G + 1) / 2;
  return (pairs + lps - 1) / lps;
}

// Heuristic kernel shape: the most lanes per track direction whose lane
// utilisation is within 5% of the best reachable with at most max_slots
// group pairs per lane (kMaxSlots for the flat-source sweep, kMaxLsSlots for
// the linear-source sweep).
void pick_shape(int G, int* lps_out, int* slots_out,
                int max_slots = moc::kMaxSlots) {
  double best = 0.0;
  for (int lps = 1; lps <= 32; lps *= 2) {
    int slots = pair_slots(G, lps);
    if (slots > max_slots) continue;
    best = std::max(best, lane_use(G, lps, slots));
  }
  int chosen = 32;
  for (int lps = 32; lps >= 1; lps /= 2) {
    int slots = pair_slots(G, lps);
    if (slots > max_slots) continue;
    if (lane_use(G, lps, slots) >= 0.95 * best) {
      chosen = lps;
      break;
    }
  }
  *lps_out = chosen;
  *slots_out = pair_slots(G, chosen);
}

int max_slots(const moc_ctx* c) {
  return c->ls ? moc::kMaxLsSlots : c->otf ? moc::kMaxOtfSlots : moc::kMaxSlots;
}

moc::OtfArgs otf_args(const moc_ctx* c) {
  moc::OtfArgs o{};
  o.trk = c->otf_trk;
  o.trk_f = c->otf_trk_f;
  o.ang = c->otf_ang;
  o.rad_segs = c->otf_rad;
  o.rad_start = c->otf_rad_start;
  o.rad_off = c->otf_rad_off;
  o.rad_total = c->otf_rad_total;
  o.above_fsr = c->otf_above_fsr;
  o.above = c->otf_above_word;
  return o;
}

int enqueue_sweep(moc_ctx* c, int check_done, bool timed, int ev_index) {
  if (c->lps == 0)
    pick_shape(c->d.num_groups, &c->lps, &c->slots, max_slots(c));
  if (timed) {
    while ((int) c->ev.size() < 2 * (ev_index + 1)) {
      cudaEvent_t e;
      MOC_CUDA(cudaEventCreate(&e));
      c->ev.push_back(e);
    }
    MOC_CUDA(cudaEventRecord(c->ev[2 * ev_index], c->stream));
  }
  moc::SweepArgs a = sweep_args(c, check_done);
  bool ok;
  if (c->otf) {
    a.order = c->otf_order;
    a.rec = nullptr;
    ok = moc::launch_otf_sweep(a, otf_args(c), c->slots, c->stream);
  } else {
    ok = c->ls ? moc::launch_ls_sweep(a, c->d.num_polar_half, c->slots,
                                      c->stream)
               : moc::launch_sweep(a, c->d.num_polar_half, c->slots,
                                   c->exp_kind, c->stream);
  }
  if (!ok)
    return fail(MOC_ERR_UNSUPPORTED,
                std::string(c->ls ? "no linear-source" : "no") +
                " sweep kernel for " + std::to_string(c->d.num_polar_half) +
                    " polar angles per half space and " +
                    std::to_string(c->slots) + " groups per lane");
  c->launches++;
  MOC_CUDA(cudaGetLastError());
  if (timed) MOC_CUDA(cudaEventRecord(c->ev[2 * ev_index + 1], c->stream));
  return MOC_OK;
}

// ---- autotuner: sweep kernel shape and exponential evaluator -----------
// Candidate shapes are every lanes-per-track-direction count with at most
// kMaxSlots groups per lane and at least half the lanes busy; each is timed
// on the context's own problem (median of three sweeps after one warm-up).
// Results are cached per problem size for the process.
struct TuneKey {
  int G, Ph, M, exp_fixed, exp_kind, ls;
  int64_t T, S, R;
  int cm;
  bool operator<(const TuneKey& o) const {
    return std::tie(G, Ph, M, exp_fixed, exp_kind, ls, T, S, R, cm) <
           std::tie(o.G, o.Ph, o.M, o.exp_fixed, o.exp_kind, o.ls, o.T, o.S,
                    o.R, o.cm);
  }
};
using TuneVal = moc_tune_entry;
std::mutex g_tune_mu;
std::map<TuneKey, TuneVal> g_tune_cache;

int time_sweep(moc_ctx* c, int reps, float* median_ms) {
  std::vector<float> t;
  MOC_TRY(enqueue_sweep(c, 0, true, 0));   // warm-up
  for (int r = 0; r < reps; r++) {
    MOC_TRY(enqueue_sweep(c, 0, true, r));
  }
  MOC_CUDA(cudaStreamSynchronize(c->stream));
  for (int r = 0; r < reps; r++) {
    float ms = 0.f;
    MOC_CUDA(cudaEventElapsedTime(&ms, c->ev[2 * r], c->ev[2 * r + 1]));
    t.push_back(ms);
  }
  std::sort(t.begin(), t.end());
  *median_ms = t[t.size() / 2];
  return MOC_OK;
}

// Leaves sweep tallies and angular-flux buffers in an undefined state: call
// only before a solve initialises them.
int autotune_sweep(moc_ctx* c, bool use_cache) {
  TuneKey key{c->d.num_groups, c->d.num_polar_half, c->d.num_materials,
              c->exp_user_set, c->exp_user_set ? c->exp_kind : -1,
              c->ls ? 1 : 0, c->d.num_tracks, c->d.num_segments,
              c->d.num_fsrs, c->cmfd ? 1 : 0};
  if (use_cache) {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto it = g_tune_cache.find(key);
    if (it != g_tune_cache.end()) {
      c->lps = it->second.lps;
      c->slots = it->second.slots;
      c->exp_kind = it->second.exp_kind;
      c->tuned = true;
      return MOC_OK;
    }
  }
  const int G = c->d.num_groups;
  std::vector<int> kinds;
  // the linear-source and on-the-fly sweeps have one exponential evaluator
  if (c->exp_user_set || c->ls || c->otf || c->cmfd)
    kinds.push_back(c->exp_kind);
  else kinds = {MOC_EXP_TABLE, MOC_EXP_INTRINSIC};
  TuneVal best{0, 0, 0, 1e30f};
  c->tune_log.clear();
  for (int kind : kinds) {
    for (int lps = 1; lps <= 32; lps *= 2) {
      const int slots = pair_slots(G, lps);
      if (slots > max_slots(c) || lane_use(G, lps, slots) < 0.5) continue;
      c->lps = lps;
      c->slots = slots;
      c->exp_kind = kind;
      float ms = 0.f;
      MOC_TRY(time_sweep(c, 3, &ms));
      c->tune_log.push_back({lps, slots, kind, ms});
      if (ms < best.ms) best = {lps, slots, kind, ms};
    }
  }
  MOC_CHECK(best.lps > 0, MOC_ERR_UNSUPPORTED, "no sweep kernel shape fits");
  c->lps = best.lps;
  c->slots = best.slots;
  c->exp_kind = best.exp_kind;
  c->tuned = true;
  std::lock_guard<std::mutex> lk(g_tune_mu);
  g_tune_cache[key] = best;
  return MOC_OK;
}

// the tallies and sources of the next sweep (fused: zero the tallies first)
void enqueue_sources(moc_ctx* c, const moc::SolverArgs& a, int iteration,
                     int fused) {
  if (c->ls)
    moc::launch_ls_sources(a, iteration, fused, c->stream);
  else
    moc::launch_compute_sources(a, iteration, fused, c->stream);
  c->launches++;
}

// addSourceToScalarFlux; update = 1 also updates keff and the normalisation
// (and, with a linear source, normalises the moments)
void enqueue_add_source(moc_ctx* c, const moc::SolverArgs& a, int update) {
  if (c->ls) {
    moc::launch_ls_add_source(a, update, c->stream);
    c->launches++;
    if (update == 1) {
      moc::launch_ls_scale_moments(a, c->stream);
      c->launches++;
    }
  } else {
    moc::launch_add_source(a, update, c->stream);
    c->launches++;
  }
}

// zero flux tallies (and moments) without computing sources; skipped, like
// every kernel of the loop, once the device reports the solve done
int enqueue_zero_tallies(moc_ctx* c, const moc::SolverArgs& a) {
  moc::launch_zero_phi(a, c->stream);
  c->launches++;
  return MOC_OK;
}

// the flux moments of a flattened flux are zero
int zero_moments(moc_ctx* c) {
  if (c->ls)
    MOC_CUDA(cudaMemsetAsync(c->mom, 0, 8 * num_flux(c), c->stream));
  if (c->ls3d)
    MOC_CUDA(cudaMemsetAsync(c->momz, 0, 4 * num_flux(c), c->stream));
  return MOC_OK;
}

int maybe_autotune(moc_ctx* c) {
  if (c->autotune && !c->tuned && !c->shape_user_set)
    return autotune_sweep(c, true);
  return MOC_OK;
}

int collect_sweep_times(moc_ctx* c, int n) {
  for (int i = 0; i < n; i++) {
    float ms = 0.f;
    MOC_CUDA(cudaEventElapsedTime(&ms, c->ev[2 * i], c->ev[2 * i + 1]));
    c->sweep_ms += ms;
  }
  return MOC_OK;
}

// Resets the device state machine for a new solve.
int begin_solve(moc_ctx* c, int mode, int max_iters, int res_type,
                double keff) {
  MOC_TRY(pull(c));
  moc::DevScalars& s = *c->hsc;
  s.keff = keff;
  s.k_prev = keff;
  s.factor = 1.0;
  s.residual = 0.0;
  s.accum_rate = 0.0;
  s.accum_res = 0.0;
  s.threshold = c->threshold;
  s.ticket_rate = s.ticket_res = s.ticket_sweep = 0;
  s.iteration = 0;
  s.max_iters = max_iters;
  s.done = 0;
  s.converged = 0;
  s.dk = 0;
  s.mode = mode;
  s.res_type = res_type;
  s.neg_sources = 0;
  s.neg_fluxes = 0;
  s.num_fissionable = c->num_fissionable;
  s.tc_error = 0;
  s.accum_abs = 0.0;
  s.leakage = 0.0;
  MOC_TRY(push(c));
  c->sweep_ms = 0.0;
  c->num_sweeps = 0;
  return MOC_OK;
}

int zero_track_fluxes(moc_ctx* c) {
  size_t bytes = sizeof(float) * (size_t) num_psi(c);
  MOC_CUDA(cudaMemsetAsync(c->psi[0], 0, bytes, c->stream));
  MOC_CUDA(cudaMemsetAsync(c->psi[1], 0, bytes, c->stream));
  MOC_TRY(pull(c));
  c->hsc->scale[0] = c->hsc->scale[1] = 1.0f;
  c->hsc->cur = 0;
  MOC_TRY(push(c));
  return MOC_OK;
}

// Whether the linear source's moments are stabilized: CPULSSolver's
// YAMAMOTO branch for the moments assigns `ratio = max_ratio` where the flat
// branch raises max_ratio, so its ratio stays 0 and the moments are left as
// they are (src/CPULSSolver.cpp:924-941, 1010-1031).
bool stab_moments(const moc_ctx* c) {
  return c->stab_on && c->ls && c->stab_type != MOC_STABILIZE_YAMAMOTO;
}

// The flux moments at the start of an eigenvalue iteration, kept as the base
// of their stabilization (CPULSSolver::computeStabilizingFlux takes them
// before the sources of the iteration; the flat flux's base is phi_old).
int enqueue_stab_moments_base(moc_ctx* c) {
  if (!stab_moments(c)) return MOC_OK;
  if (!c->stab_mom) MOC_TRY(dalloc(&c->stab_mom, 2 * num_flux(c)));
  MOC_CUDA(cudaMemcpyAsync(c->stab_mom, c->mom, 8 * num_flux(c),
                           cudaMemcpyDeviceToDevice, c->stream));
  if (c->ls3d) {
    if (!c->stab_momz) MOC_TRY(dalloc(&c->stab_momz, num_flux(c)));
    MOC_CUDA(cudaMemcpyAsync(c->stab_momz, c->momz, 4 * num_flux(c),
                             cudaMemcpyDeviceToDevice, c->stream));
  }
  return MOC_OK;
}

// addSourceToScalarFlux, computeKeff, stabilizeFlux and the normalisation
// factor of an eigenvalue iteration (the residual kernel then normalises).
void enqueue_eigen_update(moc_ctx* c, const moc::SolverArgs& a) {
  if (c->stab_on) {
    // keff first; the stabilized flux sets the normalisation, which then
    // scales the stabilized moments of a linear source
    enqueue_add_source(c, a, 2);
    moc::launch_stabilize(a, c->phi_old, 1, c->stream,
                          stab_moments(c) ? c->stab_mom : nullptr,
                          stab_moments(c) && c->ls3d ? c->stab_momz : nullptr);
    c->launches++;
    if (c->ls) {
      moc::launch_ls_scale_moments(a, c->stream);
      c->launches++;
    }
  } else if (c->num_instances) {
    // each instance's keff and normalisation
    enqueue_add_source(c, a, 0);
    moc::launch_instance_rates(a, 0, c->stream);
    c->launches++;
  } else {
    enqueue_add_source(c, a, 1);
  }
}

// The starting flux of an eigenvalue solve: flat, normalised (per instance
// with instances).
void enqueue_initial_guess(moc_ctx* c, const moc::SolverArgs& a) {
  moc::launch_fill(c->phi, num_flux(c), 1.0f, c->stream);
  if (c->num_instances) {
    moc::launch_instance_rates(a, 1, c->stream);
  } else {
    moc::launch_fission_rate(a, 1, c->stream);
    moc::launch_scale_phi(a, c->stream);
  }
  c->launches += 3;
}

// The device loop: iterations of `kind` until the device reports done.
int run_iterations(moc_ctx* c, int kind, int res_type) {
  MOC_TRY(ensure_stab(c));
  moc::SolverArgs a = solver_args(c, 1);
  int completed = 0;
  for (;;) {
    const int k = c->iters_per_sync;
    for (int i = 0; i < k; i++) {
      if (kind == moc::kModeFlux) {
        MOC_TRY(enqueue_zero_tallies(c, a));
      } else {
        if (kind == moc::kModeEigen) MOC_TRY(enqueue_stab_moments_base(c));
        enqueue_sources(c, a, -1, 1);
      }
      MOC_TRY(enqueue_sweep(c, 1, true, i));
      if (kind == moc::kModeEigen)
        enqueue_eigen_update(c, a);
      else
        enqueue_add_source(c, a, 0);
      moc::launch_residual(a, res_type, kind == moc::kModeEigen ? 1 : 0, 1, 1,
                           c->stream);
      c->launches++;
      MOC_CUDA(cudaGetLastError());
    }
    MOC_TRY(pull(c));
    MOC_CHECK(!c->hsc->tc_error, MOC_ERR_TIMEOUT,
              "a tensor-core source launch gave up waiting for its copies");
    // sweeps that returned at once after convergence still record events;
    // count only the iterations the device performed
    const int done_now = c->hsc->iteration - completed;
    MOC_TRY(collect_sweep_times(c, std::min(done_now, k)));
    c->num_sweeps += done_now;
    completed = c->hsc->iteration;
    if (c->hsc->done) break;
  }
  c->keff = c->hsc->keff;
  c->residual = c->hsc->residual;
  return MOC_OK;
}

// Once tracks and FSR materials are both on the device, fold each
// segment's material into its FSR word so the sweep needs no dependent
// material lookup.
int pack_materials(moc_ctx* c) {
  c->mat_packed = 0;
  if (!(c->have_tracks && c->have_fsrs)) return MOC_OK;
  if (c->d.num_fsrs >= (1LL << 24) || c->d.num_materials > 256) return MOC_OK;
  moc::launch_pack_materials(c->segs, c->d.num_segments, c->fsr_mat,
                             c->stream);
  c->launches++;
  MOC_CUDA(cudaGetLastError());
  MOC_CUDA(cudaStreamSynchronize(c->stream));
  c->mat_packed = 1;
  return MOC_OK;
}

void cmfd_release(moc_ctx* c) {
  dfree(c->cm_cell);
  dfree(c->cm_end);
  dfree(c->cm_cur);
  dfree(c->cm_group);
  dfree(c->cm_pair_off);
  dfree(c->cm_pair_fsr);
  dfree(c->cm_sums);
  dfree(c->cm_ratio);
  dfree(c->cm_state);
  dfree(c->cm_work);
  dfree(c->cm_dcorr);
  dfree(c->cm_flux_old);
  dfree(c->cm_flux_new);
  dfree(c->cm_cell_pair);
  dfree(c->cm_color_cells);
  dfree(c->cm_cell_pos);
  dfree(c->cm_nbr_j);
  dfree(c->cm_map_j);
  dfree(c->cm_map_nslot);
  dfree(c->cm_map_push);
  c->cm_map_nb = 0;
  dfree(c->cm_pair_mat);
  dfree(c->cm_chi_m);
  dfree(c->cm_ss_m);
  dfree(c->cm_cell_vol);
  dfree(c->cm_wx);
  dfree(c->cm_wy);
  dfree(c->cm_gstart);
  dfree(c->cm_edc_mu);
  dfree(c->cm_pro_off);
  dfree(c->cm_pro_cell);
  dfree(c->cm_pro_coef);
  dfree(c->cm_edc_w);
  if (c->h_cm_sums) cudaFreeHost(c->h_cm_sums);
  if (c->h_cm_cur) cudaFreeHost(c->h_cm_cur);
  c->h_cm_sums = nullptr;
  c->h_cm_cur = nullptr;
  c->cm_sums_n = 0;
  c->h_cm_cell.clear();
  delete c->cmfd;
  c->cmfd = nullptr;
}

// Per solve: the cross sections and FSR data the coarse solve collapses
// (read back from the device, so that any upload since is seen), the
// (cell, material) pairs with their FSR lists, and the pair-sum buffers.
int cmfd_prepare(moc_ctx* c) {
  moc_cmfd::Solver& S = *c->cmfd;
  const int M = c->d.num_materials, G = c->d.num_groups;
  const int64_t R = c->d.num_fsrs;
  const int64_t MG = (int64_t) M * G;
  std::vector<float> st(MG), nf(MG), ss(MG * G), vol(R);
  std::vector<int32_t> mat(R);
  MOC_CUDA(cudaMemcpy(st.data(), c->sigma_t, 4 * MG, cudaMemcpyDeviceToHost));
  MOC_CUDA(cudaMemcpy(nf.data(), c->nu_sigma_f, 4 * MG,
                      cudaMemcpyDeviceToHost));
  MOC_CUDA(cudaMemcpy(ss.data(), c->sigma_s, 4 * MG * G,
                      cudaMemcpyDeviceToHost));
  MOC_CUDA(cudaMemcpy(vol.data(), c->fsr_vol, 4 * R, cudaMemcpyDeviceToHost));
  MOC_CUDA(cudaMemcpy(mat.data(), c->fsr_mat, 4 * R, cudaMemcpyDeviceToHost));
  moc_cmfd::Fine& F = S.fine;
  F.M = M;
  F.st.assign(st.begin(), st.end());
  F.nf.assign(nf.begin(), nf.end());
  F.ss.assign(ss.begin(), ss.end());
  F.chi.assign(c->h_chi.begin(), c->h_chi.end());
  const int C = S.cfg.cells();
  F.cell_vol.assign(C, 0.0);
  // pair id of every (cell, material) in use, in cell-major order
  std::vector<int32_t> pid((size_t) C * M, -1);
  for (int64_t r = 0; r < R; r++) {
    pid[(size_t) c->h_cm_cell[r] * M + mat[r]] = 0;
    F.cell_vol[c->h_cm_cell[r]] += (double) vol[r];
  }
  F.pair_cell.clear();
  F.pair_mat.clear();
  for (int cell = 0; cell < C; cell++)
    for (int m = 0; m < M; m++)
      if (pid[(size_t) cell * M + m] == 0) {
        pid[(size_t) cell * M + m] = F.pairs();
        F.pair_cell.push_back(cell);
        F.pair_mat.push_back(m);
      }
  const int P = F.pairs();
  std::vector<int32_t> off(P + 1, 0), list(R);
  for (int64_t r = 0; r < R; r++)
    off[pid[(size_t) c->h_cm_cell[r] * M + mat[r]] + 1]++;
  for (int p = 0; p < P; p++) off[p + 1] += off[p];
  std::vector<int32_t> fill(off.begin(), off.end() - 1);
  for (int64_t r = 0; r < R; r++)
    list[fill[pid[(size_t) c->h_cm_cell[r] * M + mat[r]]]++] = (int32_t) r;
  dfree(c->cm_pair_off);
  dfree(c->cm_pair_fsr);
  MOC_TRY(dalloc(&c->cm_pair_off, P + 1));
  MOC_TRY(dalloc(&c->cm_pair_fsr, R));
  MOC_CUDA(cudaMemcpy(c->cm_pair_off, off.data(), 4 * (P + 1),
                      cudaMemcpyHostToDevice));
  MOC_CUDA(cudaMemcpy(c->cm_pair_fsr, list.data(), 4 * R,
                      cudaMemcpyHostToDevice));
  const int64_t n = (int64_t) P * G;
  if (n != c->cm_sums_n) {
    dfree(c->cm_sums);
    if (c->h_cm_sums) cudaFreeHost(c->h_cm_sums);
    c->h_cm_sums = nullptr;
    MOC_TRY(dalloc(&c->cm_sums, n));
    if (c->cm_host) MOC_CUDA(cudaMallocHost(&c->h_cm_sums, 8 * n));
    c->cm_sums_n = n;
  }
  // Larsen's factor is for flat sources only (Cmfd::
  // getSurfaceDiffusionCoefficient, src/Cmfd.cpp:1082-1083, 1125-1126)
  S.cfg.edc_mu = c->ls ? std::vector<double>() : c->cm_edc_mu_h;
  S.cfg.edc_w = c->ls ? std::vector<double>() : c->cm_edc_w_h;
  S.reset();
  S.source_threshold = 0.1 * c->threshold;   // Solver::initializeCmfd
  if (c->cm_host) return MOC_OK;
  // the device solve's inputs
  const moc_cmfd::Config& cf = S.cfg;
  const int E = cf.E;
  std::vector<int32_t> cell_pair(C + 1, 0);
  for (int p = 0; p < P; p++) cell_pair[F.pair_cell[p] + 1]++;
  for (int i = 0; i < C; i++) cell_pair[i + 1] += cell_pair[i];
  std::vector<float> chi_m((size_t) M * E, 0.0f), ss_m((size_t) MG * E, 0.0f);
  for (int m = 0; m < M; m++)
    for (int h = 0; h < G; h++) {
      chi_m[(size_t) m * E + cf.group_of[h]] += c->h_chi[(size_t) m * G + h];
      // scattering from h into each coarse group (sigma_s is [m][dest][orig])
      for (int g = 0; g < G; g++)
        ss_m[((size_t) m * G + h) * E + cf.group_of[g]] +=
            ss[((size_t) m * G + g) * G + h];
    }
  std::vector<float> cvol(F.cell_vol.begin(), F.cell_vol.end());
  std::vector<float> wx(cf.wx.begin(), cf.wx.end()), wy(cf.wy.begin(), cf.wy.end());
  std::vector<float> mu(cf.edc_mu.begin(), cf.edc_mu.end());
  std::vector<float> ew(cf.edc_w.begin(), cf.edc_w.end());
  std::vector<int32_t> gstart(cf.gstart.begin(), cf.gstart.end());
  auto up = [&](auto** dst, const auto& v) -> int {
    dfree(*dst);
    MOC_TRY(dalloc(dst, std::max<int64_t>(1, (int64_t) v.size())));
    if (!v.empty())
      MOC_CUDA(cudaMemcpy(*dst, v.data(), sizeof(v[0]) * v.size(),
                          cudaMemcpyHostToDevice));
    return MOC_OK;
  };
  MOC_TRY(up(&c->cm_cell_pair, cell_pair));
  std::vector<int32_t> colors;
  for (int k = 0; k < 2; k++) {
    for (int cell = 0; cell < C; cell++)
      if (((cell % cf.nx) + (cell / cf.nx)) % 2 == k) colors.push_back(cell);
    if (k == 0) c->cm_n_color0 = (int) colors.size();
  }
  MOC_TRY(up(&c->cm_color_cells, colors));
  std::vector<int32_t> pos(C), nbr_j(4 * (size_t) C, -1);
  for (int jj = 0; jj < C; jj++) pos[colors[jj]] = jj;
  for (int jj = 0; jj < C; jj++) {
    const int cell = colors[jj], ix = cell % cf.nx, iy = cell / cf.nx;
    const int nb[4] = {ix > 0 ? cell - 1 : -1, iy > 0 ? cell - cf.nx : -1,
                       ix + 1 < cf.nx ? cell + 1 : -1,
                       iy + 1 < cf.ny ? cell + cf.nx : -1};
    for (int f = 0; f < 4; f++)
      nbr_j[(size_t) f * C + jj] = nb[f] >= 0 ? pos[nb[f]] : -1;
  }
  MOC_TRY(up(&c->cm_cell_pos, pos));
  MOC_TRY(up(&c->cm_nbr_j, nbr_j));
  // the cell-parallel solve: cells in runs of cell order over the blocks
  // of a cluster, each block's red cells first
  c->cm_map_nb = 0;
  if (E <= moc::kCmfdMaxCellGroups) {
    const int cap = moc::cmfd_cells_threads(E);
    const int nb = (C + cap - 1) / cap;
    const int per = (C + nb - 1) / std::max(nb, 1);
    std::vector<int> owner(C), slot(C);
    std::vector<std::vector<int>> own(nb);
    for (int k = 0; k < 2; k++)
      for (int cell = 0; cell < C; cell++)
        if (((cell % cf.nx) + (cell / cf.nx)) % 2 == k) {
          const int r = cell / per;
          owner[cell] = r;
          slot[cell] = (int) own[r].size();
          own[r].push_back(cell);
        }
    int threads = 32;
    for (int r = 0; r < nb; r++)
      threads = std::max(threads, ((int) own[r].size() + 31) / 32 * 32);
    // halo copies: each block's copy of a bordering cell of another block
    std::vector<std::vector<std::pair<int, int>>> copies(C);   // (block, slot)
    std::vector<int> halo(nb, 0);
    std::vector<std::vector<int>> halo_slot(nb);
    bool ok = nb <= moc::kCmfdMaxClusterBlocks;
    const int NT = nb * threads;
    std::vector<int32_t> mj(NT, -1), mns(4 * (size_t) NT), mpush(2 * (size_t) NT, -1);
    for (int r = 0; ok && r < nb; r++) {
      std::vector<int> local(C, -1);   // slot in block r of each cell it reads
      for (int q = 0; q < (int) own[r].size(); q++) local[own[r][q]] = q;
      for (int q = 0; q < (int) own[r].size(); q++) {
        const int cell = own[r][q], ix = cell % cf.nx, iy = cell / cf.nx;
        const int nbc[4] = {ix > 0 ? cell - 1 : -1, iy > 0 ? cell - cf.nx : -1,
                            ix + 1 < cf.nx ? cell + 1 : -1,
                            iy + 1 < cf.ny ? cell + cf.nx : -1};
        const int gid = r * threads + q;
        mj[gid] = pos[cell];
        for (int f = 0; f < 4; f++) {
          int sl = q;
          if (nbc[f] >= 0) {
            if (local[nbc[f]] < 0) {
              local[nbc[f]] = threads + halo[r]++;
              copies[nbc[f]].push_back({r, local[nbc[f]]});
            }
            sl = local[nbc[f]];
          }
          mns[(size_t) f * NT + gid] = sl;
        }
      }
      for (int q = (int) own[r].size(); q < threads; q++)
        for (int f = 0; f < 4; f++) mns[(size_t) f * NT + r * threads + q] = q;
    }
    for (int cell = 0; ok && cell < C; cell++) {
      if (copies[cell].size() > 2) { ok = false; break; }
      const int gid = owner[cell] * threads + slot[cell];
      for (size_t q = 0; q < copies[cell].size(); q++)
        mpush[q * NT + gid] = (copies[cell][q].first << 24) | copies[cell][q].second;
    }
    int slots = threads;
    for (int r = 0; r < nb; r++) slots = std::max(slots, threads + halo[r]);
    if (ok && moc::cmfd_cells_smem(E, threads, slots) > 200 * 1024) ok = false;
    if (ok) {
      MOC_TRY(up(&c->cm_map_j, mj));
      MOC_TRY(up(&c->cm_map_nslot, mns));
      MOC_TRY(up(&c->cm_map_push, mpush));
      c->cm_map_nb = nb;
      c->cm_map_threads = threads;
      c->cm_map_slots = slots;
    }
  }
  MOC_CHECK(c->cm_solve_kind != 3 || c->cm_map_nb > 0, MOC_ERR_UNSUPPORTED,
            "the cell-parallel coarse solve takes up to " +
                std::to_string(moc::kCmfdMaxCellGroups) + " coarse groups and " +
                std::to_string(moc::kCmfdMaxClusterBlocks) + " blocks of cells");
  MOC_TRY(up(&c->cm_pair_mat, F.pair_mat));
  MOC_TRY(up(&c->cm_chi_m, chi_m));
  MOC_TRY(up(&c->cm_ss_m, ss_m));
  MOC_TRY(up(&c->cm_cell_vol, cvol));
  MOC_TRY(up(&c->cm_wx, wx));
  MOC_TRY(up(&c->cm_wy, wy));
  MOC_TRY(up(&c->cm_gstart, gstart));
  MOC_TRY(up(&c->cm_edc_mu, mu));
  MOC_TRY(up(&c->cm_edc_w, ew));
  const int64_t CE = (int64_t) C * E;
  dfree(c->cm_work);
  dfree(c->cm_dcorr);
  dfree(c->cm_flux_old);
  dfree(c->cm_flux_new);
  dfree(c->cm_state);
  MOC_TRY(dalloc(&c->cm_work, moc::cmfd_work_floats(C, E)));
  MOC_TRY(dalloc(&c->cm_dcorr, 4 * CE));
  MOC_TRY(dalloc(&c->cm_flux_old, CE));
  MOC_TRY(dalloc(&c->cm_flux_new, CE));
  MOC_TRY(dalloc(&c->cm_state, 1));
  MOC_CUDA(cudaMemset(c->cm_dcorr, 0, 16 * CE));
  MOC_CUDA(cudaMemset(c->cm_flux_old, 0, 4 * CE));
  MOC_CUDA(cudaMemset(c->cm_flux_new, 0, 4 * CE));
  moc::CmfdDevState st0{};
  st0.keff = 1.0;
  st0.max_ratio = 1.0f;
  MOC_CUDA(cudaMemcpy(c->cm_state, &st0, sizeof(st0), cudaMemcpyHostToDevice));
  return MOC_OK;
}

moc::CmfdArgs cmfd_args(moc_ctx* c) {
  const moc_cmfd::Config& cf = c->cmfd->cfg;
  moc::CmfdArgs a{};
  a.nx = cf.nx;
  a.ny = cf.ny;
  a.C = cf.cells();
  a.E = cf.E;
  a.G = cf.G;
  a.P = c->cmfd->fine.pairs();
  a.n_edc = (int) cf.edc_mu.size();
  a.ld = row_stride(c);
  for (int f = 0; f < 4; f++) a.bc[f] = cf.bc[f];
  a.relax = (float) cf.relaxation;
  a.sor = (float) cf.sor;
  a.flux_limiting = cf.flux_limiting ? 1 : 0;
  a.unbounded = cf.unbounded;
  a.wx = c->cm_wx;
  a.wy = c->cm_wy;
  a.gstart = c->cm_gstart;
  a.cell_pair = c->cm_cell_pair;
  a.color_cells = c->cm_color_cells;
  a.cell_pos = c->cm_cell_pos;
  a.nbr_j = c->cm_nbr_j;
  a.n_color0 = c->cm_n_color0;
  a.map_j = c->cm_map_j;
  a.map_nslot = c->cm_map_nslot;
  a.map_push = c->cm_map_push;
  a.map_nb = c->cm_map_nb;
  a.map_threads = c->cm_map_threads;
  a.map_slots = c->cm_map_slots;
  a.solve_kind = c->cm_solve_kind == 2 ? 2 : 0;
  a.pair_mat = c->cm_pair_mat;
  a.st = c->sigma_t;
  a.nf = c->nu_sigma_f;
  a.chi_m = c->cm_chi_m;
  a.ss_m = c->cm_ss_m;
  a.cell_vol = c->cm_cell_vol;
  a.edc_mu = c->cm_edc_mu;
  a.edc_w = c->cm_edc_w;
  a.S = c->cm_sums;
  a.cur = c->cm_cur;
  a.work = c->cm_work;
  a.dcorr_old = c->cm_dcorr;
  a.ratio = c->cm_ratio;
  a.flux_old = c->cm_flux_old;
  a.flux_new = c->cm_flux_new;
  a.cm = c->cm_state;
  a.sc = c->sc;
  return a;
}

// computeEigenvalue with CMFD (src/Solver.cpp:1591-1647): per iteration
// sources, sweep with current tallies, addSourceToScalarFlux, the coarse
// solve in place of computeKeff and the prolongation, normalizeFluxes,
// residual and store.  The device solve keeps the whole loop on the GPU
// (the host checks the state once per block of iterations, as without
// CMFD); the host solve reads the tallies back every iteration.
int run_cmfd_iterations(moc_ctx* c, int res_type) {
  MOC_TRY(ensure_stab(c));
  moc_cmfd::Solver& S = *c->cmfd;
  moc::SolverArgs a = solver_args(c, 1);
  const int C = S.cfg.cells(), E = S.cfg.E;
  const int ld = row_stride(c);
  const int64_t ncur = (int64_t) C * moc_cmfd::kFaces * ld;
  const moc::CmfdArgs ca = cmfd_args(c);
  int completed = 0;
  for (;;) {
    const int k = c->cm_host ? 1 : c->iters_per_sync;
    for (int i = 0; i < k; i++) {
      MOC_TRY(enqueue_stab_moments_base(c));
      enqueue_sources(c, a, -1, 1);
      MOC_CUDA(cudaMemsetAsync(c->cm_cur, 0, 4 * ncur, c->stream));
      MOC_TRY(enqueue_sweep(c, 1, true, i));
      enqueue_add_source(c, a, 0);
      moc::launch_cmfd_pair_sums(c->phi, c->fsr_vol, c->cm_pair_off,
                                 c->cm_pair_fsr, S.fine.pairs(),
                                 c->d.num_groups, ld, c->cm_sums, c->sc,
                                 c->stream);
      c->launches += 3;
      MOC_CUDA(cudaGetLastError());
      if (c->cm_host) {
        MOC_CUDA(cudaMemcpyAsync(c->h_cm_sums, c->cm_sums, 8 * c->cm_sums_n,
                                 cudaMemcpyDeviceToHost, c->stream));
        MOC_CUDA(cudaMemcpyAsync(c->h_cm_cur, c->cm_cur, 4 * ncur,
                                 cudaMemcpyDeviceToHost, c->stream));
        MOC_TRY(pull(c));
        if (c->hsc->done) break;
        S.source_threshold = c->hsc->iteration == 0
                                 ? 0.1 * c->threshold
                                 : 0.01 * (c->hsc->residual > 0.0
                                               ? c->hsc->residual : 1e-6);
        const double kc = S.step(c->hsc->iteration, c->h_cm_sums,
                                 c->h_cm_cur, ld);
        c->h_cm_ratio.assign(S.ratio.begin(), S.ratio.end());
        MOC_CUDA(cudaMemcpyAsync(c->cm_ratio, c->h_cm_ratio.data(),
                                 4 * (int64_t) C * E, cudaMemcpyHostToDevice,
                                 c->stream));
        c->hsc->keff = kc;
        MOC_CUDA(cudaMemcpyAsync(&c->sc->keff, &c->hsc->keff, sizeof(double),
                                 cudaMemcpyHostToDevice, c->stream));
      } else {
        // collapse, build, solve
        const bool as_asked = moc::launch_cmfd_solve(ca, c->stream);
        c->launches += 3;
        MOC_CUDA(cudaGetLastError());
        MOC_CHECK(as_asked || c->cm_solve_kind != 3, MOC_ERR_CUDA,
                  "the cell-parallel coarse solve could not be launched");
      }
      moc::launch_cmfd_prolong(c->phi, c->ls ? c->mom : nullptr, c->cm_cell,
                               c->cm_group, c->cm_ratio,
                               moc::CmfdStencil{c->cm_pro_off, c->cm_pro_cell,
                                                c->cm_pro_coef},
                               c->d.num_fsrs, c->d.num_groups, ld, E,
                               S.cfg.unbounded, c->sc, c->stream);
      if (c->stab_on)   // stabilizeFlux follows the CMFD update; the
                        // normalisation factor is the stabilized flux's
        moc::launch_stabilize(a, c->phi_old, 1, c->stream,
                              stab_moments(c) ? c->stab_mom : nullptr,
                              stab_moments(c) && c->ls3d ? c->stab_momz : nullptr);
      else
        moc::launch_fission_rate(a, 1, c->stream);
      c->launches += 2;
      if (c->ls) {     // normalizeFluxes scales the moments too
        moc::launch_ls_scale_moments(a, c->stream);
        c->launches++;
      }
      moc::launch_residual(a, res_type, 1, 1, 1, c->stream);
      c->launches++;
      MOC_CUDA(cudaGetLastError());
    }
    MOC_TRY(pull(c));
    const int done_now = c->hsc->iteration - completed;
    MOC_TRY(collect_sweep_times(c, std::min(done_now, k)));
    c->num_sweeps += done_now;
    completed = c->hsc->iteration;
    if (c->hsc->done) break;
  }
  c->keff = c->hsc->keff;
  c->residual = c->hsc->residual;
  return MOC_OK;
}

// Drops the on-the-fly description (new tracks invalidate it).
void otf_release(moc_ctx* c) {
  dfree(c->otf_trk);
  dfree(c->otf_trk_f);
  dfree(c->otf_ang);
  dfree(c->otf_rad);
  dfree(c->otf_rad_start);
  dfree(c->otf_rad_off);
  dfree(c->otf_rad_total);
  dfree(c->otf_order);
  if (c->otf && !c->shape_user_set) c->lps = c->slots = 0;
  if (c->otf) c->tuned = false;
  c->otf = false;
}

// The material of the region above the cut, packed with its id.
int otf_above_word(moc_ctx* c) {
  int32_t m = 0;
  MOC_CUDA(cudaMemcpy(&m, c->fsr_mat + c->otf_above_fsr, 4,
                      cudaMemcpyDeviceToHost));
  c->otf_above_word = c->otf_above_fsr | (m << 24);
  return MOC_OK;
}

// Drops the linear source (new tracks invalidate the start positions).
void ls_release(moc_ctx* c) {
  dfree(c->segs_ls);
  dfree(c->ls_ang);
  dfree(c->ls_dir);
  dfree(c->mom);
  dfree(c->qxy);
  dfree(c->ls_ilem);
  dfree(c->ls_const);
  dfree(c->fixed_xy);
  dfree(c->ls_segz);
  dfree(c->ls_dir3);
  dfree(c->momz);
  dfree(c->qz);
  dfree(c->fixed_z);
  c->ls3d = false;
  if (c->ls && !c->shape_user_set) c->lps = c->slots = 0;
  if (c->ls) c->tuned = false;
  c->ls = false;
  c->ls_num_flat = 0;
}

// The linear expansion constants from the uploaded segments, quadrature,
// cross sections and volumes (re-run when any of the last two change).
int ls_constants(moc_ctx* c) {
  const int64_t R = c->d.num_fsrs, T = c->d.num_tracks;
  const int G = c->d.num_groups, A = c->d.num_angles;
  const int Ph = c->d.num_polar_half;
  unsigned int* nflat = nullptr;
  MOC_TRY(dalloc(&nflat, 1));
  const double* ang = c->ls_ang;
  const int rc = moc::launch_ls_constants(
      c->segs_ls, c->seg_off, c->track_ang, T, c->d.num_segments, ang,
      ang + 2 * A, ang + 3 * A, ang + 3 * A + A * Ph, Ph, c->sigma_t,
      c->fsr_vol, c->fsr_mat, R, G, row_stride(c), c->ls_ilem, c->ls_const,
      nflat, c->stream, c->ls3d ? c->ls_segz : nullptr,
      c->ls3d ? ang + 3 * A + 2 * A * Ph : nullptr);
  c->launches += 4;
  unsigned int h = 0;
  cudaError_t e = (cudaError_t) rc;
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(&h, nflat, sizeof(h), cudaMemcpyDeviceToHost,
                        c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  dfree(nflat);
  if (e != cudaSuccess)
    return fail(MOC_ERR_CUDA, std::string("linear expansion constants: ") +
                                  cudaGetErrorString(e));
  c->ls_num_flat = h;
  return MOC_OK;
}

// Nodes of the attenuation table: 1 - exp(-x_i) then exp(-x_i), both from
// double precision, x_i = i * h.
void build_exp_table(std::vector<float>& t) {
  const int n = moc::kExpTableSize;
  t.resize(2 * n);
  for (int i = 0; i < n; i++) {
    const double x = (double) i * (double) moc::kExpTableH;
    t[i] = (float) (-std::expm1(-x));
    t[n + i] = (float) std::exp(-x);
  }
}

}  // namespace

extern "C" {

const char* moc_last_error(void) { return g_error.c_str(); }

const char* moc_version(void) { return "openmoc_gb300 0.1 (sm_103a)"; }

int moc_release_cached_memory(void) {
  release_idle(-1);
  {
    std::lock_guard<std::mutex> lk(g_bounce_mu);
    if (g_bounce) cudaFreeHost(g_bounce);
    g_bounce = nullptr;
    g_bounce_bytes = 0;
  }
  std::lock_guard<std::mutex> lk(g_pinned_mu);
  for (void* h : g_pinned_scalars) cudaFreeHost(h);
  g_pinned_scalars.clear();
  return MOC_OK;
}

int moc_create(const moc_dims* dims, moc_ctx** out) {
  MOC_CHECK(dims != nullptr && out != nullptr, MOC_ERR_ARG, "null argument");
  *out = nullptr;
  const moc_dims& d = *dims;
  MOC_CHECK(d.num_groups >= 1 && d.num_groups <= 64 * moc::kMaxSlots,
            MOC_ERR_ARG, "num_groups must be in [1, 384]");
  MOC_CHECK(d.num_polar_half >= 1 && moc::sweep_max_slots(d.num_polar_half) > 0,
            MOC_ERR_UNSUPPORTED,
            "num_polar_half must be 1, 2 or 3 (2, 4 or 6 polar angles in 2D)");
  MOC_CHECK(d.num_angles >= 1 && d.num_materials >= 1 && d.num_fsrs >= 1 &&
                d.num_tracks >= 1 && d.num_segments >= 0,
            MOC_ERR_ARG, "empty problem dimension");
  MOC_CHECK(d.num_tracks < (1LL << 31) && d.num_fsrs < (1LL << 31),
            MOC_ERR_ARG, "tracks and FSRs are limited to 2^31");
  MOC_CHECK((int64_t) d.num_materials * d.num_groups <= 16384, MOC_ERR_ARG,
            "num_materials * num_groups is limited to 16384");
  int ndev = 0;
  MOC_CUDA(cudaGetDeviceCount(&ndev));
  MOC_CHECK(d.device >= 0 && d.device < ndev, MOC_ERR_ARG,
            "no CUDA device " + std::to_string(d.device));
  MOC_CUDA(cudaSetDevice(d.device));
  moc::configure_kernels();

  moc_ctx* c = new moc_ctx();
  c->d = d;
  int st = MOC_OK;
  auto bail = [&](int s) {
    moc_destroy(c);
    return s;
  };
  if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) !=
      cudaSuccess)
    return bail(fail(MOC_ERR_CUDA, "cudaStreamCreate failed"));
  const int64_t R = d.num_fsrs, G = row_stride(c);
  const int64_t npsi = num_psi(c);
  // memory budget: state arrays plus tracks
  size_t need = sizeof(float) * (size_t) (3 * R * G + 2 * npsi) +
                sizeof(int2) * (size_t) d.num_segments +
                (sizeof(int64_t) + 4 * sizeof(int32_t) + 1) *
                    (size_t) d.num_tracks;
  size_t free_b = 0, total_b = 0;
  if (cudaMemGetInfo(&free_b, &total_b) == cudaSuccess &&
      need > free_b + idle_bytes_on(d.device))
    return bail(fail(MOC_ERR_MEMORY,
                     "problem needs " + std::to_string(need) +
                         " bytes of device memory, " +
                         std::to_string(free_b) + " free"));
  if ((st = dalloc(&c->phi, R * G)) || (st = dalloc(&c->phi_old, R * G)) ||
      (st = dalloc(&c->qt, R * G)) || (st = dalloc(&c->psi[0], npsi)) ||
      (st = dalloc(&c->psi[1], npsi)) ||
      (st = dalloc(&c->exp_table, 2 * moc::kExpTableSize)) ||
      (st = dalloc(&c->rates, R)) || (st = dalloc(&c->sc, 1)))
    return bail(st);
  {
    std::lock_guard<std::mutex> lk(g_pinned_mu);
    if (!g_pinned_scalars.empty()) {
      c->hsc = static_cast<moc::DevScalars*>(g_pinned_scalars.back());
      g_pinned_scalars.pop_back();
    }
  }
  if (!c->hsc && cudaMallocHost((void**) &c->hsc, sizeof(moc::DevScalars)) !=
                     cudaSuccess)
    return bail(fail(MOC_ERR_CUDA, "cudaMallocHost failed"));
  std::memset(c->hsc, 0, sizeof(moc::DevScalars));
  c->hsc->keff = 1.0;
  c->hsc->k_prev = 1.0;
  c->hsc->factor = 1.0;
  c->hsc->scale[0] = c->hsc->scale[1] = 1.0f;
  c->hsc->threshold = c->threshold;
  std::vector<float> tab;
  build_exp_table(tab);
  if (cudaMemcpy(c->exp_table, tab.data(), sizeof(float) * tab.size(),
                 cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(c->sc, c->hsc, sizeof(moc::DevScalars),
                 cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemset(c->phi, 0, sizeof(float) * R * G) != cudaSuccess ||
      cudaMemset(c->phi_old, 0, sizeof(float) * R * G) != cudaSuccess ||
      cudaMemset(c->qt, 0, sizeof(float) * R * G) != cudaSuccess ||
      cudaMemset(c->psi[0], 0, sizeof(float) * npsi) != cudaSuccess ||
      cudaMemset(c->psi[1], 0, sizeof(float) * npsi) != cudaSuccess)
    return bail(fail(MOC_ERR_CUDA, "device initialisation failed"));
  *out = c;
  return MOC_OK;
}

int moc_destroy(moc_ctx* c) {
  if (!c) return MOC_OK;
  cudaSetDevice(c->d.device);
  if (c->stream) cudaStreamSynchronize(c->stream);
  // nothing of this context runs any more: its blocks go back to the cache
  // without a device synchronisation each
  struct IdleScope {
    IdleScope() { g_device_idle = true; }
    ~IdleScope() { g_device_idle = false; }
  } idle_scope;
  dfree(c->segs);
  dfree(c->seg_off);
  dfree(c->order);
  dfree(c->track_ang);
  dfree(c->next);
  dfree(c->flags);
  dfree(c->trec);
  dfree(c->weights);
  dfree(c->inv_sin);
  dfree(c->sigma_t);
  dfree(c->sigma_s);
  dfree(c->sigma_s_T);
  dfree(c->nu_sigma_f);
  dfree(c->chi);
  dfree(c->scat_out);
  dfree(c->sigma_f);
  dfree(c->fissile);
  dfree(c->fsr_mat);
  dfree(c->fsr_vol);
  dfree(c->fixed);
  dfree(c->phi);
  dfree(c->phi_old);
  dfree(c->qt);
  dfree(c->psi[0]);
  dfree(c->psi[1]);
  dfree(c->exp_table);
  dfree(c->rates);
  dfree(c->flush);
  dfree(c->tc_rows);
  dfree(c->tc_tile_mat);
  dfree(c->tc_b);
  dfree(c->stab);
  dfree(c->stab_base);
  dfree(c->stab_mom);
  dfree(c->stab_momz);
  dfree(c->inst);
  dfree(c->segs_ls);
  dfree(c->ls_ang);
  dfree(c->ls_dir);
  dfree(c->mom);
  dfree(c->qxy);
  dfree(c->ls_ilem);
  dfree(c->ls_const);
  dfree(c->fixed_xy);
  dfree(c->ls_segz);
  dfree(c->ls_dir3);
  dfree(c->momz);
  dfree(c->qz);
  dfree(c->fixed_z);
  dfree(c->otf_trk);
  dfree(c->otf_trk_f);
  dfree(c->otf_ang);
  dfree(c->otf_rad);
  dfree(c->otf_rad_start);
  dfree(c->otf_rad_off);
  dfree(c->otf_rad_total);
  dfree(c->otf_order);
  cmfd_release(c);
  dfree(c->sc);
  if (c->hsc) {
    std::lock_guard<std::mutex> lk(g_pinned_mu);
    if (g_pinned_scalars.size() < 64) g_pinned_scalars.push_back(c->hsc);
    else cudaFreeHost(c->hsc);
  }
  for (cudaEvent_t e : c->ev) cudaEventDestroy(e);
  if (c->stream) cudaStreamDestroy(c->stream);
  delete c;
  return MOC_OK;
}

int moc_upload_tracks(moc_ctx* c, const float* seg_len, const int32_t* seg_fsr,
                      const int64_t* seg_off, const int32_t* track_ang,
                      const int64_t* next, const uint8_t* flags) {
  MOC_CHECK(c && seg_off && track_ang && next && flags, MOC_ERR_ARG,
            "null argument");
  const int64_t T = c->d.num_tracks, S = c->d.num_segments;
  const int64_t R = c->d.num_fsrs;
  MOC_CHECK(S == 0 || (seg_len && seg_fsr), MOC_ERR_ARG, "null segments");
  MOC_CHECK(seg_off[0] == 0 && seg_off[T] == S, MOC_ERR_ARG,
            "seg_off must run from 0 to num_segments");
  std::vector<int64_t> count(T);
  for (int64_t t = 0; t < T; t++) {
    count[t] = seg_off[t + 1] - seg_off[t];
    MOC_CHECK(count[t] >= 0 && count[t] < (1LL << 31), MOC_ERR_ARG,
              "bad segment count on track " + std::to_string(t));
    MOC_CHECK(track_ang[t] >= 0 && track_ang[t] < c->d.num_angles,
              MOC_ERR_ARG, "track angle index out of range");
    for (int d = 0; d < 2; d++)
      MOC_CHECK(next[2 * t + d] >= 0 && next[2 * t + d] < T, MOC_ERR_ARG,
                "next-track index out of range on track " +
                    std::to_string(t));
  }
  // longest tracks first (stable, so equal lengths keep UID order)
  std::vector<int32_t> order(T);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int32_t a, int32_t b) {
    return count[a] > count[b];
  });
  std::vector<int32_t> next32(2 * T);
  for (int64_t i = 0; i < 2 * T; i++) next32[i] = (int32_t) next[i];
  MOC_CUDA(cudaSetDevice(c->d.device));
  dfree(c->segs);
  dfree(c->seg_off);
  dfree(c->order);
  dfree(c->track_ang);
  dfree(c->next);
  dfree(c->flags);
  dfree(c->trec);
  MOC_TRY(dalloc(&c->segs, S));
  // segments: raw lengths and FSR ids up, packed and checked on the device
  {
    float* d_len = nullptr;
    int32_t* d_fsr = nullptr;
    unsigned long long* d_chk = nullptr;   // [0] first bad index, [1..] tail
    int st = dalloc(&d_len, S);
    if (!st) st = dalloc(&d_fsr, S);
    if (!st) st = dalloc(&d_chk, 1 + moc::kMaxHotFsrs);
    std::vector<unsigned long long> chk(1 + moc::kMaxHotFsrs, 0);
    chk[0] = ~0ull;
    cudaError_t e = cudaSuccess;
    if (!st && S > 0) {
      e = cudaMemcpy(d_len, seg_len, 4 * S, cudaMemcpyHostToDevice);
      if (e == cudaSuccess)
        e = cudaMemcpy(d_fsr, seg_fsr, 4 * S, cudaMemcpyHostToDevice);
      if (e == cudaSuccess)
        e = cudaMemcpy(d_chk, chk.data(), 8 * chk.size(), cudaMemcpyHostToDevice);
      if (e == cudaSuccess) {
        moc::launch_pack_segments(d_len, d_fsr, c->segs, S, R, d_chk, d_chk + 1,
                                  c->stream);
        e = cudaStreamSynchronize(c->stream);
      }
      if (e == cudaSuccess)
        e = cudaMemcpy(chk.data(), d_chk, 8 * chk.size(), cudaMemcpyDeviceToHost);
    }
    dfree(d_len);
    dfree(d_fsr);
    dfree(d_chk);
    MOC_TRY(st);
    MOC_CUDA(e);
    if (chk[0] != ~0ull) {
      const int64_t i = (int64_t) chk[0];
      dfree(c->segs);
      MOC_CHECK(seg_fsr[i] >= 0 && seg_fsr[i] < R, MOC_ERR_ARG,
                "segment FSR id out of range at segment " + std::to_string(i));
      return fail(MOC_ERR_ARG, "bad segment length at segment " +
                                   std::to_string(i));
    }
    // trailing FSR ids crossed by at least 0.2 % of all segments each
    c->hot_count = 0;
    while (c->hot_count < moc::kMaxHotFsrs && c->hot_count < R && S > 0) {
      const int64_t r = R - 1 - c->hot_count;          // FSR id
      const int64_t slot = r - (R - moc::kMaxHotFsrs);  // its tail counter
      if (slot < 0 || chk[1 + slot] * 500 < (unsigned long long) S) break;
      c->hot_count++;
    }
    c->hot_base = (int) (R - c->hot_count);
  }
  MOC_TRY(dalloc(&c->seg_off, T + 1));
  MOC_TRY(dalloc(&c->order, T));
  MOC_TRY(dalloc(&c->track_ang, T));
  MOC_TRY(dalloc(&c->next, 2 * T));
  MOC_TRY(dalloc(&c->flags, T));
  MOC_CUDA(cudaMemcpy(c->seg_off, seg_off, sizeof(int64_t) * (T + 1),
                      cudaMemcpyHostToDevice));
  MOC_CUDA(cudaMemcpy(c->order, order.data(), sizeof(int32_t) * T,
                      cudaMemcpyHostToDevice));
  {
    std::vector<moc::TrackRec> rec(T);
    for (int64_t i = 0; i < T; i++) {
      const int32_t t = order[i];
      moc::TrackRec& r = rec[i];
      r.off = seg_off[t];
      r.t = t;
      r.n = (int32_t) count[t];
      r.ang = track_ang[t];
      r.flags = flags[t];
      r.next[0] = next32[2 * t];
      r.next[1] = next32[2 * t + 1];
    }
    MOC_TRY(dalloc(&c->trec, T));
    MOC_CUDA(cudaMemcpy(c->trec, rec.data(), sizeof(moc::TrackRec) * T,
                        cudaMemcpyHostToDevice));
  }
  MOC_CUDA(cudaMemcpy(c->track_ang, track_ang, sizeof(int32_t) * T,
                      cudaMemcpyHostToDevice));
  MOC_CUDA(cudaMemcpy(c->next, next32.data(), sizeof(int32_t) * 2 * T,
                      cudaMemcpyHostToDevice));
  MOC_CUDA(cudaMemcpy(c->flags, flags, T, cudaMemcpyHostToDevice));
  ls_release(c);
  otf_release(c);
  cmfd_release(c);
  c->have_tracks = true;
  MOC_TRY(pack_materials(c));
  return MOC_OK;
}

int moc_upload_quadrature(moc_ctx* c, const float* weights,
                          const float* inv_sin) {
  MOC_CHECK(c && weights && inv_sin, MOC_ERR_ARG, "null argument");
  const int64_t n = (int64_t) c->d.num_angles * c->d.num_polar_half;
  for (int64_t i = 0; i < n; i++)
    MOC_CHECK(std::isfinite(weights[i]) && std::isfinite(inv_sin[i]) &&
                  inv_sin[i] >= 1.0f,
              MOC_ERR_ARG, "bad quadrature entry " + std::to_string(i));
  MOC_CUDA(cudaSetDevice(c->d.device));
  dfree(c->weights);
  dfree(c->inv_sin);
  MOC_TRY(dalloc(&c->weights, n));
  MOC_TRY(dalloc(&c->inv_sin, n));
  MOC_CUDA(cudaMemcpy(c->weights, weights, sizeof(float) * n,
                      cudaMemcpyHostToDevice));
  MOC_CUDA(cudaMemcpy(c->inv_sin, inv_sin, sizeof(float) * n,
                      cudaMemcpyHostToDevice));
  c->have_quad = true;
  return MOC_OK;
}

static void count_fissionable(moc_ctx* c, const int32_t* fsr_mat) {
  c->num_fissionable = 0;
  for (int64_t r = 0; r < c->d.num_fsrs; r++)
    c->num_fissionable += c->h_fissile[fsr_mat[r]] ? 1 : 0;
}

int moc_upload_materials(moc_ctx* c, const float* sigma_t,
                         const float* sigma_s, const float* nu_sigma_f,
                         const float* chi) {
  MOC_CHECK(c && sigma_t && sigma_s && nu_sigma_f && chi, MOC_ERR_ARG,
            "null argument");
  const int M = c->d.num_materials, G = c->d.num_groups;
  const int64_t MG = (int64_t) M * G;
  std::vector<float> scat_out(MG, 0.0f);
  std::vector<float> ssT((size_t) MG * G);
  std::vector<uint8_t> fis(M, 0);
  for (int m = 0; m < M; m++) {
    for (int g = 0; g < G; g++) {
      const int64_t i = (int64_t) m * G + g;
      MOC_CHECK(std::isfinite(sigma_t[i]) && sigma_t[i] > 0.0f, MOC_ERR_ARG,
                "sigma_t must be positive and finite (material " +
                    std::to_string(m) + ", group " + std::to_string(g + 1) +
                    ")");
      MOC_CHECK(std::isfinite(nu_sigma_f[i]) && std::isfinite(chi[i]),
                MOC_ERR_ARG, "non-finite fission data in material " +
                                 std::to_string(m));
      if (nu_sigma_f[i] > 0.0f) fis[m] = 1;
    }
    for (int gd = 0; gd < G; gd++)
      for (int g = 0; g < G; g++) {
        const float v = sigma_s[((int64_t) m * G + gd) * G + g];
        MOC_CHECK(std::isfinite(v), MOC_ERR_ARG,
                  "non-finite scattering data in material " +
                      std::to_string(m));
        scat_out[(int64_t) m * G + g] += v;
        ssT[((int64_t) m * G + g) * G + gd] = v;
      }
  }
  c->h_sigma_t.assign(sigma_t, sigma_t + MG);
  c->h_scat_diag.resize(MG);
  for (int m = 0; m < M; m++)
    for (int g = 0; g < G; g++)
      c->h_scat_diag[(int64_t) m * G + g] =
          sigma_s[((int64_t) m * G + g) * G + g];
  c->stab_dirty = true;
  MOC_CUDA(cudaSetDevice(c->d.device));
  dfree(c->sigma_t);
  dfree(c->sigma_s);
  dfree(c->sigma_s_T);
  dfree(c->nu_sigma_f);
  dfree(c->chi);
  dfree(c->scat_out);
  dfree(c->fissile);
  MOC_TRY(dalloc(&c->sigma_t, MG));
  MOC_TRY(dalloc(&c->sigma_s, MG * G));
  // padded to whole 16-byte words: the source kernel stages it as float4
  MOC_TRY(dalloc(&c->sigma_s_T, MG * G + 4));
  MOC_CUDA(cudaMemset(c->sigma_s_T, 0, 4 * (MG * G + 4)));
  MOC_CUDA(cudaMemcpy(c->sigma_s_T, ssT.data(), 4 * MG * G,
                      cudaMemcpyHostToDevice));
  MOC_TRY(dalloc(&c->nu_sigma_f, MG));
  MOC_TRY(dalloc(&c->chi, MG));
  MOC_TRY(dalloc(&c->scat_out, MG));
  MOC_TRY(dalloc(&c->fissile, M));
  MOC_CUDA(cudaMemcpy(c->sigma_t, sigma_t, 4 * MG, cudaMemcpyHostToDevice));
  MOC_CUDA(cudaMemcpy(c->sigma_s, sigma_s, 4 * MG * G, cudaMemcpyHostToDevice));
  MOC_CUDA(cudaMemcpy(c->nu_sigma_f, nu_sigma_f, 4 * MG,
                      cudaMemcpyHostToDevice));
  MOC_CUDA(cudaMemcpy(c->chi, chi, 4 * MG, cudaMemcpyHostToDevice));
  MOC_CUDA(cudaMemcpy(c->scat_out, scat_out.data(), 4 * MG,
                      cudaMemcpyHostToDevice));
  MOC_CUDA(cudaMemcpy(c->fissile, fis.data(), M, cudaMemcpyHostToDevice));
  dfree(c->tc_b);
  if (moc::tc_sources_supported(G)) {
    std::vector<float> b;
    moc::tc_pack_scattering(sigma_s, M, G, b);
    MOC_TRY(dalloc(&c->tc_b, b.size()));
    MOC_CUDA(cudaMemcpy(c->tc_b, b.data(), 4 * b.size(), cudaMemcpyHostToDevice));
  }
  c->h_fissile = fis;
  c->h_chi.assign(chi, chi + MG);
  c->have_mats = true;
  if (c->ls && c->have_fsrs) MOC_TRY(ls_constants(c));
  return MOC_OK;
}

int moc_upload_sigma_f(moc_ctx* c, const float* sigma_f) {
  MOC_CHECK(c && sigma_f, MOC_ERR_ARG, "null argument");
  const int64_t MG = (int64_t) c->d.num_materials * c->d.num_groups;
  MOC_CUDA(cudaSetDevice(c->d.device));
  dfree(c->sigma_f);
  MOC_TRY(dalloc(&c->sigma_f, MG));
  MOC_CUDA(cudaMemcpy(c->sigma_f, sigma_f, 4 * MG, cudaMemcpyHostToDevice));
  return MOC_OK;
}

int moc_upload_fsrs(moc_ctx* c, const int32_t* fsr_mat, const float* fsr_vol) {
  MOC_CHECK(c && fsr_mat && fsr_vol, MOC_ERR_ARG, "null argument");
  MOC_CHECK(c->have_mats, MOC_ERR_STATE, "upload materials before FSRs");
  const int64_t R = c->d.num_fsrs;
  for (int64_t r = 0; r < R; r++) {
    MOC_CHECK(fsr_mat[r] >= 0 && fsr_mat[r] < c->d.num_materials, MOC_ERR_ARG,
              "FSR material index out of range at FSR " + std::to_string(r));
    MOC_CHECK(std::isfinite(fsr_vol[r]) && fsr_vol[r] >= 0.0f, MOC_ERR_ARG,
              "bad FSR volume at FSR " + std::to_string(r));
  }
  MOC_CUDA(cudaSetDevice(c->d.device));
  dfree(c->fsr_mat);
  dfree(c->fsr_vol);
  MOC_TRY(dalloc(&c->fsr_mat, R));
  MOC_TRY(dalloc(&c->fsr_vol, R));
  MOC_CUDA(cudaMemcpy(c->fsr_mat, fsr_mat, 4 * R, cudaMemcpyHostToDevice));
  MOC_CUDA(cudaMemcpy(c->fsr_vol, fsr_vol, 4 * R, cudaMemcpyHostToDevice));
  c->h_mat_used.assign(c->d.num_materials, 0);
  for (int64_t r = 0; r < R; r++) c->h_mat_used[fsr_mat[r]] = 1;
  c->stab_dirty = true;
  count_fissionable(c, fsr_mat);
  // tensor-core source tiles: FSR ids grouped by material, each material's
  // list padded to whole tiles with -1
  dfree(c->tc_rows);
  dfree(c->tc_tile_mat);
  c->tc_tiles = 0;
  if (moc::tc_sources_supported(c->d.num_groups)) {
    std::vector<std::vector<int32_t>> by_mat(c->d.num_materials);
    for (int64_t r = 0; r < R; r++) by_mat[fsr_mat[r]].push_back((int32_t) r);
    std::vector<int32_t> rows, tile_mat;
    for (int m = 0; m < c->d.num_materials; m++) {
      const int64_t n = (int64_t) by_mat[m].size();
      for (int64_t t0 = 0; t0 < n; t0 += moc::kTcRows) {
        tile_mat.push_back(m);
        for (int64_t i = 0; i < moc::kTcRows; i++)
          rows.push_back(t0 + i < n ? by_mat[m][t0 + i] : -1);
      }
    }
    c->tc_tiles = (int) tile_mat.size();
    MOC_TRY(dalloc(&c->tc_rows, rows.size()));
    MOC_TRY(dalloc(&c->tc_tile_mat, tile_mat.size()));
    MOC_CUDA(cudaMemcpy(c->tc_rows, rows.data(), 4 * rows.size(),
                        cudaMemcpyHostToDevice));
    MOC_CUDA(cudaMemcpy(c->tc_tile_mat, tile_mat.data(), 4 * tile_mat.size(),
                        cudaMemcpyHostToDevice));
  }
  // the FISSION_SOURCE residual norm is read on the device by every
  // residual launch, hooks included
  MOC_TRY(pull(c));
  c->hsc->num_fissionable = c->num_fissionable;
  MOC_TRY(push(c));
  c->have_fsrs = true;
  MOC_TRY(pack_materials(c));
  if (c->ls) {
    // new FSR materials: refresh the material bits of the segment words
    moc::launch_ls_refresh_ids(c->segs, c->segs_ls, c->d.num_segments,
                               c->stream);
    c->launches++;
    MOC_TRY(ls_constants(c));
  }
  if (c->otf) {
    moc::launch_pack_materials(c->otf_rad, c->otf_S2, c->fsr_mat, c->stream);
    c->launches++;
    MOC_CUDA(cudaStreamSynchronize(c->stream));
    MOC_TRY(otf_above_word(c));
  }
  return MOC_OK;
}

int moc_set_fixed_sources(moc_ctx* c, const float* q) {
  MOC_CHECK(c, MOC_ERR_ARG, "null context");
  MOC_CUDA(cudaSetDevice(c->d.device));
  if (!q) {
    dfree(c->fixed);
    return MOC_OK;
  }
  const int64_t n = num_host_flux(c);
  for (int64_t i = 0; i < n; i++)
    MOC_CHECK(std::isfinite(q[i]), MOC_ERR_ARG, "non-finite fixed source");
  if (!c->fixed) {
    MOC_TRY(dalloc(&c->fixed, num_flux(c)));
    MOC_CUDA(cudaMemset(c->fixed, 0, 4 * num_flux(c)));
  }
  const int G = c->d.num_groups, ld = row_stride(c);
  MOC_CUDA(cudaMemcpy2D(c->fixed, 4 * ld, q, 4 * G, 4 * G, c->d.num_fsrs,
                        cudaMemcpyHostToDevice));
  return MOC_OK;
}

int moc_set_convergence_threshold(moc_ctx* c, double threshold) {
  MOC_CHECK(c, MOC_ERR_ARG, "null context");
  MOC_CHECK(threshold > 0.0 && std::isfinite(threshold), MOC_ERR_ARG,
            "the convergence threshold must be positive");
  c->threshold = threshold;
  return MOC_OK;
}

int moc_set_exponential(moc_ctx* c, int kind) {
  MOC_CHECK(c, MOC_ERR_ARG, "null context");
  MOC_CHECK(kind == MOC_EXP_TABLE || kind == MOC_EXP_INTRINSIC, MOC_ERR_ARG,
            "unknown exponential evaluator");
  c->exp_kind = kind;
  c->exp_user_set = 1;
  c->tuned = false;
  return MOC_OK;
}

int moc_get_exponential(moc_ctx* c, int* kind) {
  MOC_CHECK(c && kind, MOC_ERR_ARG, "null argument");
  *kind = c->exp_kind;
  return MOC_OK;
}

int moc_set_autotune(moc_ctx* c, int on) {
  MOC_CHECK(c, MOC_ERR_ARG, "null context");
  c->autotune = on ? 1 : 0;
  if (on) c->tuned = false;
  return MOC_OK;
}

int moc_autotune(moc_ctx* c, int* lps, int* slots, int* exp_kind) {
  MOC_TRY(ready(c));
  c->tuned = false;
  const int user_shape = c->shape_user_set;
  c->shape_user_set = 0;
  int st = autotune_sweep(c, false);
  c->shape_user_set = user_shape;
  MOC_TRY(st);
  // the timing sweeps leave undefined tallies and angular fluxes behind
  MOC_TRY(zero_track_fluxes(c));
  MOC_CUDA(cudaMemsetAsync(c->phi, 0, 4 * num_flux(c), c->stream));
  MOC_TRY(zero_moments(c));
  if (lps) *lps = c->lps;
  if (slots) *slots = c->slots;
  if (exp_kind) *exp_kind = c->exp_kind;
  return MOC_OK;
}

int moc_get_tuning_log(moc_ctx* c, int* lps, int* slots, int* exp_kind,
                       float* ms, int capacity, int* count) {
  MOC_CHECK(c && count, MOC_ERR_ARG, "null argument");
  *count = (int) c->tune_log.size();
  for (int i = 0; i < (int) c->tune_log.size() && i < capacity; i++) {
    lps[i] = c->tune_log[i].lps;
    slots[i] = c->tune_log[i].slots;
    exp_kind[i] = c->tune_log[i].exp_kind;
    ms[i] = c->tune_log[i].ms;
  }
  return MOC_OK;
}

int moc_set_sweep_shape(moc_ctx* c, int lps, int slots) {
  MOC_CHECK(c, MOC_ERR_ARG, "null context");
  if (lps == 0) {
    c->lps = 0;
    c->slots = 0;
    c->shape_user_set = 0;
    c->tuned = false;
    return MOC_OK;
  }
  MOC_CHECK(moc::sweep_lps_supported(lps), MOC_ERR_ARG,
            "lanes per track direction must be 1, 2, 4, 8, 16 or 32");
  MOC_CHECK(slots >= 1 && slots <= max_slots(c) &&
                2 * (int64_t) lps * slots >= c->d.num_groups,
            MOC_ERR_ARG,
            "lanes x group pairs per lane must cover every group");
  MOC_CHECK(slots == pair_slots(c->d.num_groups, lps), MOC_ERR_ARG,
            "group pairs per lane must be the fewest that cover the groups, "
            "ceil(ceil(G / 2) / lanes)");
  c->lps = lps;
  c->slots = slots;
  c->shape_user_set = 1;
  return MOC_OK;
}

int moc_get_sweep_shape(moc_ctx* c, int* lps, int* slots) {
  MOC_CHECK(c && lps && slots, MOC_ERR_ARG, "null argument");
  if (c->lps == 0)
    pick_shape(c->d.num_groups, &c->lps, &c->slots, max_slots(c));
  *lps = c->lps;
  *slots = c->slots;
  return MOC_OK;
}

int moc_set_tensor_wait_limit(moc_ctx* c, int64_t polls) {
  MOC_CHECK(c, MOC_ERR_ARG, "null context");
  MOC_CHECK(polls <= (int64_t) 0xFFFFFFFFu, MOC_ERR_ARG,
            "the wait limit must fit 32 bits");
  c->tc_wait_limit = polls < 0 ? -1 : polls;
  return MOC_OK;
}

int moc_set_source_kernel(moc_ctx* c, int kind) {
  MOC_CHECK(c, MOC_ERR_ARG, "null context");
  MOC_CHECK(kind == MOC_SOURCES_AUTO || kind == MOC_SOURCES_FP32 ||
                kind == MOC_SOURCES_TF32X3,
            MOC_ERR_ARG, "unknown source kernel");
  MOC_CHECK(kind != MOC_SOURCES_TF32X3 ||
                moc::tc_sources_supported(c->d.num_groups),
            MOC_ERR_UNSUPPORTED,
            "the tensor-core source kernel takes 64 to 96 groups");
  c->source_kind = kind;
  return MOC_OK;
}

int moc_get_source_kernel(moc_ctx* c, int* kind) {
  MOC_CHECK(c && kind, MOC_ERR_ARG, "null argument");
  *kind = use_tc_sources(c) ? MOC_SOURCES_TF32X3 : MOC_SOURCES_FP32;
  return MOC_OK;
}

int moc_set_iterations_per_sync(moc_ctx* c, int k) {
  MOC_CHECK(c && k >= 1 && k <= 1024, MOC_ERR_ARG, "k must be in [1, 1024]");
  c->iters_per_sync = k;
  return MOC_OK;
}

// ---------------------------------------------------------------- solves
int moc_compute_eigenvalue(moc_ctx* c, int max_iters, int res_type) {
  MOC_TRY(ready(c));
  MOC_CHECK(max_iters >= 1, MOC_ERR_ARG, "max_iters must be positive");
  MOC_CHECK(res_type >= 0 && res_type <= 2, MOC_ERR_ARG, "bad residual type");
  MOC_CHECK(res_type != MOC_FISSION_SOURCE || c->num_fissionable > 0,
            MOC_ERR_ARG,
            "The Solver is unable to compute a FISSION_SOURCE residual "
            "without fissionable FSRs");
  MOC_CHECK(c->num_fissionable > 0, MOC_ERR_ARG,
            "an eigenvalue solve needs fissionable material");
  MOC_CHECK(!c->num_instances || !(c->ls || c->otf || c->cmfd || c->stab_on ||
                                   c->keff_balance),
            MOC_ERR_UNSUPPORTED,
            "instances are built for the flat-source eigenvalue loop of stored "
            "segments (no linear source, on-the-fly segments, CMFD, "
            "stabilization or neutron-balance keff)");
  if (c->cmfd) {
    MOC_CHECK(!c->otf, MOC_ERR_UNSUPPORTED,
              "CMFD acceleration of an on-the-fly solve is not supported");
    MOC_TRY(cmfd_prepare(c));
  }
  MOC_TRY(maybe_autotune(c));
  // Solver::computeInitialFluxGuess: flat flux 1, normalised, stored;
  // zero boundary fluxes (src/Solver.cpp:1710-1757)
  MOC_TRY(zero_track_fluxes(c));
  MOC_TRY(begin_solve(c, moc::kModeEigen, max_iters, res_type, 1.0));
  if (c->num_instances) MOC_TRY(reset_instances(c));
  moc::SolverArgs a = solver_args(c, 0);
  enqueue_initial_guess(c, a);
  MOC_TRY(zero_moments(c));
  MOC_CUDA(cudaMemcpyAsync(c->phi_old, c->phi, 4 * num_flux(c),
                           cudaMemcpyDeviceToDevice, c->stream));
  MOC_CUDA(cudaGetLastError());
  if (c->cmfd)
    MOC_TRY(run_cmfd_iterations(c, res_type));
  else
    MOC_TRY(run_iterations(c, moc::kModeEigen, res_type));
  c->num_iterations = c->hsc->iteration;
  return MOC_OK;
}

int moc_compute_source(moc_ctx* c, int max_iters, double k_eff,
                       int res_type) {
  MOC_TRY(ready(c));
  MOC_CHECK(!c->num_instances, MOC_ERR_UNSUPPORTED,
            "instances are solved by moc_compute_eigenvalue only");
  MOC_CHECK(max_iters >= 1, MOC_ERR_ARG, "max_iters must be positive");
  MOC_CHECK(k_eff > 0.0, MOC_ERR_ARG,
            "The Solver is unable to compute the source with a non-positive "
            "keff");
  MOC_CHECK(res_type >= 0 && res_type <= 2, MOC_ERR_ARG, "bad residual type");
  MOC_TRY(maybe_autotune(c));
  MOC_TRY(zero_track_fluxes(c));
  MOC_TRY(begin_solve(c, moc::kModeSource, max_iters, res_type, k_eff));
  moc::launch_fill(c->phi, num_flux(c), 1.0f, c->stream);
  MOC_TRY(zero_moments(c));
  c->launches++;
  MOC_CUDA(cudaMemcpyAsync(c->phi_old, c->phi, 4 * num_flux(c),
                           cudaMemcpyDeviceToDevice, c->stream));
  MOC_TRY(run_iterations(c, moc::kModeSource, res_type));
  c->num_iterations =
      c->hsc->converged ? c->hsc->iteration - 1 : max_iters;
  return MOC_OK;
}

int moc_compute_flux(moc_ctx* c, int max_iters, int only_fixed_source) {
  MOC_TRY(ready(c));
  MOC_CHECK(!c->num_instances, MOC_ERR_UNSUPPORTED,
            "instances are solved by moc_compute_eigenvalue only");
  MOC_CHECK(max_iters >= 1, MOC_ERR_ARG, "max_iters must be positive");
  MOC_CHECK(only_fixed_source, MOC_ERR_UNSUPPORTED,
            "computeFlux without only_fixed_source needs a previous "
            "eigenvalue solve; use the hooks");
  MOC_TRY(maybe_autotune(c));
  MOC_TRY(zero_track_fluxes(c));
  MOC_TRY(begin_solve(c, moc::kModeFlux, max_iters, MOC_SCALAR_FLUX, 1.0));
  moc::SolverArgs a = solver_args(c, 0);
  moc::launch_fill(c->phi, num_flux(c), 0.0f, c->stream);
  MOC_TRY(zero_moments(c));
  MOC_CUDA(cudaMemcpyAsync(c->phi_old, c->phi, 4 * num_flux(c),
                           cudaMemcpyDeviceToDevice, c->stream));
  enqueue_sources(c, a, 0, 0);
  c->launches++;
  MOC_TRY(run_iterations(c, moc::kModeFlux, MOC_SCALAR_FLUX));
  c->num_iterations =
      c->hsc->converged ? c->hsc->iteration - 1 : max_iters;
  return MOC_OK;
}

// Fixed-count eigenvalue iterations for measurement: the loop body of
// computeEigenvalue with the convergence exit disabled, each iteration
// bracketed by CUDA events on the solver's stream (and its sweep by a second
// pair).  With flush_l2, a buffer twice the L2 size is overwritten before
// every iteration, outside the timed interval.
int moc_bench_iterations(moc_ctx* c, int steps, int res_type, int flush_l2,
                         double* step_ms, double* sweep_ms) {
  MOC_TRY(ready(c));
  MOC_CHECK(steps >= 1 && step_ms && sweep_ms, MOC_ERR_ARG, "bad arguments");
  if (flush_l2 && !c->flush) {
    int l2 = 0;
    MOC_CUDA(cudaDeviceGetAttribute(&l2, cudaDevAttrL2CacheSize,
                                    c->d.device));
    c->flush_n = std::max<int64_t>(2 * (int64_t) l2 / 4, 1 << 20);
    MOC_TRY(dalloc(&c->flush, c->flush_n));
  }
  MOC_TRY(maybe_autotune(c));
  // initial state as computeEigenvalue's first iteration sees it
  MOC_TRY(zero_track_fluxes(c));
  MOC_TRY(begin_solve(c, moc::kModeEigen, 1 << 30, res_type, 1.0));
  c->hsc->threshold = -1.0;  // never converged: every iteration runs
  MOC_TRY(push(c));
  if (c->num_instances) MOC_TRY(reset_instances(c));
  MOC_TRY(ensure_stab(c));
  moc::SolverArgs a = solver_args(c, 1);
  enqueue_initial_guess(c, a);
  MOC_TRY(zero_moments(c));
  MOC_CUDA(cudaMemcpyAsync(c->phi_old, c->phi, 4 * num_flux(c),
                           cudaMemcpyDeviceToDevice, c->stream));
  std::vector<cudaEvent_t> ev(4 * steps);
  for (auto& e : ev) MOC_CUDA(cudaEventCreate(&e));
  for (int i = 0; i < steps; i++) {
    if (flush_l2) moc::launch_fill(c->flush, c->flush_n, (float) i, c->stream);
    MOC_CUDA(cudaEventRecord(ev[4 * i], c->stream));
    MOC_TRY(enqueue_stab_moments_base(c));
    enqueue_sources(c, a, -1, 1);
    MOC_CUDA(cudaEventRecord(ev[4 * i + 1], c->stream));
    MOC_TRY(enqueue_sweep(c, 1, false, 0));
    MOC_CUDA(cudaEventRecord(ev[4 * i + 2], c->stream));
    enqueue_eigen_update(c, a);
    moc::launch_residual(a, res_type, 1, 1, 1, c->stream);
    MOC_CUDA(cudaEventRecord(ev[4 * i + 3], c->stream));
    c->launches++;
  }
  MOC_CUDA(cudaGetLastError());
  MOC_CUDA(cudaStreamSynchronize(c->stream));
  for (int i = 0; i < steps; i++) {
    float t = 0.f, s = 0.f;
    MOC_CUDA(cudaEventElapsedTime(&t, ev[4 * i], ev[4 * i + 3]));
    MOC_CUDA(cudaEventElapsedTime(&s, ev[4 * i + 1], ev[4 * i + 2]));
    step_ms[i] = t;
    sweep_ms[i] = s;
  }
  for (auto& e : ev) cudaEventDestroy(e);
  MOC_TRY(pull(c));
  c->keff = c->hsc->keff;
  c->num_iterations = c->hsc->iteration;
  return MOC_OK;
}

// --------------------------------------------------------------- results
int moc_get_keff(moc_ctx* c, double* keff) {
  MOC_CHECK(c && keff, MOC_ERR_ARG, "null argument");
  MOC_TRY(pull(c));
  *keff = c->hsc->keff;
  return MOC_OK;
}

int moc_get_num_iterations(moc_ctx* c, int* iters) {
  MOC_CHECK(c && iters, MOC_ERR_ARG, "null argument");
  *iters = c->num_iterations;
  return MOC_OK;
}

int moc_get_residual(moc_ctx* c, double* residual) {
  MOC_CHECK(c && residual, MOC_ERR_ARG, "null argument");
  MOC_TRY(pull(c));
  *residual = c->hsc->residual;
  return MOC_OK;
}

static int copy_out(moc_ctx* c, const float* src, float* out, int64_t n,
                    int64_t expected) {
  MOC_CHECK(c && out, MOC_ERR_ARG, "null argument");
  MOC_CHECK(n == expected, MOC_ERR_ARG,
            "expected " + std::to_string(expected) + " values, got " +
                std::to_string(n));
  MOC_CUDA(cudaSetDevice(c->d.device));
  MOC_CUDA(cudaMemcpyAsync(out, src, 4 * n, cudaMemcpyDeviceToHost, c->stream));
  MOC_CUDA(cudaStreamSynchronize(c->stream));
  return MOC_OK;
}

static int copy_in(moc_ctx* c, float* dst, const float* in, int64_t n,
                   int64_t expected) {
  MOC_CHECK(c && in, MOC_ERR_ARG, "null argument");
  MOC_CHECK(n == expected, MOC_ERR_ARG,
            "expected " + std::to_string(expected) + " values, got " +
                std::to_string(n));
  MOC_CUDA(cudaSetDevice(c->d.device));
  MOC_CUDA(cudaMemcpyAsync(dst, in, 4 * n, cudaMemcpyHostToDevice, c->stream));
  MOC_CUDA(cudaStreamSynchronize(c->stream));
  return MOC_OK;
}

// [R][G] host rows from / to the [R][ld] device layout.
static int copy_rows_out(moc_ctx* c, const float* src, float* out, int64_t n) {
  MOC_CHECK(c && out, MOC_ERR_ARG, "null argument");
  MOC_CHECK(n == num_host_flux(c), MOC_ERR_ARG,
            "expected " + std::to_string(num_host_flux(c)) + " values, got " +
                std::to_string(n));
  const int G = c->d.num_groups, ld = row_stride(c);
  const int64_t R = c->d.num_fsrs;
  MOC_CUDA(cudaSetDevice(c->d.device));
  cudaPointerAttributes attr;
  const bool locked = cudaPointerGetAttributes(&attr, out) == cudaSuccess &&
                      attr.type == cudaMemoryTypeHost;
  cudaGetLastError();
  const size_t bytes = sizeof(float) * (size_t) R * ld;
  if (!locked) {
    // the rows as they lie into the bounce buffer, then de-pitched here
    std::lock_guard<std::mutex> lk(g_bounce_mu);
    if (g_bounce_bytes < bytes) {
      if (g_bounce) cudaFreeHost(g_bounce);
      g_bounce = nullptr;
      g_bounce_bytes = 0;
      if (cudaMallocHost(&g_bounce, bytes) == cudaSuccess) {
        g_bounce_bytes = bytes;
      } else {
        cudaGetLastError();
        g_bounce = nullptr;
      }
    }
    if (g_bounce) {
      MOC_CUDA(cudaMemcpyAsync(g_bounce, src, bytes, cudaMemcpyDeviceToHost,
                               c->stream));
      MOC_CUDA(cudaStreamSynchronize(c->stream));
      const float* b = static_cast<const float*>(g_bounce);
      if (ld == G)
        std::memcpy(out, b, sizeof(float) * (size_t) R * G);
      else
        for (int64_t r = 0; r < R; r++)
          std::memcpy(out + r * G, b + r * ld, sizeof(float) * G);
      return MOC_OK;
    }
  }
  MOC_CUDA(cudaMemcpy2DAsync(out, 4 * G, src, 4 * ld, 4 * G, R,
                             cudaMemcpyDeviceToHost, c->stream));
  MOC_CUDA(cudaStreamSynchronize(c->stream));
  return MOC_OK;
}

static int copy_rows_in(moc_ctx* c, float* dst, const float* in, int64_t n) {
  MOC_CHECK(c && in, MOC_ERR_ARG, "null argument");
  MOC_CHECK(n == num_host_flux(c), MOC_ERR_ARG,
            "expected " + std::to_string(num_host_flux(c)) + " values, got " +
                std::to_string(n));
  const int G = c->d.num_groups, ld = row_stride(c);
  MOC_CUDA(cudaSetDevice(c->d.device));
  MOC_CUDA(cudaMemcpy2DAsync(dst, 4 * ld, in, 4 * G, 4 * G, c->d.num_fsrs,
                             cudaMemcpyHostToDevice, c->stream));
  MOC_CUDA(cudaStreamSynchronize(c->stream));
  return MOC_OK;
}

int moc_get_fluxes(moc_ctx* c, float* out, int64_t n) {
  MOC_CHECK(c, MOC_ERR_ARG, "null context");
  return copy_rows_out(c, c->phi, out, n);
}

int moc_set_fluxes(moc_ctx* c, const float* in, int64_t n) {
  MOC_CHECK(c, MOC_ERR_ARG, "null context");
  MOC_TRY(copy_rows_in(c, c->phi, in, n));
  return copy_rows_in(c, c->phi_old, in, n);
}

int moc_get_old_fluxes(moc_ctx* c, float* out, int64_t n) {
  MOC_CHECK(c, MOC_ERR_ARG, "null context");
  return copy_rows_out(c, c->phi_old, out, n);
}

int moc_set_old_fluxes(moc_ctx* c, const float* in, int64_t n) {
  MOC_CHECK(c, MOC_ERR_ARG, "null context");
  return copy_rows_in(c, c->phi_old, in, n);
}

int moc_get_reduced_sources(moc_ctx* c, float* out, int64_t n) {
  MOC_CHECK(c, MOC_ERR_ARG, "null context");
  MOC_TRY(copy_rows_out(c, c->qt, out, n));
  // the device keeps Q / (4 pi sigma_t); report Q / (4 pi)
  std::vector<float> st((size_t) c->d.num_materials * c->d.num_groups);
  std::vector<int32_t> mat(c->d.num_fsrs);
  MOC_CUDA(cudaMemcpy(st.data(), c->sigma_t, 4 * st.size(),
                      cudaMemcpyDeviceToHost));
  MOC_CUDA(cudaMemcpy(mat.data(), c->fsr_mat, 4 * mat.size(),
                      cudaMemcpyDeviceToHost));
  const int G = c->d.num_groups;
  for (int64_t r = 0; r < c->d.num_fsrs; r++)
    for (int g = 0; g < G; g++)
      out[r * G + g] *= st[(int64_t) mat[r] * G + g];
  return MOC_OK;
}

int moc_get_start_flux(moc_ctx* c, float* out, int64_t n) {
  MOC_CHECK(c, MOC_ERR_ARG, "null context");
  MOC_TRY(pull(c));
  const int cur = c->hsc->cur;
  const float scale = c->hsc->scale[cur];
  MOC_TRY(copy_out(c, c->psi[cur], out, n, num_psi(c)));
  if (scale != 1.0f)
    for (int64_t i = 0; i < n; i++) out[i] *= scale;
  return MOC_OK;
}

int moc_set_start_flux(moc_ctx* c, const float* in, int64_t n) {
  MOC_CHECK(c, MOC_ERR_ARG, "null context");
  MOC_TRY(copy_in(c, c->psi[0], in, n, num_psi(c)));
  MOC_TRY(copy_in(c, c->psi[1], in, n, num_psi(c)));
  MOC_TRY(pull(c));
  c->hsc->scale[0] = c->hsc->scale[1] = 1.0f;
  return push(c);
}

int moc_get_sweep_time(moc_ctx* c, double* ms, int64_t* num_sweeps) {
  MOC_CHECK(c && ms && num_sweeps, MOC_ERR_ARG, "null argument");
  *ms = c->sweep_ms;
  *num_sweeps = c->num_sweeps;
  return MOC_OK;
}

int moc_eval_attenuation(moc_ctx* c, int kind, const float* x, float* g,
                         int64_t n) {
  MOC_CHECK(c && x && g && n >= 0, MOC_ERR_ARG, "bad arguments");
  MOC_CHECK(kind == MOC_EXP_TABLE || kind == MOC_EXP_INTRINSIC, MOC_ERR_ARG,
            "unknown exponential evaluator");
  if (n == 0) return MOC_OK;
  MOC_CUDA(cudaSetDevice(c->d.device));
  float *dx = nullptr, *dg = nullptr;
  MOC_TRY(dalloc(&dx, n));
  int st = dalloc(&dg, n);
  if (st != MOC_OK) {
    dfree(dx);
    return st;
  }
  cudaError_t e = cudaMemcpyAsync(dx, x, 4 * n, cudaMemcpyHostToDevice,
                                  c->stream);
  if (e == cudaSuccess) {
    moc::launch_attenuation(kind, dx, dg, n, c->exp_table, c->stream);
    c->launches++;
    e = cudaGetLastError();
  }
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(g, dg, 4 * n, cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  dfree(dx);
  dfree(dg);
  MOC_CUDA(e);
  return MOC_OK;
}

int moc_get_launch_count(moc_ctx* c, int64_t* launches) {
  MOC_CHECK(c && launches, MOC_ERR_ARG, "null argument");
  *launches = c->launches;
  return MOC_OK;
}

// ----------------------------------------------------------------- hooks
int moc_zero_track_fluxes(moc_ctx* c) {
  MOC_TRY(ready(c));
  return zero_track_fluxes(c);
}

int moc_flatten_fsr_fluxes(moc_ctx* c, float value) {
  MOC_TRY(ready(c));
  moc::launch_fill(c->phi, num_flux(c), value, c->stream);
  c->launches++;
  MOC_TRY(zero_moments(c));
  MOC_CUDA(cudaGetLastError());
  return MOC_OK;
}

int moc_flatten_fsr_fluxes_chi(moc_ctx* c, int material) {
  MOC_TRY(ready(c));
  MOC_CHECK(material >= 0 && material < c->d.num_materials, MOC_ERR_ARG,
            "chi spectrum material out of range");
  float* d_chi = c->chi + (int64_t) material * c->d.num_groups;
  moc::launch_fill_chi(c->phi, d_chi, c->d.num_fsrs, c->d.num_groups,
                       row_stride(c), c->stream);
  c->launches++;
  MOC_TRY(zero_moments(c));
  MOC_CUDA(cudaGetLastError());
  return MOC_OK;
}

int moc_store_fsr_fluxes(moc_ctx* c) {
  MOC_TRY(ready(c));
  MOC_CUDA(cudaMemcpyAsync(c->phi_old, c->phi, 4 * num_flux(c),
                           cudaMemcpyDeviceToDevice, c->stream));
  return MOC_OK;
}

int moc_normalize_fluxes(moc_ctx* c, double* factor) {
  MOC_TRY(ready(c));
  MOC_CHECK(!c->num_instances, MOC_ERR_UNSUPPORTED,
            "instances are solved by moc_compute_eigenvalue only");
  moc::SolverArgs a = solver_args(c, 0);
  moc::launch_fission_rate(a, 1, c->stream);
  moc::launch_scale_phi(a, c->stream);
  c->launches += 2;
  if (c->ls) {
    moc::launch_ls_scale_moments(a, c->stream);
    c->launches++;
  }
  MOC_CUDA(cudaGetLastError());
  MOC_TRY(pull(c));
  if (factor) *factor = c->hsc->factor;
  return MOC_OK;
}

int moc_compute_fsr_sources(moc_ctx* c, int iteration) {
  MOC_TRY(ready(c));
  MOC_CHECK(iteration >= 0, MOC_ERR_ARG, "iteration must be non-negative");
  moc::SolverArgs a = solver_args(c, 0);
  enqueue_sources(c, a, iteration, 0);
  MOC_CUDA(cudaGetLastError());
  return MOC_OK;
}

int moc_transport_sweep(moc_ctx* c) {
  MOC_TRY(ready(c));
  MOC_CUDA(cudaMemsetAsync(c->phi, 0, 4 * num_flux(c), c->stream));
  // the leakage tally starts afresh with every sweep (src/CPUSolver.cpp:2360)
  MOC_CUDA(cudaMemsetAsync(&c->sc->leakage, 0, sizeof(double), c->stream));
  MOC_TRY(zero_moments(c));
  MOC_TRY(enqueue_sweep(c, 0, true, 0));
  MOC_CUDA(cudaStreamSynchronize(c->stream));
  MOC_TRY(collect_sweep_times(c, 1));
  c->num_sweeps++;
  return MOC_OK;
}

int moc_add_source_to_scalar_flux(moc_ctx* c) {
  MOC_TRY(ready(c));
  moc::SolverArgs a = solver_args(c, 0);
  enqueue_add_source(c, a, 0);
  MOC_CUDA(cudaGetLastError());
  return MOC_OK;
}

int moc_compute_keff(moc_ctx* c) {
  MOC_TRY(ready(c));
  MOC_CHECK(!c->num_instances, MOC_ERR_UNSUPPORTED,
            "instances are solved by moc_compute_eigenvalue only");
  moc::SolverArgs a = solver_args(c, 0);
  moc::launch_fission_rate(a, 0, c->stream);
  c->launches++;
  MOC_CUDA(cudaGetLastError());
  MOC_TRY(pull(c));
  c->keff = c->hsc->keff;
  return MOC_OK;
}

int moc_compute_residual(moc_ctx* c, int res_type, double* residual) {
  MOC_TRY(ready(c));
  MOC_CHECK(res_type >= 0 && res_type <= 2, MOC_ERR_ARG, "bad residual type");
  moc::SolverArgs a = solver_args(c, 0);
  moc::launch_residual(a, res_type, 0, 0, 0, c->stream);
  c->launches++;
  MOC_CUDA(cudaGetLastError());
  MOC_TRY(pull(c));
  if (residual) *residual = c->hsc->residual;
  return MOC_OK;
}

int moc_set_keff(moc_ctx* c, double keff) {
  MOC_CHECK(c, MOC_ERR_ARG, "null context");
  MOC_CHECK(keff > 0.0 && std::isfinite(keff), MOC_ERR_ARG,
            "keff must be positive");
  MOC_TRY(pull(c));
  c->hsc->keff = keff;
  c->hsc->k_prev = keff;
  c->keff = keff;
  return push(c);
}

int moc_compute_fsr_fission_rates(moc_ctx* c, double* rates, int64_t n,
                                  int nu) {
  MOC_TRY(ready(c));
  MOC_CHECK(rates && n == c->d.num_fsrs, MOC_ERR_ARG,
            "rates must hold num_fsrs values");
  MOC_CHECK(nu || c->sigma_f, MOC_ERR_STATE,
            "fission (not nu-fission) rates need moc_upload_sigma_f");
  moc::SolverArgs a = solver_args(c, 0);
  moc::launch_fsr_rates(a, c->rates, nu, c->stream);
  c->launches++;
  MOC_CUDA(cudaGetLastError());
  MOC_CUDA(cudaMemcpyAsync(rates, c->rates, 8 * n, cudaMemcpyDeviceToHost,
                           c->stream));
  MOC_CUDA(cudaStreamSynchronize(c->stream));
  return MOC_OK;
}

// ------------------------------------------------------------ linear source
int moc_set_linear_source(moc_ctx* c, const moc_ls_geometry* g) {
  MOC_TRY(ready(c));
  if (!g) {
    ls_release(c);
    return MOC_OK;
  }
  const bool d3 = c->d.solve_3d != 0;
  MOC_CHECK(!d3 || (g->seg_z && g->pol_cos), MOC_ERR_ARG,
            "the linear source on 3D tracks needs seg_z and pol_cos");
  MOC_CHECK(!d3 || c->d.num_polar_half == 1, MOC_ERR_UNSUPPORTED,
            "the linear source on 3D tracks takes one polar value per track");
  MOC_CHECK(!d3 || !c->otf, MOC_ERR_UNSUPPORTED,
            "on-the-fly segmentation and the linear source do not combine");
  MOC_CHECK(!c->keff_balance, MOC_ERR_UNSUPPORTED,
            "keff from the neutron balance is built for the flat source");
  MOC_CHECK(c->d.num_polar_half >= 1 && c->d.num_polar_half <= 3,
            MOC_ERR_UNSUPPORTED,
            "the linear-source sweep takes 1 to 3 polar angles per half space");
  MOC_CHECK(c->mat_packed, MOC_ERR_UNSUPPORTED,
            "the linear-source sweep needs fewer than 2^24 FSRs and at most "
            "256 materials");
  MOC_CHECK(c->d.num_groups <= 256 && c->d.num_segments < (1LL << 31),
            MOC_ERR_UNSUPPORTED,
            "the linear source takes at most 256 groups and 2^31 segments");
  MOC_CHECK(g->seg_x && g->seg_y && g->ang_dir && g->ang_wgt && g->pol_sin &&
                g->pol_wgt,
            MOC_ERR_ARG, "null linear-source array");
  const int64_t S = c->d.num_segments, R = c->d.num_fsrs;
  const int A = c->d.num_angles, Ph = c->d.num_polar_half;
  for (int64_t i = 0; i < S; i++)
    MOC_CHECK(std::isfinite(g->seg_x[i]) && std::isfinite(g->seg_y[i]) &&
                  (!d3 || std::isfinite(g->seg_z[i])),
              MOC_ERR_ARG,
              "non-finite segment start position at segment " +
                  std::to_string(i));
  for (int a = 0; a < A && d3; a++) {
    const double sn = g->pol_sin[a], cs = g->pol_cos[a];
    MOC_CHECK(std::isfinite(cs) && std::fabs(sn * sn + cs * cs - 1.0) < 1e-6,
              MOC_ERR_ARG,
              "sin and cos theta of angle row " + std::to_string(a) +
                  " do not make a unit vector");
  }
  for (int a = 0; a < A; a++) {
    const double cx = g->ang_dir[2 * a], cy = g->ang_dir[2 * a + 1];
    MOC_CHECK(std::isfinite(cx) && std::isfinite(cy) &&
                  std::fabs(cx * cx + cy * cy - 1.0) < 1e-6,
              MOC_ERR_ARG,
              "track direction of angle " + std::to_string(a) +
                  " is not a unit vector");
    MOC_CHECK(std::isfinite(g->ang_wgt[a]) && g->ang_wgt[a] > 0.0,
              MOC_ERR_ARG, "azimuthal weight must be positive");
    for (int p = 0; p < Ph; p++) {
      const double sn = g->pol_sin[a * Ph + p], w = g->pol_wgt[a * Ph + p];
      MOC_CHECK(std::isfinite(sn) && sn > 0.0 && sn <= 1.0, MOC_ERR_ARG,
                "sin(theta) must lie in (0, 1]");
      MOC_CHECK(std::isfinite(w) && w >= 0.0, MOC_ERR_ARG,
                "polar weight must be non-negative");
    }
  }
  ls_release(c);
  const int64_t nf = num_flux(c);
  const size_t nang = 3 * (size_t) A + 2 * (size_t) A * Ph + (d3 ? A : 0);
  std::vector<double> ang(nang);
  std::vector<float2> dir(A);
  std::vector<float4> dir3(d3 ? A : 0);
  for (int a = 0; a < A; a++) {
    ang[2 * a] = g->ang_dir[2 * a];
    ang[2 * a + 1] = g->ang_dir[2 * a + 1];
    ang[2 * A + a] = g->ang_wgt[a];
    dir[a] = make_float2((float) g->ang_dir[2 * a], (float) g->ang_dir[2 * a + 1]);
    for (int p = 0; p < Ph; p++) {
      ang[3 * A + a * Ph + p] = g->pol_sin[a * Ph + p];
      ang[3 * A + A * Ph + a * Ph + p] = g->pol_wgt[a * Ph + p];
    }
    if (d3) {
      // TransportSweep::onTrack: cos(phi) sin(theta), sin(phi) sin(theta),
      // cos(theta) in double, then rounded
      // (src/TrackTraversingAlgorithms.cpp:913-926)
      ang[3 * A + 2 * A * Ph + a] = g->pol_cos[a];
      dir3[a] = make_float4((float) (g->ang_dir[2 * a] * g->pol_sin[a]),
                            (float) (g->ang_dir[2 * a + 1] * g->pol_sin[a]),
                            (float) g->pol_cos[a], 0.0f);
    }
  }
  const int NC = d3 ? 6 : 3;
  float* dx = nullptr;
  float* dy = nullptr;
  int st = MOC_OK;
  auto step = [&](int r) { if (st == MOC_OK) st = r; };
  step(dalloc(&c->segs_ls, S > 0 ? S : 1));
  step(dalloc(&c->ls_ang, nang));
  step(dalloc(&c->ls_dir, A));
  step(dalloc(&c->mom, 2 * nf));
  step(dalloc(&c->qxy, 2 * nf));
  step(dalloc(&c->ls_ilem, NC * R));
  step(dalloc(&c->ls_const, NC * nf));
  step(dalloc(&dx, S > 0 ? S : 1));
  step(dalloc(&dy, S > 0 ? S : 1));
  if (d3) {
    step(dalloc(&c->ls_segz, S > 0 ? S : 1));
    step(dalloc(&c->ls_dir3, A));
    step(dalloc(&c->momz, nf));
    step(dalloc(&c->qz, nf));
  }
  if (st != MOC_OK) {
    dfree(dx);
    dfree(dy);
    ls_release(c);
    return st;
  }
  cudaError_t e = cudaMemcpy(dx, g->seg_x, 4 * S, cudaMemcpyHostToDevice);
  if (e == cudaSuccess)
    e = cudaMemcpy(dy, g->seg_y, 4 * S, cudaMemcpyHostToDevice);
  if (e == cudaSuccess)
    e = cudaMemcpy(c->ls_ang, ang.data(), 8 * nang, cudaMemcpyHostToDevice);
  if (e == cudaSuccess)
    e = cudaMemcpy(c->ls_dir, dir.data(), 8 * (size_t) A,
                   cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemset(c->mom, 0, 8 * nf);
  if (e == cudaSuccess) e = cudaMemset(c->qxy, 0, 8 * nf);
  if (d3 && e == cudaSuccess)
    e = cudaMemcpy(c->ls_segz, g->seg_z, 4 * S, cudaMemcpyHostToDevice);
  if (d3 && e == cudaSuccess)
    e = cudaMemcpy(c->ls_dir3, dir3.data(), 16 * (size_t) A,
                   cudaMemcpyHostToDevice);
  if (d3 && e == cudaSuccess) e = cudaMemset(c->momz, 0, 4 * nf);
  if (d3 && e == cudaSuccess) e = cudaMemset(c->qz, 0, 4 * nf);
  if (e == cudaSuccess) {
    moc::launch_ls_pack_segments(c->segs, dx, dy, c->segs_ls, S, c->stream);
    c->launches++;
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  dfree(dx);
  dfree(dy);
  if (e != cudaSuccess) {
    ls_release(c);
    return fail(MOC_ERR_CUDA, std::string("linear source upload: ") +
                                  cudaGetErrorString(e));
  }
  c->ls = true;
  c->ls3d = d3;
  if (!c->shape_user_set) c->lps = c->slots = 0;
  c->tuned = false;
  st = ls_constants(c);
  if (st != MOC_OK) ls_release(c);
  return st;
}

int moc_get_linear_source(moc_ctx* c, int* enabled, int64_t* num_flat) {
  MOC_CHECK(c, MOC_ERR_ARG, "null context");
  if (enabled) *enabled = c->ls ? 1 : 0;
  if (num_flat) *num_flat = c->ls_num_flat;
  return MOC_OK;
}

int moc_set_negative_fluxes_allowed(moc_ctx* c, int allowed) {
  MOC_CHECK(c, MOC_ERR_ARG, "null context");
  c->negative_ok = allowed ? 1 : 0;
  return MOC_OK;
}

int moc_set_transport_stabilization(moc_ctx* c, int on, double factor,
                                    int type) {
  MOC_CHECK(c, MOC_ERR_ARG, "null context");
  if (!on) {
    c->stab_on = 0;
    return MOC_OK;
  }
  MOC_CHECK(std::isfinite(factor) && factor > 0.0, MOC_ERR_ARG,
            "the stabilization factor must be positive");
  MOC_CHECK(type == MOC_STABILIZE_DIAGONAL || type == MOC_STABILIZE_YAMAMOTO ||
                type == MOC_STABILIZE_GLOBAL,
            MOC_ERR_ARG, "unknown stabilization type");
  if (c->stab && c->d.num_materials > 0) {
    // the coefficients depend on the factor and type
    dfree(c->stab);
    c->stab = nullptr;
  }
  c->stab_on = 1;
  c->stab_factor = factor;
  c->stab_type = type;
  c->stab_dirty = true;
  return MOC_OK;
}

int moc_compute_stabilizing_flux(moc_ctx* c) {
  MOC_TRY(ready(c));
  MOC_CHECK(c->stab_on, MOC_ERR_STATE, "transport stabilization is off");
  MOC_TRY(ensure_stab(c));
  if (!c->stab_base) MOC_TRY(dalloc(&c->stab_base, num_flux(c)));
  MOC_CUDA(cudaMemcpyAsync(c->stab_base, c->phi, 4 * num_flux(c),
                           cudaMemcpyDeviceToDevice, c->stream));
  MOC_TRY(enqueue_stab_moments_base(c));
  return MOC_OK;
}

int moc_stabilize_flux(moc_ctx* c) {
  MOC_TRY(ready(c));
  MOC_CHECK(c->stab_on, MOC_ERR_STATE, "transport stabilization is off");
  MOC_CHECK(c->stab_base, MOC_ERR_STATE,
            "computeStabilizingFlux must come before stabilizeFlux");
  MOC_TRY(ensure_stab(c));
  moc::SolverArgs a = solver_args(c, 0);
  MOC_CHECK(!stab_moments(c) || c->stab_mom, MOC_ERR_STATE,
            "computeStabilizingFlux must come before stabilizeFlux");
  moc::launch_stabilize(a, c->stab_base, 0, c->stream,
                        stab_moments(c) ? c->stab_mom : nullptr,
                        stab_moments(c) && c->ls3d ? c->stab_momz : nullptr);
  c->launches++;
  MOC_CUDA(cudaGetLastError());
  return MOC_OK;
}

int moc_compute_fsr_fission_sources(moc_ctx* c) {
  MOC_TRY(ready(c));
  moc::SolverArgs a = solver_args(c, 0);
  moc::launch_partial_sources(a, 0, c->stream);
  c->launches++;
  MOC_CUDA(cudaGetLastError());
  return MOC_OK;
}

int moc_compute_fsr_scatter_sources(moc_ctx* c) {
  MOC_TRY(ready(c));
  moc::SolverArgs a = solver_args(c, 0);
  moc::launch_partial_sources(a, 1, c->stream);
  c->launches++;
  MOC_CUDA(cudaGetLastError());
  return MOC_OK;
}

int moc_set_instances(moc_ctx* c, int num_instances) {
  MOC_CHECK(c, MOC_ERR_ARG, "null context");
  if (num_instances == 0) {
    c->num_instances = 0;
    c->inst_groups = 0;
    return MOC_OK;
  }
  MOC_CHECK(num_instances >= 1 && num_instances <= moc::kMaxInstances,
            MOC_ERR_ARG, "1 to 16 instances");
  MOC_CHECK(c->d.num_groups % num_instances == 0, MOC_ERR_ARG,
            "the problem's groups must be the instances' groups side by side "
            "(num_groups a multiple of the instance count)");
  if (!c->inst) MOC_TRY(dalloc(&c->inst, 1));
  c->num_instances = num_instances;
  c->inst_groups = c->d.num_groups / num_instances;
  return reset_instances(c);
}

int moc_get_instance_keffs(moc_ctx* c, double* keffs, int num_instances) {
  MOC_CHECK(c && keffs, MOC_ERR_ARG, "null argument");
  MOC_CHECK(c->num_instances > 0 && num_instances == c->num_instances,
            MOC_ERR_ARG, "num_instances must be the context's instance count");
  moc::InstState h;
  MOC_CUDA(cudaMemcpyAsync(&h, c->inst, sizeof(h), cudaMemcpyDeviceToHost,
                           c->stream));
  MOC_CUDA(cudaStreamSynchronize(c->stream));
  for (int k = 0; k < num_instances; k++) keffs[k] = h.keff[k];
  return MOC_OK;
}

int moc_set_keff_from_neutron_balance(moc_ctx* c, int on) {
  MOC_CHECK(c, MOC_ERR_ARG, "null context");
  MOC_CHECK(!on || (!c->ls && !c->otf), MOC_ERR_UNSUPPORTED,
            "keff from the neutron balance is built for the flat-source sweep "
            "of stored segments (not the linear source or on-the-fly 3D "
            "segments)");
  c->keff_balance = on ? 1 : 0;
  return MOC_OK;
}

// host [R][3][G] (x, y, z) <-> device [R][ld][2] (x, y adjacent per group)
// and, on 3D tracks, [R][ld] (z; dev_z null: z = 0)
static int moments_out(moc_ctx* c, const float* dev, float* out, int64_t n,
                       float scale_by_sigma_t, const float* dev_z = nullptr) {
  const int64_t R = c->d.num_fsrs;
  const int G = c->d.num_groups, ld = row_stride(c);
  MOC_CHECK(out && n == 3 * R * G, MOC_ERR_ARG,
            "moments need num_fsrs x 3 x num_groups values");
  std::vector<float> h((size_t) 2 * R * ld), hz(dev_z ? (size_t) R * ld : 0);
  MOC_CUDA(cudaMemcpyAsync(h.data(), dev, 8 * (size_t) R * ld,
                           cudaMemcpyDeviceToHost, c->stream));
  if (dev_z)
    MOC_CUDA(cudaMemcpyAsync(hz.data(), dev_z, 4 * (size_t) R * ld,
                             cudaMemcpyDeviceToHost, c->stream));
  std::vector<float> st;
  std::vector<int32_t> fm;
  if (scale_by_sigma_t != 0.0f) {
    st.resize((size_t) c->d.num_materials * G);
    fm.resize(R);
    MOC_CUDA(cudaMemcpyAsync(st.data(), c->sigma_t, 4 * st.size(),
                             cudaMemcpyDeviceToHost, c->stream));
    MOC_CUDA(cudaMemcpyAsync(fm.data(), c->fsr_mat, 4 * (size_t) R,
                             cudaMemcpyDeviceToHost, c->stream));
  }
  MOC_CUDA(cudaStreamSynchronize(c->stream));
  for (int64_t r = 0; r < R; r++)
    for (int g = 0; g < G; g++) {
      float x = h[(r * ld + g) * 2], y = h[(r * ld + g) * 2 + 1];
      float z = dev_z ? hz[r * ld + g] : 0.0f;
      if (scale_by_sigma_t != 0.0f) {
        const float s = st[(size_t) fm[r] * G + g];
        x *= s;
        y *= s;
        z *= s;
      }
      out[(r * 3 + 0) * G + g] = x;
      out[(r * 3 + 1) * G + g] = y;
      out[(r * 3 + 2) * G + g] = z;
    }
  return MOC_OK;
}

static int moments_in(moc_ctx* c, float* dev, const float* in, int64_t n,
                      float* dev_z = nullptr) {
  const int64_t R = c->d.num_fsrs;
  const int G = c->d.num_groups, ld = row_stride(c);
  MOC_CHECK(in && n == 3 * R * G, MOC_ERR_ARG,
            "moments need num_fsrs x 3 x num_groups values");
  std::vector<float> h((size_t) 2 * R * ld, 0.0f), hz((size_t) R * ld, 0.0f);
  for (int64_t r = 0; r < R; r++)
    for (int g = 0; g < G; g++) {
      const float x = in[(r * 3 + 0) * G + g], y = in[(r * 3 + 1) * G + g];
      const float z = in[(r * 3 + 2) * G + g];
      MOC_CHECK(std::isfinite(x) && std::isfinite(y) &&
                    (!dev_z || std::isfinite(z)),
                MOC_ERR_ARG, "non-finite moment");
      h[(r * ld + g) * 2] = x;
      h[(r * ld + g) * 2 + 1] = y;
      hz[r * ld + g] = z;
    }
  MOC_CUDA(cudaMemcpyAsync(dev, h.data(), 8 * (size_t) R * ld,
                           cudaMemcpyHostToDevice, c->stream));
  if (dev_z)
    MOC_CUDA(cudaMemcpyAsync(dev_z, hz.data(), 4 * (size_t) R * ld,
                             cudaMemcpyHostToDevice, c->stream));
  MOC_CUDA(cudaStreamSynchronize(c->stream));
  return MOC_OK;
}

int moc_get_flux_moments(moc_ctx* c, float* out, int64_t n) {
  MOC_TRY(ready(c));
  MOC_CHECK(c->ls, MOC_ERR_STATE, "no linear source set");
  return moments_out(c, c->mom, out, n, 0.0f, c->ls3d ? c->momz : nullptr);
}

int moc_set_flux_moments(moc_ctx* c, const float* in, int64_t n) {
  MOC_TRY(ready(c));
  MOC_CHECK(c->ls, MOC_ERR_STATE, "no linear source set");
  return moments_in(c, c->mom, in, n, c->ls3d ? c->momz : nullptr);
}

int moc_get_source_moments(moc_ctx* c, float* out, int64_t n) {
  MOC_TRY(ready(c));
  MOC_CHECK(c->ls, MOC_ERR_STATE, "no linear source set");
  return moments_out(c, c->qxy, out, n, 1.0f, c->ls3d ? c->qz : nullptr);
}

int moc_set_fixed_source_moments(moc_ctx* c, const float* in, int64_t n) {
  MOC_TRY(ready(c));
  MOC_CHECK(c->ls, MOC_ERR_STATE, "no linear source set");
  if (!in) {
    dfree(c->fixed_xy);
    dfree(c->fixed_z);
    return MOC_OK;
  }
  if (!c->fixed_xy) MOC_TRY(dalloc(&c->fixed_xy, 2 * num_flux(c)));
  if (c->ls3d && !c->fixed_z) MOC_TRY(dalloc(&c->fixed_z, num_flux(c)));
  return moments_in(c, c->fixed_xy, in, n, c->ls3d ? c->fixed_z : nullptr);
}

int moc_get_linear_expansion(moc_ctx* c, double* ilem, float* src_const) {
  MOC_TRY(ready(c));
  MOC_CHECK(c->ls, MOC_ERR_STATE, "no linear source set");
  const int64_t R = c->d.num_fsrs;
  const int G = c->d.num_groups, ld = row_stride(c);
  const int NC = c->ls3d ? 6 : 3;
  if (ilem) {
    std::vector<float> h(NC * (size_t) R);
    MOC_CUDA(cudaMemcpy(h.data(), c->ls_ilem, 4 * h.size(),
                        cudaMemcpyDeviceToHost));
    for (size_t i = 0; i < h.size(); i++) ilem[i] = h[i];
  }
  if (src_const)
    MOC_CUDA(cudaMemcpy2D(src_const, 4 * G, c->ls_const, 4 * ld, 4 * G,
                          NC * R, cudaMemcpyDeviceToHost));
  return MOC_OK;
}

// ------------------------------------------------- on-the-fly 3D tracks
int moc_set_otf_tracks(moc_ctx* c, const moc_otf_tracks* d) {
  MOC_TRY(ready(c));
  if (!d) {
    otf_release(c);
    return MOC_OK;
  }
  MOC_CHECK(c->d.solve_3d && c->d.num_polar_half == 1, MOC_ERR_UNSUPPORTED,
            "on-the-fly segmentation takes 3D tracks");
  MOC_CHECK(!c->ls, MOC_ERR_UNSUPPORTED,
            "on-the-fly segmentation and the linear source do not combine");
  MOC_CHECK(!c->keff_balance, MOC_ERR_UNSUPPORTED,
            "keff from the neutron balance is built for stored segments");
  MOC_CHECK(c->d.num_fsrs < (1LL << 24) && c->d.num_materials <= 256,
            MOC_ERR_UNSUPPORTED,
            "on-the-fly segmentation needs fewer than 2^24 FSRs and at most "
            "256 materials");
  MOC_CHECK(d->trk && d->trk_f && d->ang && d->rad_len && d->rad_fsr &&
                d->rad_off && d->rad_start && d->rad_total,
            MOC_ERR_ARG, "null on-the-fly array");
  const int64_t T = c->d.num_tracks, T2 = d->num_radial_tracks;
  const int64_t S2 = d->num_radial_segments, R = c->d.num_fsrs;
  const int A = c->d.num_angles;
  MOC_CHECK(T2 >= 1 && S2 >= 0 && d->rad_off[0] == 0 && d->rad_off[T2] == S2,
            MOC_ERR_ARG, "radial segment offsets must run from 0 to S2");
  MOC_CHECK(d->above_fsr >= 0 && d->above_fsr < R, MOC_ERR_ARG,
            "above_fsr out of range");
  for (int64_t t = 0; t < T2; t++)
    MOC_CHECK(d->rad_off[t + 1] >= d->rad_off[t] && std::isfinite(d->rad_total[t]),
              MOC_ERR_ARG, "bad radial track " + std::to_string(t));
  for (int64_t k = 0; k < S2; k++)
    MOC_CHECK(d->rad_fsr[k] >= 0 && d->rad_fsr[k] < R &&
                  std::isfinite(d->rad_len[k]) && d->rad_len[k] >= 0.0f &&
                  std::isfinite(d->rad_start[k]),
              MOC_ERR_ARG, "bad radial segment " + std::to_string(k));
  std::vector<int32_t> cnt(T);
  for (int64_t t = 0; t < T; t++) {
    const int32_t* q = d->trk + 4 * t;
    const float* f = d->trk_f + 4 * t;
    MOC_CHECK(q[0] >= 0 && q[0] < T2 && q[2] >= 0 && (q[3] == 0 || q[3] == 1),
              MOC_ERR_ARG, "bad on-the-fly track " + std::to_string(t));
    const int64_t n = d->rad_off[q[0] + 1] - d->rad_off[q[0]];
    const int64_t lo = q[3] ? q[1] - q[2] + 1 : q[1];
    const int64_t hi = q[3] ? q[1] : q[1] + q[2] - 1;
    MOC_CHECK(q[2] == 0 || (lo >= 0 && hi < n), MOC_ERR_ARG,
              "on-the-fly track " + std::to_string(t) +
                  " crosses radial segments outside its radial track");
    MOC_CHECK(std::isfinite(f[0]) && std::isfinite(f[1]) && f[1] >= 0.0f &&
                  std::isfinite(f[2]),
              MOC_ERR_ARG, "bad on-the-fly track " + std::to_string(t));
    cnt[t] = q[2];
  }
  for (int a = 0; a < 4 * A; a++)
    MOC_CHECK(std::isfinite(d->ang[a]), MOC_ERR_ARG, "bad on-the-fly angle data");
  std::vector<int32_t> order(T);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(),
                   [&](int32_t x, int32_t y) { return cnt[x] > cnt[y]; });
  std::vector<int2> rad(S2);
  for (int64_t k = 0; k < S2; k++)
    rad[k] = make_int2(__builtin_bit_cast(int, d->rad_len[k]), d->rad_fsr[k]);
  otf_release(c);
  int st = MOC_OK;
  auto step = [&](int r) { if (st == MOC_OK) st = r; };
  step(dalloc(&c->otf_trk, T > 0 ? T : 1));
  step(dalloc(&c->otf_trk_f, T > 0 ? T : 1));
  step(dalloc(&c->otf_ang, A));
  step(dalloc(&c->otf_rad, S2 > 0 ? S2 : 1));
  step(dalloc(&c->otf_rad_start, S2 > 0 ? S2 : 1));
  step(dalloc(&c->otf_rad_off, T2 + 1));
  step(dalloc(&c->otf_rad_total, T2));
  step(dalloc(&c->otf_order, T > 0 ? T : 1));
  if (st != MOC_OK) {
    otf_release(c);
    return st;
  }
  cudaError_t e = cudaMemcpy(c->otf_trk, d->trk, 16 * T, cudaMemcpyHostToDevice);
  if (e == cudaSuccess)
    e = cudaMemcpy(c->otf_trk_f, d->trk_f, 16 * T, cudaMemcpyHostToDevice);
  if (e == cudaSuccess)
    e = cudaMemcpy(c->otf_ang, d->ang, 16 * (size_t) A, cudaMemcpyHostToDevice);
  if (e == cudaSuccess)
    e = cudaMemcpy(c->otf_rad, rad.data(), 8 * S2, cudaMemcpyHostToDevice);
  if (e == cudaSuccess)
    e = cudaMemcpy(c->otf_rad_start, d->rad_start, 4 * S2,
                   cudaMemcpyHostToDevice);
  if (e == cudaSuccess)
    e = cudaMemcpy(c->otf_rad_off, d->rad_off, 8 * (T2 + 1),
                   cudaMemcpyHostToDevice);
  if (e == cudaSuccess)
    e = cudaMemcpy(c->otf_rad_total, d->rad_total, 4 * T2,
                   cudaMemcpyHostToDevice);
  if (e == cudaSuccess)
    e = cudaMemcpy(c->otf_order, order.data(), 4 * T, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    otf_release(c);
    return fail(MOC_ERR_CUDA, std::string("on-the-fly upload: ") +
                                  cudaGetErrorString(e));
  }
  c->otf_S2 = S2;
  c->otf_above_fsr = d->above_fsr;
  moc::launch_pack_materials(c->otf_rad, S2, c->fsr_mat, c->stream);
  c->launches++;
  MOC_CUDA(cudaStreamSynchronize(c->stream));
  MOC_TRY(otf_above_word(c));
  c->otf = true;
  if (!c->shape_user_set) c->lps = c->slots = 0;
  c->tuned = false;
  return MOC_OK;
}

int moc_get_otf_tracks(moc_ctx* c, int* enabled) {
  MOC_CHECK(c && enabled, MOC_ERR_ARG, "null argument");
  *enabled = c->otf ? 1 : 0;
  return MOC_OK;
}

int moc_set_cmfd(moc_ctx* c, const moc_cmfd_mesh* m) {
  MOC_TRY(ready(c));
  if (!m) {
    if (c->cmfd) {
      cmfd_release(c);
      c->tuned = false;
      if (!c->exp_user_set) c->exp_kind = MOC_EXP_TABLE;
    }
    return MOC_OK;
  }
  MOC_CHECK(!c->otf, MOC_ERR_UNSUPPORTED,
            "CMFD is supported for 2D solves with stored segments");
  MOC_CHECK(!(c->exp_user_set && c->exp_kind == MOC_EXP_TABLE),
            MOC_ERR_UNSUPPORTED,
            "CMFD current tallies use the hardware exponential");
  const int64_t R = c->d.num_fsrs, T = c->d.num_tracks;
  const int G = c->d.num_groups;
  MOC_CHECK(m->num_x >= 1 && m->num_y >= 1 &&
                (int64_t) m->num_x * m->num_y <= (1 << 24),
            MOC_ERR_ARG, "bad CMFD lattice structure");
  MOC_CHECK(m->widths_x && m->widths_y && m->fsr_cell && m->track_end_face,
            MOC_ERR_ARG, "null CMFD mesh array");
  const int C = m->num_x * m->num_y;
  for (int i = 0; i < m->num_x; i++)
    MOC_CHECK(std::isfinite(m->widths_x[i]) && m->widths_x[i] > 0.0,
              MOC_ERR_ARG, "CMFD cell widths must be positive");
  for (int i = 0; i < m->num_y; i++)
    MOC_CHECK(std::isfinite(m->widths_y[i]) && m->widths_y[i] > 0.0,
              MOC_ERR_ARG, "CMFD cell widths must be positive");
  for (int64_t r = 0; r < R; r++)
    MOC_CHECK(m->fsr_cell[r] >= 0 && m->fsr_cell[r] < C, MOC_ERR_ARG,
              "CMFD cell out of range at FSR " + std::to_string(r));
  for (int64_t i = 0; i < 2 * T; i++)
    MOC_CHECK(m->track_end_face[i] >= -1 && m->track_end_face[i] < 4,
              MOC_ERR_ARG, "bad track end face");
  for (int f = 0; f < 4; f++)
    MOC_CHECK(m->boundary[f] == MOC_BC_VACUUM ||
                  m->boundary[f] == MOC_BC_REFLECTIVE,
              MOC_ERR_UNSUPPORTED,
              "CMFD boundaries must be vacuum or reflective");
  const int E = m->group_of ? m->num_cmfd_groups : G;
  MOC_CHECK(E >= 1 && E <= G, MOC_ERR_ARG, "bad number of CMFD groups");
  std::vector<int> group_of(G);
  for (int g = 0; g < G; g++) group_of[g] = m->group_of ? m->group_of[g] : g;
  MOC_CHECK(group_of[0] == 0 && group_of[G - 1] == E - 1, MOC_ERR_ARG,
            "CMFD groups must cover 0 .. E-1");
  for (int g = 1; g < G; g++)
    MOC_CHECK(group_of[g] == group_of[g - 1] ||
                  group_of[g] == group_of[g - 1] + 1,
              MOC_ERR_ARG,
              "CMFD groups must be contiguous ranges of groups");
  MOC_CHECK(m->num_edc_angles >= 0 &&
                (m->num_edc_angles == 0 || (m->edc_mu && m->edc_weight)),
            MOC_ERR_ARG, "bad EDC quadrature");
  for (int i = 0; i < m->num_edc_angles; i++)
    MOC_CHECK(m->edc_mu[i] > 0.0 && m->edc_mu[i] <= 1.0 &&
                  std::isfinite(m->edc_weight[i]),
              MOC_ERR_ARG, "bad EDC quadrature");
  MOC_CHECK(std::isfinite(m->relaxation) && m->relaxation > 0.0 &&
                m->relaxation <= 1.0,
            MOC_ERR_ARG, "the CMFD relaxation factor must be in (0, 1]");
  MOC_CHECK(std::isfinite(m->sor_factor) && m->sor_factor > 0.0 &&
                m->sor_factor < 2.0,
            MOC_ERR_ARG, "the SOR factor must be in (0, 2)");
  MOC_CHECK(m->num_unbounded_iterations >= 0, MOC_ERR_ARG,
            "negative number of unbounded iterations");
  MOC_CHECK(m->solve_on_host >= 0 && m->solve_on_host <= 3, MOC_ERR_ARG,
            "solve_on_host must be 0 (device, automatic), 1 (host), 2 (device, "
            "one block) or 3 (device, cell-parallel)");
  MOC_CHECK(m->k_nearest >= 0 && m->k_nearest <= 9, MOC_ERR_ARG,
            "k_nearest must be in 0..9 (Cmfd::setKNearest takes 1..9)");
  MOC_CHECK(m->k_nearest == 0 || m->fsr_centroid, MOC_ERR_ARG,
            "the k-nearest update needs the FSR centroids");
  if (m->k_nearest > 0)
    for (int64_t i = 0; i < 2 * R; i++)
      MOC_CHECK(std::isfinite(m->fsr_centroid[i]), MOC_ERR_ARG,
                "non-finite FSR centroid");
  cmfd_release(c);
  auto* S = new moc_cmfd::Solver();
  moc_cmfd::Config& cf = S->cfg;
  cf.nx = m->num_x;
  cf.ny = m->num_y;
  cf.G = G;
  cf.E = E;
  cf.wx.assign(m->widths_x, m->widths_x + m->num_x);
  cf.wy.assign(m->widths_y, m->widths_y + m->num_y);
  cf.group_of = group_of;
  cf.gstart.assign(E + 1, G);
  for (int g = G - 1; g >= 0; g--) cf.gstart[group_of[g]] = g;
  c->cm_edc_mu_h.assign(m->edc_mu, m->edc_mu + m->num_edc_angles);
  c->cm_edc_w_h.assign(m->edc_weight, m->edc_weight + m->num_edc_angles);
  for (int f = 0; f < 4; f++) cf.bc[f] = m->boundary[f];
  cf.relaxation = m->relaxation;
  cf.sor = m->sor_factor;
  cf.flux_limiting = m->flux_limiting != 0;
  cf.unbounded = m->num_unbounded_iterations;
  c->cmfd = S;
  c->cm_host = m->solve_on_host == 1;
  c->cm_solve_kind = m->solve_on_host;
  c->h_cm_cell.assign(m->fsr_cell, m->fsr_cell + R);
  const int ld = row_stride(c);
  const int64_t ncur = (int64_t) C * moc_cmfd::kFaces * ld;
  int st = MOC_OK;
  auto step = [&](int r) { if (st == MOC_OK) st = r; };
  step(dalloc(&c->cm_cell, R));
  step(dalloc(&c->cm_end, 2 * T));
  step(dalloc(&c->cm_cur, ncur));
  step(dalloc(&c->cm_group, G));
  step(dalloc(&c->cm_ratio, (int64_t) C * E));
  if (st == MOC_OK && c->cm_host &&
      cudaMallocHost(&c->h_cm_cur, 4 * ncur) != cudaSuccess)
    st = fail(MOC_ERR_MEMORY, "pinned host buffer for CMFD currents");
  if (st != MOC_OK) {
    cmfd_release(c);
    return st;
  }
  cudaError_t e = cudaMemcpy(c->cm_cell, m->fsr_cell, 4 * R,
                             cudaMemcpyHostToDevice);
  if (e == cudaSuccess)
    e = cudaMemcpy(c->cm_end, m->track_end_face, 2 * T,
                   cudaMemcpyHostToDevice);
  if (e == cudaSuccess)
    e = cudaMemcpy(c->cm_group, group_of.data(), 4 * G,
                   cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemset(c->cm_cur, 0, 4 * ncur);
  if (e == cudaSuccess && m->k_nearest > 0) {
    std::vector<int32_t> off, cell;
    std::vector<float> coef;
    moc_cmfd::knearest_coefficients(cf, m->k_nearest, m->origin_x,
                                    m->origin_y, m->fsr_centroid,
                                    m->fsr_cell, R, off, cell, coef);
    int st2 = dalloc(&c->cm_pro_off, R + 1);
    if (st2 == MOC_OK) st2 = dalloc(&c->cm_pro_cell, (int64_t) cell.size());
    if (st2 == MOC_OK) st2 = dalloc(&c->cm_pro_coef, (int64_t) coef.size());
    if (st2 != MOC_OK) {
      cmfd_release(c);
      return st2;
    }
    e = cudaMemcpy(c->cm_pro_off, off.data(), 4 * (R + 1),
                   cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
      e = cudaMemcpy(c->cm_pro_cell, cell.data(), 4 * cell.size(),
                     cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
      e = cudaMemcpy(c->cm_pro_coef, coef.data(), 4 * coef.size(),
                     cudaMemcpyHostToDevice);
  }
  if (e != cudaSuccess) {
    cmfd_release(c);
    return fail(MOC_ERR_CUDA, cudaGetErrorString(e));
  }
  S->reset();
  c->exp_kind = MOC_EXP_INTRINSIC;
  c->tuned = false;
  return MOC_OK;
}

int moc_get_cmfd_info(moc_ctx* c, int* enabled, double* keff,
                      int* power_iterations, int* linear_iterations,
                      double* max_ratio, int* failed) {
  MOC_CHECK(c, MOC_ERR_ARG, "null context");
  const moc_cmfd::Solver* S = c->cmfd;
  double k = S ? S->keff : 0.0, mr = 1.0;
  int pi = S ? S->stats.power_iterations : 0;
  int li = S ? S->stats.linear_iterations : 0;
  int fl = S ? (S->stats.failed ? 1 : 0) : 0;
  if (S && !c->cm_host && c->cm_state) {
    moc::CmfdDevState d{};
    MOC_CUDA(cudaSetDevice(c->d.device));
    MOC_CUDA(cudaStreamSynchronize(c->stream));
    MOC_CUDA(cudaMemcpy(&d, c->cm_state, sizeof(d), cudaMemcpyDeviceToHost));
    k = d.keff;
    pi = d.power_iters;
    li = d.linear_iters;
    mr = d.max_ratio;
    fl = d.failed;
  } else if (S) {
    mr = S->stats.max_ratio;
  }
  if (enabled) *enabled = S ? 1 : 0;
  if (keff) *keff = k;
  if (power_iterations) *power_iterations = pi;
  if (linear_iterations) *linear_iterations = li;
  if (max_ratio) *max_ratio = mr;
  if (failed) *failed = fl;
  return MOC_OK;
}

int moc_get_cmfd_fluxes(moc_ctx* c, double* old_flux, double* new_flux,
                        int64_t n) {
  MOC_CHECK(c && c->cmfd, MOC_ERR_STATE, "CMFD is not attached");
  const moc_cmfd::Solver& S = *c->cmfd;
  const int64_t need = (int64_t) S.cfg.cells() * S.cfg.E;
  MOC_CHECK(n == need, MOC_ERR_ARG,
            "expected " + std::to_string(need) + " coarse fluxes");
  if (!c->cm_host) {
    MOC_CHECK(c->cm_flux_old != nullptr, MOC_ERR_STATE,
              "no coarse solve has run");
    std::vector<float> t(need);
    MOC_CUDA(cudaSetDevice(c->d.device));
    MOC_CUDA(cudaStreamSynchronize(c->stream));
    if (old_flux) {
      MOC_CUDA(cudaMemcpy(t.data(), c->cm_flux_old, 4 * need,
                          cudaMemcpyDeviceToHost));
      std::copy(t.begin(), t.end(), old_flux);
    }
    if (new_flux) {
      MOC_CUDA(cudaMemcpy(t.data(), c->cm_flux_new, 4 * need,
                          cudaMemcpyDeviceToHost));
      std::copy(t.begin(), t.end(), new_flux);
    }
    return MOC_OK;
  }
  if (old_flux && (int64_t) S.phi_old.size() == need)
    std::copy(S.phi_old.begin(), S.phi_old.end(), old_flux);
  if (new_flux && (int64_t) S.phi_new.size() == need)
    std::copy(S.phi_new.begin(), S.phi_new.end(), new_flux);
  return MOC_OK;
}

}  // extern "C"
