// The batched solve server of include/openmoc_gb300_serve.h: a
// device-resident request loop that runs many independent solves of uneven
// size on one GPU.
//
// Each pool (one group count and polar count) keeps the solves it holds in
// shared device arrays.  A solve owns contiguous ranges of FSR rows, track
// entries, segments, materials and angle rows, handed out by first-fit
// allocators over the pool's capacity; its track data are uploaded in its
// own numbering and rebased on the device.  An iteration of the pool is one
// launch of each kernel for every live solve (solver_kernels.cu batch_*,
// and the tuned sweep kernel over the concatenated track list, longest
// tracks first), and blocks of iterations are replayed as captured CUDA
// graphs.  Per solve, the loop body and convergence test are those of
// Solver::computeEigenvalue / computeSource (src/Solver.cpp:1459-1700): the
// same kernels' arithmetic, with reductions split per solve.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "../../include/openmoc_gb300.h"
#include "../../include/openmoc_gb300_serve.h"
#include "moc_internal.cuh"

namespace {

// Group pairs per lane for G groups over lps lanes.
int pairs_for(int G, int lps) { return ((G + 1) / 2 + lps - 1) / lps; }

// Group pairs per lane of the linear-source sweep instances.
constexpr int kLsMaxPairs = 5;

#define SV_FAIL(code, msg) moc::set_error(code, std::string(msg).c_str())

#define SV_CHECK(cond, code, msg)          \
  do {                                     \
    if (!(cond)) return SV_FAIL(code, msg); \
  } while (0)

#define SV_CUDA(call)                                                     \
  do {                                                                    \
    cudaError_t e_ = (call);                                              \
    if (e_ != cudaSuccess)                                                \
      return SV_FAIL(MOC_ERR_CUDA,                                        \
                     std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

#define SV_TRY(expr)               \
  do {                             \
    int s_ = (expr);               \
    if (s_ != MOC_OK) return s_;   \
  } while (0)

double now_s() {
  return std::chrono::duration<double>(
             std::chrono::steady_clock::now().time_since_epoch())
      .count();
}

template <typename T>
int dev_alloc(T** p, size_t n) {
  *p = nullptr;
  if (n == 0) n = 1;
  cudaError_t e = cudaMalloc((void**) p, n * sizeof(T));
  if (e == cudaErrorMemoryAllocation) {
    cudaGetLastError();
    return SV_FAIL(MOC_ERR_MEMORY, "device memory exhausted creating a pool (" +
                                       std::to_string(n * sizeof(T)) +
                                       " bytes)");
  }
  SV_CUDA(e);
  return MOC_OK;
}

template <typename T>
void dev_free(T*& p) {
  if (p) cudaFree((void*) p);
  p = nullptr;
}

// First-fit allocator of ranges of [0, capacity).
class RangeAlloc {
 public:
  void reset(int64_t cap) {
    cap_ = cap;
    free_.clear();
    if (cap > 0) free_[0] = cap;
  }
  // offset of a free range of n >= 1 entries, or -1
  int64_t alloc(int64_t n) {
    n = std::max<int64_t>(n, 1);
    for (auto it = free_.begin(); it != free_.end(); ++it) {
      if (it->second < n) continue;
      const int64_t off = it->first, len = it->second;
      free_.erase(it);
      if (len > n) free_[off + n] = len - n;
      return off;
    }
    return -1;
  }
  void release(int64_t off, int64_t n) {
    n = std::max<int64_t>(n, 1);
    auto next = free_.lower_bound(off);
    if (next != free_.end() && next->first == off + n) {
      n += next->second;
      next = free_.erase(next);
    }
    if (next != free_.begin()) {
      auto prev = std::prev(next);
      if (prev->first + prev->second == off) {
        prev->second += n;
        return;
      }
    }
    free_[off] = n;
  }
 private:
  int64_t cap_ = 0;
  std::map<int64_t, int64_t> free_;
};

// Page-locked host blocks in power-of-two size classes, kept for reuse:
// each request's arrays are copied into one on submission (on the
// submitting thread), so that admission only enqueues asynchronous copies.
class PinnedCache {
 public:
  ~PinnedCache() {
    for (auto& b : all_) cudaFreeHost(b.first);
  }
  char* get(size_t n, size_t* cap) {
    size_t c = (size_t) 1 << 16;
    while (c < n) c <<= 1;
    *cap = c;
    {
      std::lock_guard<std::mutex> lk(mu_);
      auto it = free_.find(c);
      if (it != free_.end()) {
        char* q = it->second;
        free_.erase(it);
        return q;
      }
    }
    void* q = nullptr;
    if (cudaHostAlloc(&q, c, cudaHostAllocPortable) != cudaSuccess) {
      cudaGetLastError();
      return nullptr;
    }
    std::lock_guard<std::mutex> lk(mu_);
    all_.emplace_back((char*) q, c);
    return (char*) q;
  }
  void put(char* q, size_t cap) {
    if (!q) return;
    std::lock_guard<std::mutex> lk(mu_);
    free_.emplace(cap, q);
  }
 private:
  std::mutex mu_;
  std::multimap<size_t, char*> free_;
  std::vector<std::pair<char*, size_t>> all_;
};

// The arrays of a request in its pinned block, in this order.
enum Part {
  kSegs, kSegOff, kNext, kTrackAng, kFlags, kWeights, kInvSin, kSigmaT,
  kSigmaST, kNuSigmaF, kChi, kScatOut, kFissile, kFsrMat, kFsrVol, kFixed,
  kSegX, kSegY, kLsAng, kLsDir, kFixedXY, kLsList, kNumParts
};

// A validated request, packed in its own numbering, waiting for or holding
// a pool slot.
struct Staged {
  int64_t ticket = 0;
  moc_request req{};
  int pool = -1;
  int G = 0, Ph = 0, A = 0, M = 0, ld = 0;
  int64_t R = 0, T = 0, S = 0;
  std::vector<int2> segs;          // {length bits, local FSR}
  std::vector<int64_t> seg_off;    // [T + 1]
  std::vector<int32_t> next;       // [2T]
  std::vector<int32_t> track_ang;  // [T]
  std::vector<int32_t> nseg;       // [T]
  std::vector<uint8_t> flags;      // [T + 1]
  std::vector<float> weights, inv_sin;
  std::vector<float> sigma_t, sigma_s_T, nu_sigma_f, chi, scat_out;
  std::vector<uint8_t> fissile;
  std::vector<int32_t> fsr_mat;
  std::vector<float> fsr_vol;
  std::vector<float> fixed;        // [R][ld] or empty
  // linear source: segment starts relative to the FSR centroids, the angle
  // data in moc_set_linear_source's layout ([A][2] directions, [A] weights,
  // [A][Ph] sin(theta), [A][Ph] polar weights), and the fixed source
  // moments as [R][ld][2] (empty: none)
  bool ls = false;
  std::vector<float> seg_x, seg_y;
  std::vector<double> ls_ang;
  std::vector<float2> ls_dir;
  std::vector<float> fixed_xy;
  // segment ids sorted by FSR (ascending within an FSR) for the expansion
  // constants, built here so that admission only copies and launches
  std::vector<int32_t> ls_list;
  long long num_fissionable = 0;
  double init_flux = 1.0;          // flat starting flux (normalised)
  double t_submit = 0.0, t_admit = 0.0;
  // the pinned copy of the arrays (offset, bytes per Part), until the
  // copies to the pool have run
  PinnedCache* cache = nullptr;
  char* pin = nullptr;
  size_t pin_cap = 0;
  size_t off[kNumParts] = {}, len[kNumParts] = {};
  const char* part(int i) const { return pin + off[i]; }
  // returns the pinned block (its copies have run: the pool's stream was
  // waited on since they were enqueued)
  void release_pin() {
    if (pin && cache) cache->put(pin, pin_cap);
    pin = nullptr;
  }
  ~Staged() { release_pin(); }

  void release_arrays() {
    std::vector<int2>().swap(segs);
    std::vector<int64_t>().swap(seg_off);
    std::vector<int32_t>().swap(next);
    std::vector<int32_t>().swap(track_ang);
    std::vector<uint8_t>().swap(flags);
    std::vector<float>().swap(weights);
    std::vector<float>().swap(inv_sin);
    std::vector<float>().swap(sigma_t);
    std::vector<float>().swap(sigma_s_T);
    std::vector<float>().swap(nu_sigma_f);
    std::vector<float>().swap(chi);
    std::vector<float>().swap(scat_out);
    std::vector<uint8_t>().swap(fissile);
    std::vector<float>().swap(fsr_vol);
    std::vector<float>().swap(fixed);
    std::vector<float>().swap(seg_x);
    std::vector<float>().swap(seg_y);
    std::vector<double>().swap(ls_ang);
    std::vector<float2>().swap(ls_dir);
    std::vector<float>().swap(fixed_xy);
    std::vector<int32_t>().swap(ls_list);
    std::vector<int32_t>().swap(fsr_mat);
  }
};

// Copies a staged request's arrays into one pinned block (16-byte aligned
// parts, in Part order) and frees the pageable ones.
int pin_request(PinnedCache& cache, Staged& s) {
  const void* src[kNumParts] = {};
  size_t n[kNumParts] = {};
  auto set = [&](int i, const void* q, size_t b) {
    src[i] = q;
    n[i] = b;
  };
  set(kSegs, s.segs.data(), sizeof(int2) * s.segs.size());
  set(kSegOff, s.seg_off.data(), sizeof(int64_t) * s.seg_off.size());
  set(kNext, s.next.data(), sizeof(int32_t) * s.next.size());
  set(kTrackAng, s.track_ang.data(), sizeof(int32_t) * s.track_ang.size());
  set(kFlags, s.flags.data(), s.flags.size());
  set(kWeights, s.weights.data(), sizeof(float) * s.weights.size());
  set(kInvSin, s.inv_sin.data(), sizeof(float) * s.inv_sin.size());
  set(kSigmaT, s.sigma_t.data(), sizeof(float) * s.sigma_t.size());
  set(kSigmaST, s.sigma_s_T.data(), sizeof(float) * s.sigma_s_T.size());
  set(kNuSigmaF, s.nu_sigma_f.data(), sizeof(float) * s.nu_sigma_f.size());
  set(kChi, s.chi.data(), sizeof(float) * s.chi.size());
  set(kScatOut, s.scat_out.data(), sizeof(float) * s.scat_out.size());
  set(kFissile, s.fissile.data(), s.fissile.size());
  set(kFsrMat, s.fsr_mat.data(), sizeof(int32_t) * s.fsr_mat.size());
  set(kFsrVol, s.fsr_vol.data(), sizeof(float) * s.fsr_vol.size());
  set(kFixed, s.fixed.data(), sizeof(float) * s.fixed.size());
  set(kSegX, s.seg_x.data(), sizeof(float) * s.seg_x.size());
  set(kSegY, s.seg_y.data(), sizeof(float) * s.seg_y.size());
  set(kLsAng, s.ls_ang.data(), sizeof(double) * s.ls_ang.size());
  set(kLsDir, s.ls_dir.data(), sizeof(float2) * s.ls_dir.size());
  set(kFixedXY, s.fixed_xy.data(), sizeof(float) * s.fixed_xy.size());
  set(kLsList, s.ls_list.data(), sizeof(int32_t) * s.ls_list.size());
  size_t total = 0;
  for (int i = 0; i < kNumParts; i++) {
    s.off[i] = total;
    s.len[i] = n[i];
    total += (n[i] + 15) & ~(size_t) 15;
  }
  s.cache = &cache;
  s.pin = cache.get(total > 0 ? total : 16, &s.pin_cap);
  SV_CHECK(s.pin, MOC_ERR_MEMORY,
           "no page-locked host memory for the request's arrays");
  for (int i = 0; i < kNumParts; i++)
    if (n[i]) std::memcpy(s.pin + s.off[i], src[i], n[i]);
  s.release_arrays();
  return MOC_OK;
}

// The linear-source part of a request, checked as moc_set_linear_source and
// moc_set_fixed_source_moments check theirs (same limits and messages).
int stage_linear_source(const moc_request& q, Staged& s) {
  const moc_ls_geometry* g = q.linear_source;
  const int64_t S = s.S, R = s.R;
  const int A = s.A, Ph = s.Ph, G = s.G, ld = s.ld;
  SV_CHECK(G <= 256, MOC_ERR_UNSUPPORTED,
           "the linear source takes at most 256 groups and 2^31 segments");
  SV_CHECK(S == 0 || (g->seg_x && g->seg_y), MOC_ERR_ARG,
           "null linear-source array");
  SV_CHECK(g->ang_dir && g->ang_wgt && g->pol_sin && g->pol_wgt, MOC_ERR_ARG,
           "null linear-source array");
  SV_CHECK(!g->seg_z && !g->pol_cos, MOC_ERR_UNSUPPORTED,
           "linear-source pools take 2D tracks");
  s.seg_x.resize(S);
  s.seg_y.resize(S);
  for (int64_t i = 0; i < S; i++) {
    SV_CHECK(std::isfinite(g->seg_x[i]) && std::isfinite(g->seg_y[i]),
             MOC_ERR_ARG,
             "non-finite segment start position at segment " +
                 std::to_string(i));
    s.seg_x[i] = g->seg_x[i];
    s.seg_y[i] = g->seg_y[i];
  }
  s.ls_ang.assign(3 * (size_t) A + 2 * (size_t) A * Ph, 0.0);
  s.ls_dir.resize(A);
  for (int a = 0; a < A; a++) {
    const double cx = g->ang_dir[2 * a], cy = g->ang_dir[2 * a + 1];
    SV_CHECK(std::isfinite(cx) && std::isfinite(cy) &&
                 std::fabs(cx * cx + cy * cy - 1.0) < 1e-6,
             MOC_ERR_ARG,
             "track direction of angle " + std::to_string(a) +
                 " is not a unit vector");
    SV_CHECK(std::isfinite(g->ang_wgt[a]) && g->ang_wgt[a] > 0.0, MOC_ERR_ARG,
             "azimuthal weight must be positive");
    s.ls_ang[2 * a] = cx;
    s.ls_ang[2 * a + 1] = cy;
    s.ls_ang[2 * A + a] = g->ang_wgt[a];
    s.ls_dir[a] = make_float2((float) cx, (float) cy);
    for (int p = 0; p < Ph; p++) {
      const double sn = g->pol_sin[a * Ph + p], w = g->pol_wgt[a * Ph + p];
      SV_CHECK(std::isfinite(sn) && sn > 0.0 && sn <= 1.0, MOC_ERR_ARG,
               "sin(theta) must lie in (0, 1]");
      SV_CHECK(std::isfinite(w) && w >= 0.0, MOC_ERR_ARG,
               "polar weight must be non-negative");
      s.ls_ang[3 * A + a * Ph + p] = sn;
      s.ls_ang[3 * A + A * Ph + a * Ph + p] = w;
    }
  }
  if (q.fixed_source_moments) {
    s.fixed_xy.assign(2 * (size_t) R * ld, 0.0f);
    for (int64_t r = 0; r < R; r++)
      for (int gg = 0; gg < G; gg++) {
        const float x = q.fixed_source_moments[(r * 3 + 0) * G + gg];
        const float y = q.fixed_source_moments[(r * 3 + 1) * G + gg];
        SV_CHECK(std::isfinite(x) && std::isfinite(y), MOC_ERR_ARG,
                 "non-finite moment");
        s.fixed_xy[2 * (r * ld + gg)] = x;
        s.fixed_xy[2 * (r * ld + gg) + 1] = y;
      }
  }
  // a counting sort of the segment ids by FSR
  std::vector<int64_t> fill(R + 1, 0);
  for (int64_t i = 0; i < S; i++) fill[s.segs[i].y + 1]++;
  for (int64_t r = 0; r < R; r++) fill[r + 1] += fill[r];
  s.ls_list.resize(S);
  for (int64_t i = 0; i < S; i++) s.ls_list[fill[s.segs[i].y]++] = (int32_t) i;
  s.ls = true;
  return MOC_OK;
}

// Checks a request as moc_upload_* check a context's inputs and packs it.
int stage_request(const moc_request& q, Staged& s) {
  SV_CHECK(q.num_groups >= 1 && q.num_groups <= 64 * moc::kMaxSlots,
           MOC_ERR_ARG, "num_groups must be in [1, 384]");
  SV_CHECK(q.num_polar_half >= 1 && q.num_polar_half <= 3, MOC_ERR_UNSUPPORTED,
           "num_polar_half must be 1, 2 or 3");
  SV_CHECK(q.num_angles >= 1 && q.num_materials >= 1 && q.num_fsrs >= 1 &&
               q.num_tracks >= 1 && q.num_segments >= 0,
           MOC_ERR_ARG, "empty problem dimension");
  SV_CHECK(q.num_materials <= 256 && q.num_fsrs < (1LL << 24) &&
               q.num_tracks < (1LL << 30),
           MOC_ERR_ARG, "request too large for a pool");
  SV_CHECK(q.seg_off && q.track_ang && q.next && q.flags && q.weights &&
               q.inv_sin && q.sigma_t && q.sigma_s && q.nu_sigma_f && q.chi &&
               q.fsr_mat && q.fsr_vol && q.flux_out,
           MOC_ERR_ARG, "null array in request");
  SV_CHECK(q.num_segments == 0 || (q.seg_len && q.seg_fsr), MOC_ERR_ARG,
           "null segments");
  SV_CHECK(q.kind == MOC_SOLVE_EIGENVALUE || q.kind == MOC_SOLVE_SOURCE ||
               q.kind == MOC_SOLVE_FLUX,
           MOC_ERR_ARG, "unknown solve kind");
  SV_CHECK(q.max_iters >= 1, MOC_ERR_ARG, "max_iters must be positive");
  SV_CHECK(q.res_type >= 0 && q.res_type <= 2, MOC_ERR_ARG,
           "bad residual type");
  SV_CHECK(q.threshold > 0.0 && std::isfinite(q.threshold), MOC_ERR_ARG,
           "the convergence threshold must be positive");
  SV_CHECK(q.kind != MOC_SOLVE_SOURCE || q.k_eff > 0.0, MOC_ERR_ARG,
           "The Solver is unable to compute the source with a non-positive "
           "keff");
  SV_CHECK(!q.linear_source || q.num_segments < (1LL << 31),
           MOC_ERR_UNSUPPORTED,
           "the linear source takes at most 256 groups and 2^31 segments");
  SV_CHECK(q.linear_source || (!q.fixed_source_moments && !q.moments_out),
           MOC_ERR_ARG, "flux moments need a linear-source request");
  const int G = q.num_groups, M = q.num_materials, Ph = q.num_polar_half;
  const int64_t R = q.num_fsrs, T = q.num_tracks, S = q.num_segments;
  s.req = q;
  s.G = G;
  s.Ph = Ph;
  s.A = q.num_angles;
  s.M = M;
  s.R = R;
  s.T = T;
  s.S = S;
  s.ld = G + (G & 1);

  // tracks
  SV_CHECK(q.seg_off[0] == 0 && q.seg_off[T] == S, MOC_ERR_ARG,
           "seg_off must run from 0 to num_segments");
  s.seg_off.assign(q.seg_off, q.seg_off + T + 1);
  s.nseg.resize(T);
  s.next.resize(2 * T);
  s.track_ang.resize(T);
  s.flags.assign(q.flags, q.flags + T);
  s.flags.push_back(0);
  for (int64_t t = 0; t < T; t++) {
    const int64_t n = q.seg_off[t + 1] - q.seg_off[t];
    SV_CHECK(n >= 0 && n < (1LL << 31), MOC_ERR_ARG,
             "bad segment count on track " + std::to_string(t));
    s.nseg[t] = (int32_t) n;
    SV_CHECK(q.track_ang[t] >= 0 && q.track_ang[t] < q.num_angles,
             MOC_ERR_ARG, "track angle index out of range");
    s.track_ang[t] = q.track_ang[t];
    for (int d = 0; d < 2; d++) {
      SV_CHECK(q.next[2 * t + d] >= 0 && q.next[2 * t + d] < T, MOC_ERR_ARG,
               "next-track index out of range on track " + std::to_string(t));
      s.next[2 * t + d] = (int32_t) q.next[2 * t + d];
    }
  }
  s.segs.resize(S);
  for (int64_t i = 0; i < S; i++) {
    SV_CHECK(q.seg_fsr[i] >= 0 && q.seg_fsr[i] < R, MOC_ERR_ARG,
             "segment FSR id out of range at segment " + std::to_string(i));
    SV_CHECK(std::isfinite(q.seg_len[i]) && q.seg_len[i] >= 0.0f, MOC_ERR_ARG,
             "bad segment length at segment " + std::to_string(i));
    int2 v;
    std::memcpy(&v.x, &q.seg_len[i], 4);
    v.y = q.seg_fsr[i];
    s.segs[i] = v;
  }

  // quadrature
  const int64_t nq = (int64_t) q.num_angles * Ph;
  s.weights.assign(q.weights, q.weights + nq);
  s.inv_sin.assign(q.inv_sin, q.inv_sin + nq);
  for (int64_t i = 0; i < nq; i++)
    SV_CHECK(std::isfinite(q.weights[i]) && std::isfinite(q.inv_sin[i]) &&
                 q.inv_sin[i] >= 1.0f,
             MOC_ERR_ARG, "bad quadrature entry " + std::to_string(i));

  // materials
  const int64_t MG = (int64_t) M * G;
  s.sigma_t.assign(q.sigma_t, q.sigma_t + MG);
  s.nu_sigma_f.assign(q.nu_sigma_f, q.nu_sigma_f + MG);
  s.chi.assign(q.chi, q.chi + MG);
  s.scat_out.assign(MG, 0.0f);
  s.sigma_s_T.assign(MG * G, 0.0f);
  s.fissile.assign(M, 0);
  for (int m = 0; m < M; m++) {
    for (int g = 0; g < G; g++) {
      const int64_t i = (int64_t) m * G + g;
      SV_CHECK(std::isfinite(q.sigma_t[i]) && q.sigma_t[i] > 0.0f,
               MOC_ERR_ARG, "sigma_t must be positive and finite (material " +
                                std::to_string(m) + ")");
      SV_CHECK(std::isfinite(q.nu_sigma_f[i]) && std::isfinite(q.chi[i]),
               MOC_ERR_ARG, "non-finite fission data in material " +
                                std::to_string(m));
      if (q.nu_sigma_f[i] > 0.0f) s.fissile[m] = 1;
    }
    for (int gd = 0; gd < G; gd++)
      for (int g = 0; g < G; g++) {
        const float v = q.sigma_s[((int64_t) m * G + gd) * G + g];
        SV_CHECK(std::isfinite(v), MOC_ERR_ARG,
                 "non-finite scattering data in material " +
                     std::to_string(m));
        s.scat_out[(int64_t) m * G + g] += v;
        s.sigma_s_T[((int64_t) m * G + g) * G + gd] = v;
      }
  }

  // FSRs
  s.fsr_mat.assign(q.fsr_mat, q.fsr_mat + R);
  s.fsr_vol.assign(q.fsr_vol, q.fsr_vol + R);
  double total = 0.0;
  for (int64_t r = 0; r < R; r++) {
    SV_CHECK(q.fsr_mat[r] >= 0 && q.fsr_mat[r] < M, MOC_ERR_ARG,
             "FSR material index out of range at FSR " + std::to_string(r));
    SV_CHECK(std::isfinite(q.fsr_vol[r]) && q.fsr_vol[r] >= 0.0f, MOC_ERR_ARG,
             "bad FSR volume at FSR " + std::to_string(r));
    const int m = q.fsr_mat[r];
    if (s.fissile[m]) {
      s.num_fissionable++;
      double row = 0.0;
      for (int g = 0; g < G; g++) row += (double) q.nu_sigma_f[(int64_t) m * G + g];
      total += row * (double) q.fsr_vol[r];
    }
  }
  if (q.kind == MOC_SOLVE_EIGENVALUE) {
    SV_CHECK(s.num_fissionable > 0 && total > 0.0, MOC_ERR_ARG,
             "an eigenvalue solve needs fissionable material");
    // Solver::computeInitialFluxGuess then normalizeFluxes: a flat flux of
    // one scaled by R / (total fission source)
    s.init_flux = (double) (float) ((double) R / total);
  } else if (q.kind == MOC_SOLVE_FLUX) {
    // Solver::computeFlux: flattenFSRFluxes(0), and the SCALAR_FLUX
    // residual whatever the request says (src/Solver.cpp:1380-1440)
    s.init_flux = 0.0;
    s.req.res_type = MOC_SCALAR_FLUX;
  } else {
    s.init_flux = 1.0;
  }
  SV_CHECK(q.res_type != MOC_FISSION_SOURCE || s.num_fissionable > 0,
           MOC_ERR_ARG,
           "The Solver is unable to compute a FISSION_SOURCE residual "
           "without fissionable FSRs");
  if (q.fixed_source) {
    s.fixed.assign((size_t) R * s.ld, 0.0f);
    for (int64_t r = 0; r < R; r++)
      for (int g = 0; g < G; g++) {
        const float v = q.fixed_source[r * G + g];
        SV_CHECK(std::isfinite(v), MOC_ERR_ARG, "non-finite fixed source");
        s.fixed[r * s.ld + g] = v;
      }
  }
  return q.linear_source ? stage_linear_source(q, s) : MOC_OK;
}

}  // namespace

struct moc_server;

namespace {

// A pool slot: one live solve and the ranges it owns.
struct Slot {
  std::unique_ptr<Staged> st;
  int64_t r0 = 0, t0 = 0, s0 = 0;
  int64_t m0 = 0, a0 = 0;
  bool live = false;
  bool uploaded = false;    // data copied into the pool's arrays
  bool needs_init = false;  // starting state not yet written
};

struct Pool {
  moc_pool_config cfg{};
  int index = 0;
  int G = 0, Ph = 0, ld = 0, F = 0;
  cudaStream_t stream = nullptr;
  cudaEvent_t block_start = nullptr;
  cudaEvent_t block_done = nullptr;
  std::vector<cudaEvent_t> tune_ev;

  // device arrays over the pool's capacity
  int2* segs = nullptr;
  int64_t* seg_off = nullptr;
  int32_t* order = nullptr;
  int32_t* track_ang = nullptr;
  int32_t* next = nullptr;
  int32_t* track_slot = nullptr;
  uint8_t* flags = nullptr;
  float* weights = nullptr;
  float* inv_sin = nullptr;
  float* sigma_t = nullptr;
  float* sigma_s_T = nullptr;
  float* nu_sigma_f = nullptr;
  float* chi = nullptr;
  float* scat_out = nullptr;
  uint8_t* fissile = nullptr;
  int32_t* fsr_mat = nullptr;
  int32_t* row_slot = nullptr;
  float* fsr_vol = nullptr;
  float* fixed = nullptr;
  float* phi = nullptr;
  float* phi_old = nullptr;
  float* qt = nullptr;
  float* psi[2] = {nullptr, nullptr};
  float* exp_table = nullptr;
  double* row_val = nullptr;
  moc::DevScalars* sc = nullptr;       // pool: buffer index and ticket
  moc::DevScalars* slots_d = nullptr;  // per-solve states
  moc::DevScalars* slots_h = nullptr;  // pinned: states read back per block
  moc::DevScalars* init_h = nullptr;   // pinned: states written at admission
  float* retire_h = nullptr;           // pinned: fluxes of retired solves
  // linear source (ls): 16-byte segment words, angle directions, inverse
  // expansion matrices, source constants, source and flux moments, fixed
  // source moments; admission scratch (segment starts, angle data, the
  // count of flat FSRs); the moments of retired solves
  bool ls = false;
  int4* segs_ls = nullptr;
  float2* ang_dir = nullptr;
  float* ls_ilem = nullptr;
  float* ls_const = nullptr;
  float* qxy = nullptr;
  float* mom = nullptr;
  float* fixed_xy = nullptr;
  float* ls_xy = nullptr;
  double* ls_ang = nullptr;
  double* ls_scratch = nullptr;
  int32_t* ls_list = nullptr;
  int32_t* ls_seg_track = nullptr;
  unsigned int* ls_flat = nullptr;
  float* retire_mom_h = nullptr;

  RangeAlloc rows, tracks, segments, mats, angles;
  std::vector<int> free_slots;
  std::vector<Slot> slots;
  std::deque<std::unique_ptr<Staged>> queue;  // guarded by the server mutex

  bool in_flight = false;
  bool dirty = false;
  int64_t active_tracks = 0;
  int64_t rows_hi = 0;
  int64_t mats_hi = 0;
  cudaGraphExec_t graph = nullptr;
  int graph_iters = 0;

  int lps = 0, pairs = 0, exp_kind = MOC_EXP_INTRINSIC;
  int graph_lps = 0, graph_pairs = 0;          // shape of the captured graph
  std::map<int, std::pair<int, int>> shape_by_class;
  // autotuner scratch outputs
  float* tune_psi = nullptr;
  float* tune_phi = nullptr;
  float* tune_mom = nullptr;
  moc::DevScalars* tune_sc = nullptr;
  moc::DevScalars* tune_slots = nullptr;
  // counters (read under the server mutex)
  int64_t n_admitted = 0, n_completed = 0, n_blocks = 0, n_tunes = 0;
  double busy_s = 0.0;
};

}  // namespace

struct moc_server {
  PinnedCache pinned;                // requests' host arrays (outlives pools)
  moc_server_config cfg{};
  int64_t hot_live = 0;              // sweep-gathered bytes of live solves
  std::vector<std::unique_ptr<Pool>> pools;
  std::mutex mu;                     // queues, results, counters
  std::condition_variable cv;
  std::map<int64_t, moc_result> results;
  std::vector<int64_t> completed;    // since the last poll
  int64_t next_ticket = 1;
  moc_server_stats stats{};
  std::thread loop;
  std::atomic<bool> running{false};
  std::string loop_error;
  std::vector<float> exp_table_h;
};

namespace {

void destroy_pool(Pool& p) {
  if (p.stream) cudaStreamSynchronize(p.stream);
  if (p.graph) cudaGraphExecDestroy(p.graph);
  dev_free(p.segs);
  dev_free(p.seg_off);
  dev_free(p.order);
  dev_free(p.track_ang);
  dev_free(p.next);
  dev_free(p.track_slot);
  dev_free(p.flags);
  dev_free(p.weights);
  dev_free(p.inv_sin);
  dev_free(p.sigma_t);
  dev_free(p.sigma_s_T);
  dev_free(p.nu_sigma_f);
  dev_free(p.chi);
  dev_free(p.scat_out);
  dev_free(p.fissile);
  dev_free(p.fsr_mat);
  dev_free(p.row_slot);
  dev_free(p.fsr_vol);
  dev_free(p.fixed);
  dev_free(p.phi);
  dev_free(p.phi_old);
  dev_free(p.qt);
  dev_free(p.psi[0]);
  dev_free(p.psi[1]);
  dev_free(p.exp_table);
  dev_free(p.row_val);
  dev_free(p.sc);
  dev_free(p.slots_d);
  dev_free(p.tune_psi);
  dev_free(p.tune_phi);
  dev_free(p.tune_mom);
  dev_free(p.tune_sc);
  dev_free(p.tune_slots);
  dev_free(p.segs_ls);
  dev_free(p.ang_dir);
  dev_free(p.ls_ilem);
  dev_free(p.ls_const);
  dev_free(p.qxy);
  dev_free(p.mom);
  dev_free(p.fixed_xy);
  dev_free(p.ls_xy);
  dev_free(p.ls_ang);
  dev_free(p.ls_scratch);
  dev_free(p.ls_list);
  dev_free(p.ls_seg_track);
  dev_free(p.ls_flat);
  if (p.slots_h) cudaFreeHost(p.slots_h);
  if (p.init_h) cudaFreeHost(p.init_h);
  if (p.retire_h) cudaFreeHost(p.retire_h);
  if (p.retire_mom_h) cudaFreeHost(p.retire_mom_h);
  p.slots_h = p.init_h = nullptr;
  p.retire_h = p.retire_mom_h = nullptr;
  for (cudaEvent_t e : p.tune_ev) cudaEventDestroy(e);
  if (p.block_start) cudaEventDestroy(p.block_start);
  if (p.block_done) cudaEventDestroy(p.block_done);
  if (p.stream) cudaStreamDestroy(p.stream);
  p.stream = nullptr;
}

int create_pool(moc_server* srv, const moc_pool_config& c, Pool& p) {
  SV_CHECK(c.num_groups >= 1 && c.num_groups <= 64 * moc::kMaxSlots,
           MOC_ERR_ARG, "num_groups must be in [1, 384]");
  SV_CHECK(c.num_polar_half >= 1 && c.num_polar_half <= 3,
           MOC_ERR_UNSUPPORTED, "num_polar_half must be 1, 2 or 3");
  SV_CHECK(c.max_solves >= 1 && c.max_solves <= 4096 && c.max_materials >= 1 &&
               c.max_materials <= 256 && c.max_angles >= 1 &&
               c.max_fsrs >= 1 && c.max_fsrs < (1LL << 24) &&
               c.max_tracks >= 2 && c.max_tracks < (1LL << 30) &&
               c.max_segments >= 1,
           MOC_ERR_ARG, "bad pool capacity");
  const int ld = c.num_groups + (c.num_groups & 1);
  SV_CHECK((int64_t) c.max_materials * ld * 4 <= 200 * 1024, MOC_ERR_ARG,
           "max_materials x groups exceeds the sweep's shared-memory table");
  SV_CHECK(c.linear_source == 0 || c.linear_source == 1, MOC_ERR_ARG,
           "linear_source must be 0 or 1");
  SV_CHECK(!c.linear_source || c.num_groups <= 256, MOC_ERR_UNSUPPORTED,
           "the linear source takes at most 256 groups and 2^31 segments");
  SV_CHECK(!c.linear_source || c.max_segments < (1LL << 31),
           MOC_ERR_UNSUPPORTED,
           "the linear source takes at most 256 groups and 2^31 segments");
  if (c.lanes != 0) {
    SV_CHECK(!c.linear_source || c.pairs <= kLsMaxPairs, MOC_ERR_ARG,
             "the linear-source sweep takes at most 5 group pairs per lane");
    SV_CHECK(moc::sweep_lps_supported(c.lanes), MOC_ERR_ARG,
             "lanes per track direction must be 1, 2, 4, 8, 16 or 32");
    SV_CHECK(c.pairs >= 1 && c.pairs <= moc::kMaxSlots &&
                 2 * (int64_t) c.lanes * c.pairs >= c.num_groups,
             MOC_ERR_ARG, "lanes x group pairs per lane must cover every group");
    SV_CHECK(c.pairs == pairs_for(c.num_groups, c.lanes), MOC_ERR_ARG,
             "group pairs per lane must be the fewest that cover the groups, "
             "ceil(ceil(G / 2) / lanes)");
    SV_CHECK(c.exp_kind == MOC_EXP_INTRINSIC, MOC_ERR_UNSUPPORTED,
             "pools sweep with the hardware-ex2 evaluator (MOC_EXP_INTRINSIC)");
  }
  p.cfg = c;
  p.G = c.num_groups;
  p.Ph = c.num_polar_half;
  p.ld = ld;
  p.F = p.G * p.Ph;
  p.ls = c.linear_source != 0;
  if (c.lanes != 0) {
    p.lps = c.lanes;
    p.pairs = c.pairs;
    p.exp_kind = c.exp_kind;
  }
  // pools of few fluxes per track run short, latency-bound kernels: with
  // priorities on they go ahead of the long sweeps of the wide pools
  int prio_low = 0, prio_high = 0;
  SV_CUDA(cudaDeviceGetStreamPriorityRange(&prio_low, &prio_high));
  const bool high = srv->cfg.priorities && p.F <= 48;
  SV_CUDA(cudaStreamCreateWithPriority(&p.stream, cudaStreamNonBlocking,
                                       high ? prio_high : prio_low));
  SV_CUDA(cudaEventCreate(&p.block_start));
  SV_CUDA(cudaEventCreate(&p.block_done));
  const int64_t R = c.max_fsrs, T = c.max_tracks, S = c.max_segments;
  const int64_t M = c.max_materials, A = c.max_angles, N = c.max_solves;
  const int64_t MG = M * p.G, npsi = T * 2 * p.F;
  SV_TRY(dev_alloc(&p.segs, S));
  SV_TRY(dev_alloc(&p.seg_off, T));
  SV_TRY(dev_alloc(&p.order, T));
  SV_TRY(dev_alloc(&p.track_ang, T));
  SV_TRY(dev_alloc(&p.next, 2 * T));
  SV_TRY(dev_alloc(&p.track_slot, T));
  SV_TRY(dev_alloc(&p.flags, T));
  SV_TRY(dev_alloc(&p.weights, A * p.Ph));
  SV_TRY(dev_alloc(&p.inv_sin, A * p.Ph));
  SV_TRY(dev_alloc(&p.sigma_t, MG));
  SV_TRY(dev_alloc(&p.sigma_s_T, MG * p.G + 4));
  SV_TRY(dev_alloc(&p.nu_sigma_f, MG));
  SV_TRY(dev_alloc(&p.chi, MG));
  SV_TRY(dev_alloc(&p.scat_out, MG));
  SV_TRY(dev_alloc(&p.fissile, M));
  SV_TRY(dev_alloc(&p.fsr_mat, R));
  SV_TRY(dev_alloc(&p.row_slot, R));
  SV_TRY(dev_alloc(&p.fsr_vol, R));
  SV_TRY(dev_alloc(&p.fixed, R * ld));
  SV_TRY(dev_alloc(&p.phi, R * ld));
  SV_TRY(dev_alloc(&p.phi_old, R * ld));
  SV_TRY(dev_alloc(&p.qt, R * ld));
  SV_TRY(dev_alloc(&p.psi[0], npsi));
  SV_TRY(dev_alloc(&p.psi[1], npsi));
  SV_TRY(dev_alloc(&p.exp_table, 2 * moc::kExpTableSize));
  SV_TRY(dev_alloc(&p.row_val, R));
  SV_TRY(dev_alloc(&p.sc, 1));
  SV_TRY(dev_alloc(&p.slots_d, N));
  SV_CUDA(cudaMallocHost((void**) &p.slots_h, sizeof(moc::DevScalars) * N));
  SV_CUDA(cudaMallocHost((void**) &p.init_h, sizeof(moc::DevScalars) * N));
  SV_CUDA(cudaMallocHost((void**) &p.retire_h, sizeof(float) * R * ld));
  // every slot starts free: done, so every kernel skips it
  std::vector<moc::DevScalars> st(N);
  std::memset(st.data(), 0, sizeof(moc::DevScalars) * N);
  for (auto& s : st) {
    s.done = 1;
    s.keff = 1.0;
    s.scale[0] = s.scale[1] = 1.0f;
  }
  std::memcpy(p.slots_h, st.data(), sizeof(moc::DevScalars) * N);
  moc::DevScalars pool_sc;
  std::memset(&pool_sc, 0, sizeof(pool_sc));
  pool_sc.keff = 1.0;
  pool_sc.scale[0] = pool_sc.scale[1] = 1.0f;
  SV_CUDA(cudaMemcpy(p.slots_d, st.data(), sizeof(moc::DevScalars) * N,
                     cudaMemcpyHostToDevice));
  SV_CUDA(cudaMemcpy(p.sc, &pool_sc, sizeof(pool_sc), cudaMemcpyHostToDevice));
  SV_CUDA(cudaMemcpy(p.exp_table, srv->exp_table_h.data(),
                     sizeof(float) * srv->exp_table_h.size(),
                     cudaMemcpyHostToDevice));
  SV_CUDA(cudaMemset(p.row_slot, 0xFF, sizeof(int32_t) * R));
  SV_CUDA(cudaMemset(p.fixed, 0, sizeof(float) * R * ld));
  SV_CUDA(cudaMemset(p.phi, 0, sizeof(float) * R * ld));
  SV_CUDA(cudaMemset(p.phi_old, 0, sizeof(float) * R * ld));
  SV_CUDA(cudaMemset(p.qt, 0, sizeof(float) * R * ld));
  SV_CUDA(cudaMemset(p.psi[0], 0, sizeof(float) * npsi));
  SV_CUDA(cudaMemset(p.psi[1], 0, sizeof(float) * npsi));
  SV_CUDA(cudaMemset(p.sigma_s_T, 0, sizeof(float) * (MG * p.G + 4)));
  if (p.ls) {
    SV_TRY(dev_alloc(&p.segs_ls, S));
    SV_TRY(dev_alloc(&p.ang_dir, A));
    SV_TRY(dev_alloc(&p.ls_ilem, 3 * R));
    SV_TRY(dev_alloc(&p.ls_const, 3 * R * ld));
    SV_TRY(dev_alloc(&p.qxy, 2 * R * ld));
    SV_TRY(dev_alloc(&p.mom, 2 * R * ld));
    SV_TRY(dev_alloc(&p.fixed_xy, 2 * R * ld));
    SV_TRY(dev_alloc(&p.ls_xy, 2 * S));
    SV_TRY(dev_alloc(&p.ls_ang, A * (3 + 2 * p.Ph)));
    SV_TRY(dev_alloc(&p.ls_scratch, moc::ls_constants_scratch(R, ld, false)));
    SV_TRY(dev_alloc(&p.ls_list, S));
    SV_TRY(dev_alloc(&p.ls_seg_track, S));
    SV_TRY(dev_alloc(&p.ls_flat, 1));
    SV_CUDA(cudaMallocHost((void**) &p.retire_mom_h,
                           sizeof(float) * 2 * R * ld));
    SV_CUDA(cudaMemset(p.qxy, 0, sizeof(float) * 2 * R * ld));
    SV_CUDA(cudaMemset(p.mom, 0, sizeof(float) * 2 * R * ld));
    SV_CUDA(cudaMemset(p.fixed_xy, 0, sizeof(float) * 2 * R * ld));
    SV_CUDA(cudaMemset(p.ls_ilem, 0, sizeof(float) * 3 * R));
    SV_CUDA(cudaMemset(p.ls_const, 0, sizeof(float) * 3 * R * ld));
  }
  p.rows.reset(R);
  p.tracks.reset(T);
  p.segments.reset(S);
  p.mats.reset(M);
  p.angles.reset(A);
  p.slots.resize(N);
  for (int i = (int) N - 1; i >= 0; i--) p.free_slots.push_back(i);
  return MOC_OK;
}

moc::SweepArgs pool_sweep_args(Pool& p) {
  moc::SweepArgs a{};
  a.segs = p.segs;
  a.seg_off = p.seg_off;
  a.order = p.order;
  a.track_ang = p.track_ang;
  a.next = p.next;
  a.flags = p.flags;
  a.weights = p.weights;
  a.inv_sin = p.inv_sin;
  a.sigma_t = p.sigma_t;
  a.fsr_mat = p.fsr_mat;
  a.qt = p.qt;
  a.exp_table = p.exp_table;
  a.phi = p.phi;
  a.psi[0] = p.psi[0];
  a.psi[1] = p.psi[1];
  a.sc = p.sc;
  a.num_tracks = p.active_tracks;
  a.num_groups = p.G;
  a.ld = p.ld;
  a.num_materials = (int) std::max<int64_t>(p.mats_hi, 1);
  a.lps = p.lps;
  a.check_done = 0;
  a.mat_packed = 1;
  a.track_slot = p.track_slot;
  a.slots = p.slots_d;
  a.num_slots = p.cfg.max_solves;
  a.hot_base = 0x7FFFFFFF;   // no shared-memory tallies in pools
  a.hot_count = 0;
  if (p.ls) {
    a.segs_ls = p.segs_ls;
    a.ang_dir = p.ang_dir;
    a.qxy = p.qxy;
    a.mom = p.mom;
  }
  return a;
}

moc::SolverArgs pool_solver_args(Pool& p) {
  moc::SolverArgs a{};
  a.sigma_t = p.sigma_t;
  a.sigma_s = nullptr;
  a.sigma_s_T = p.sigma_s_T;
  a.nu_sigma_f = p.nu_sigma_f;
  a.chi = p.chi;
  a.fissile = p.fissile;
  a.fsr_mat = p.fsr_mat;
  a.fsr_vol = p.fsr_vol;
  a.fixed = p.fixed;
  a.scat_out = p.scat_out;
  a.sigma_f = nullptr;
  a.phi = p.phi;
  a.phi_old = p.phi_old;
  a.qt = p.qt;
  a.psi[0] = p.psi[0];
  a.psi[1] = p.psi[1];
  a.sc = p.sc;
  a.num_fsrs = p.rows_hi;
  a.num_psi = p.cfg.max_tracks * 2 * p.F;
  a.num_groups = p.G;
  a.ld = p.ld;
  a.num_materials = (int) std::max<int64_t>(p.mats_hi, 1);
  a.check_done = 0;
  a.row_slot = p.row_slot;
  a.slots = p.slots_d;
  a.row_val = p.row_val;
  a.num_slots = p.cfg.max_solves;
  if (p.ls) {
    a.mom = p.mom;
    a.qxy = p.qxy;
    a.ls_ilem = p.ls_ilem;
    a.ls_const = p.ls_const;
    a.fixed_xy = p.fixed_xy;
  }
  return a;
}

}  // namespace

namespace {

void add_launches(moc_server* srv, int64_t n) {
  std::lock_guard<std::mutex> lk(srv->mu);
  srv->stats.kernel_launches += n;
}

void publish(moc_server* srv, const Staged& st, const moc_result& r) {
  std::lock_guard<std::mutex> lk(srv->mu);
  srv->results[st.ticket] = r;
  srv->completed.push_back(st.ticket);
  if (r.status == MOC_OK) srv->stats.completed++;
  else srv->stats.failed++;
  srv->stats.live--;
  srv->cv.notify_all();
}

// Bytes of a solve that the sweep gathers and scatters by FSR id: its
// reduced sources and tallies, and with a linear source their x and y
// moments too.
int64_t hot_bytes(const Staged& s) { return (s.ls ? 24 : 8) * s.R * s.ld; }

// The pool material numbers of an admitted solve's FSRs (its own + m0),
// and the owner of its rows.
__global__ void offset_i32_kernel(int32_t* v, int64_t n, int32_t add) {
  for (int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t) gridDim.x * blockDim.x)
    v[i] += add;
}

__global__ void fill_i32_kernel(int32_t* v, int64_t n, int32_t value) {
  for (int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t) gridDim.x * blockDim.x)
    v[i] = value;
}

unsigned small_grid(int64_t n) {
  int64_t b = (n + 255) / 256;
  return (unsigned) (b < 1 ? 1 : b > 1024 ? 1024 : b);
}

// The linear-source data of an admitted solve, while its segments and track
// data are still in its own numbering: the 16-byte segment words, its angle
// directions and fixed source moments, and its expansion matrices and
// source constants (CPULSSolver::initializeFSRs with
// LinearExpansionGenerator, src/CPULSSolver.cpp:136-146), computed over its
// own segments into its rows from the buckets staged on submission.  All
// copies and launches are in the pool's stream order, so the admission
// scratch is reused by the next admission without a synchronisation.
int upload_linear_source(moc_server* srv, Pool& p, const Slot& sl) {
  const Staged& s = *sl.st;
  cudaStream_t st = p.stream;
  const int64_t S = s.S, R = s.R, ld = p.ld;
  const int A = s.A, Ph = s.Ph;
  auto put = [&](void* dst, int part) -> int {
    if (s.len[part])
      SV_CUDA(cudaMemcpyAsync(dst, s.part(part), s.len[part],
                              cudaMemcpyHostToDevice, st));
    return MOC_OK;
  };
  if (S > 0) {
    float* dx = p.ls_xy;
    float* dy = p.ls_xy + S;
    SV_TRY(put(dx, kSegX));
    SV_TRY(put(dy, kSegY));
    moc::launch_ls_pack_segments(p.segs + sl.s0, dx, dy, p.segs_ls + sl.s0,
                                 S, st);
  }
  SV_TRY(put(p.ls_ang, kLsAng));
  SV_TRY(put(p.ang_dir + sl.a0, kLsDir));
  if (s.len[kFixedXY] == 0)
    SV_CUDA(cudaMemsetAsync(p.fixed_xy + 2 * sl.r0 * ld, 0,
                            sizeof(float) * 2 * R * ld, st));
  else
    SV_TRY(put(p.fixed_xy + 2 * sl.r0 * ld, kFixedXY));
  if (S > 0) {
    SV_TRY(put(p.ls_list, kLsList));
    moc::launch_ls_seg_track(p.seg_off + sl.t0, s.T, p.ls_seg_track, st);
  }
  const double* ang = p.ls_ang;
  moc::launch_ls_constants_bucketed(
      p.segs_ls + sl.s0, p.ls_list, S, p.ls_seg_track, p.track_ang + sl.t0,
      ang, ang + 2 * A, ang + 3 * A, ang + 3 * A + A * Ph, Ph, p.sigma_t,
      p.fsr_vol + sl.r0, p.fsr_mat + sl.r0, R, s.G, (int) ld,
      p.ls_ilem + 3 * sl.r0, p.ls_const + 3 * sl.r0 * ld, p.ls_flat,
      p.ls_scratch, st);
  SV_CUDA(cudaGetLastError());
  add_launches(srv, S > 0 ? 3 : 1);
  return MOC_OK;
}

// Copies a solve's data from its pinned block into the ranges given to it
// (asynchronous copies only) and rebases them.
int upload_slot(moc_server* srv, Pool& p, int slot_index) {
  Slot& sl = p.slots[slot_index];
  Staged& s = *sl.st;
  cudaStream_t st = p.stream;
  const int64_t T = s.T, S = s.S, R = s.R, G = s.G;
  auto put = [&](void* dst, int part) -> int {
    if (s.len[part])
      SV_CUDA(cudaMemcpyAsync(dst, s.part(part), s.len[part],
                              cudaMemcpyHostToDevice, st));
    return MOC_OK;
  };
  SV_TRY(put(p.segs + sl.s0, kSegs));
  SV_TRY(put(p.seg_off + sl.t0, kSegOff));
  SV_TRY(put(p.next + 2 * sl.t0, kNext));
  SV_TRY(put(p.track_ang + sl.t0, kTrackAng));
  SV_TRY(put(p.flags + sl.t0, kFlags));
  SV_TRY(put(p.weights + sl.a0 * p.Ph, kWeights));
  SV_TRY(put(p.inv_sin + sl.a0 * p.Ph, kInvSin));
  SV_TRY(put(p.sigma_t + sl.m0 * G, kSigmaT));
  SV_TRY(put(p.sigma_s_T + sl.m0 * G * G, kSigmaST));
  SV_TRY(put(p.nu_sigma_f + sl.m0 * G, kNuSigmaF));
  SV_TRY(put(p.chi + sl.m0 * G, kChi));
  SV_TRY(put(p.scat_out + sl.m0 * G, kScatOut));
  SV_TRY(put(p.fissile + sl.m0, kFissile));
  SV_TRY(put(p.fsr_mat + sl.r0, kFsrMat));
  offset_i32_kernel<<<small_grid(R), 256, 0, st>>>(p.fsr_mat + sl.r0, R,
                                                   (int32_t) sl.m0);
  SV_TRY(put(p.fsr_vol + sl.r0, kFsrVol));
  if (s.len[kFixed] == 0)
    SV_CUDA(cudaMemsetAsync(p.fixed + sl.r0 * p.ld, 0,
                            sizeof(float) * R * p.ld, st));
  else
    SV_TRY(put(p.fixed + sl.r0 * p.ld, kFixed));
  if (p.ls) SV_TRY(upload_linear_source(srv, p, sl));
  moc::launch_batch_rebase(p.segs + sl.s0, S, p.fsr_mat, (int32_t) sl.r0,
                           p.seg_off + sl.t0, p.next + 2 * sl.t0,
                           p.track_ang + sl.t0, p.track_slot + sl.t0, T, sl.s0,
                           (int32_t) sl.t0, (int32_t) sl.a0, slot_index, st);
  // the linear-source words take the rebased FSR ids and materials
  if (p.ls) moc::launch_ls_refresh_ids(p.segs + sl.s0, p.segs_ls + sl.s0, S, st);
  // rows become visible to the row kernels only with their owner set, after
  // the data above in stream order
  fill_i32_kernel<<<small_grid(R), 256, 0, st>>>(p.row_slot + sl.r0, R,
                                                 slot_index);
  SV_CUDA(cudaGetLastError());
  add_launches(srv, 3);
  return MOC_OK;
}

// Starting state of an admitted solve (Solver::computeEigenvalue /
// computeSource before their loops, src/Solver.cpp:1459-1580): flat flux,
// normalised for an eigenvalue solve, stored as the old flux; zero boundary
// fluxes; keff 1 or the given one.
int init_slot(moc_server* srv, Pool& p, int slot_index) {
  Slot& sl = p.slots[slot_index];
  Staged& s = *sl.st;
  moc::SolverArgs a = pool_solver_args(p);
  moc::launch_batch_init_rows(a, sl.r0, s.R, (float) s.init_flux, p.stream);
  SV_CUDA(cudaGetLastError());
  const size_t psi_bytes = sizeof(float) * (size_t) (s.T + 1) * 2 * p.F;
  for (int b = 0; b < 2; b++)
    SV_CUDA(cudaMemsetAsync(p.psi[b] + sl.t0 * 2 * p.F, 0, psi_bytes,
                            p.stream));
  moc::DevScalars& d = p.init_h[slot_index];
  std::memset(&d, 0, sizeof(d));
  const bool eigen = s.req.kind == MOC_SOLVE_EIGENVALUE;
  d.keff = eigen ? 1.0 : s.req.k_eff;
  d.k_prev = d.keff;
  d.factor = 1.0;
  d.threshold = s.req.threshold;
  d.scale[0] = d.scale[1] = 1.0f;
  d.max_iters = s.req.max_iters;
  d.mode = eigen ? moc::kModeEigen
                 : s.req.kind == MOC_SOLVE_FLUX ? moc::kModeFlux
                                                : moc::kModeSource;
  d.res_type = s.req.res_type;
  d.num_fissionable = s.num_fissionable;
  d.negative_ok = s.req.allow_negative_fluxes ? 1 : 0;
  d.row0 = sl.r0;
  d.nrows = s.R;
  SV_CUDA(cudaMemcpyAsync(p.slots_d + slot_index, &d, sizeof(d),
                          cudaMemcpyHostToDevice, p.stream));
  sl.needs_init = false;
  add_launches(srv, 1);
  return MOC_OK;
}

// Admits queued requests while a slot and every range fit.
int admit(moc_server* srv, Pool& p) {
  {
    std::lock_guard<std::mutex> lk(srv->mu);
    bool pool_empty = true;
    for (const Slot& sl : p.slots) pool_empty = pool_empty && !sl.live;
    for (auto it = p.queue.begin(); it != p.queue.end();) {
      Staged& s = **it;
      if (p.free_slots.empty()) break;
      // sources and tallies are gathered and scattered by FSR id in every
      // sweep: admit while the live solves' share of them fits the budget
      const int64_t hot = hot_bytes(s);
      if (srv->cfg.hot_bytes > 0 && !pool_empty &&
          srv->hot_live + hot > srv->cfg.hot_bytes) {
        ++it;
        continue;
      }
      const int64_t r0 = p.rows.alloc(s.R);
      const int64_t t0 = (r0 >= 0) ? p.tracks.alloc(s.T + 1) : -1;
      const int64_t s0 = (t0 >= 0) ? p.segments.alloc(s.S) : -1;
      const int64_t m0 = (s0 >= 0) ? p.mats.alloc(s.M) : -1;
      const int64_t a0 = (m0 >= 0) ? p.angles.alloc(s.A) : -1;
      if (a0 < 0) {
        if (r0 >= 0) p.rows.release(r0, s.R);
        if (t0 >= 0) p.tracks.release(t0, s.T + 1);
        if (s0 >= 0) p.segments.release(s0, s.S);
        if (m0 >= 0) p.mats.release(m0, s.M);
        ++it;
        continue;
      }
      const int idx = p.free_slots.back();
      p.free_slots.pop_back();
      Slot& sl = p.slots[idx];
      sl.r0 = r0;
      sl.t0 = t0;
      sl.s0 = s0;
      sl.m0 = m0;
      sl.a0 = a0;
      sl.live = true;
      sl.uploaded = false;
      sl.needs_init = true;
      s.t_admit = now_s();
      sl.st = std::move(*it);
      it = p.queue.erase(it);
      srv->hot_live += hot;
      pool_empty = false;
      srv->stats.admitted++;
      p.n_admitted++;
      srv->stats.queued--;
      srv->stats.live++;
      p.dirty = true;
    }
  }
  for (int i = 0; i < (int) p.slots.size(); i++) {
    Slot& sl = p.slots[i];
    if (!sl.live || sl.uploaded) continue;
    SV_TRY(upload_slot(srv, p, i));
    sl.uploaded = true;
  }
  return MOC_OK;
}

// Copies out and publishes every solve that the last block finished: all
// their flux rows are copied into the pinned buffer at their own row
// offsets, with one synchronisation.
int retire(moc_server* srv, Pool& p) {
  std::vector<int> done;
  for (int i = 0; i < (int) p.slots.size(); i++) {
    const Slot& sl = p.slots[i];
    if (sl.live && !sl.needs_init && p.slots_h[i].done) done.push_back(i);
  }
  if (done.empty()) return MOC_OK;
  for (int i : done) {
    const Slot& sl = p.slots[i];
    const int64_t R = sl.st->R;
    SV_CUDA(cudaMemcpyAsync(p.retire_h + sl.r0 * p.ld, p.phi + sl.r0 * p.ld,
                            sizeof(float) * R * p.ld, cudaMemcpyDeviceToHost,
                            p.stream));
    if (p.ls && sl.st->req.moments_out)
      SV_CUDA(cudaMemcpyAsync(p.retire_mom_h + 2 * sl.r0 * p.ld,
                              p.mom + 2 * sl.r0 * p.ld,
                              sizeof(float) * 2 * R * p.ld,
                              cudaMemcpyDeviceToHost, p.stream));
    // the rows leave the row kernels' view before they are reused
    SV_CUDA(cudaMemsetAsync(p.row_slot + sl.r0, 0xFF, sizeof(int32_t) * R,
                            p.stream));
  }
  SV_CUDA(cudaStreamSynchronize(p.stream));
  for (int i : done) {
    Slot& sl = p.slots[i];
    Staged& s = *sl.st;
    const moc::DevScalars& d = p.slots_h[i];
    const float* rows = p.retire_h + sl.r0 * p.ld;
    for (int64_t r = 0; r < s.R; r++)
      std::memcpy(s.req.flux_out + r * s.G, rows + r * p.ld,
                  sizeof(float) * s.G);
    if (p.ls && s.req.moments_out) {
      // [R][ld][2] (x, y adjacent) -> [R][3][G] with z = 0
      const float* m = p.retire_mom_h + 2 * sl.r0 * p.ld;
      float* out = s.req.moments_out;
      for (int64_t r = 0; r < s.R; r++)
        for (int g = 0; g < s.G; g++) {
          out[(r * 3 + 0) * s.G + g] = m[2 * (r * p.ld + g)];
          out[(r * 3 + 1) * s.G + g] = m[2 * (r * p.ld + g) + 1];
          out[(r * 3 + 2) * s.G + g] = 0.0f;
        }
    }
    moc_result res{};
    res.status = MOC_OK;
    res.converged = d.converged;
    res.iterations = (s.req.kind == MOC_SOLVE_EIGENVALUE)
                         ? d.iteration
                         : (d.converged ? d.iteration - 1 : s.req.max_iters);
    res.pool = p.index;
    res.keff = d.keff;
    res.residual = d.residual;
    res.t_submit = s.t_submit;
    res.t_admit = s.t_admit;
    res.t_done = now_s();
    p.rows.release(sl.r0, s.R);
    p.tracks.release(sl.t0, s.T + 1);
    p.segments.release(sl.s0, s.S);
    p.mats.release(sl.m0, s.M);
    p.angles.release(sl.a0, s.A);
    srv->hot_live -= hot_bytes(s);
    sl.live = false;
    {
      std::lock_guard<std::mutex> lk(srv->mu);
      p.n_completed++;
    }
    publish(srv, s, res);
    sl.st.reset();
    p.free_slots.push_back(i);
    p.dirty = true;
  }
  return MOC_OK;
}

}  // namespace

namespace {

// Track list of every live solve, longest tracks first, and the extents of
// the rows and materials in use.
int rebuild_order(Pool& p) {
  std::vector<std::pair<int32_t, int32_t>> keyed;  // (-segments, track)
  int64_t rows_hi = 0, mats_hi = 0;
  for (const Slot& sl : p.slots) {
    if (!sl.live) continue;
    const Staged& s = *sl.st;
    for (int64_t t = 0; t < s.T; t++)
      keyed.emplace_back(-s.nseg[t], (int32_t) (sl.t0 + t));
    rows_hi = std::max(rows_hi, sl.r0 + s.R);
    mats_hi = std::max(mats_hi, sl.m0 + s.M);
  }
  std::sort(keyed.begin(), keyed.end());
  std::vector<int32_t> order(keyed.size());
  for (size_t i = 0; i < keyed.size(); i++) order[i] = keyed[i].second;
  if (!order.empty())
    SV_CUDA(cudaMemcpyAsync(p.order, order.data(),
                            sizeof(int32_t) * order.size(),
                            cudaMemcpyHostToDevice, p.stream));
  p.active_tracks = (int64_t) order.size();
  p.rows_hi = rows_hi;
  p.mats_hi = mats_hi;
  p.dirty = false;
  if (p.graph) {
    cudaGraphExecDestroy(p.graph);
    p.graph = nullptr;
  }
  return MOC_OK;
}


// The pool's sweep (flat or linear source) with the given shape.
bool pool_sweep(Pool& p, const moc::SweepArgs& a, int pairs) {
  if (p.ls) return moc::launch_ls_sweep(a, p.Ph, pairs, p.stream);
  return moc::launch_sweep(a, p.Ph, pairs, MOC_EXP_INTRINSIC, p.stream);
}

// Times every sweep shape with at most kMaxSlots pairs per lane (5 with a
// linear source) and at
// least half of its lanes busy on the pool's current solves (the faster of
// two sweeps after a warm-up) and keeps the fastest.  The timing sweeps read
// the live tracks and sources but write tallies, angular fluxes, the buffer
// index and the solves' scales into scratch copies, so the live state is
// untouched and a pool can be retuned whenever its track count changes
// scale.  Pools sweep with the hardware-ex2 evaluator, the faster one on
// every workload measured.
int autotune_pool(moc_server* srv, Pool& p) {
  if (p.tune_ev.empty()) {
    p.tune_ev.resize(2);
    for (auto& e : p.tune_ev) SV_CUDA(cudaEventCreate(&e));
  }
  const int N = p.cfg.max_solves;
  if (!p.tune_psi) {
    const int64_t npsi = p.cfg.max_tracks * 2 * p.F;
    SV_TRY(dev_alloc(&p.tune_psi, npsi));
    SV_TRY(dev_alloc(&p.tune_phi, p.cfg.max_fsrs * p.ld));
    if (p.ls) SV_TRY(dev_alloc(&p.tune_mom, 2 * p.cfg.max_fsrs * p.ld));
    SV_TRY(dev_alloc(&p.tune_sc, 1));
    SV_TRY(dev_alloc(&p.tune_slots, N));
    SV_CUDA(cudaMemsetAsync(p.tune_psi, 0, sizeof(float) * npsi, p.stream));
  }
  SV_CUDA(cudaMemcpyAsync(p.tune_sc, p.sc, sizeof(moc::DevScalars),
                          cudaMemcpyDeviceToDevice, p.stream));
  SV_CUDA(cudaMemcpyAsync(p.tune_slots, p.slots_d, sizeof(moc::DevScalars) * N,
                          cudaMemcpyDeviceToDevice, p.stream));
  float best_ms = 1e30f;
  int best_lps = 0, best_pairs = 0;
  const int max_pairs = p.ls ? kLsMaxPairs : moc::kMaxSlots;
  for (int lps = 1; lps <= 32; lps *= 2) {
    const int pairs = pairs_for(p.G, lps);
    if (pairs > max_pairs || (double) p.G / (2.0 * lps * pairs) < 0.5)
      continue;
    p.lps = lps;
    moc::SweepArgs a = pool_sweep_args(p);
    a.phi = p.tune_phi;
    if (p.ls) a.mom = p.tune_mom;
    a.psi[0] = a.psi[1] = p.tune_psi;
    a.sc = p.tune_sc;
    a.slots = p.tune_slots;
    float best = 1e30f;
    for (int r = 0; r < 3; r++) {
      SV_CUDA(cudaEventRecord(p.tune_ev[0], p.stream));
      if (!pool_sweep(p, a, pairs))
        return SV_FAIL(MOC_ERR_UNSUPPORTED, "no sweep kernel for the pool");
      SV_CUDA(cudaEventRecord(p.tune_ev[1], p.stream));
      SV_CUDA(cudaEventSynchronize(p.tune_ev[1]));
      float t = 0.f;
      SV_CUDA(cudaEventElapsedTime(&t, p.tune_ev[0], p.tune_ev[1]));
      if (r > 0) best = std::min(best, t);
    }
    add_launches(srv, 3);
    if (best < best_ms) {
      best_ms = best;
      best_lps = lps;
      best_pairs = pairs;
    }
  }
  SV_CHECK(best_lps > 0, MOC_ERR_UNSUPPORTED, "no sweep kernel shape fits");
  p.lps = best_lps;
  p.pairs = best_pairs;
  p.exp_kind = MOC_EXP_INTRINSIC;
  std::lock_guard<std::mutex> lk(srv->mu);
  p.n_tunes++;
  return MOC_OK;
}

// Sweep shape for the pool's current track count: fixed by the pool's
// configuration, or the autotuned one of its size class (a power of two of
// live tracks), tuning that class on first use.
int choose_shape(moc_server* srv, Pool& p) {
  if (p.cfg.lanes != 0) return MOC_OK;
  int cls = 0;
  for (int64_t t = std::max<int64_t>(p.active_tracks, 1); t > 1; t >>= 1) cls++;
  auto it = p.shape_by_class.find(cls);
  int lps, pairs;
  if (it == p.shape_by_class.end()) {
    SV_TRY(autotune_pool(srv, p));
    lps = p.lps;
    pairs = p.pairs;
    p.shape_by_class[cls] = std::make_pair(lps, pairs);
  } else {
    lps = it->second.first;
    pairs = it->second.second;
  }
  if (lps != p.graph_lps || pairs != p.graph_pairs) {
    if (p.graph) cudaGraphExecDestroy(p.graph);
    p.graph = nullptr;
  }
  p.lps = lps;
  p.pairs = pairs;
  return MOC_OK;
}

// One source iteration of every live solve of the pool: six launches.
int enqueue_iteration(Pool& p) {
  moc::SolverArgs a = pool_solver_args(p);
  moc::SweepArgs w = pool_sweep_args(p);
  if (p.ls)
    moc::launch_ls_sources(a, 0, 1, p.stream);
  else
    moc::launch_batch_sources(a, p.stream);
  if (!pool_sweep(p, w, p.pairs))
    return SV_FAIL(MOC_ERR_UNSUPPORTED, "no sweep kernel for the pool");
  if (p.ls)
    moc::launch_ls_add_source(a, 0, p.stream);
  else
    moc::launch_batch_add_source(a, p.stream);
  moc::launch_batch_rate_finish(a, p.stream);
  moc::launch_batch_residual(a, p.stream);
  moc::launch_batch_residual_finish(a, p.stream);
  SV_CUDA(cudaGetLastError());
  return MOC_OK;
}

// Starts the next block of iterations of a pool and the read-back of its
// solves' states.
int launch_block(moc_server* srv, Pool& p) {
  bool any = false;
  for (const Slot& sl : p.slots) any = any || sl.live;
  if (!any) return MOC_OK;
  if (p.dirty) SV_TRY(rebuild_order(p));
  for (int i = 0; i < (int) p.slots.size(); i++)
    if (p.slots[i].live && p.slots[i].needs_init) SV_TRY(init_slot(srv, p, i));
  SV_TRY(choose_shape(srv, p));
  const int K = std::max(1, srv->cfg.iterations_per_poll);
  if (srv->cfg.use_graphs) {
    if (!p.graph || p.graph_iters != K) {
      const double t_cap = now_s();
      if (p.graph) cudaGraphExecDestroy(p.graph);
      p.graph = nullptr;
      cudaGraph_t g = nullptr;
      SV_CUDA(cudaStreamBeginCapture(p.stream, cudaStreamCaptureModeRelaxed));
      int st = MOC_OK;
      for (int k = 0; k < K && st == MOC_OK; k++) st = enqueue_iteration(p);
      cudaError_t e = cudaStreamEndCapture(p.stream, &g);
      SV_TRY(st);
      SV_CUDA(e);
      e = cudaGraphInstantiate(&p.graph, g, 0);
      cudaGraphDestroy(g);
      SV_CUDA(e);
      p.graph_iters = K;
      p.graph_lps = p.lps;
      p.graph_pairs = p.pairs;
      std::lock_guard<std::mutex> lk(srv->mu);
      srv->stats.graph_captures++;
      srv->stats.host_graph_s += now_s() - t_cap;
    }
    SV_CUDA(cudaEventRecord(p.block_start, p.stream));
    SV_CUDA(cudaGraphLaunch(p.graph, p.stream));
  } else {
    SV_CUDA(cudaEventRecord(p.block_start, p.stream));
    for (int k = 0; k < K; k++) SV_TRY(enqueue_iteration(p));
  }
  SV_CUDA(cudaMemcpyAsync(p.slots_h, p.slots_d,
                          sizeof(moc::DevScalars) * p.cfg.max_solves,
                          cudaMemcpyDeviceToHost, p.stream));
  SV_CUDA(cudaEventRecord(p.block_done, p.stream));
  p.in_flight = true;
  {
    std::lock_guard<std::mutex> lk(srv->mu);
    srv->stats.blocks++;
    p.n_blocks++;
    srv->stats.kernel_launches += 6 * K;
  }
  return MOC_OK;
}

// Fails every live and queued request of a pool after an error in the loop.
void fail_pool(moc_server* srv, Pool& p, int status) {
  std::vector<std::unique_ptr<Staged>> dead;
  for (Slot& sl : p.slots)
    if (sl.live) {
      srv->hot_live -= hot_bytes(*sl.st);
      dead.push_back(std::move(sl.st));
      sl.live = false;
    }
  {
    std::lock_guard<std::mutex> lk(srv->mu);
    for (auto& q : p.queue) {
      dead.push_back(std::move(q));
      srv->stats.queued--;
      srv->stats.live++;
    }
    p.queue.clear();
  }
  for (auto& s : dead) {
    moc_result r{};
    r.status = status;
    r.pool = p.index;
    r.t_submit = s->t_submit;
    r.t_admit = s->t_admit;
    r.t_done = now_s();
    publish(srv, *s, r);
  }
}

// One pass over a pool; with wait, blocks on its running block.  Returns
// the number of live and queued solves, or a negative status.
int service(moc_server* srv, Pool& p, bool wait, bool* progressed) {
  if (p.in_flight) {
    if (wait) {
      SV_CUDA(cudaEventSynchronize(p.block_done));
    } else {
      cudaError_t e = cudaEventQuery(p.block_done);
      if (e == cudaErrorNotReady) return MOC_OK;
      SV_CUDA(e);
    }
    p.in_flight = false;
    // the copies of the solves admitted before this block have run
    for (Slot& sl : p.slots)
      if (sl.live && sl.uploaded) sl.st->release_pin();
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, p.block_start, p.block_done) == cudaSuccess) {
      std::lock_guard<std::mutex> lk(srv->mu);
      srv->stats.gpu_busy_s += 1e-3 * ms;
      p.busy_s += 1e-3 * ms;
    }
    const double t_ret = now_s();
    SV_TRY(retire(srv, p));
    {
      std::lock_guard<std::mutex> lk(srv->mu);
      srv->stats.host_retire_s += now_s() - t_ret;
    }
    *progressed = true;
  }
  const double t_adm = now_s();
  SV_TRY(admit(srv, p));
  {
    std::lock_guard<std::mutex> lk(srv->mu);
    srv->stats.host_admit_s += now_s() - t_adm;
  }
  const bool had = p.in_flight;
  SV_TRY(launch_block(srv, p));
  if (p.in_flight && !had) *progressed = true;
  return MOC_OK;
}

int step_all(moc_server* srv, bool wait, bool* progressed) {
  for (auto& pp : srv->pools) {
    Pool& p = *pp;
    cudaSetDevice(srv->cfg.device);
    int st = service(srv, p, wait, progressed);
    if (st != MOC_OK) {
      const char* msg = moc_last_error();
      {
        std::lock_guard<std::mutex> lk(srv->mu);
        srv->loop_error = msg ? msg : "";
      }
      cudaStreamSynchronize(p.stream);
      p.in_flight = false;
      fail_pool(srv, p, st);
    }
  }
  return MOC_OK;
}

int64_t pending(moc_server* srv) {
  std::lock_guard<std::mutex> lk(srv->mu);
  return srv->stats.live + srv->stats.queued;
}

}  // namespace

extern "C" {

int moc_server_create(const moc_server_config* cfg, moc_server** out) {
  SV_CHECK(cfg && out, MOC_ERR_ARG, "null argument");
  *out = nullptr;
  SV_CHECK(cfg->iterations_per_poll >= 1 && cfg->iterations_per_poll <= 1024,
           MOC_ERR_ARG, "iterations_per_poll must be in [1, 1024]");
  int ndev = 0;
  SV_CUDA(cudaGetDeviceCount(&ndev));
  SV_CHECK(cfg->device >= 0 && cfg->device < ndev, MOC_ERR_ARG,
           "no CUDA device " + std::to_string(cfg->device));
  SV_CUDA(cudaSetDevice(cfg->device));
  moc::configure_kernels();   // before any launch is captured into a graph
  moc_server* srv = new moc_server();
  srv->cfg = *cfg;
  // nodes of the attenuation table, as in moc_create
  const int n = moc::kExpTableSize;
  srv->exp_table_h.resize(2 * n);
  for (int i = 0; i < n; i++) {
    const double x = (double) i * (double) moc::kExpTableH;
    srv->exp_table_h[i] = (float) (-std::expm1(-x));
    srv->exp_table_h[n + i] = (float) std::exp(-x);
  }
  *out = srv;
  return MOC_OK;
}

int moc_server_destroy(moc_server* srv) {
  if (!srv) return MOC_OK;
  moc_server_stop(srv);
  cudaSetDevice(srv->cfg.device);
  for (auto& p : srv->pools) destroy_pool(*p);
  delete srv;
  return MOC_OK;
}

int moc_server_add_pool(moc_server* srv, const moc_pool_config* cfg,
                        int* pool) {
  SV_CHECK(srv && cfg, MOC_ERR_ARG, "null argument");
  SV_CHECK(!srv->running.load(), MOC_ERR_STATE,
           "add pools before starting the loop");
  for (auto& p : srv->pools)
    SV_CHECK(p->G != cfg->num_groups || p->Ph != cfg->num_polar_half ||
                 p->ls != (cfg->linear_source != 0),
             MOC_ERR_ARG,
             "a pool for this group count, polar count and source kind "
             "exists");
  SV_CUDA(cudaSetDevice(srv->cfg.device));
  std::unique_ptr<Pool> p(new Pool());
  p->index = (int) srv->pools.size();
  int st = create_pool(srv, *cfg, *p);
  if (st != MOC_OK) {
    std::string msg = moc_last_error();
    destroy_pool(*p);
    return SV_FAIL(st, msg);
  }
  if (pool) *pool = p->index;
  srv->pools.push_back(std::move(p));
  return MOC_OK;
}

int moc_server_submit(moc_server* srv, const moc_request* req,
                      int64_t* ticket) {
  SV_CHECK(srv && req, MOC_ERR_ARG, "null argument");
  Pool* target = nullptr;
  const bool ls = req->linear_source != nullptr;
  for (auto& p : srv->pools)
    if (p->G == req->num_groups && p->Ph == req->num_polar_half && p->ls == ls)
      target = p.get();
  SV_CHECK(target, MOC_ERR_UNSUPPORTED,
           "no " + std::string(ls ? "linear-source" : "flat-source") +
               " pool for " + std::to_string(req->num_groups) +
               " groups and " + std::to_string(req->num_polar_half) +
               " polar angles");
  std::unique_ptr<Staged> s(new Staged());
  SV_TRY(stage_request(*req, *s));
  const moc_pool_config& c = target->cfg;
  SV_CHECK(s->R <= c.max_fsrs && s->T + 1 <= c.max_tracks &&
               s->S <= c.max_segments && s->M <= c.max_materials &&
               s->A <= c.max_angles,
           MOC_ERR_MEMORY, "request exceeds its pool's capacity");
  SV_TRY(pin_request(srv->pinned, *s));
  s->pool = target->index;
  s->t_submit = now_s();
  std::lock_guard<std::mutex> lk(srv->mu);
  s->ticket = srv->next_ticket++;
  if (ticket) *ticket = s->ticket;
  srv->stats.submitted++;
  srv->stats.queued++;
  target->queue.push_back(std::move(s));
  srv->cv.notify_all();
  return MOC_OK;
}

int moc_server_step(moc_server* srv, int64_t* pend) {
  SV_CHECK(srv, MOC_ERR_ARG, "null server");
  SV_CHECK(!srv->running.load(), MOC_ERR_STATE,
           "the loop thread is running");
  bool progressed = false;
  SV_TRY(step_all(srv, true, &progressed));
  if (pend) *pend = pending(srv);
  return MOC_OK;
}

int moc_server_start(moc_server* srv) {
  SV_CHECK(srv, MOC_ERR_ARG, "null server");
  SV_CHECK(!srv->running.load(), MOC_ERR_STATE, "already running");
  srv->running.store(true);
  srv->loop = std::thread([srv]() {
    cudaSetDevice(srv->cfg.device);
    while (srv->running.load()) {
      bool progressed = false;
      step_all(srv, false, &progressed);
      if (!progressed) {
        // nothing finished and nothing new: wait briefly for a submission
        // or for the device
        std::unique_lock<std::mutex> lk(srv->mu);
        if (srv->stats.live == 0 && srv->running.load())
          srv->cv.wait_for(lk, std::chrono::milliseconds(2));
        else
          std::this_thread::yield();
      }
    }
  });
  return MOC_OK;
}

int moc_server_stop(moc_server* srv) {
  SV_CHECK(srv, MOC_ERR_ARG, "null server");
  if (!srv->running.load()) return MOC_OK;
  srv->running.store(false);
  srv->cv.notify_all();
  if (srv->loop.joinable()) srv->loop.join();
  // finish the blocks in flight so that the server can be stepped or
  // destroyed
  for (auto& p : srv->pools)
    if (p->stream) cudaStreamSynchronize(p->stream);
  return MOC_OK;
}

int moc_server_wait(moc_server* srv, int64_t ticket, double timeout_s,
                    moc_result* out) {
  SV_CHECK(srv && out, MOC_ERR_ARG, "null argument");
  std::unique_lock<std::mutex> lk(srv->mu);
  SV_CHECK(ticket >= 1 && ticket < srv->next_ticket, MOC_ERR_ARG,
           "unknown ticket");
  auto ready = [&] { return srv->results.count(ticket) > 0; };
  if (timeout_s < 0) {
    srv->cv.wait(lk, ready);
  } else if (!srv->cv.wait_for(lk, std::chrono::duration<double>(timeout_s),
                               ready)) {
    lk.unlock();
    return SV_FAIL(MOC_ERR_TIMEOUT, "request not completed");
  }
  *out = srv->results[ticket];
  return MOC_OK;
}

int moc_server_poll(moc_server* srv, int64_t* tickets, int capacity,
                    int* count) {
  SV_CHECK(srv && count && (capacity == 0 || tickets), MOC_ERR_ARG,
           "null argument");
  std::lock_guard<std::mutex> lk(srv->mu);
  const int n = std::min<int>(capacity, (int) srv->completed.size());
  for (int i = 0; i < n; i++) tickets[i] = srv->completed[i];
  srv->completed.erase(srv->completed.begin(), srv->completed.begin() + n);
  *count = n;
  return MOC_OK;
}

int moc_server_pool_stats(moc_server* srv, int pool, moc_pool_stats* out) {
  SV_CHECK(srv && out, MOC_ERR_ARG, "null argument");
  SV_CHECK(pool >= 0 && pool < (int) srv->pools.size(), MOC_ERR_ARG,
           "no pool " + std::to_string(pool));
  std::lock_guard<std::mutex> lk(srv->mu);
  const Pool& p = *srv->pools[pool];
  out->num_groups = p.G;
  out->num_polar_half = p.Ph;
  out->lanes = p.lps;
  out->pairs = p.pairs;
  out->exp_kind = p.exp_kind;
  out->live = 0;
  for (const Slot& sl : p.slots) out->live += sl.live ? 1 : 0;
  out->admitted = p.n_admitted;
  out->completed = p.n_completed;
  out->blocks = p.n_blocks;
  out->tunes = p.n_tunes;
  out->gpu_busy_s = p.busy_s;
  return MOC_OK;
}

int moc_server_stats_get(moc_server* srv, moc_server_stats* out) {
  SV_CHECK(srv && out, MOC_ERR_ARG, "null argument");
  std::lock_guard<std::mutex> lk(srv->mu);
  *out = srv->stats;
  return MOC_OK;
}

const char* moc_server_loop_error(moc_server* srv) {
  thread_local std::string copy;
  if (!srv) return "";
  std::lock_guard<std::mutex> lk(srv->mu);
  copy = srv->loop_error;
  return copy.c_str();
}

}  // extern "C"
