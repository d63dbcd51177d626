// Ray tracing of pin-cell lattices on the GPU: the segmentation step of
// moc_lattice_generate (lattice.cpp) -- OpenMOC's Geometry::segmentize2D for
// this geometry family (src/Geometry.cpp:2085-2230) -- one thread per track,
// with FSR ids by first touch over tracks in UID order and FSR volumes
// (VolumeKernel, src/MOCKernel.cpp:86-170).  The laydown (angles, tracks,
// links) stays on the host: it is O(tracks).
//
// The arithmetic is the host generator's, operation for operation, with no
// contraction into FMA (this file and lattice.cpp are compiled without it),
// so segment lengths and FSR ids come out bit for bit as on the host; the
// track directions and sector-line directions are computed once on the host
// and passed in.  Lattice-line crossings along a track are two monotone
// sequences, merged in order instead of sorted; the crossings inside a pin
// cell are sorted by insertion.  Volumes are summed with FP64 atomics, so
// their order (and possibly the last bit of a float volume) differs from the
// host's sequential sum.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include <cuda_runtime.h>

#include "lattice_internal.h"

namespace {

using moc_lat::kPi;
using moc_lat::kTinyMove;

constexpr int kMaxRings = 16;
constexpr int kMaxLines = 64;
constexpr int kMaxPts = 2 * kMaxRings + kMaxLines + 2;
constexpr int kMaxRingsMax = 16;

struct GpuLattice {
  int nx, ny;
  double pitch, xmin, ymin;
  int rings, fuel_sectors, mod_sectors, nlines, sec;   // sec: max sectors
  double r2[kMaxRings];
  double radii[kMaxRings];
  double vx[kMaxLines], vy[kMaxLines];
};

struct GpuTrack {
  double x0, y0, ux, uy, len;
};

__device__ int dev_sector_of(double ang, int n) {
  if (n <= 1) return 0;
  const double d = 2.0 * kPi / n;
  double x = ang + kPi / 4.0;
  x = fmod(x, 2.0 * kPi);
  if (x < 0) x += 2.0 * kPi;
  int s = (int) floor(x / d);
  if (s >= n) s = n - 1;
  return s;
}

__device__ uint32_t dev_classify(const GpuLattice& g, double dx, double dy) {
  const double rr = dx * dx + dy * dy;
  int ring = g.rings;
  if (rr < g.r2[0]) {
    ring = 0;
    for (int k = 1; k < g.rings; k++)
      if (rr < g.r2[k]) ring = k;
  }
  const double ang = atan2(dy, dx);
  const int sec = dev_sector_of(ang, ring < g.rings ? g.fuel_sectors
                                                    : g.mod_sectors);
  return (uint32_t) ring << 16 | (uint32_t) sec;
}

// The next lattice-line crossing of a track along one axis: crossings at
// (lo + k * pitch - p0) / u for k = 1 .. n - 1, visited in increasing order
// of the parameter (k up when u > 0, down when u < 0).
struct AxisCrossings {
  int k, step, end;
  double lo, p0, u;
  __device__ void init(int n, double lo_, double pitch, double p0_, double u_) {
    lo = lo_;
    p0 = p0_;
    u = u_;
    if (fabs(u) < 1e-300 || n < 2) {
      k = end = 0;
      step = 1;
    } else if (u > 0) {
      k = 1;
      end = n;
      step = 1;
    } else {
      k = n - 1;
      end = 0;
      step = -1;
    }
    (void) pitch;
  }
  __device__ bool has() const { return k != end; }
  __device__ double value(double pitch) const {
    return (lo + k * pitch - p0) / u;
  }
};

// Walks one track: calls emit(len, key) for every merged segment in order.
template <typename Emit>
__device__ void trace_track(const GpuLattice& g, const GpuTrack& tr,
                            Emit emit) {
  AxisCrossings xa, ya;
  xa.init(g.nx, g.xmin, g.pitch, tr.x0, tr.ux);
  ya.init(g.ny, g.ymin, g.pitch, tr.y0, tr.uy);
  auto next_cut = [&](double& t) -> bool {
    // the smallest remaining crossing in (0, len), or len at the end
    for (;;) {
      const bool hx = xa.has(), hy = ya.has();
      if (!hx && !hy) return false;
      double tx = hx ? xa.value(g.pitch) : 0.0;
      double ty = hy ? ya.value(g.pitch) : 0.0;
      bool take_x = hx && (!hy || tx <= ty);
      double tt = take_x ? tx : ty;
      if (take_x)
        xa.k += xa.step;
      else
        ya.k += ya.step;
      if (tt > 0 && tt < tr.len) {
        t = tt;
        return true;
      }
    }
  };
  double pts[kMaxPts];
  bool have_prev = false;
  uint64_t prev_key = 0;
  double ta = 0.0;
  bool more = true;
  while (more) {
    double tb;
    if (!next_cut(tb)) {
      tb = tr.len;
      more = false;
    }
    if (tb - ta > 0) {
      const double tm = 0.5 * (ta + tb);
      const double mx = tr.x0 + tm * tr.ux, my = tr.y0 + tm * tr.uy;
      int ci = (int) floor((mx - g.xmin) / g.pitch);
      int cj = (int) floor((my - g.ymin) / g.pitch);
      ci = min(max(ci, 0), g.nx - 1);
      cj = min(max(cj, 0), g.ny - 1);
      const double cx = g.xmin + (ci + 0.5) * g.pitch;
      const double cy = g.ymin + (cj + 0.5) * g.pitch;
      int np = 0;
      pts[np++] = ta;
      const double px = tr.x0 - cx, py = tr.y0 - cy;
      const double b = px * tr.ux + py * tr.uy;
      const double pp = px * px + py * py;
      for (int i = 0; i < g.rings; i++) {
        const double r = g.radii[i];
        const double disc = b * b - (pp - r * r);
        if (disc <= 0) continue;
        const double sq = sqrt(disc);
        const double t1 = -b - sq, t2 = -b + sq;
        if (t1 > ta && t1 < tb) pts[np++] = t1;
        if (t2 > ta && t2 < tb) pts[np++] = t2;
      }
      for (int i = 0; i < g.nlines; i++) {
        const double vx = g.vx[i], vy = g.vy[i];
        const double den = tr.ux * vy - tr.uy * vx;
        if (fabs(den) < 1e-14) continue;
        const double qx = cx - tr.x0, qy = cy - tr.y0;
        const double tt = (qx * vy - qy * vx) / den;
        const double ss = (qx * tr.uy - qy * tr.ux) / den;
        if (ss > -1e-12 && tt > ta && tt < tb) pts[np++] = tt;
      }
      pts[np++] = tb;
      for (int i = 1; i < np; i++) {   // insertion sort
        const double v = pts[i];
        int j = i - 1;
        while (j >= 0 && pts[j] > v) {
          pts[j + 1] = pts[j];
          j--;
        }
        pts[j + 1] = v;
      }
      const uint64_t cell = (uint64_t) ((int64_t) (g.ny - 1 - cj) * g.nx + ci);
      for (int k = 0; k + 1 < np; k++) {
        const double l = pts[k + 1] - pts[k];
        if (l <= kTinyMove) continue;
        const double mm = 0.5 * (pts[k] + pts[k + 1]);
        const uint32_t rs = dev_classify(g, tr.x0 + mm * tr.ux - cx,
                                         tr.y0 + mm * tr.uy - cy);
        const uint64_t key = cell << 32 | rs;
        emit(l, key, have_prev && prev_key == key);
        have_prev = true;
        prev_key = key;
      }
    }
    ta = tb;
  }
}

__global__ void count_kernel(GpuLattice g, const GpuTrack* tracks, int64_t T,
                             int64_t* count) {
  for (int64_t t = (int64_t) blockIdx.x * blockDim.x + threadIdx.x; t < T;
       t += (int64_t) gridDim.x * blockDim.x) {
    int64_t n = 0;
    trace_track(g, tracks[t], [&](double, uint64_t, bool merge) {
      if (!merge) n++;
    });
    count[t] = n;
  }
}

__device__ __forceinline__ int64_t dense_key(const GpuLattice& g,
                                             uint64_t key) {
  const int64_t cell = (int64_t) (key >> 32);
  const int ring = (int) ((key >> 16) & 0xFFFF);
  const int sec = (int) (key & 0xFFFF);
  return (cell * (g.rings + 1) + ring) * g.sec + sec;
}

__global__ void fill_kernel(GpuLattice g, const GpuTrack* tracks, int64_t T,
                            const int64_t* seg_off, float* seg_len,
                            int32_t* seg_dense,
                            unsigned long long* first_touch) {
  for (int64_t t = (int64_t) blockIdx.x * blockDim.x + threadIdx.x; t < T;
       t += (int64_t) gridDim.x * blockDim.x) {
    int64_t i = seg_off[t] - 1;
    trace_track(g, tracks[t], [&](double l, uint64_t key, bool merge) {
      if (merge) {
        seg_len[i] = (float) ((double) seg_len[i] + l);
      } else {
        i++;
        seg_len[i] = (float) l;
        const int64_t d = dense_key(g, key);
        seg_dense[i] = (int32_t) d;
        // the first touch only decreases: skip the atomic once a smaller
        // index is already recorded (most segments, after the first tracks)
        if (*(volatile unsigned long long*) (first_touch + d) >
            (unsigned long long) i)
          atomicMin(first_touch + d, (unsigned long long) i);
      }
    });
  }
}

__global__ void finish_kernel(const int32_t* seg_dense, const int32_t* table,
                              const float* seg_len, const int32_t* seg_track,
                              const double* wgt, int64_t S, int32_t* seg_fsr,
                              double* vol) {
  for (int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x; i < S;
       i += (int64_t) gridDim.x * blockDim.x) {
    const int32_t r = table[seg_dense[i]];
    seg_fsr[i] = r;
    atomicAdd(vol + r, wgt[seg_track[i]] * (double) seg_len[i]);
  }
}

__global__ void seg_track_kernel(const int64_t* seg_off, int64_t T,
                                 int32_t* seg_track) {
  for (int64_t t = (int64_t) blockIdx.x * blockDim.x + threadIdx.x; t < T;
       t += (int64_t) gridDim.x * blockDim.x)
    for (int64_t k = seg_off[t]; k < seg_off[t + 1]; k++)
      seg_track[k] = (int32_t) t;
}

unsigned grid(int64_t n, int threads) {
  int64_t b = (n + threads - 1) / threads;
  if (b < 1) b = 1;
  if (b > 152 * 32) b = 152 * 32;
  return (unsigned) b;
}

// RAII for the device buffers of one generation
struct DevBuf {
  std::vector<void*> ptrs;
  ~DevBuf() {
    for (void* p : ptrs) cudaFree(p);
  }
  template <typename T>
  cudaError_t alloc(T** p, size_t n) {
    cudaError_t e = cudaMalloc((void**) p, sizeof(T) * (n > 0 ? n : 1));
    if (e == cudaSuccess) ptrs.push_back(*p);
    return e;
  }
};

}  // namespace

using namespace moc_lat;

extern "C" int moc_lattice_generate_device(const moc_lattice_spec* sp,
                                           int32_t device,
                                           moc_lattice** out) {
  if (!sp || !out) return lat_fail("null argument");
  *out = nullptr;
  const moc_lattice_spec& s = *sp;
  if (lat_validate(s)) return -1;
  LatCells cells;
  lat_cells(s, cells);
  if (cells.rings > kMaxRingsMax || (int) cells.line_dirs.size() > kMaxLines)
    return lat_fail("the device ray tracer takes at most 16 rings and 64 "
                    "sector lines per pin cell");
  GpuLattice g{};
  g.nx = s.nx;
  g.ny = s.ny;
  g.pitch = s.pitch;
  g.rings = cells.rings;
  g.fuel_sectors = cells.fuel_sectors;
  g.mod_sectors = cells.mod_sectors;
  g.sec = std::max(1, std::max(cells.fuel_sectors, cells.mod_sectors));
  g.nlines = (int) cells.line_dirs.size();
  for (int i = 0; i < cells.rings; i++) {
    g.r2[i] = cells.r2[i];
    g.radii[i] = cells.radii[i];
  }
  for (int i = 0; i < g.nlines; i++) {
    g.vx[i] = std::cos(cells.line_dirs[i]);
    g.vy[i] = std::sin(cells.line_dirs[i]);
  }
  moc_lattice* L = new moc_lattice();
  LatGeo X;
  lat_laydown(s, L, X);
  g.xmin = X.xmin;
  g.ymin = X.ymin;
  const int64_t T = X.T;
  std::vector<GpuTrack> ht(T);
  std::vector<double> hw(T);
  for (int64_t t = 0; t < T; t++) {
    const Track& tr = X.tracks[t];
    ht[t].x0 = tr.x0;
    ht[t].y0 = tr.y0;
    ht[t].ux = std::cos(tr.phi);
    ht[t].uy = std::sin(tr.phi);
    ht[t].len = std::sqrt((tr.x1 - tr.x0) * (tr.x1 - tr.x0) +
                          (tr.y1 - tr.y0) * (tr.y1 - tr.y0));
    hw[t] = X.spac[tr.a] * X.wa[tr.a];
  }
  const int64_t K = (int64_t) s.nx * s.ny * (g.rings + 1) * g.sec;
  auto fail_cuda = [&](cudaError_t e) {
    delete L;
    return lat_fail(std::string("device ray tracing: ") + cudaGetErrorString(e));
  };
  cudaError_t e = cudaSetDevice(device);
  if (e != cudaSuccess) return fail_cuda(e);
  DevBuf buf;
  GpuTrack* d_tracks = nullptr;
  int64_t* d_count = nullptr;
  unsigned long long* d_first = nullptr;
  if ((e = buf.alloc(&d_tracks, T)) != cudaSuccess ||
      (e = buf.alloc(&d_count, T + 1)) != cudaSuccess ||
      (e = buf.alloc(&d_first, K)) != cudaSuccess)
    return fail_cuda(e);
  e = cudaMemcpy(d_tracks, ht.data(), sizeof(GpuTrack) * T,
                 cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemset(d_first, 0xFF, sizeof(uint64_t) * K);
  if (e != cudaSuccess) return fail_cuda(e);
  count_kernel<<<grid(T, 128), 128>>>(g, d_tracks, T, d_count);
  std::vector<int64_t> off(T + 1, 0);
  e = cudaMemcpy(off.data() + 1, d_count, sizeof(int64_t) * T,
                 cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return fail_cuda(e);
  for (int64_t t = 0; t < T; t++) off[t + 1] += off[t];
  const int64_t S = off[T];
  if (S >= (1LL << 31)) {
    delete L;
    return lat_fail("more than 2^31 segments");
  }
  int64_t* d_off = nullptr;
  float* d_len = nullptr;
  int32_t* d_dense = nullptr;
  int32_t* d_fsr = nullptr;
  int32_t* d_seg_track = nullptr;
  double* d_w = nullptr;
  if ((e = buf.alloc(&d_off, T + 1)) != cudaSuccess ||
      (e = buf.alloc(&d_len, S)) != cudaSuccess ||
      (e = buf.alloc(&d_dense, S)) != cudaSuccess ||
      (e = buf.alloc(&d_fsr, S)) != cudaSuccess ||
      (e = buf.alloc(&d_seg_track, S)) != cudaSuccess ||
      (e = buf.alloc(&d_w, T)) != cudaSuccess)
    return fail_cuda(e);
  e = cudaMemcpy(d_off, off.data(), sizeof(int64_t) * (T + 1),
                 cudaMemcpyHostToDevice);
  if (e == cudaSuccess)
    e = cudaMemcpy(d_w, hw.data(), sizeof(double) * T, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return fail_cuda(e);
  fill_kernel<<<grid(T, 128), 128>>>(g, d_tracks, T, d_off, d_len, d_dense,
                                     d_first);
  seg_track_kernel<<<grid(T, 128), 128>>>(d_off, T, d_seg_track);
  // FSR ids: keys ordered by the first segment that touches them
  std::vector<unsigned long long> first(K);
  e = cudaMemcpy(first.data(), d_first, sizeof(uint64_t) * K,
                 cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return fail_cuda(e);
  std::vector<std::pair<unsigned long long, int64_t>> touched;
  for (int64_t d = 0; d < K; d++)
    if (first[d] != ~0ull) touched.emplace_back(first[d], d);
  std::sort(touched.begin(), touched.end());
  const int64_t R = (int64_t) touched.size();
  std::vector<int32_t> table(K, -1);
  std::vector<uint64_t> keys(R);
  for (int64_t r = 0; r < R; r++) {
    const int64_t d = touched[r].second;
    table[d] = (int32_t) r;
    const int64_t sec = d % g.sec;
    const int64_t ring = (d / g.sec) % (g.rings + 1);
    const int64_t cell = d / g.sec / (g.rings + 1);
    keys[r] = (uint64_t) cell << 32 | (uint64_t) ring << 16 | (uint64_t) sec;
  }
  int32_t* d_table = nullptr;
  double* d_vol = nullptr;
  if ((e = buf.alloc(&d_table, K)) != cudaSuccess ||
      (e = buf.alloc(&d_vol, R)) != cudaSuccess)
    return fail_cuda(e);
  e = cudaMemcpy(d_table, table.data(), sizeof(int32_t) * K,
                 cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemset(d_vol, 0, sizeof(double) * R);
  if (e != cudaSuccess) return fail_cuda(e);
  finish_kernel<<<grid(S, 256), 256>>>(d_dense, d_table, d_len, d_seg_track,
                                       d_w, S, d_fsr, d_vol);
  L->S = S;
  L->seg_off = off;
  L->seg_len.resize(S);
  L->seg_fsr.resize(S);
  std::vector<double> vol(R);
  e = cudaMemcpy(L->seg_len.data(), d_len, sizeof(float) * S,
                 cudaMemcpyDeviceToHost);
  if (e == cudaSuccess)
    e = cudaMemcpy(L->seg_fsr.data(), d_fsr, sizeof(int32_t) * S,
                   cudaMemcpyDeviceToHost);
  if (e == cudaSuccess)
    e = cudaMemcpy(vol.data(), d_vol, sizeof(double) * R,
                   cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaGetLastError();
  if (e != cudaSuccess) return fail_cuda(e);
  lat_finish(s, L, X, keys, false);
  L->fsr_vol.resize(R);
  for (int64_t r = 0; r < R; r++) L->fsr_vol[r] = (float) vol[r];
  *out = L;
  return 0;
}
