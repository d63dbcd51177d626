/**
 * @file openmoc_gb300_serve.h
 * @brief C ABI of the batched solve server: many independent eigenvalue and
 *        fixed-source solves of uneven size sharing one GPU.
 *
 * No counterpart in the reference: OpenMOC solves one problem per Solver
 * object, one at a time (src/Solver.cpp:1352-1700).  A server is the
 * device-resident request loop that runs many such solves concurrently with
 * the same per-solve results (same loop body, same convergence test):
 *
 *   - a pool holds every live solve of one group count, polar count and
 *     source kind (flat, or linear as CPULSSolver) in shared device arrays (FSR rows, tracks, segments, materials and angle
 *     rows are contiguous ranges handed out by first-fit allocators over the
 *     pool's capacity, which is its device-memory budget);
 *   - one iteration of a pool is six launches for all of its solves
 *     (sources, one transport sweep over every live track, add-source,
 *     per-solve keff/normalisation, residual terms, per-solve convergence),
 *     and a block of iterations is captured once as a CUDA graph and
 *     replayed until the set of live solves changes;
 *   - between blocks the loop retires finished solves (their fluxes are
 *     copied out and their ranges freed) and admits queued requests into the
 *     freed ranges (continuous batching); pools run on their own streams, so
 *     their work overlaps on the device;
 *   - the sweep shape of a pool (lanes per track, group pairs per lane;
 *     hardware-ex2 evaluator) is autotuned on the live solves, once per
 *     size class (power of two of live tracks), unless fixed; the timing
 *     sweeps write into scratch buffers, so live state is untouched.
 *
 * Requests reference host arrays owned by the caller: the input arrays are
 * copied by moc_server_submit, flux_out and moments_out must stay writable
 * until the request completes.  Every entry point
 * returns MOC_OK or a negative MOC_ERR_* status; moc_last_error() gives the
 * text.  moc_server_submit, moc_server_wait, moc_server_poll and
 * moc_server_stats may be called from any thread; moc_server_step only when
 * no loop thread is running.
 */
#ifndef OPENMOC_GB300_SERVE_H_
#define OPENMOC_GB300_SERVE_H_

#include <stdint.h>

#include "openmoc_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Solve kinds of a request. */
#define MOC_SOLVE_EIGENVALUE 0 /* Solver::computeEigenvalue */
#define MOC_SOLVE_SOURCE 1     /* Solver::computeSource with a fixed keff */
#define MOC_SOLVE_FLUX 2       /* Solver::computeFlux(max_iters, true): the
                                  fixed source alone, computed once from a
                                  zero flux; SCALAR_FLUX residual */

typedef struct moc_server moc_server;

typedef struct {
  int32_t device;              /* CUDA device ordinal */
  int32_t iterations_per_poll; /* iterations per pool between host polls */
  int32_t use_graphs;          /* 1: replay each block as a CUDA graph */
  int32_t priorities;          /* 1: pools of few fluxes per track (short,
                                  latency-bound kernels) get the high
                                  stream priority */
  int64_t hot_bytes;           /* cap on the sweep-gathered bytes (sources
                                  and tallies, 8 B per FSR and group) of all
                                  live solves, so that they stay in L2;
                                  0: no cap.  A pool with no live solve
                                  always admits one. */
} moc_server_config;

typedef struct {
  int32_t num_groups;     /* G of every solve in the pool */
  int32_t num_polar_half; /* Ph of every solve in the pool */
  int32_t max_solves;     /* concurrent solves */
  int32_t max_materials;  /* material rows, <= 256 */
  int32_t max_angles;     /* weight-table rows */
  int64_t max_fsrs;       /* FSR rows, < 2^24 */
  int64_t max_tracks;     /* track entries (a solve uses T + 1) */
  int64_t max_segments;   /* segments */
  int32_t lanes;          /* sweep lanes per track direction; 0: autotune */
  int32_t pairs;          /* group pairs per lane (with lanes): the fewest
                             that cover the groups, ceil(ceil(G/2)/lanes) */
  int32_t exp_kind;       /* with lanes: MOC_EXP_INTRINSIC (pools use ex2) */
  int32_t linear_source;  /* 1: the pool takes linear-source requests
                             (CPULSSolver, 2D), at most 5 group pairs per
                             lane; 0: flat-source requests */
} moc_pool_config;

typedef struct {
  /* the problem: dimensions and arrays as for moc_create / moc_upload_* */
  int32_t num_groups, num_polar_half, num_angles, num_materials;
  int64_t num_fsrs, num_tracks, num_segments;
  const float* seg_len;
  const int32_t* seg_fsr;
  const int64_t* seg_off;
  const int32_t* track_ang;
  const int64_t* next;
  const uint8_t* flags;
  const float* weights;
  const float* inv_sin;
  const float* sigma_t;
  const float* sigma_s; /* [M][dest][orig] */
  const float* nu_sigma_f;
  const float* chi;
  const int32_t* fsr_mat;
  const float* fsr_vol;
  const float* fixed_source; /* [R][G] or NULL */
  /* the solve */
  int32_t kind;      /* MOC_SOLVE_* */
  int32_t max_iters;
  int32_t res_type;  /* MOC_SCALAR_FLUX / MOC_FISSION_SOURCE / MOC_TOTAL_SOURCE */
  double k_eff;      /* MOC_SOLVE_SOURCE: the fixed eigenvalue */
  double threshold;  /* convergence threshold */
  float* flux_out;   /* [R][G] scalar fluxes, written on completion */
  int32_t allow_negative_fluxes; /* Solver::allowNegativeFluxes */
  /* linear source (NULL: flat source): the geometry moc_set_linear_source
     takes; the request goes to its (G, Ph) linear-source pool, which
     computes the expansion constants when it admits the request */
  const moc_ls_geometry* linear_source;
  const float* fixed_source_moments; /* [R][3][G] (x, y, z; z unused) or
                                        NULL (setFixedSourceMomentByFSR) */
  float* moments_out;  /* [R][3][G] flux moments (z = 0) written on
                          completion, or NULL */
} moc_request;

typedef struct {
  int32_t status;     /* MOC_OK or the error that ended the request */
  int32_t iterations; /* as Solver::getNumIterations after the solve */
  int32_t converged;
  int32_t pool;
  double keff;
  double residual;
  double t_submit, t_admit, t_done; /* seconds on a monotonic clock */
} moc_result;

typedef struct {
  int64_t submitted, admitted, completed, failed;
  int64_t blocks;          /* iteration blocks launched */
  int64_t graph_captures;  /* CUDA graphs captured */
  int64_t kernel_launches; /* kernels run, graph nodes included */
  int64_t live, queued;
  double gpu_busy_s;       /* device time of all blocks (pools overlap) */
  double host_admit_s;     /* loop time spent uploading admitted solves */
  double host_retire_s;    /* loop time spent copying out finished solves */
  double host_graph_s;     /* loop time spent capturing CUDA graphs */
} moc_server_stats;

int moc_server_create(const moc_server_config* cfg, moc_server** out);
int moc_server_destroy(moc_server* srv);

/** Adds a pool; requests go to the pool of their (G, Ph) and source
 *  kind (flat or linear). */
int moc_server_add_pool(moc_server* srv, const moc_pool_config* cfg,
                        int* pool);

/** Validates and queues a request; *ticket identifies it. */
int moc_server_submit(moc_server* srv, const moc_request* req,
                      int64_t* ticket);

/** One pass of the request loop on the calling thread: for every pool,
 *  waits for its running block, retires, admits, launches the next block.
 *  *pending = live + queued solves afterwards. */
int moc_server_step(moc_server* srv, int64_t* pending);

/** Runs the request loop on a background thread until moc_server_stop. */
int moc_server_start(moc_server* srv);
int moc_server_stop(moc_server* srv);

/** Waits up to timeout_s seconds (< 0: forever) for a request;
 *  MOC_ERR_TIMEOUT if it has not completed. */
int moc_server_wait(moc_server* srv, int64_t ticket, double timeout_s,
                    moc_result* out);

/** Tickets completed since the previous poll (up to capacity). */
int moc_server_poll(moc_server* srv, int64_t* tickets, int capacity,
                    int* count);

int moc_server_stats_get(moc_server* srv, moc_server_stats* out);
/** The message of the last error inside the request loop (the call that
 *  failed and CUDA's description), which failed the requests of its pool
 *  with that status; "" when none.  Valid until the next call on the
 *  server from this thread. */
const char* moc_server_loop_error(moc_server* srv);

typedef struct {
  int32_t num_groups, num_polar_half;
  int32_t lanes, pairs, exp_kind; /* sweep shape in use (autotuned or fixed) */
  int32_t live;
  int64_t admitted, completed, blocks;
  int64_t tunes;          /* autotuner runs (one per size class met) */
  double gpu_busy_s;
} moc_pool_stats;

/** Statistics and sweep shape of one pool. */
int moc_server_pool_stats(moc_server* srv, int pool, moc_pool_stats* out);

#ifdef __cplusplus
}
#endif

#endif /* OPENMOC_GB300_SERVE_H_ */
