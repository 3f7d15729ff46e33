/*
 * svie.h -- C ABI of the GB300 (sm_103a) narrow-band level-set erosion library.
 *
 * Every function takes plain device pointers, sizes and a cudaStream_t passed as
 * `void* stream` (NULL = legacy default stream), returns an int status
 * (SVIE_OK = 0) and allocates no device memory: scratch space is a
 * caller-provided workspace whose size the matching *_workspace_bytes() query
 * reports.  svie_last_error() returns the message of the last failure on the
 * calling thread.  Grids are dense float32 arrays in C order with axes (x, y, z)
 * (strides ny*nz, nz, 1); node lists are sorted int32 flat indices.
 *
 * Each declaration names the reference interface it replaces (paths within the
 * SVIErosion project).  The reference binds nothing natively: its hot path is
 * PyTorch functions compiled by torch.compile, so the "binding" is the Python
 * module svierosion_gb300 (ctypes), whose functions keep the reference's names
 * and argument orders.
 */
#ifndef SVIE_H
#define SVIE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------ status */
#define SVIE_OK 0
#define SVIE_ERR_ARG 1          /* bad argument / shape                        */
#define SVIE_ERR_LAUNCH 2       /* CUDA launch or runtime error                */
#define SVIE_ERR_WORKSPACE 3    /* workspace too small                         */
#define SVIE_ERR_MARGIN 4       /* narrow band reaches the grid boundary       */
#define SVIE_ERR_UNSUPPORTED 5  /* size outside what the kernels support      */
#define SVIE_ERR_CAPACITY 6     /* output capacity too small                   */

const char* svie_last_error(void);
int svie_version(void);
/* Number of kernels launched through this library so far (all threads). */
unsigned long long svie_launch_count(void);

/* ---------------------------------------------------------------- structs */
/* Speed law and integrator constants (reference svierosion/flows.py:51-213,
 * svierosion/evolve.py:70-112).  kind: 0 = SVI power law, 1 = mean curvature,
 * 2 = Gauss curvature. */
typedef struct svie_law {
  int32_t kind;
  int32_t k;             /* SVI exponent                                   */
  int32_t s;             /* SVI geometric switch (0/1)                     */
  int32_t pad0;
  double t;              /* SVI singularity                                */
  double eps;            /* additive grassfire term                        */
  double n_cap;          /* SVI cap on N (1.0 when s == 0)                 */
  double radius;         /* SVI ball radius                                */
  double alpha;          /* curvature exponent                             */
  double delta;          /* curvature regularisation                       */
  double cfl;
  double feedback_cfl;
  double parabolic_cfl;
  double h;              /* grid spacing                                   */
  double cut_a;          /* cutoff[0] * h                                  */
  double cut_b;          /* cutoff[1] * h                                  */
} svie_law;

/* Per-step statistics and scalars, written on the device and read back once
 * per step (reference svierosion/evolve.py:118-170, levelset.py:93-95,123-126).
 * Float maxima of non-negative values are stored as IEEE bits; signed minima
 * and maxima as order-preserving keys (see svierosion_gb300/_native.py). */
typedef struct svie_stats {
  double vsum_near;      /* sum of V (before cutoff) over |phi| < h       */
  double vsum_all;       /* sum of V (before cutoff) over the band        */
  double fsum;           /* sum of band cell fractions (float64)          */
  double dt;             /* stable time step computed on the device        */
  double dt_cap;         /* upper bound for dt (max_time - time or +inf)   */
  double reserved_d[3];
  uint32_t vmax;         /* max V after cutoff (float bits)               */
  uint32_t qmin_near, qmax_near, qmin_all, qmax_all;   /* ordered keys    */
  uint32_t dvmax_near, dvmax_all;                      /* float bits      */
  uint32_t dmax_near, dmax_all;                        /* float bits      */
  uint32_t capped_near, capped_all;
  uint32_t n_near;
  uint32_t any_neg, any_pos;   /* band has phi < 0 / phi > 0               */
  uint32_t n_band;
  uint32_t reserved_u;
} svie_stats;

/* Band bookkeeping written by svie_band_write (reference levelset.py:70-86,
 * evolve.py:96-105). */
typedef struct svie_band_info {
  int64_t count;             /* band size                                   */
  int64_t static_inside;     /* nodes outside the band with phi < 0          */
  int32_t lo[3], hi[3];      /* min / max band coordinate per axis           */
  int32_t ilo[3], ihi[3];    /* min / max coordinate of phi < 0 nodes        */
} svie_band_info;

/* ----------------------------------------------------- band construction */
/* LevelSet.rebuild_band (svierosion/levelset.py:70-77): clamp phi to
 * [-cap, cap] in place, then list the nodes with |phi| < thresh in ascending
 * flat order.  Two calls: svie_band_scan clamps and counts (writing the count
 * to info->count on the device); the caller reads it, sizes `band` and calls
 * svie_band_write, which also writes occ[i] = (phi[i] < 0) for every node when
 * occ is non-NULL, and fills the rest of *info (margin check data,
 * levelset.py:79-86). */
size_t svie_band_workspace_bytes(int64_t n);
int svie_band_scan(float* phi, int64_t n, float cap, float thresh, void* ws, size_t ws_bytes,
                   svie_band_info* info, void* stream);
int svie_band_write(const float* phi, int nx, int ny, int nz, float thresh, const void* ws,
                    size_t ws_bytes, int32_t* band, int64_t capacity, float* occ,
                    svie_band_info* info, void* stream);

/* Generic order-preserving compaction of mask[i] != 0 (torch.nonzero on a
 * bool mask, as in levelset.py:173).  Same two-call protocol; `count` is a
 * device int64. */
int svie_mask_scan(const uint8_t* mask, int64_t n, void* ws, size_t ws_bytes, int64_t* count,
                   void* stream);
int svie_mask_write(const uint8_t* mask, int64_t n, const void* ws, size_t ws_bytes, int32_t* out,
                    int64_t capacity, void* stream);
/* idx[mask] for an int32 index list (LevelSet.interface_nodes,
 * levelset.py:88-91): out[k] = vals[e] for the k-th e with mask[e] != 0.  Uses
 * the workspace of a preceding svie_mask_scan over the same mask. */
int svie_mask_select(const uint8_t* mask, const int32_t* vals, int64_t n, const void* ws,
                     size_t ws_bytes, int32_t* out, int64_t capacity, void* stream);
/* The same node sets in brick order (bricks of 4 x 4 x 16 nodes, x-major
 * brick order, z fastest inside a row): kind 0 selects mask[i] != 0 (uint8
 * src), kind 1 selects |phi[i]| < thresh (float src), kind 2 the set bits of
 * a bit mask in the layout of svie_reinit_bits (uint32 src).  Same two-call
 * protocol; the brick-ordered lists drive the stencil kernels, the ascending
 * lists stay the API's node lists. */
size_t svie_brick_workspace_bytes(int nx, int ny, int nz);
int svie_brick_scan(int kind, const void* src, int nx, int ny, int nz, float thresh, void* ws,
                    size_t ws_bytes, int64_t* count, void* stream);
int svie_brick_write(int kind, const void* src, int nx, int ny, int nz, float thresh,
                     const void* ws, size_t ws_bytes, int32_t* out, int64_t capacity, void* stream);
/* LevelSet.rebuild_band (levelset.py:70-86) restricted to a node list idx of m
 * nodes (the reinitialisation work set, brick order), for a phi that changed
 * only on the list since the last full rebuild: clamp and count (scan), then
 * the band entries in list order, occupancy of the listed nodes and info
 * (count, band box; static_inside and the inside box cover the listed nodes
 * only).  ws: svie_list_workspace_bytes(m). */
size_t svie_list_workspace_bytes(int64_t m);
int svie_list_band_scan(float* phi, const int32_t* idx, int64_t m, float cap, float thresh, void* ws,
                        size_t ws_bytes, svie_band_info* info, void* stream);
int svie_list_band_write(const float* phi, const int32_t* idx, int64_t m, int nx, int ny, int nz, float thresh,
                         const void* ws, size_t ws_bytes, int32_t* out, int64_t capacity, float* occ,
                         svie_band_info* info, void* stream);
/* *count = the listed nodes with phi < 0 whose bit in `marked` (layout of
 * svie_reinit_bits) is clear. */
int svie_list_inside_off_mask(const float* phi, const int32_t* idx, int64_t m, const uint32_t* marked, int nx,
                              int ny, int nz, uint64_t* count, void* stream);
/* LevelSet.rebuild_band (svierosion/levelset.py:70-86) with the band listed in
 * brick order: svie_brick_band_scan clamps phi to [-cap, cap] in place and
 * counts |phi| < thresh (info->count on the device); svie_brick_band_write
 * lists those nodes in brick order and, like svie_band_write, writes occ (when
 * non-NULL) and the rest of *info.  Two grid passes in place of four when the
 * ascending list is not needed at once.  Workspace: svie_brick_workspace_bytes. */
int svie_brick_band_scan(float* phi, int nx, int ny, int nz, float cap, float thresh, void* ws,
                         size_t ws_bytes, svie_band_info* info, void* stream);
int svie_brick_band_write(const float* phi, int nx, int ny, int nz, float thresh, const void* ws,
                          size_t ws_bytes, int32_t* out, int64_t capacity, float* occ,
                          svie_band_info* info, void* stream);

/* ------------------------------------------------- stencil kernels (API) */
/* svierosion/kernels.py:146 godunov_inward(flat, idx, sx, sy, sz, inv_h) */
int svie_godunov_inward(const float* flat, const int32_t* idx, int64_t m, int64_t sx, int64_t sy,
                        int64_t sz, float inv_h, float* out, void* stream);
/* svierosion/kernels.py:173 cell_fractions(flat, idx, sx, sy, sz) */
int svie_cell_fractions(const float* flat, const int32_t* idx, int64_t m, int64_t sx, int64_t sy,
                        int64_t sz, float* out, void* stream);
/* svierosion/kernels.py:185 closest_points(flat, idx, ny, nz, hi_x, hi_y, hi_z, h); out (m,3) */
int svie_closest_points(const float* flat, const int32_t* idx, int64_t m, int ny, int nz, float hi_x,
                        float hi_y, float hi_z, float h, float* out, void* stream);
/* svierosion/kernels.py:212 tricubic(flat, ny, nz, p) */
int svie_tricubic(const float* flat, int ny, int nz, const float* p, int64_t m, float* out,
                  void* stream);
/* svierosion/kernels.py:232 tricubic_with_gradient(flat, ny, nz, p); grad (m,3) */
int svie_tricubic_with_gradient(const float* flat, int ny, int nz, const float* p, int64_t m,
                                float* val, float* grad, void* stream);
/* svierosion/kernels.py:257 trilinear(flat, ny, nz, p) */
int svie_trilinear(const float* flat, int ny, int nz, const float* p, int64_t m, float* out,
                   void* stream);
/* svierosion/kernels.py:274 principal_curvatures(flat, idx, sx, sy, sz, h) */
int svie_principal_curvatures(const float* flat, const int32_t* idx, int64_t m, int64_t sx,
                              int64_t sy, int64_t sz, float h, float* k1, float* k2, void* stream);
/* svierosion/kernels.py:303 interface_mask(flat, idx, sx, sy, sz) */
int svie_interface_mask(const float* flat, const int32_t* idx, int64_t m, int64_t sx, int64_t sy,
                        int64_t sz, uint8_t* out, void* stream);
/* svierosion/kernels.py:382-427 _point_triangle_distance2 for m (point, triangle) pairs;
 * p (m,3), a, b, c (m,3) */
int svie_point_triangle_distance2(const float* p, const float* a, const float* b, const float* c,
                                  int64_t m, float* out, void* stream);
/* LevelSet.central_gradient (levelset.py:98-101); out (m,3) */
int svie_central_gradient(const float* flat, const int32_t* idx, int64_t m, int64_t sx, int64_t sy,
                          int64_t sz, float* out, void* stream);
/* LevelSet.closest_points(idx, newton_steps) (levelset.py:129-151); out (m,3) */
int svie_closest_points_newton(const float* flat, const int32_t* idx, int64_t m, int ny, int nz,
                               float hi_x, float hi_y, float hi_z, float h, int newton_steps,
                               float* out, void* stream);
/* phi[band] (the reference's `flat[band]`, e.g. levelset.py:123-126 and the
 * band values a caller reads back): out[k] = src[idx[k]]. */
int svie_gather(const float* src, const int32_t* idx, int64_t m, float* out, void* stream);
/* levelset.cube_plane_fraction (levelset.py:37-48, kernels.py:104-122) */
int svie_cube_plane_fraction(const float* s, const float* a, const float* b, const float* c,
                             int64_t m, float* out, void* stream);
/* SVIPowerLaw.speed/dspeed (flows.py:89-108) or the curvature laws'
 * speed_and_diffusivity (flows.py:170-206): x2 is k2 for curvature laws. */
int svie_law_eval(const float* x1, const float* x2, int64_t m, const svie_law* law, float* V,
                  float* D, void* stream);

/* ------------------------------------------- occupancy and solid volume */
/* LevelSet.dense_fractions (svierosion/levelset.py:117-121): occ[band[i]] =
 * cell fraction; occ elsewhere must already hold (phi < 0). */
int svie_scatter_fractions(const float* phi, const int32_t* band, int64_t m, int64_t sx, int64_t sy,
                           int64_t sz, float* occ, void* stream);
/* occ[i] = (phi[i] < 0) on every node (levelset.py:119). */
int svie_dense_occupancy(const float* phi, int64_t n, float* occ, void* stream);
/* LevelSet.volume (svierosion/levelset.py:123-126) minus the static count:
 * stats->fsum = float64 sum of the band cell fractions (deterministic order),
 * stats->any_neg / any_pos = has_interface flags (levelset.py:93-95); when occ
 * is non-NULL the fractions are also scattered into it. */
size_t svie_volume_workspace_bytes(int64_t m);
int svie_band_volume(const float* phi, const int32_t* band, int64_t m, int64_t sx, int64_t sy,
                     int64_t sz, float* occ, void* ws, size_t ws_bytes, svie_stats* stats,
                     void* stream);
/* svie_band_volume without a workspace: no counterpart in the reference.  For
 * callers that cannot allocate device memory (a plugin inside a host
 * framework whose pool owns all device memory, or a loop that forbids
 * cudaMalloc after start-up because it can synchronise the device).  The
 * scratch is a static 512 KiB device array held by every GPU that loads the
 * library, so m is limited to svie_band_volume_noalloc_max() band nodes
 * (16,777,216); larger m returns SVIE_ERR_CAPACITY.  The first call on a
 * device (and in each further CUDA context made current on it) looks up the
 * array's device address (cudaGetSymbolAddress), so make that first call
 * before any stream capture.  Do not reset the device between calls: a
 * recreated context may reuse its old handle, and the cached address would
 * then be stale.  All calls share the array: calls that overlap on the GPU
 * race and must be ordered by the caller. */
int64_t svie_band_volume_noalloc_max(void);
int svie_band_volume_noalloc(const float* phi, const int32_t* band, int64_t m, int64_t sx,
                             int64_t sy, int64_t sz, float* occ, svie_stats* stats, void* stream);

/* ------------------------------------------------------ SVI convolution */
/* svierosion/svi.py:24 ball_cell_weights(radius, spacing, quad): half-width
 * m = floor(r/h + 1/2) + 1, weights (2m+1)^3 float64 on the device. */
int svie_ball_half_width(double radius, double spacing);
int svie_ball_weights(double radius, double spacing, int quad, double* w, void* stream);

/* BallConvolution (svierosion/svi.py:58-93).  The plan holds the FFT twiddle
 * tables and the real, axis-even kernel spectrum K^ computed in float64 from
 * the float64 weights and rounded to float32, stored for
 * kx <= nx/2, ky <= ny/2, kz <= nz/2.  The workspace holds one complex64
 * padded half spectrum nx*ny*svie_conv_spectrum_row(nz). */
size_t svie_conv_plan_bytes(int nx, int ny, int nz);
size_t svie_conv_workspace_bytes(int nx, int ny, int nz);
int svie_conv_supported(int n);
/* The float64 intermediates of the K^ sums use a temporary workspace of
 * svie_conv_init_workspace_bytes() bytes. */
size_t svie_conv_init_workspace_bytes(int nx, int ny, int nz, int m);
int svie_conv_plan_init(void* plan, int nx, int ny, int nz, const double* w, int m, void* ws,
                        size_t ws_bytes, void* stream);
/* out = beta + alpha * (w (*) f) with unnormalised circular convolution:
 * interior_volume uses alpha = h^3, beta = 0; exterior_fraction uses
 * alpha = -h^3/|B_r|, beta = 1 (svi.py:84-93). */
int svie_conv_apply(const void* plan, int nx, int ny, int nz, const float* f, float* out,
                    double alpha, double beta, void* ws, size_t ws_bytes, void* stream);
/* Row length (complex values) of the padded half spectrum used by the
 * workspace and by svie_rfft3 / svie_irfft3: nz/2+1 rounded up to a multiple
 * of 8, so every row starts on a 64-byte boundary.  The spectrum is
 * [nx][ny][row]; entries kz >= nz/2+1 are padding. */
int svie_conv_spectrum_row(int nz);
/* Line flags for the masked convolution over the (x, y) lines of the grid
 * (lineflag: nx*ny bytes, slabflag: nx bytes, tmp: nx*ny bytes scratch):
 * bit 0 marks lines holding band nodes -- every line with solid, since the
 * padding keeps the grid boundary outside -- and bit 1 those lines dilated by
 * `dilation` lines in x and y, which covers every tricubic stencil at the
 * closest point of a band node when dilation >= 10 (the projection moves at
 * most 1.25 * 6 + 0.25 cells, the stencil reaches 2 more).  slabflag[x] ORs
 * the bits of slab x. */
int svie_conv_line_flags(const int32_t* band, int64_t m, int nx, int ny, int nz, int dilation,
                         uint8_t* lineflag, uint8_t* slabflag, uint8_t* tmp, void* stream);
/* svie_conv_apply that skips provably unneeded work: z lines without bit 0
 * are zero on input (only zeros are written for them), y slabs without bit 0
 * stay zero in the forward pass, and in the inverse passes only slabs / lines
 * with bit 1 are computed -- the other values of `out` are left unchanged and
 * must not be read.  events (optional): six cudaEvent_t recorded before,
 * between and after the five passes (z R2C, y forward, x forward*K^*inverse,
 * y inverse, z C2R). */
int svie_conv_apply_masked(const void* plan, int nx, int ny, int nz, const float* f, float* out,
                           double alpha, double beta, void* ws, size_t ws_bytes,
                           const uint8_t* lineflag, const uint8_t* slabflag,
                           void* const* events, void* stream);
/* Launch forms of the passes.  Each pass has up to three forms that group the
 * lines into CTAs differently (z: 16, 8 or 1 line pairs per CTA; y: persistent
 * 8-line tiles, one 8-line tile or one line per CTA; x: one 8-line tile,
 * persistent 8-line tiles or one line per CTA).  All forms run the same radix
 * stages; the z forms give the same bits, and so do the 8-line forms of y and
 * x, while the one-line y and x forms (2) may differ from those in the last
 * bit.
 * svie_conv_tune times the forms that fit shared memory on this grid shape,
 * the one-line y and x forms only where no 8-line form fits, so that a tuned
 * shape gives the fixed rule's bits (`reps` timed launches after one untimed
 * one, shortest kept; f is transformed, out and ws are overwritten; the
 * stream is synchronised, so not while it is being captured).  It keeps the
 * fastest forms per (device, nx, ny, nz) for every later call on that shape.
 * svie_conv_get_choice returns 1 and the kept forms when the shape was tuned
 * or set, else 0 and the fixed rule's forms (z 16 line pairs, y and x one
 * 8-line tile per CTA, where they fit).  svie_conv_set_choice sets them
 * (SVIE_ERR_ARG for a form that does not exist or fit); a negative value
 * clears the entry.  Replaces nothing in the reference, whose transforms are
 * torch.fft calls (svi.py:84-93). */
int svie_conv_tune(const void* plan, int nx, int ny, int nz, const float* f, float* out, void* ws,
                   size_t ws_bytes, int reps, void* stream);
/* The 8-line y and x passes load their tiles with TMA boxes of a tensor map
 * over the spectrum (cp.async when the axis length is odd or SVIE_TMA=0) and
 * wait for them on an mbarrier with a bounded poll; this returns how many
 * tiles ran out of that bound since the library was loaded (0 in a healthy
 * run; such a tile is skipped), synchronising the device.  0xFFFFFFFF when the
 * count could not be read. */
unsigned int svie_conv_tma_timeouts(void);
int svie_conv_get_choice(int nx, int ny, int nz, int* z, int* y, int* x);
/* Passes compiled for the axis lengths.  svie_conv_jit starts compiling
 * (NVRTC, on background threads, in the current context) the 8-line y and x
 * passes for ny and nx and the z passes for nz, with every stage's radix,
 * column count and span as constants, and makes the shape use each of them as
 * soon as it is loaded (the library's passes run until then; the bits are the
 * same).  SVIE_OK, or SVIE_ERR_UNSUPPORTED when NVRTC or the driver functions
 * are missing or the 8-line forms do not fit.  svie_conv_jit_enabled reports
 * whether the shape is set to use them, svie_conv_jit_ready whether all three
 * are loaded, svie_conv_jit_wait waits up to timeout_ms for every compilation
 * started (SVIE_ERR_LAUNCH when some still run).  svie_conv_jit_source writes
 * the generated source for an axis length into buf (minb 0: the z passes, else
 * the strided pass for minb CTAs per SM; no device needed).  Replace nothing
 * in the reference. */
int svie_conv_jit(int nx, int ny, int nz);
int svie_conv_jit_enabled(int nx, int ny, int nz);
int svie_conv_jit_ready(int nx, int ny, int nz);
int svie_conv_jit_wait(int timeout_ms);
/* Stops the compile worker: drops the queued compilations, waits (at most
 * 10 s) for the one in progress and joins the thread; later svie_conv_jit
 * requests run the library's passes.  A host calls it on its exit path before
 * the process tears its libraries down, so that no compilation runs inside
 * NVRTC during that teardown (the Python package registers it at interpreter
 * exit). */
int svie_conv_jit_stop(void);
int svie_conv_jit_source(int n, int minb, char* buf, size_t buf_bytes);
int svie_conv_set_choice(int nx, int ny, int nz, int z, int y, int x);
/* Full complex64 half spectrum K^ (rfftn of the wrapped kernel, svi.py:76-81). */
int svie_conv_kernel_hat(const void* plan, int nx, int ny, int nz, void* out_c64, void* stream);
/* Forward rfftn (complex64 nx*ny*(nz/2+1)) and inverse irfftn with
 * out = beta + alpha * irfftn_unnormalised(spec); spec is overwritten. */
int svie_rfft3(const void* plan, int nx, int ny, int nz, const float* f, void* spec, void* stream);
int svie_irfft3(const void* plan, int nx, int ny, int nz, void* spec, float* out, double alpha,
                double beta, void* stream);

/* ---------------------------------------------------- fused RK3 stages */
/* ErosionSimulation._rhs for the SVI law (svierosion/evolve.py:118-160):
 * closest point -> tricubic N -> speed law -> cutoff -> WENO5/Godunov ->
 * L = V |grad phi|.  u0 (phi at the band, optional) and V (after cutoff,
 * optional) are also written.  When stats is non-NULL the stage-0 statistics
 * are accumulated (the struct must be cleared first with svie_stats_reset). */
size_t svie_stage_workspace_bytes(int64_t m);
int svie_stats_reset(svie_stats* stats, double dt_cap, void* stream);
int svie_stage_svi(const float* phi, const int32_t* band, int64_t m, int nx, int ny, int nz,
                   const float* N, const svie_law* law, float* L, float* u0, float* V,
                   svie_stats* stats, void* ws, size_t ws_bytes, void* stream);
/* Curvature laws: principal curvatures into an interleaved (k1, k2) dense
 * field (zero off the band), then trilinear at closest points
 * (evolve.py:137-151). */
int svie_curvature_scatter(const float* phi, const int32_t* band, int64_t m, int nx, int ny, int nz,
                           float h, float* kdense, void* stream);
int svie_stage_curvature(const float* phi, const int32_t* band, int64_t m, int nx, int ny, int nz,
                         const float* kdense, const svie_law* law, float* L, float* u0, float* V,
                         svie_stats* stats, void* ws, size_t ws_bytes, void* stream);
/* stable_dt (evolve.py:162-170) on the device: stats->dt. */
int svie_stats_finalize(svie_stats* stats, const svie_law* law, const void* ws, size_t ws_bytes,
                        int64_t m, void* stream);
/* _rk3 stage updates (evolve.py:172-179); stage 1: phi = u0 + dt L;
 * 2: phi = 3/4 u0 + 1/4 (phi + dt L); 3: phi = u0/3 + 2/3 (phi + dt L).
 * dt is read from *dt on the device; nothing is written unless dt is finite
 * and positive.  stage 0 restores phi[band] = u0. */
int svie_rk_stage(float* phi, const int32_t* band, int64_t m, const float* u0, const float* L,
                  const double* dt, int stage, void* stream);
int svie_set_f64(double* dst, double value, void* stream);

/* ------------------------------------------- many level sets in one launch */
/* The per-step band work of svierosion/evolve.py:118-179 (stage right-hand
 * sides, statistics and time step, RK combinations, occupancy refresh, the
 * float64 volume of levelset.py:123-126) for a group of independent level
 * sets -- the batched form of ErosionSimulation.run (evolve.py:182-250), which
 * the reference runs one solid at a time.  Every member's band is cut into
 * tiles of 256 entries, the CTAs of the one-level-set kernels, and each launch
 * takes the packed (member, tile) list of all members: one launch per pass
 * instead of one per member.  A member's arithmetic is the one-level-set
 * kernels' own, so its results equal svie_stage_* / svie_rk_stage /
 * svie_band_volume bit for bit.  Members keep their own arrays; time steps
 * (stats->dt) are per member and never leave the device.  No time cap: a
 * member's stats->dt_cap is +inf. */
typedef struct svie_group_member {
  float* phi;               /* the member's dense level set                  */
  const int32_t* band;      /* its band (work order), m entries              */
  int64_t m;
  int32_t nx, ny, nz;
  int32_t kind;             /* 0: SVI law, field = N; 1: curvature law,
                               field = interleaved (k1, k2) (zero off band)  */
  float* field;
  float* occ;               /* the maintained occupancy                      */
  float* u0;                /* phi at the band at the start of the step      */
  float* L[3];              /* stage right-hand sides                        */
  svie_stats* stats;        /* stage statistics and dt                       */
  svie_stats* vstats;       /* volume statistics                             */
  void* stage_ws;           /* >= svie_stage_workspace_bytes(m)              */
  size_t stage_ws_bytes;
  void* volume_ws;          /* >= svie_volume_workspace_bytes(m)             */
  size_t volume_ws_bytes;
  svie_law law;
} svie_group_member;

typedef struct svie_group {  /* a built group (filled by svie_group_build)  */
  void* table;              /* device table of member records and tiles      */
  int32_t n;                /* members                                       */
  int32_t pad;
  int64_t tiles;            /* tiles of all members                          */
  int64_t tiles_svi;        /* of which the first tiles_svi are SVI members' */
} svie_group;

int64_t svie_group_tiles(const svie_group_member* members, int32_t n);
size_t svie_group_table_bytes(int32_t n, int64_t tiles);
/* Packs the table into host_staging (table_bytes, caller-owned; pinned memory
 * for an asynchronous copy, which must stay untouched until the copy has run)
 * and copies it to the device table on `stream`. */
int svie_group_build(const svie_group_member* members, int32_t n, void* table, size_t table_bytes,
                     void* host_staging, svie_group* out, void* stream);
int svie_group_stats_reset(const svie_group* g, void* stream);
/* occupancy refresh of the SVI members (svie_scatter_fractions) */
int svie_group_scatter_fractions(const svie_group* g, void* stream);
/* principal curvatures of the curvature members (svie_curvature_scatter) */
int svie_group_curvature_scatter(const svie_group* g, void* stream);
/* stage right-hand side into L[stage] (0..2); stage 0 also writes u0 and the
 * statistics (svie_stage_svi / svie_stage_curvature) */
int svie_group_stage(const svie_group* g, int stage, void* stream);
/* every member's dt from its statistics (svie_stats_finalize) */
int svie_group_stats_finalize(const svie_group* g, void* stream);
/* RK combination `stage` (1..3; 0 restores u0) with L[stage - 1] and the
 * member's own dt (svie_rk_stage) */
int svie_group_rk(const svie_group* g, int stage, void* stream);
/* float64 band volume, interface flags and occupancy (svie_band_volume) */
int svie_group_volume(const svie_group* g, void* stream);
/* copies member k's stats and vstats to dst[2k] and dst[2k + 1] */
int svie_group_gather_stats(const svie_group* g, svie_stats* dst, void* stream);

/* ------------------------------------------------- point-to-mesh distance */
/* point_mesh_distance (svierosion/api.py:104-168), exact: the T pieces (T x 9
 * floats) are binned by centroid into a gx x gy x gz grid of cells of side cs
 * from (ox, oy, oz), with the bounding box of each cell's pieces, an occupancy
 * bit per cell and each piece's bounding sphere (svie_piece_grid_build,
 * workspace svie_piece_grid_bytes);
 * svie_point_mesh_distance walks Chebyshev shells of cells around each point
 * (one warp per point), visiting the cells whose piece box is not farther than
 * the best distance so far and testing their pieces against their bounding
 * spheres first, until no unvisited piece can be closer (rho bounds
 * centroid-to-piece distances), and writes the distance (float32, sqrt of the
 * float32 squared distance of kernels.py:382-427). */
/* The triangles of a device mesh relative to (sx, sy, sz) as float32 pieces (T x 9), the first-edge
 * lengths (float32 [T]) and the largest edge and centroid-to-vertex distance (float bits in
 * maxbits[0], maxbits[1]). */
int svie_mesh_pieces(const double* vertices, const int32_t* faces, int64_t T, double sx, double sy, double sz,
                     float* out, float* first_edge, uint32_t* maxbits, void* stream);
/* The (T, 3) int64 faces of a host mesh as int32 on the device (the upload of meshio.TriMesh's faces);
 * *bad = the number of indices outside [0, V), which are written as 0. */
int svie_mesh_faces_i32(const int64_t* faces64, int64_t T, int64_t V, int32_t* faces, int* bad, void* stream);
/* Exact bounding box of V float64 vertices (V, 3): out = (min x, min y, min z, max x, max y, max z),
 * numpy's per-column min / max (TriMesh.bounds, meshio.py:35-37); ws holds 48 bytes. */
int svie_mesh_bounds(const double* vertices, int64_t V, void* ws, size_t ws_bytes, double* out, void* stream);
/* out[0], out[1] = the k0-th and k1-th smallest of n floats (0-based; np.partition's kth values) by
 * an exact radix select over order-preserving keys: the middle values of np.median over the
 * first-edge lengths of api.py:122-126.  Workspace svie_order_stats_bytes(). */
size_t svie_order_stats_bytes(void);
int svie_order_stats_f32(const float* x, int64_t n, int64_t k0, int64_t k1, void* ws, size_t ws_bytes, float* out,
                         void* stream);
size_t svie_piece_grid_bytes(int64_t T, int gx, int gy, int gz);
int svie_piece_grid_build(const float* tri, int64_t T, float ox, float oy, float oz, float cs, int gx, int gy,
                          int gz, void* ws, size_t ws_bytes, void* stream);
int svie_point_mesh_distance(const float* pts, int64_t n, const float* tri, int64_t T, float ox, float oy,
                             float oz, float cs, int gx, int gy, int gz, const void* ws, size_t ws_bytes,
                             float rho, float* out, void* stream);

/* ------------------------------------------------- surface extraction */
/* extract_surface (svierosion/surface.py:16-56): marching cubes over the cells
 * whose lower corner is one of the m band nodes (ascending), with a case table
 * generated from the method's definition (svie_surface_table returns it:
 * tri[256][16] cell-edge triples, -1 after the last; ntri[256] triangle
 * counts).  svie_surface_scan counts vertices and faces (device int64
 * totals[2]); svie_surface_write fills verts (nv, 3) in index coordinates and
 * faces (nt, 3), using vinfo (int32, one per grid node) as scratch; ids follow
 * the band order.  svie_surface_project moves every vertex by one Newton step
 * on the tricubic interpolant, limited to max_shift cells (surface.py:44-51). */
int svie_surface_table(int8_t* tri, uint8_t* ntri);
size_t svie_surface_workspace_bytes(int64_t m);
int svie_surface_scan(const float* phi, const int32_t* band, int64_t m, int nx, int ny, int nz,
                      void* ws, size_t ws_bytes, int64_t* totals, void* stream);
int svie_surface_write(const float* phi, const int32_t* band, int64_t m, int nx, int ny, int nz,
                       const void* ws, size_t ws_bytes, int32_t* vinfo, float* verts, int64_t nv,
                       int32_t* faces, int64_t nt, void* stream);
int svie_surface_project(const float* phi, int ny, int nz, float* verts, int64_t nv, float max_shift,
                         void* stream);
/* Signed volume (float64) of the mesh (verts in index coordinates) about (cx, cy, cz), for the
 * orientation test of surface.py:54-55. */
int svie_surface_signed_volume(const float* verts, const int32_t* faces, int64_t nt, double cx, double cy,
                               double cz, double* out, void* stream);
/* The host mesh of surface.py:52-56 written on the device: world = origin + h * verts (float64,
 * rounded as numpy rounds it), faces64 (int64) reversed when *vol < 0, and *bad = the number of
 * faces with a negative vertex index (a crossing outside the band, an error). */
int svie_surface_finish(const float* verts, int64_t nv, const int32_t* faces, int64_t nt, const double* vol,
                        double ox, double oy, double oz, double h, double* world, int64_t* faces64, int* bad,
                        void* stream);
/* out = float32((points - (sx, sy, sz)) / scale) for n float64 points (n, 3): the query points of
 * api.py:147-153 (scale 1, shifted by the pieces' centre) and Grid.to_index before the float32
 * cast of surface.py:59-67 (shift = origin, scale = h), computed as numpy computes them. */
int svie_points_f32(const double* points, int64_t n, double sx, double sy, double sz, double scale, float* out,
                    void* stream);

/* ------------------------------------------------------ reinitialisation */
/* LevelSet.reinitialize (svierosion/levelset.py:154-183): work mask = band
 * dilated by `dilation` cells with the `margin` outer layers cleared. */
int svie_reinit_mask(const int32_t* band, int64_t m, int nx, int ny, int nz, int dilation, int margin,
                     uint8_t* mask, uint8_t* tmp, void* stream);
/* The same work mask as bits (rows (x, y) of ceil(nz / 32) words, bit z % 32
 * of word z / 32; dilation <= 31), for svie_brick_scan / svie_brick_write
 * kind 2.  bits, tmp and marked: svie_reinit_bits_bytes(nx, ny, nz) each;
 * marked (may be NULL) receives the undilated band's bits. */
size_t svie_reinit_bits_bytes(int nx, int ny, int nz);
int svie_reinit_bits(const int32_t* band, int64_t m, int nx, int ny, int nz, int dilation, int margin,
                     uint32_t* bits, uint32_t* tmp, uint32_t* marked, void* stream);
/* reinit_geometry (kernels.py:335-359) packed over the m work-set nodes for
 * svie_reinit_iterate / svie_reinit_rhs: meta uint8[m] (bits 0-5 crossing
 * flags cp/cm per axis, bit 6 phi0 > 0, bit 7 phi0 < 0), per-warp offsets and
 * the subcell distances of the flagged crossings only (compact, in work-set
 * order), and the two entry lists of the sweeps: the plain entries (no
 * crossing, a sign) by grid index and sign, the others by grid index with
 * their flags and distance offsets.  The pseudo-time step is not stored: it is
 * rebuilt from the distances where it is used.
 * geo: svie_reinit_geometry_bytes(m), 16-byte aligned. */
size_t svie_reinit_geometry_bytes(int64_t m);
int svie_reinit_geometry(const float* phi, const int32_t* idx, int64_t m, int64_t sx, int64_t sy,
                         int64_t sz, float h, float cfl, void* geo, void* stream);
/* `iterations` TVD-RK2 pseudo-time steps (levelset.py:178-182); phi_tmp is a
 * dense grid used as the second buffer (it is overwritten). */
int svie_reinit_iterate(float* phi, float* phi_tmp, int64_t n, const int32_t* idx, int64_t m,
                        int64_t sx, int64_t sy, int64_t sz, float h, const void* geo, int iterations,
                        void* stream);
/* kernels.reinit_rhs (kernels.py:363-379) for API parity. */
int svie_reinit_rhs(const float* phi, const int32_t* idx, int64_t m, int64_t sx, int64_t sy, int64_t sz,
                    float h, const void* geo, float* out, void* stream);
/* The 14 arrays of kernels.reinit_geometry (kernels.py:335-359): sgn, dtau
 * float[m]; flags uint8[6][m] and dist6 float[6][m] in the order cp_x cm_x
 * cp_y cm_y cp_z cm_z / xp_x xm_x xp_y xm_y xp_z xm_z (distances of every
 * node, clamped below to 1e-6 h). */
int svie_reinit_geometry_arrays(const float* phi, const int32_t* idx, int64_t m, int64_t sx, int64_t sy,
                                int64_t sz, float h, float cfl, float* sgn, float* dtau, uint8_t* flags,
                                float* dist6, void* stream);
/* Packed geometry from those arrays (kernels.reinit_rhs takes them from the
 * caller) for svie_reinit_rhs; dtau is not used (may be NULL).  Without the
 * grid indices the sweep lists stay empty: svie_reinit_iterate takes the
 * geometry of svie_reinit_geometry. */
int svie_reinit_geometry_pack(const float* sgn, const float* dtau, const uint8_t* flags, const float* dist6,
                              int64_t m, void* geo, void* stream);
/* levelset.dilate (levelset.py:25-34); tmp is a same-size scratch grid. */
int svie_dilate(const uint8_t* mask, int nx, int ny, int nz, int steps, uint8_t* out, uint8_t* tmp,
                void* stream);

/* ------------------------------------------------------------------ SDF */
/* mesh_to_sdf (svierosion/sdf.py:365-415).  tri: (T,3,3) float32 and tri64:
 * (T,3,3) float64 triangle vertices in index coordinates (after
 * split_long_triangles).  keys: dense int64 (dist bits << 32 | id),
 * initialised to INT64_MAX by svie_sdf_keys_init. */
int svie_sdf_keys_init(int64_t* keys, int64_t n, void* stream);
/* _exact_near_field (sdf.py:100-145): nodes within exact_band cells of a
 * triangle's bounding box, kept when dist <= eb_keep.  A warp takes 32
 * triangles; `slices` (1-32) warps share them (more for larger triangles). */
int svie_sdf_near_field(const float* tri, const double* tri64, int64_t ntri, int nx, int ny, int nz,
                        double exact_band, float eb_keep, int slices, int64_t* keys, void* stream);
/* keys -> dist (inf where empty), tid (-1 where empty), known mask */
int svie_sdf_unpack(const int64_t* keys, int64_t n, float* dist, int32_t* tid, uint8_t* known,
                    void* stream);
/* _propagate (sdf.py:163-202), one ring: ring = dilate26(known) & ~known
 * without the outer grid layer; update = best over the neighbours' closest
 * triangles (new values into new_dist/new_tid); scatter writes them back and
 * marks the nodes known. */
int svie_sdf_ring_mask(const uint8_t* known, int nx, int ny, int nz, uint8_t* ring, void* stream);
/* The same ring from the previous ring's node list `last` (m nodes): ring = 1 at the unknown
 * interior neighbours of those nodes, 0 elsewhere.  For every ring after the first this is
 * svie_sdf_ring_mask's set (an unknown node next to an older known node is in an older ring). */
int svie_sdf_ring_mark(const int32_t* last, int64_t m, const uint8_t* known, int nx, int ny, int nz, uint8_t* ring,
                       void* stream);
int svie_sdf_ring_update(const int32_t* upd, int64_t m, int nx, int ny, int nz, const float* tri,
                         const float* dist, const int32_t* tid, float* new_dist, int32_t* new_tid,
                         void* stream);
int svie_sdf_scatter(const int32_t* upd, int64_t m, const float* new_dist, const int32_t* new_tid,
                     float* dist, int32_t* tid, uint8_t* known, void* stream);
/* mask = (dist > lo) & (dist <= hi)  (sdf.py:403) */
int svie_sdf_outer_mask(const float* dist, int64_t n, float lo, float hi, uint8_t* mask, void* stream);
/* _refine_with_stars, one pass (sdf.py:211-265); star CSR: first/deg per
 * vertex, star = triangle ids grouped by vertex; vid (T,3); changed: device
 * int64 counter (accumulated). */
int svie_sdf_star_pass(const int32_t* nodes, int64_t m, int nx, int ny, int nz, const float* tri,
                       const int32_t* vid, const int32_t* first, const int32_t* deg,
                       const int32_t* star, float* dist, int32_t* tid, int64_t* changed,
                       void* stream);
/* _crossings_along_axis (sdf.py:285-340): acc int32 (n_axis+1) x n_b x n_c,
 * zeroed by the caller, accumulates the crossings of the grid lines parallel
 * to `axis`; svie_sdf_inside adds 1 to votes[x,y,z] where the prefix sum says
 * inside (signed_rule = winding number, else parity).  A warp takes 32
 * triangles and their (triangle, line) pairs; `slices` (1-1024) warps share the
 * pairs of one group (more for triangles that cover many lines). */
int svie_sdf_crossings(const double* tri64, int64_t ntri, int nx, int ny, int nz, int axis,
                       int signed_rule, int slices, int32_t* acc, void* stream);
int svie_sdf_inside(const int32_t* acc, int nx, int ny, int nz, int axis, int signed_rule,
                    uint8_t* votes, void* stream);
/* Mesh preprocessing (the host numpy work of sdf.py:205-208,385,398-402
 * and meshio.py:80-105).  svie_mesh_tri_index: triangle soup in index
 * coordinates (T,3,3) float64 and float32 and the longest edge (float bits,
 * atomically maxed into *max_edge_bits, which the caller zeroes). */
int svie_mesh_tri_index(const double* vertices, const int32_t* faces, int64_t T, double ox, double oy,
                        double oz, double h, double* tri64, float* tri32, uint32_t* max_edge_bits,
                        void* stream);
/* Vertex welding (np.unique over rows): ids[i] = representative index of the
 * points exactly equal to point i (-0.0 == +0.0).  *overflow is set if the
 * table is too full (it is sized by svie_mesh_weld_table_bytes). */
size_t svie_mesh_weld_table_bytes(int64_t n);
int svie_mesh_weld(const double* points, int64_t n, void* table, size_t table_bytes, int32_t* ids,
                   int* overflow, void* stream);
/* Vertex stars as CSR over nv vertex ids: vid = weld[faces] (faces NULL: weld
 * is per soup corner), deg, first (exclusive scan), star = triangle ids
 * grouped by vertex; cursor is nv ints of scratch. */
int svie_mesh_stars(const int32_t* faces, const int32_t* weld, int64_t T, int64_t nv, int32_t* vid,
                    int32_t* deg, int32_t* first, int32_t* cursor, int32_t* star, void* stream);
/* Edge topology of the faces as given: out4 = {edges, boundary, non-manifold,
 * misoriented}. */
size_t svie_mesh_edge_table_bytes(int64_t T);
int svie_mesh_edge_topology(const int32_t* faces, int64_t T, void* table, size_t table_bytes,
                            uint64_t* out4, int* overflow, void* stream);
/* Signed volume about the point c (meshio.py:80-83), float64. */
int svie_mesh_signed_volume(const double* vertices, const int32_t* faces, int64_t T, double cx,
                            double cy, double cz, double* out, void* stream);
/* phi = inside ? -(min(dist, band) * h) : +(...), inside = 2*votes > naxes
 * (sdf.py:361, 409-410). */
int svie_sdf_finalize(const float* dist, const uint8_t* votes, int64_t n, int naxes, float band,
                      float h, float* phi, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* SVIE_H */
