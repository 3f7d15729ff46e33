// Per-node stencil and interpolation kernels behind svierosion_gb300.kernels,
// plus the band occupancy scatter and the float64 solid-volume reduction.
//
// One thread per listed node; the node list is sorted, so neighbouring threads
// read neighbouring phi values and the +-stride stencil taps of a warp fall in
// the same few cache lines.  All of these are gather-bound (L2/HBM).
#include "common.cuh"

namespace svie {

constexpr int ST_THREADS = 256;

__global__ void k_godunov(const float* __restrict__ f, const int32_t* __restrict__ idx, long long m,
                          long long sx, long long sy, long long sz, float inv_h, float* __restrict__ out) {
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= m) return;
  out[t] = godunov_at(f, idx[t], sx, sy, sz, inv_h);
}

__global__ void k_fractions(const float* __restrict__ f, const int32_t* __restrict__ idx, long long m,
                            long long sx, long long sy, long long sz, float* __restrict__ out,
                            int scatter) {
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= m) return;
  long long i = idx[t];
  float v = cell_fraction_at(f, i, sx, sy, sz);
  if (scatter) out[i] = v; else out[t] = v;
}

__global__ void k_closest(const float* __restrict__ f, const int32_t* __restrict__ idx, long long m, CpGeom G,
                          float* __restrict__ out) {
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= m) return;
  float3 p = closest_point_at(f, idx[t], G);
  out[3 * t] = p.x;
  out[3 * t + 1] = p.y;
  out[3 * t + 2] = p.z;
}

__global__ void k_tricubic(const float* __restrict__ g, int ny, int nz, const float* __restrict__ p,
                           long long m, float* __restrict__ out) {
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= m) return;
  out[t] = tricubic_at(g, ny, nz, make_float3(p[3 * t], p[3 * t + 1], p[3 * t + 2]));
}

__global__ void k_tricubic_grad(const float* __restrict__ g, int ny, int nz, const float* __restrict__ p,
                                long long m, float* __restrict__ val, float* __restrict__ grad) {
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= m) return;
  float v, gx, gy, gz;
  tricubic_grad_at(g, ny, nz, make_float3(p[3 * t], p[3 * t + 1], p[3 * t + 2]), &v, &gx, &gy, &gz);
  val[t] = v;
  grad[3 * t] = gx;
  grad[3 * t + 1] = gy;
  grad[3 * t + 2] = gz;
}

__global__ void k_trilinear(const float* __restrict__ g, int ny, int nz, const float* __restrict__ p,
                            long long m, float* __restrict__ out) {
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= m) return;
  out[t] = trilinear_at(g, ny, nz, make_float3(p[3 * t], p[3 * t + 1], p[3 * t + 2]), 1, 0);
}

__global__ void k_curvatures(const float* __restrict__ f, const int32_t* __restrict__ idx, long long m,
                             long long sx, long long sy, long long sz, float h, float* __restrict__ k1,
                             float* __restrict__ k2) {
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= m) return;
  float2 k = principal_curvatures_at(f, idx[t], sx, sy, sz, h);
  k1[t] = k.x;
  k2[t] = k.y;
}

__global__ void k_interface(const float* __restrict__ f, const int32_t* __restrict__ idx, long long m,
                            long long sx, long long sy, long long sz, uint8_t* __restrict__ out) {
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= m) return;
  long long i = idx[t];
  float c = __ldg(f + i);
  bool hit = false;
  const long long st[3] = {sx, sy, sz};
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    hit = hit || (__ldg(f + i + st[a]) * c <= 0.0f) || (__ldg(f + i - st[a]) * c <= 0.0f);
  }
  out[t] = hit ? 1 : 0;
}


__global__ void k_pt_tri(const float* __restrict__ p, const float* __restrict__ a, const float* __restrict__ b,
                         const float* __restrict__ c, long long m, float* __restrict__ out) {
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= m) return;
  auto ld = [&](const float* q) { return make_float3(q[3 * t], q[3 * t + 1], q[3 * t + 2]); };
  out[t] = point_triangle_d2(ld(p), ld(a), ld(b), ld(c));
}

// Band volume: per-CTA float64 partial sums of the cell fractions, reduced in a
// fixed order by a second one-CTA kernel (deterministic); also the
// has_interface flags and (optionally) the occupancy scatter.
// One tile (ST_THREADS consecutive band entries, the tile-th) of the band
// volume: its double-float partial into slot `tile`, the interface flags by
// atomics, the cell fractions into occ when given.
SVIE_DEV void volume_tile(long long tile, const float* __restrict__ f, const int32_t* __restrict__ idx, long long m,
                          long long sx, long long sy, long long sz, float* __restrict__ occ, double* partial,
                          svie_stats* stats) {
  __shared__ DF shd[ST_THREADS / 32];
  const long long t = tile * ST_THREADS + threadIdx.x;
  float v = 0.0f;
  int neg = 0, pos = 0;
  if (t < m) {
    const int i = idx[t];
    const float fr = cell_fraction_at(f, i, (int)sx, (int)sy, (int)sz);
    if (occ) occ[i] = fr;
    v = fr;
    const float c = __ldg(f + i);
    neg = c < 0.0f;
    pos = c > 0.0f;
  }
  const DF s = block_sum_df(v, shd);
  const int an = __syncthreads_or(neg), ap = __syncthreads_or(pos);
  if (threadIdx.x == 0) {
    reinterpret_cast<float2*>(partial)[tile] = make_float2(s.hi, s.lo);
    if (an) atomicOr(&stats->any_neg, 1u);
    if (ap) atomicOr(&stats->any_pos, 1u);
  }
}

__global__ void __launch_bounds__(ST_THREADS) k_volume_partial(const float* __restrict__ f,
                                                               const int32_t* __restrict__ idx, long long m,
                                                               long long sx, long long sy, long long sz,
                                                               float* __restrict__ occ, double* partial,
                                                               svie_stats* stats) {
  pdl_wait();
  pdl_release();
  volume_tile(blockIdx.x, f, idx, m, sx, sy, sz, occ, partial, stats);
}

// The per-CTA double-float partials (stored in the 8 bytes of a double each)
// summed in a fixed order: deterministic run to run.
__global__ void __launch_bounds__(SUM_THREADS) k_sum_partials(const double* partial, long long nb, double* out) {
  pdl_wait();
  pdl_release();
  __shared__ DF sh[SUM_THREADS / 32];
  const DF s = block_sum_partials_df(reinterpret_cast<const float2*>(partial), nb, sh);
  if (threadIdx.x == 0) *out = df_value(s);
}

__global__ void k_clear_flags(svie_stats* stats, unsigned int n_band) {
  pdl_wait();
  pdl_release();
  stats->any_neg = 0;
  stats->any_pos = 0;
  stats->n_band = n_band;
}

}  // namespace svie

using namespace svie;

#define SVIE_CHECK_M(name, m)                                 \
  if ((m) < 0) {                                              \
    set_error("%s: negative size", name);                     \
    return SVIE_ERR_ARG;                                      \
  }                                                           \
  if ((m) == 0) return SVIE_OK;

extern "C" {

int svie_godunov_inward(const float* flat, const int32_t* idx, int64_t m, int64_t sx, int64_t sy,
                        int64_t sz, float inv_h, float* out, void* stream) {
  SVIE_CHECK_M("svie_godunov_inward", m);
  k_godunov<<<blocks_for(m, ST_THREADS), ST_THREADS, 0, (cudaStream_t)stream>>>(flat, idx, m, sx, sy, sz,
                                                                                 inv_h, out);
  return launch_status("svie_godunov_inward");
}

int svie_cell_fractions(const float* flat, const int32_t* idx, int64_t m, int64_t sx, int64_t sy,
                        int64_t sz, float* out, void* stream) {
  SVIE_CHECK_M("svie_cell_fractions", m);
  k_fractions<<<blocks_for(m, ST_THREADS), ST_THREADS, 0, (cudaStream_t)stream>>>(flat, idx, m, sx, sy, sz,
                                                                                   out, 0);
  return launch_status("svie_cell_fractions");
}

int svie_scatter_fractions(const float* phi, const int32_t* band, int64_t m, int64_t sx, int64_t sy,
                           int64_t sz, float* occ, void* stream) {
  SVIE_CHECK_M("svie_scatter_fractions", m);
  k_fractions<<<blocks_for(m, ST_THREADS), ST_THREADS, 0, (cudaStream_t)stream>>>(phi, band, m, sx, sy, sz,
                                                                                   occ, 1);
  return launch_status("svie_scatter_fractions");
}

int svie_closest_points(const float* flat, const int32_t* idx, int64_t m, int ny, int nz, float hi_x,
                        float hi_y, float hi_z, float h, float* out, void* stream) {
  SVIE_CHECK_M("svie_closest_points", m);
  k_closest<<<blocks_for(m, ST_THREADS), ST_THREADS, 0, (cudaStream_t)stream>>>(
      flat, idx, m, cp_geom(ny, nz, hi_x, hi_y, hi_z, h), out);
  return launch_status("svie_closest_points");
}

int svie_tricubic(const float* flat, int ny, int nz, const float* p, int64_t m, float* out, void* stream) {
  SVIE_CHECK_M("svie_tricubic", m);
  k_tricubic<<<blocks_for(m, ST_THREADS), ST_THREADS, 0, (cudaStream_t)stream>>>(flat, ny, nz, p, m, out);
  return launch_status("svie_tricubic");
}

int svie_tricubic_with_gradient(const float* flat, int ny, int nz, const float* p, int64_t m, float* val,
                                float* grad, void* stream) {
  SVIE_CHECK_M("svie_tricubic_with_gradient", m);
  k_tricubic_grad<<<blocks_for(m, ST_THREADS), ST_THREADS, 0, (cudaStream_t)stream>>>(flat, ny, nz, p, m,
                                                                                       val, grad);
  return launch_status("svie_tricubic_with_gradient");
}

int svie_trilinear(const float* flat, int ny, int nz, const float* p, int64_t m, float* out, void* stream) {
  SVIE_CHECK_M("svie_trilinear", m);
  k_trilinear<<<blocks_for(m, ST_THREADS), ST_THREADS, 0, (cudaStream_t)stream>>>(flat, ny, nz, p, m, out);
  return launch_status("svie_trilinear");
}

int svie_principal_curvatures(const float* flat, const int32_t* idx, int64_t m, int64_t sx, int64_t sy,
                              int64_t sz, float h, float* k1, float* k2, void* stream) {
  SVIE_CHECK_M("svie_principal_curvatures", m);
  k_curvatures<<<blocks_for(m, ST_THREADS), ST_THREADS, 0, (cudaStream_t)stream>>>(flat, idx, m, sx, sy, sz,
                                                                                    h, k1, k2);
  return launch_status("svie_principal_curvatures");
}

int svie_interface_mask(const float* flat, const int32_t* idx, int64_t m, int64_t sx, int64_t sy,
                        int64_t sz, uint8_t* out, void* stream) {
  SVIE_CHECK_M("svie_interface_mask", m);
  k_interface<<<blocks_for(m, ST_THREADS), ST_THREADS, 0, (cudaStream_t)stream>>>(flat, idx, m, sx, sy, sz,
                                                                                   out);
  return launch_status("svie_interface_mask");
}

int svie_point_triangle_distance2(const float* p, const float* a, const float* b, const float* c, int64_t m,
                                  float* out, void* stream) {
  SVIE_CHECK_M("svie_point_triangle_distance2", m);
  k_pt_tri<<<blocks_for(m, ST_THREADS), ST_THREADS, 0, (cudaStream_t)stream>>>(p, a, b, c, m, out);
  return launch_status("svie_point_triangle_distance2");
}

size_t svie_volume_workspace_bytes(int64_t m) {
  long long nb = (m + ST_THREADS - 1) / ST_THREADS;
  if (nb < 1) nb = 1;
  return (size_t)nb * sizeof(double) + 256;
}

int svie_band_volume(const float* phi, const int32_t* band, int64_t m, int64_t sx, int64_t sy, int64_t sz,
                     float* occ, void* ws, size_t ws_bytes, svie_stats* stats, void* stream) {
  if (m < 0 || !stats || m >= (1LL << 31)) {
    set_error("svie_band_volume: bad arguments");
    return SVIE_ERR_ARG;
  }
  if (!ws || ws_bytes < svie_volume_workspace_bytes(m)) {
    set_error("svie_band_volume: workspace too small");
    return SVIE_ERR_WORKSPACE;
  }
  cudaStream_t s = (cudaStream_t)stream;
  long long nb = (m + ST_THREADS - 1) / ST_THREADS;
  cudaError_t e = launch_dependent(false, k_clear_flags, dim3(1), dim3(1), 0, s, stats, (unsigned)m);
  if (nb > 0 && e == cudaSuccess)
    e = launch_dependent(true, k_volume_partial, dim3((unsigned)nb), dim3(ST_THREADS), 0, s, phi, band,
                         (long long)m, (long long)sx, (long long)sy, (long long)sz, occ, (double*)ws, stats);
  if (e == cudaSuccess)
    e = launch_dependent(true, k_sum_partials, dim3(1), dim3(SUM_THREADS), 0, s, (const double*)ws, nb,
                         &stats->fsum);
  return dependent_status(e, "svie_band_volume", nb > 0 ? 3 : 2);
}

}  // extern "C"

// ------------------------------------------------------------ API helpers
namespace svie {

__global__ void k_central_gradient(const float* __restrict__ f, const int32_t* __restrict__ idx, long long m,
                                   long long sx, long long sy, long long sz, float* __restrict__ out) {
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= m) return;
  long long i = idx[t];
  out[3 * t] = 0.5f * (__ldg(f + i + sx) - __ldg(f + i - sx));
  out[3 * t + 1] = 0.5f * (__ldg(f + i + sy) - __ldg(f + i - sy));
  out[3 * t + 2] = 0.5f * (__ldg(f + i + sz) - __ldg(f + i - sz));
}

// LevelSet.closest_points with newton_steps >= 1 (levelset.py:129-151): the
// first projection from the central gradient, then Newton steps on the
// tricubic interpolant with the same step cap, clamped to [1, n - 3.001].
__global__ void k_closest_newton(const float* __restrict__ f, const int32_t* __restrict__ idx, long long m, int ny,
                                 int nz, CpGeom G, int steps, float* __restrict__ out) {
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= m) return;
  float3 p = closest_point_at(f, idx[t], G);
  const float hx = G.hx, hy = G.hy, hz = G.hz, h = G.h;
  const long long syz = (long long)ny * nz;
  for (int s = 1; s < steps; ++s) {
    float fx = floorf(p.x), fy = floorf(p.y), fz = floorf(p.z);
    float wx[4], wy[4], wz[4], dx[4], dy[4], dz[4];
    cubic_w(p.x - fx, wx); cubic_w(p.y - fy, wy); cubic_w(p.z - fz, wz);
    cubic_dw(p.x - fx, dx); cubic_dw(p.y - fy, dy); cubic_dw(p.z - fz, dz);
    const long long b0 = ((long long)fx - 1) * syz + ((long long)fy - 1) * nz + ((long long)fz - 1);
    float v = 0.f, gx = 0.f, gy = 0.f, gz = 0.f;
    for (int a = 0; a < 4; ++a)
      for (int b = 0; b < 4; ++b)
        for (int c = 0; c < 4; ++c) {
          float q = __ldg(f + b0 + a * syz + b * nz + c);
          v = v + wx[a] * wy[b] * wz[c] * q;
          gx = gx + dx[a] * wy[b] * wz[c] * q;
          gy = gy + wx[a] * dy[b] * wz[c] * q;
          gz = gz + wx[a] * wy[b] * dz[c] * q;
        }
    float g2 = fmaxf(gx * gx + gy * gy + gz * gz, 1e-30f);
    float length = fabsf(v) / sqrtf(g2);
    float cap = 1.25f * fabsf(v) / h + 0.25f;
    float sc = v / g2 * fminf(cap / fmaxf(length, 1e-30f), 1.0f);
    p.x = fminf(fmaxf(p.x - sc * gx, 1.0f), hx);
    p.y = fminf(fmaxf(p.y - sc * gy, 1.0f), hy);
    p.z = fminf(fmaxf(p.z - sc * gz, 1.0f), hz);
  }
  out[3 * t] = p.x;
  out[3 * t + 1] = p.y;
  out[3 * t + 2] = p.z;
}

__global__ void k_gather(const float* __restrict__ src, const int32_t* __restrict__ idx, long long m,
                         float* __restrict__ out) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < m) out[t] = __ldg(src + __ldg(idx + t));
}

__global__ void k_cube_plane(const float* __restrict__ s, const float* __restrict__ a, const float* __restrict__ b,
                             const float* __restrict__ c, long long m, float* __restrict__ out) {
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= m) return;
  out[t] = cube_plane_fraction(s[t], a[t], b[t], c[t]);
}

}  // namespace svie

extern "C" {

int svie_central_gradient(const float* flat, const int32_t* idx, int64_t m, int64_t sx, int64_t sy, int64_t sz,
                          float* out, void* stream) {
  SVIE_CHECK_M("svie_central_gradient", m);
  k_central_gradient<<<blocks_for(m, ST_THREADS), ST_THREADS, 0, (cudaStream_t)stream>>>(flat, idx, m, sx, sy, sz,
                                                                                          out);
  return launch_status("svie_central_gradient");
}

int svie_closest_points_newton(const float* flat, const int32_t* idx, int64_t m, int ny, int nz, float hi_x,
                               float hi_y, float hi_z, float h, int newton_steps, float* out, void* stream) {
  SVIE_CHECK_M("svie_closest_points_newton", m);
  if (newton_steps < 1) {
    set_error("svie_closest_points_newton: newton_steps must be >= 1");
    return SVIE_ERR_ARG;
  }
  k_closest_newton<<<blocks_for(m, ST_THREADS), ST_THREADS, 0, (cudaStream_t)stream>>>(
      flat, idx, m, ny, nz, cp_geom(ny, nz, hi_x, hi_y, hi_z, h), newton_steps, out);
  return launch_status("svie_closest_points_newton");
}

int svie_gather(const float* src, const int32_t* idx, int64_t m, float* out, void* stream) {
  SVIE_CHECK_M("svie_gather", m);
  if (m > 0 && (!src || !idx || !out)) {
    set_error("svie_gather: null pointer");
    return SVIE_ERR_ARG;
  }
  k_gather<<<blocks_for(m, ST_THREADS), ST_THREADS, 0, (cudaStream_t)stream>>>(src, idx, m, out);
  return launch_status("svie_gather");
}

int svie_cube_plane_fraction(const float* s, const float* a, const float* b, const float* c, int64_t m, float* out,
                             void* stream) {
  SVIE_CHECK_M("svie_cube_plane_fraction", m);
  k_cube_plane<<<blocks_for(m, ST_THREADS), ST_THREADS, 0, (cudaStream_t)stream>>>(s, a, b, c, m, out);
  return launch_status("svie_cube_plane_fraction");
}

}  // extern "C"

namespace svie {
__global__ void k_dense_occ(const float* __restrict__ phi, long long n, float* __restrict__ occ) {
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x)
    occ[e] = phi[e] < 0.0f ? 1.0f : 0.0f;
}
}  // namespace svie

// occ = (phi < 0) on every node (the dense part of levelset.py:119).
extern "C" int svie_dense_occupancy(const float* phi, int64_t n, float* occ, void* stream) {
  if (!phi || !occ || n <= 0) {
    svie::set_error("svie_dense_occupancy: bad arguments");
    return SVIE_ERR_ARG;
  }
  svie::k_dense_occ<<<svie::blocks_for(n, 256, 152 * 32), 256, 0, (cudaStream_t)stream>>>(phi, n, occ);
  return svie::launch_status("svie_dense_occupancy");
}

// ------------------------------------------------- allocation-free volume
// svie_band_volume_noalloc: the same float64 volume reduction as
// svie_band_volume, for callers that must not allocate device memory and have
// no workspace to hand over -- for example a plugin living inside a host
// framework whose own memory pool owns every device allocation, or a
// latency-critical loop that forbids cudaMalloc after start-up because the
// allocator may synchronise the device.  Its scratch (one float64 partial sum
// per CTA) is the file-scope array below, which every GPU that loads this
// library keeps for the life of the process.
#include <mutex>

namespace svie {

constexpr long long VOLUME_NOALLOC_MAX_CTAS = 65536;  // 512 KiB of float64 partial sums

static __device__ __align__(256) double g_volume_partials[VOLUME_NOALLOC_MAX_CTAS];

static std::mutex g_volume_symbol_mutex;

// One resolved address per (device, context).  A driver-API context made
// current by a host framework loads this library's module anew, so the array
// has another address there; the context handle tells the cases apart.  A
// context destroyed and created again (cudaDeviceReset) may reuse its old
// handle value, which this cache cannot tell from the old context: callers
// must not reset the device between calls.
struct VolumeSymbol {
  int dev;
  void* ctx;
  double* addr;
};
static VolumeSymbol g_volume_symbol[64];
static int g_volume_symbol_n = 0;

typedef int (*CtxGetCurrentFn)(void**);

// The current context's handle through the driver entry point (no link to
// libcuda); nullptr when it cannot be had, and then the device alone keys the
// cache.  Called with g_volume_symbol_mutex held.
static void* current_context() {
  static CtxGetCurrentFn fn = nullptr;
  static bool tried = false;
  if (!tried) {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = (CtxGetCurrentFn)f;
    tried = true;
  }
  void* ctx = nullptr;
  if (fn && fn(&ctx) != 0) ctx = nullptr;
  return ctx;
}

// Device address of g_volume_partials in the current device's context, looked
// up once per device and context (the array's name in host code is only a
// stand-in for the symbol).
static int volume_partials_address(double** out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0) {
    set_error("svie_band_volume_noalloc: no usable current CUDA device");
    return SVIE_ERR_LAUNCH;
  }
  std::lock_guard<std::mutex> lock(g_volume_symbol_mutex);
  // nullptr while no context is current: the runtime then works in the
  // device's primary context, which that key stands for
  void* ctx = current_context();
  for (int i = 0; i < g_volume_symbol_n; ++i) {
    if (g_volume_symbol[i].dev == dev && g_volume_symbol[i].ctx == ctx) {
      *out = g_volume_symbol[i].addr;
      return SVIE_OK;
    }
  }
  void* p = nullptr;
  const cudaError_t e = cudaGetSymbolAddress(&p, g_volume_partials);
  if (e != cudaSuccess || !p) {
    set_error("svie_band_volume_noalloc: cudaGetSymbolAddress failed: %s", cudaGetErrorString(e));
    return SVIE_ERR_LAUNCH;
  }
  // a full table (more than 64 device/context pairs) keeps working uncached
  if (g_volume_symbol_n < 64) g_volume_symbol[g_volume_symbol_n++] = VolumeSymbol{dev, ctx, (double*)p};
  *out = (double*)p;
  return SVIE_OK;
}

}  // namespace svie

extern "C" {

int64_t svie_band_volume_noalloc_max(void) { return (int64_t)svie::VOLUME_NOALLOC_MAX_CTAS * svie::ST_THREADS; }

int svie_band_volume_noalloc(const float* phi, const int32_t* band, int64_t m, int64_t sx, int64_t sy, int64_t sz,
                             float* occ, svie_stats* stats, void* stream) {
  using namespace svie;
  // the size limit is checked first, before any pointer is looked at
  if (m > svie_band_volume_noalloc_max()) {
    set_error("svie_band_volume_noalloc: %lld band nodes exceed the static scratch limit of %lld; use "
              "svie_band_volume with a workspace", (long long)m, (long long)svie_band_volume_noalloc_max());
    return SVIE_ERR_CAPACITY;
  }
  if (m < 0 || !stats || (m > 0 && (!phi || !band))) {
    set_error("svie_band_volume_noalloc: bad arguments");
    return SVIE_ERR_ARG;
  }
  double* partials = nullptr;
  int st = volume_partials_address(&partials);
  if (st) return st;
  cudaStream_t s = (cudaStream_t)stream;
  const long long nb = (m + ST_THREADS - 1) / ST_THREADS;
  k_clear_flags<<<1, 1, 0, s>>>(stats, (unsigned)m);
  // every CTA overwrites its own partial, and the sum reads exactly those nb
  // entries, so nothing left from an earlier call is read
  if (nb > 0)
    k_volume_partial<<<(unsigned)nb, ST_THREADS, 0, s>>>(phi, band, m, sx, sy, sz, occ, partials, stats);
  k_sum_partials<<<1, SUM_THREADS, 0, s>>>(partials, nb, &stats->fsum);
  return launch_status("svie_band_volume_noalloc", nb > 0 ? 3 : 2);
}

}  // extern "C"

// ------------------------------------------------ many level sets in one launch
namespace svie {

static_assert(ST_THREADS == GROUP_TILE, "group tiles are the volume kernel's CTAs");

__global__ void __launch_bounds__(GROUP_TILE) k_group_fractions(const void* table, int n) {
  const int2 tl = ((const int2*)((const char*)table + group_tiles_offset(n)))[blockIdx.x];
  const GroupInst* I = (const GroupInst*)table + tl.x;
  const long long t = (long long)tl.y * GROUP_TILE + threadIdx.x;
  if (t >= I->m) return;
  const long long syz = (long long)I->ny * I->nz;
  const int i = I->band[t];
  I->occ[i] = cell_fraction_at(I->phi, i, syz, I->nz, 1);
}

__global__ void k_group_clear_flags(const void* table, int n) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const GroupInst* I = (const GroupInst*)table + k;
  I->vstats->any_neg = 0;
  I->vstats->any_pos = 0;
  I->vstats->n_band = (unsigned)I->m;
}

__global__ void __launch_bounds__(GROUP_TILE) k_group_volume_partial(const void* table, int n) {
  __shared__ GroupInst I;
  const int2 tl = ((const int2*)((const char*)table + group_tiles_offset(n)))[blockIdx.x];
  load_group_inst(I, (const GroupInst*)table + tl.x);
  volume_tile(tl.y, I.phi, I.band, I.m, (long long)I.ny * I.nz, I.nz, 1, I.occ, I.vol_part, I.vstats);
}

// one CTA per member
__global__ void __launch_bounds__(SUM_THREADS) k_group_sum_partials(const void* table) {
  __shared__ DF sh[SUM_THREADS / 32];
  const GroupInst* I = (const GroupInst*)table + blockIdx.x;
  const long long nb = (I->m + GROUP_TILE - 1) / GROUP_TILE;
  const DF s = block_sum_partials_df(reinterpret_cast<const float2*>(I->vol_part), nb, sh);
  if (threadIdx.x == 0) I->vstats->fsum = df_value(s);
}

}  // namespace svie

extern "C" {

int svie_group_scatter_fractions(const svie_group* g, void* stream) {
  if (!g || g->n < 0 || (g->n > 0 && !g->table) || g->tiles_svi < 0) {
    set_error("svie_group_scatter_fractions: bad group");
    return SVIE_ERR_ARG;
  }
  if (g->tiles_svi == 0) return SVIE_OK;
  k_group_fractions<<<(unsigned)g->tiles_svi, GROUP_TILE, 0, (cudaStream_t)stream>>>(g->table, g->n);
  return launch_status("svie_group_scatter_fractions");
}

int svie_group_volume(const svie_group* g, void* stream) {
  if (!g || g->n < 0 || (g->n > 0 && !g->table) || g->tiles < 0) {
    set_error("svie_group_volume: bad group");
    return SVIE_ERR_ARG;
  }
  if (g->n == 0) return SVIE_OK;
  cudaStream_t s = (cudaStream_t)stream;
  k_group_clear_flags<<<(g->n + 127) / 128, 128, 0, s>>>(g->table, g->n);
  if (g->tiles > 0) k_group_volume_partial<<<(unsigned)g->tiles, GROUP_TILE, 0, s>>>(g->table, g->n);
  k_group_sum_partials<<<g->n, SUM_THREADS, 0, s>>>(g->table);
  return launch_status("svie_group_volume", g->tiles > 0 ? 3 : 2);
}

}  // extern "C"
