// Fused right-hand side of one TVD-RK3 stage on the narrow band
// (reference svierosion/evolve.py:118-179).
//
// SVI law, one thread per band node:
//   closest point (7-point stencil) -> tricubic N at it (64 taps of the dense N
//   field) -> speed law (t - N in float64 when s = 1) -> statistics ->
//   smoothstep cutoff -> WENO5/Godunov |grad phi| (19 taps) -> L = V |grad phi|.
// Curvature laws replace the N lookup by principal curvatures scattered into an
// interleaved dense (k1, k2) field and trilinear lookups at the closest point.
//
// Statistics: maxima/minima with one atomic per CTA on order-preserving
// integer keys (exact, order independent); sums as per-CTA float64 partials
// reduced in a fixed order, so every run gives the same bits.
#include "common.cuh"

namespace svie {

constexpr int SG_THREADS = 256;

static StageConst stage_const(const svie_law& L, int nx, int ny, int nz) {
  StageConst c;
  c.h = (float)L.h;
  c.inv_h = (float)(1.0 / L.h);
  c.hx = (float)(nx - 3.001);
  c.hy = (float)(ny - 3.001);
  c.hz = (float)(nz - 3.001);
  c.n_cap = (float)L.n_cap;
  c.eps = (float)L.eps;
  c.cut_b = (float)L.cut_b;
  c.cut_scale = (float)(1.0 / (L.cut_b - L.cut_a));
  c.t = (float)L.t;
  c.alpha = (float)L.alpha;
  c.am1 = (float)(L.alpha - 1.0);
  c.am2 = (float)(L.alpha - 2.0);
  c.delta = (float)L.delta;
  c.amode = L.alpha == 1.0 ? 0 : (L.alpha < 1.0 ? 1 : 2);
  c.cp = cp_geom(ny, nz, c.hx, c.hy, c.hz, c.h);
  return c;
}

SVIE_DEV float powk(float x, int k) {
  if (k == 0) return 1.0f;
  if (k == 1) return x;
  if (k == 2) return x * x;
  if (k == 3) return x * x * x;
  return powf(x, (float)k);
}

// SVIPowerLaw.speed (flows.py:89-96).  t - N in float32 with t rounded to
// float, as the reference computes it on float32 tensors (N <= n_cap < t, so
// the difference stays well away from zero).
SVIE_DEV float svi_speed(float N, const svie_law& L, const StageConst& C) {
  N = fminf(fmaxf(N, 0.0f), 1.0f);
  float V;
  if (L.s) {
    N = fminf(N, C.n_cap);
    V = powk(N, L.k) / (C.t - N);
  } else {
    V = L.k ? powk(N, L.k) : 1.0f;
  }
  return C.eps != 0.0f ? V + C.eps : V;
}

// SVIPowerLaw.dspeed (flows.py:98-108)
SVIE_DEV float svi_dspeed(float N, const svie_law& L, const StageConst& C) {
  N = fminf(fmaxf(N, 1e-12f), 1.0f);
  if (L.s) {
    N = fminf(N, C.n_cap);
    const float d = C.t - N;
    const float V = powk(N, L.k) / d;
    return V * ((float)L.k / N + 1.0f / d);
  }
  if (L.k == 0) return 0.0f;
  return (float)L.k * powk(N, L.k - 1);
}

// _CurvatureLaw._power / _dpower (flows.py:139-158)
SVIE_DEV float curv_power(float x, const StageConst& C) {
  if (C.amode == 0) return x;
  if (C.amode == 1) return x * powf(x + C.delta, C.am1);
  return powf(x, C.alpha);
}
SVIE_DEV float curv_dpower(float x, const StageConst& C) {
  if (C.amode == 0) return 1.0f;
  if (C.amode == 1) {
    float y = x + C.delta;
    return powf(y, C.am2) * (C.alpha * x + C.delta);
  }
  return C.alpha * powf(fmaxf(x, 0.0f), C.am1);
}

// Speed and diffusivity of the curvature laws (flows.py:170-206).
SVIE_DEV void curv_speed(float k1, float k2, const svie_law& L, const StageConst& C, float* V, float* D) {
  if (L.kind == 1) {
    float H = 0.5f * (k1 + k2);
    float Hp = fmaxf(H, 0.0f);
    *V = curv_power(Hp, C) + C.eps;
    *D = H > 0.0f ? curv_dpower(Hp, C) : 0.0f;
  } else {
    float a = fmaxf(k1, 0.0f), b = fmaxf(k2, 0.0f);
    float Kc = a * b;
    *V = curv_power(Kc, C) + C.eps;
    float dF = curv_dpower(Kc, C);
    *D = Kc > 0.0f ? dF * (a + b) : dF * 0.0f;
  }
}

// Smoothstep cutoff (evolve.py:108-112): t = clamp((b - |phi|)/(b - a), 0, 1).
SVIE_DEV float cutoff(float phi, const StageConst& C) {
  float x = fabsf(phi);
  float t = (C.cut_b - x) * C.cut_scale;
  t = fminf(fmaxf(t, 0.0f), 1.0f);
  return t * t * (3.0f - 2.0f * t);
}

struct StatAcc {
  float vmax;          // after cutoff, all nodes
  float qmin_n, qmax_n, qmin_a, qmax_a;
  float dv_n, dv_a;    // dspeed (svi) or diffusivity (curvature)
  unsigned int cap_n, cap_a, n_near;
  float vs_n, vs_a;    // V of this node (summed with compensated block sums)
};

SVIE_DEV void stat_init(StatAcc& s) {
  s.vmax = 0.0f;
  s.qmin_n = s.qmin_a = INFINITY;
  s.qmax_n = s.qmax_a = -INFINITY;
  s.dv_n = s.dv_a = 0.0f;
  s.cap_n = s.cap_a = s.n_near = 0;
  s.vs_n = s.vs_a = 0.0f;
}

// Per-CTA reduction of the statistics and one atomic / partial write per CTA:
// every quantity is reduced across its warp first, then warp 0 combines the
// warps after a single barrier.  Maxima, minima and counts are exact in any
// order; the two float64 partials are added in warp order.
SVIE_DEV void stat_commit(StatAcc& a, svie_stats* st, double* partial, long long tile) {
  constexpr int NW = SG_THREADS / 32;
  __shared__ float shf[7][NW];
  __shared__ unsigned int shu[3][NW];
  __shared__ DF shd[2][NW];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  float f[7] = {a.vmax, a.qmin_n, a.qmax_n, a.qmin_a, a.qmax_a, a.dv_n, a.dv_a};
  unsigned int u[3] = {a.cap_n, a.cap_a, a.n_near};
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
    for (int k = 0; k < 7; ++k) {
      const float w = __shfl_xor_sync(0xffffffffu, f[k], o);
      f[k] = (k == 1 || k == 3) ? fminf(f[k], w) : fmaxf(f[k], w);
    }
#pragma unroll
    for (int k = 0; k < 3; ++k) u[k] += __shfl_xor_sync(0xffffffffu, u[k], o);
  }
  const DF d0 = warp_sum_df(DF{a.vs_n, 0.0f}), d1 = warp_sum_df(DF{a.vs_a, 0.0f});
  if (lane == 0) {
#pragma unroll
    for (int k = 0; k < 7; ++k) shf[k][wid] = f[k];
#pragma unroll
    for (int k = 0; k < 3; ++k) shu[k][wid] = u[k];
    shd[0][wid] = d0;
    shd[1][wid] = d1;
  }
  __syncthreads();
  if (wid != 0) return;
  const bool in = lane < NW;
  const float fid[7] = {0.0f, INFINITY, -INFINITY, INFINITY, -INFINITY, 0.0f, 0.0f};
#pragma unroll
  for (int k = 0; k < 7; ++k) f[k] = in ? shf[k][lane] : fid[k];
#pragma unroll
  for (int k = 0; k < 3; ++k) u[k] = in ? shu[k][lane] : 0u;
#pragma unroll
  for (int o = NW / 2; o > 0; o >>= 1) {
#pragma unroll
    for (int k = 0; k < 7; ++k) {
      const float w = __shfl_xor_sync(0xffffffffu, f[k], o);
      f[k] = (k == 1 || k == 3) ? fminf(f[k], w) : fmaxf(f[k], w);
    }
#pragma unroll
    for (int k = 0; k < 3; ++k) u[k] += __shfl_xor_sync(0xffffffffu, u[k], o);
  }
  if (lane != 0) return;
  if (f[0] > 0.0f) atomicMax(&st->vmax, __float_as_uint(f[0]));
  if (f[1] < INFINITY) atomicMin(&st->qmin_near, float_to_ordered(f[1]));
  if (f[2] > -INFINITY) atomicMax(&st->qmax_near, float_to_ordered(f[2]));
  if (f[3] < INFINITY) atomicMin(&st->qmin_all, float_to_ordered(f[3]));
  if (f[4] > -INFINITY) atomicMax(&st->qmax_all, float_to_ordered(f[4]));
  if (f[5] > 0.0f) atomicMax(&st->dvmax_near, __float_as_uint(f[5]));
  if (f[6] > 0.0f) atomicMax(&st->dvmax_all, __float_as_uint(f[6]));
  if (u[0]) atomicAdd(&st->capped_near, u[0]);
  if (u[1]) atomicAdd(&st->capped_all, u[1]);
  if (u[2]) atomicAdd(&st->n_near, u[2]);
  DF r0 = shd[0][0], r1 = shd[1][0];
  for (int i = 1; i < NW; ++i) {
    r0 = df_add(r0, shd[0][i]);
    r1 = df_add(r1, shd[1][i]);
  }
  // double-float partials, two per CTA (near, all), in the 16 bytes of two doubles
  float2* pp = reinterpret_cast<float2*>(partial);
  pp[2 * tile] = make_float2(r0.hi, r0.lo);
  pp[2 * tile + 1] = make_float2(r1.hi, r1.lo);
}

// One tile (SG_THREADS consecutive band entries, the tile-th) of the SVI stage;
// the statistics partial of the tile goes to slot `tile` of `partial`.
SVIE_DEV void stage_svi_tile(long long tile, const float* __restrict__ phi, const int32_t* __restrict__ band,
                             long long m, int ny, int nz, const float* __restrict__ Nd, const svie_law& L,
                             const StageConst& C, float* __restrict__ Lout, float* __restrict__ u0,
                             float* __restrict__ Vout, svie_stats* st, double* partial) {
  const long long t = tile * SG_THREADS + threadIdx.x;
  const int syz = ny * nz;
  StatAcc acc;
  if (st) stat_init(acc);
  if (t < m) {
    const int i = band[t];
    const float c = __ldg(phi + i);
    const float3 p = closest_point_at(phi, i, C.cp);
    const float N = tricubic_at(Nd, ny, nz, p);
    float V = svi_speed(N, L, C);
    if (st) {
      const bool near = fabsf(c) < C.h;
      const float dv = svi_dspeed(N, L, C);
      const bool capped = N > C.n_cap;
      acc.qmin_a = N; acc.qmax_a = N; acc.dv_a = dv; acc.cap_a = capped; acc.vs_a = V;
      if (near) {
        acc.qmin_n = N; acc.qmax_n = N; acc.dv_n = dv; acc.cap_n = capped; acc.vs_n = V; acc.n_near = 1;
      }
    }
    V = V * cutoff(c, C);
    const float G = godunov_at(phi, i, syz, nz, 1, C.inv_h);
    Lout[t] = V * G;
    if (u0) u0[t] = c;
    if (Vout) Vout[t] = V;
    if (st) acc.vmax = V;
  }
  if (st) stat_commit(acc, st, partial, tile);
}

__global__ void __launch_bounds__(SG_THREADS, 6) k_stage_svi(const float* __restrict__ phi,
                                                          const int32_t* __restrict__ band, long long m, int nx,
                                                          int ny, int nz, const float* __restrict__ Nd,
                                                          svie_law L, StageConst C, float* __restrict__ Lout,
                                                          float* __restrict__ u0, float* __restrict__ Vout,
                                                          svie_stats* st, double* partial) {
  stage_svi_tile(blockIdx.x, phi, band, m, ny, nz, Nd, L, C, Lout, u0, Vout, st, partial);
}

SVIE_DEV void curv_scatter_tile(long long tile, const float* __restrict__ phi, const int32_t* __restrict__ band,
                                long long m, int ny, int nz, float h, float* __restrict__ kd) {
  const long long t = tile * SG_THREADS + threadIdx.x;
  if (t >= m) return;
  const int i = band[t];
  reinterpret_cast<float2*>(kd)[i] = principal_curvatures_at(phi, i, ny * nz, nz, 1, h);
}

__global__ void k_curv_scatter(const float* __restrict__ phi, const int32_t* __restrict__ band, long long m,
                               int ny, int nz, float h, float* __restrict__ kd) {
  curv_scatter_tile(blockIdx.x, phi, band, m, ny, nz, h, kd);
}

SVIE_DEV void stage_curv_tile(long long tile, const float* __restrict__ phi, const int32_t* __restrict__ band,
                              long long m, int ny, int nz, const float* __restrict__ kd, const svie_law& L,
                              const StageConst& C, float* __restrict__ Lout, float* __restrict__ u0,
                              float* __restrict__ Vout, svie_stats* st, double* partial) {
  const long long t = tile * SG_THREADS + threadIdx.x;
  const int syz = ny * nz;
  StatAcc acc;
  if (st) stat_init(acc);
  if (t < m) {
    const int i = band[t];
    const float c = __ldg(phi + i);
    const float3 p = closest_point_at(phi, i, C.cp);
    const float2 kk = trilinear2_at(reinterpret_cast<const float2*>(kd), ny, nz, p);
    const float k1 = kk.x, k2 = kk.y;
    float V, D;
    curv_speed(k1, k2, L, C, &V, &D);
    if (st) {
      const bool near = fabsf(c) < C.h;
      const float H = 0.5f * (k1 + k2);
      acc.qmin_a = H; acc.qmax_a = H; acc.dv_a = D; acc.vs_a = V;
      if (near) { acc.qmin_n = H; acc.qmax_n = H; acc.dv_n = D; acc.vs_n = V; acc.n_near = 1; }
    }
    V = V * cutoff(c, C);
    const float G = godunov_at(phi, i, syz, nz, 1, C.inv_h);
    Lout[t] = V * G;
    if (u0) u0[t] = c;
    if (Vout) Vout[t] = V;
    if (st) acc.vmax = V;
  }
  if (st) stat_commit(acc, st, partial, tile);
}

__global__ void __launch_bounds__(SG_THREADS) k_stage_curv(const float* __restrict__ phi,
                                                           const int32_t* __restrict__ band, long long m, int nx,
                                                           int ny, int nz, const float* __restrict__ kd,
                                                           svie_law L, StageConst C, float* __restrict__ Lout,
                                                           float* __restrict__ u0, float* __restrict__ Vout,
                                                           svie_stats* st, double* partial) {
  stage_curv_tile(blockIdx.x, phi, band, m, ny, nz, kd, L, C, Lout, u0, Vout, st, partial);
}

SVIE_DEV void stats_reset_at(svie_stats* st, double dt_cap) {
  st->vsum_near = st->vsum_all = 0.0;
  st->dt = 0.0;
  st->dt_cap = dt_cap;
  st->vmax = 0u;
  st->qmin_near = st->qmin_all = 0xffffffffu;
  st->qmax_near = st->qmax_all = 0u;
  st->dvmax_near = st->dvmax_all = 0u;
  st->dmax_near = st->dmax_all = 0u;
  st->capped_near = st->capped_all = 0u;
  st->n_near = 0u;
}

__global__ void k_stats_reset(svie_stats* st, double dt_cap) { stats_reset_at(st, dt_cap); }

// stable_dt (evolve.py:162-170) plus the float64 sums of V.
SVIE_DEV void stats_finalize_block(svie_stats* st, const svie_law& L, const double* partial, long long nb,
                                   long long m) {
  __shared__ DF sh[SUM_THREADS / 32];
  // the (near, all) double-float partials interleaved per CTA: sum each stream in a fixed order
  const float2* pp = reinterpret_cast<const float2*>(partial);
  DF a{0.0f, 0.0f}, b{0.0f, 0.0f};
  for (long long i = threadIdx.x; i < nb; i += blockDim.x) {
    const float2 x = pp[2 * i], y = pp[2 * i + 1];
    a = df_add(a, DF{x.x, x.y});
    b = df_add(b, DF{y.x, y.y});
  }
  a = warp_sum_df(a);
  b = warp_sum_df(b);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) sh[wid] = a;
  __syncthreads();
  if (wid == 0) a = warp_sum_df(lane < SUM_THREADS / 32 ? sh[lane] : DF{0.0f, 0.0f});
  __syncthreads();
  if (lane == 0) sh[wid] = b;
  __syncthreads();
  if (wid == 0) b = warp_sum_df(lane < SUM_THREADS / 32 ? sh[lane] : DF{0.0f, 0.0f});
  if (threadIdx.x != 0) return;
  st->vsum_near = df_value(a);
  st->vsum_all = df_value(b);
  const bool any_near = st->n_near > 0;
  const double vmax = m > 0 ? (double)__uint_as_float(st->vmax) : 0.0;
  const double h = L.h;
  double dt = vmax > 0 ? L.cfl * h / vmax : INFINITY;
  if (L.kind == 0) {
    const double dv = (double)__uint_as_float(any_near ? st->dvmax_near : st->dvmax_all);
    if (dv > 0) dt = fmin(dt, L.feedback_cfl * (4.0 * L.radius / 3.0) / dv);
  } else {
    const double dm = (double)__uint_as_float(any_near ? st->dvmax_near : st->dvmax_all);
    st->dmax_near = st->dvmax_near;
    st->dmax_all = st->dvmax_all;
    if (dm > 0) dt = fmin(dt, L.parabolic_cfl * h * h / dm);
  }
  dt = fmin(dt, st->dt_cap);
  st->dt = dt;
}

__global__ void __launch_bounds__(SUM_THREADS) k_stats_finalize(svie_stats* st, svie_law L, const double* partial,
                                                                long long nb, long long m) {
  stats_finalize_block(st, L, partial, nb, m);
}

// TVD-RK3 stage combinations (evolve.py:175-179): the new value from u0 (a),
// L (l) and the current phi (p; stages 2 and 3), for stages 1-3.  Every
// operation is rounded on its own, in the reference's float32 order (its
// tensor arithmetic fuses no multiply-add), so that every kernel that calls
// this gives the same bits whatever the compiler would contract.
SVIE_DEV float rk_value(int stage, float a, float l, float p, float dt) {
  const float dl = __fmul_rn(dt, l);
  if (stage == 1) return __fadd_rn(a, dl);
  if (stage == 2) return __fadd_rn(__fmul_rn(0.75f, a), __fmul_rn(0.25f, __fadd_rn(p, dl)));
  return __fadd_rn(__fdiv_rn(a, 3.0f), __fmul_rn((float)(2.0 / 3.0), __fadd_rn(p, dl)));
}

// One entry (dt read from the device; stage 0 copies u0 back).
SVIE_DEV void rk_at(long long t, float* __restrict__ phi, const int32_t* __restrict__ band, long long m,
                    const float* __restrict__ u0, const float* __restrict__ L, const double* dtp, int stage) {
  if (t >= m) return;
  const long long i = band[t];
  if (stage == 0) {
    phi[i] = u0[t];
    return;
  }
  const double dtd = *dtp;
  if (!(dtd > 0.0) || !isfinite(dtd)) return;
  phi[i] = rk_value(stage, u0[t], L[t], stage >= 2 ? phi[i] : 0.0f, (float)dtd);
}

// RK_PER entries per thread, at a stride of the block size (coalesced list
// reads): every list read of the thread is issued before the dependent reads
// of phi, so that RK_PER independent chains of two loads are in flight
// instead of one.  The same values as rk_at.
constexpr int RK_PER = 4;

__global__ void __launch_bounds__(256) k_rk(float* __restrict__ phi, const int32_t* __restrict__ band, long long m,
                                            const float* __restrict__ u0, const float* __restrict__ L,
                                            const double* dtp, int stage) {
  const long long t0 = (long long)blockIdx.x * blockDim.x * RK_PER + threadIdx.x;
  if (stage == 0) {
#pragma unroll
    for (int u = 0; u < RK_PER; ++u) {
      const long long t = t0 + (long long)u * blockDim.x;
      if (t < m) phi[band[t]] = u0[t];
    }
    return;
  }
  const double dtd = *dtp;
  if (!(dtd > 0.0) || !isfinite(dtd)) return;
  const float dt = (float)dtd;
  int i[RK_PER];
  float a[RK_PER], l[RK_PER], p[RK_PER];
#pragma unroll
  for (int u = 0; u < RK_PER; ++u) {
    const long long t = t0 + (long long)u * blockDim.x;
    const bool in = t < m;
    i[u] = in ? band[t] : -1;
    a[u] = in ? u0[t] : 0.0f;
    l[u] = in ? L[t] : 0.0f;
  }
#pragma unroll
  for (int u = 0; u < RK_PER; ++u) p[u] = (stage >= 2 && i[u] >= 0) ? phi[i[u]] : 0.0f;
#pragma unroll
  for (int u = 0; u < RK_PER; ++u)
    if (i[u] >= 0) phi[i[u]] = rk_value(stage, a[u], l[u], p[u], dt);
}

}  // namespace svie

using namespace svie;

extern "C" {

size_t svie_stage_workspace_bytes(int64_t m) {
  long long nb = (m + SG_THREADS - 1) / SG_THREADS;
  if (nb < 1) nb = 1;
  return (size_t)nb * 2 * sizeof(double) + 256;
}

int svie_stats_reset(svie_stats* stats, double dt_cap, void* stream) {
  if (!stats) {
    set_error("svie_stats_reset: null stats");
    return SVIE_ERR_ARG;
  }
  k_stats_reset<<<1, 1, 0, (cudaStream_t)stream>>>(stats, dt_cap);
  return launch_status("svie_stats_reset");
}

static int stage_check(const char* name, int64_t m, int nx, int ny, int nz, const svie_law* law, svie_stats* st,
                       void* ws, size_t ws_bytes) {
  if (m < 0 || m >= (1LL << 31) || nx < 8 || ny < 8 || nz < 8 || !law) {
    set_error("%s: bad arguments", name);
    return SVIE_ERR_ARG;
  }
  if (st && (!ws || ws_bytes < svie_stage_workspace_bytes(m))) {
    set_error("%s: workspace too small", name);
    return SVIE_ERR_WORKSPACE;
  }
  return SVIE_OK;
}

int svie_stage_svi(const float* phi, const int32_t* band, int64_t m, int nx, int ny, int nz, const float* N,
                   const svie_law* law, float* L, float* u0, float* V, svie_stats* stats, void* ws,
                   size_t ws_bytes, void* stream) {
  int s = stage_check("svie_stage_svi", m, nx, ny, nz, law, stats, ws, ws_bytes);
  if (s) return s;
  const long long nb = (m + SG_THREADS - 1) / SG_THREADS;
  if (nb == 0) return SVIE_OK;
  k_stage_svi<<<(unsigned)nb, SG_THREADS, 0, (cudaStream_t)stream>>>(phi, band, m, nx, ny, nz, N, *law,
                                                                     stage_const(*law, nx, ny, nz), L, u0, V, stats,
                                                                     (double*)ws);
  return launch_status("svie_stage_svi");
}

int svie_curvature_scatter(const float* phi, const int32_t* band, int64_t m, int nx, int ny, int nz, float h,
                           float* kdense, void* stream) {
  (void)nx;
  if (m <= 0) return m < 0 ? SVIE_ERR_ARG : SVIE_OK;
  k_curv_scatter<<<blocks_for(m, SG_THREADS), SG_THREADS, 0, (cudaStream_t)stream>>>(phi, band, m, ny, nz, h,
                                                                                      kdense);
  return launch_status("svie_curvature_scatter");
}

int svie_stage_curvature(const float* phi, const int32_t* band, int64_t m, int nx, int ny, int nz,
                         const float* kdense, const svie_law* law, float* L, float* u0, float* V,
                         svie_stats* stats, void* ws, size_t ws_bytes, void* stream) {
  int s = stage_check("svie_stage_curvature", m, nx, ny, nz, law, stats, ws, ws_bytes);
  if (s) return s;
  const long long nb = (m + SG_THREADS - 1) / SG_THREADS;
  if (nb == 0) return SVIE_OK;
  k_stage_curv<<<(unsigned)nb, SG_THREADS, 0, (cudaStream_t)stream>>>(phi, band, m, nx, ny, nz, kdense, *law,
                                                                      stage_const(*law, nx, ny, nz), L, u0, V, stats,
                                                                      (double*)ws);
  return launch_status("svie_stage_curvature");
}

int svie_stats_finalize(svie_stats* stats, const svie_law* law, const void* ws, size_t ws_bytes, int64_t m,
                        void* stream) {
  if (!stats || !law || m < 0) {
    set_error("svie_stats_finalize: bad arguments");
    return SVIE_ERR_ARG;
  }
  if (!ws || ws_bytes < svie_stage_workspace_bytes(m)) {
    set_error("svie_stats_finalize: workspace too small");
    return SVIE_ERR_WORKSPACE;
  }
  const long long nb = (m + SG_THREADS - 1) / SG_THREADS;
  k_stats_finalize<<<1, SUM_THREADS, 0, (cudaStream_t)stream>>>(stats, *law, (const double*)ws, nb, m);
  return launch_status("svie_stats_finalize");
}

int svie_rk_stage(float* phi, const int32_t* band, int64_t m, const float* u0, const float* L, const double* dt,
                  int stage, void* stream) {
  if (m < 0 || stage < 0 || stage > 3 || (stage > 0 && (!L || !dt))) {
    set_error("svie_rk_stage: bad arguments");
    return SVIE_ERR_ARG;
  }
  if (m == 0) return SVIE_OK;
  k_rk<<<blocks_for((m + RK_PER - 1) / RK_PER, 256), 256, 0, (cudaStream_t)stream>>>(phi, band, m, u0, L, dt, stage);
  return launch_status("svie_rk_stage");
}

}  // extern "C"

namespace svie {
// Elementwise law evaluation: SVI: V = speed(x1), D = dspeed(x1); curvature
// laws: V, D = speed_and_diffusivity(x1 = k1, x2 = k2).
__global__ void k_law_eval(const float* __restrict__ x1, const float* __restrict__ x2, long long m, svie_law L,
                           StageConst C, float* __restrict__ V, float* __restrict__ D) {
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= m) return;
  if (L.kind == 0) {
    if (V) V[t] = svi_speed(x1[t], L, C);
    if (D) D[t] = svi_dspeed(x1[t], L, C);
  } else {
    float v, d;
    curv_speed(x1[t], x2[t], L, C, &v, &d);
    if (V) V[t] = v;
    if (D) D[t] = d;
  }
}
}  // namespace svie

extern "C" int svie_law_eval(const float* x1, const float* x2, int64_t m, const svie_law* law, float* V, float* D,
                             void* stream) {
  if (m < 0 || !law || (m > 0 && !x1) || (law->kind != 0 && m > 0 && !x2)) {
    svie::set_error("svie_law_eval: bad arguments");
    return SVIE_ERR_ARG;
  }
  if (m == 0) return SVIE_OK;
  // the law's float constants (the grid-dependent ones are unused here)
  const svie::StageConst C = svie::stage_const(*law, 4, 4, 4);
  svie::k_law_eval<<<svie::blocks_for(m, 256), 256, 0, (cudaStream_t)stream>>>(x1, x2, m, *law, C, V, D);
  return svie::launch_status("svie_law_eval");
}

// ------------------------------------------------ many level sets in one launch
namespace svie {

static_assert(SG_THREADS == GROUP_TILE, "group tiles are the stage kernels' CTAs");

SVIE_DEV const GroupInst* group_members(const void* table) { return (const GroupInst*)table; }
SVIE_DEV const int2* group_tile_list(const void* table, int n) {
  return (const int2*)((const char*)table + group_tiles_offset(n));
}

__global__ void k_group_stats_reset(const void* table, int n) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) stats_reset_at(group_members(table)[k].stats, INFINITY);
}

__global__ void __launch_bounds__(SG_THREADS) k_group_curv_scatter(const void* table, int n, long long first) {
  __shared__ GroupInst I;
  const int2 tl = group_tile_list(table, n)[first + blockIdx.x];
  load_group_inst(I, group_members(table) + tl.x);
  curv_scatter_tile(tl.y, I.phi, I.band, I.m, I.ny, I.nz, (float)I.law.h, I.field);
}

__global__ void __launch_bounds__(SG_THREADS, 6) k_group_stage_svi(const void* table, int n, int stage) {
  __shared__ GroupInst I;
  const int2 tl = group_tile_list(table, n)[blockIdx.x];
  load_group_inst(I, group_members(table) + tl.x);
  const bool first = stage == 0;
  stage_svi_tile(tl.y, I.phi, I.band, I.m, I.ny, I.nz, I.field, I.law, I.C, I.L[stage], first ? I.u0 : nullptr,
                 nullptr, first ? I.stats : nullptr, I.stage_part);
}

__global__ void __launch_bounds__(SG_THREADS) k_group_stage_curv(const void* table, int n, long long first_tile,
                                                                 int stage) {
  __shared__ GroupInst I;
  const int2 tl = group_tile_list(table, n)[first_tile + blockIdx.x];
  load_group_inst(I, group_members(table) + tl.x);
  const bool first = stage == 0;
  stage_curv_tile(tl.y, I.phi, I.band, I.m, I.ny, I.nz, I.field, I.law, I.C, I.L[stage], first ? I.u0 : nullptr,
                  nullptr, first ? I.stats : nullptr, I.stage_part);
}

// one CTA per member
__global__ void __launch_bounds__(SUM_THREADS) k_group_stats_finalize(const void* table) {
  const GroupInst* I = group_members(table) + blockIdx.x;
  const long long m = I->m;
  stats_finalize_block(I->stats, I->law, I->stage_part, (m + SG_THREADS - 1) / SG_THREADS, m);
}

__global__ void __launch_bounds__(GROUP_TILE) k_group_rk(const void* table, int n, int stage) {
  const int2 tl = group_tile_list(table, n)[blockIdx.x];
  const GroupInst* I = group_members(table) + tl.x;
  rk_at((long long)tl.y * GROUP_TILE + threadIdx.x, I->phi, I->band, I->m, I->u0,
        stage > 0 ? I->L[stage - 1] : nullptr, &I->stats->dt, stage);
}

__global__ void k_group_gather_stats(const void* table, svie_stats* dst) {
  const GroupInst* I = group_members(table) + blockIdx.x;
  constexpr int W = (int)(sizeof(svie_stats) / 4);
  const int* a = (const int*)I->stats;
  const int* b = (const int*)I->vstats;
  int* o = (int*)(dst + 2 * blockIdx.x);
  for (int k = threadIdx.x; k < 2 * W; k += blockDim.x) o[k] = k < W ? a[k] : b[k - W];
}

static bool group_ok(const char* name, const svie_group* g) {
  if (!g || (g->n > 0 && !g->table) || g->n < 0 || g->tiles < 0 || g->tiles_svi < 0 || g->tiles_svi > g->tiles) {
    set_error("%s: bad group", name);
    return false;
  }
  return true;
}

}  // namespace svie

extern "C" {

int64_t svie_group_tiles(const svie_group_member* members, int32_t n) {
  if (!members || n < 0) return -1;
  int64_t t = 0;
  for (int k = 0; k < n; ++k) t += (members[k].m + GROUP_TILE - 1) / GROUP_TILE;
  return t;
}

size_t svie_group_table_bytes(int32_t n, int64_t tiles) {
  if (n < 0 || tiles < 0) return 0;
  return group_tiles_offset(n) + (size_t)tiles * sizeof(int2) + 16;
}

int svie_group_build(const svie_group_member* members, int32_t n, void* table, size_t table_bytes,
                     void* host_staging, svie_group* out, void* stream) {
  if (!out || n < 0 || (n > 0 && (!members || !table || !host_staging)) || ((uintptr_t)table & 15) ||
      ((uintptr_t)host_staging & 15)) {
    set_error("svie_group_build: bad arguments (table and staging 16-byte aligned)");
    return SVIE_ERR_ARG;
  }
  const int64_t tiles = svie_group_tiles(members, n);
  if (table_bytes < svie_group_table_bytes(n, tiles)) {
    set_error("svie_group_build: table of %zu bytes, %zu needed", table_bytes, svie_group_table_bytes(n, tiles));
    return SVIE_ERR_WORKSPACE;
  }
  GroupInst* rec = (GroupInst*)host_staging;
  int2* tl = (int2*)((char*)host_staging + group_tiles_offset(n));
  int64_t w = 0;
  for (int pass = 0; pass < 2; ++pass) {  // SVI members' tiles first
    for (int k = 0; k < n; ++k) {
      const svie_group_member& M = members[k];
      if (M.kind != pass) continue;
      if (M.m < 0 || M.m >= (1LL << 31) || M.nx < 8 || M.ny < 8 || M.nz < 8 || (M.kind != 0 && M.kind != 1) ||
          (M.m > 0 && (!M.phi || !M.band || !M.field || !M.occ || !M.u0 || !M.L[0] || !M.L[1] || !M.L[2])) ||
          !M.stats || !M.vstats || (long long)M.nx * M.ny * M.nz >= (1LL << 31)) {
        set_error("svie_group_build: member %d: bad arguments", k);
        return SVIE_ERR_ARG;
      }
      if (!M.stage_ws || M.stage_ws_bytes < svie_stage_workspace_bytes(M.m) || !M.volume_ws ||
          M.volume_ws_bytes < svie_volume_workspace_bytes(M.m)) {
        set_error("svie_group_build: member %d: workspace too small", k);
        return SVIE_ERR_WORKSPACE;
      }
      GroupInst& r = rec[k];
      r.phi = M.phi;
      r.band = M.band;
      r.field = M.field;
      r.occ = M.occ;
      r.u0 = M.u0;
      for (int j = 0; j < 3; ++j) r.L[j] = M.L[j];
      r.stats = M.stats;
      r.vstats = M.vstats;
      r.stage_part = (double*)M.stage_ws;
      r.vol_part = (double*)M.volume_ws;
      r.m = M.m;
      r.nx = M.nx;
      r.ny = M.ny;
      r.nz = M.nz;
      r.kind = M.kind;
      r.law = M.law;
      r.C = stage_const(M.law, M.nx, M.ny, M.nz);
      const long long nt = (M.m + GROUP_TILE - 1) / GROUP_TILE;
      for (long long j = 0; j < nt; ++j) tl[w++] = make_int2(k, (int)j);
    }
    if (pass == 0) out->tiles_svi = w;
  }
  out->table = table;
  out->n = n;
  out->pad = 0;
  out->tiles = w;
  if (n > 0 && cudaMemcpyAsync(table, host_staging, svie_group_table_bytes(n, tiles), cudaMemcpyHostToDevice,
                               (cudaStream_t)stream) != cudaSuccess) {
    set_error("svie_group_build: table copy failed");
    return SVIE_ERR_LAUNCH;
  }
  return SVIE_OK;
}

int svie_group_stats_reset(const svie_group* g, void* stream) {
  if (!group_ok("svie_group_stats_reset", g)) return SVIE_ERR_ARG;
  if (g->n == 0) return SVIE_OK;
  k_group_stats_reset<<<(g->n + 127) / 128, 128, 0, (cudaStream_t)stream>>>(g->table, g->n);
  return launch_status("svie_group_stats_reset");
}

int svie_group_curvature_scatter(const svie_group* g, void* stream) {
  if (!group_ok("svie_group_curvature_scatter", g)) return SVIE_ERR_ARG;
  const long long nt = g->tiles - g->tiles_svi;
  if (nt == 0) return SVIE_OK;
  k_group_curv_scatter<<<(unsigned)nt, SG_THREADS, 0, (cudaStream_t)stream>>>(g->table, g->n, g->tiles_svi);
  return launch_status("svie_group_curvature_scatter");
}

int svie_group_stage(const svie_group* g, int stage, void* stream) {
  if (!group_ok("svie_group_stage", g) || stage < 0 || stage > 2) {
    set_error("svie_group_stage: bad arguments");
    return SVIE_ERR_ARG;
  }
  cudaStream_t s = (cudaStream_t)stream;
  int launches = 0;
  if (g->tiles_svi > 0) {
    k_group_stage_svi<<<(unsigned)g->tiles_svi, SG_THREADS, 0, s>>>(g->table, g->n, stage);
    ++launches;
  }
  const long long nc = g->tiles - g->tiles_svi;
  if (nc > 0) {
    k_group_stage_curv<<<(unsigned)nc, SG_THREADS, 0, s>>>(g->table, g->n, g->tiles_svi, stage);
    ++launches;
  }
  return launch_status("svie_group_stage", launches);
}

int svie_group_stats_finalize(const svie_group* g, void* stream) {
  if (!group_ok("svie_group_stats_finalize", g)) return SVIE_ERR_ARG;
  if (g->n == 0) return SVIE_OK;
  k_group_stats_finalize<<<g->n, SUM_THREADS, 0, (cudaStream_t)stream>>>(g->table);
  return launch_status("svie_group_stats_finalize");
}

int svie_group_rk(const svie_group* g, int stage, void* stream) {
  if (!group_ok("svie_group_rk", g) || stage < 0 || stage > 3) {
    set_error("svie_group_rk: bad arguments");
    return SVIE_ERR_ARG;
  }
  if (g->tiles == 0) return SVIE_OK;
  k_group_rk<<<(unsigned)g->tiles, GROUP_TILE, 0, (cudaStream_t)stream>>>(g->table, g->n, stage);
  return launch_status("svie_group_rk");
}

int svie_group_gather_stats(const svie_group* g, svie_stats* dst, void* stream) {
  if (!group_ok("svie_group_gather_stats", g) || (g->n > 0 && !dst)) {
    set_error("svie_group_gather_stats: bad arguments");
    return SVIE_ERR_ARG;
  }
  if (g->n == 0) return SVIE_OK;
  k_group_gather_stats<<<g->n, 64, 0, (cudaStream_t)stream>>>(g->table, dst);
  return launch_status("svie_group_gather_stats");
}

}  // extern "C"
