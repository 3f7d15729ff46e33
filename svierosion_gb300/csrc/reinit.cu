// PDE reinitialisation with subcell fix (Min 2010), reference
// svierosion/levelset.py:154-183 and svierosion/kernels.py:312-379.
//
// Work set: band dilated by `dilation` cells (box), outer `margin` layers
// cleared, compacted in brick order.  Geometry (sign, local pseudo-time step,
// per-axis crossing flags and subcell interface distances) is computed once
// from the initial phi (layout at struct Geo below).
// Each TVD-RK2 iteration is two Jacobi sweeps between the level-set grid A and
// a second dense grid B that mirrors A off the work set:
//   B[idx] = u0 + dtau rhs(A);   A[idx] = (u0 + B[idx] + dtau rhs(B)) / 2.
#include "common.cuh"

namespace svie {

constexpr int RI_THREADS = 256;

SVIE_DEV float minmod(float a, float b) {
  return (a * b > 0.0f) ? (fabsf(a) < fabsf(b) ? a : b) : 0.0f;
}

// _interface_distance (kernels.py:312-331)
SVIE_DEV float interface_distance(float p0, float p1, float dd, float h) {
  float den = p0 - p1;
  float lin = h * p0 / (den != 0.0f ? den : 1e-30f);
  float c2 = 0.5f * dd / (h * h);
  float c1 = (p1 - p0) / h;
  float c0 = 0.5f * (p0 + p1) - c2 * h * h / 4.0f;
  float disc = c1 * c1 - 4.0f * c2 * c0;
  float sq = sqrtf(fmaxf(disc, 0.0f));
  float q = -0.5f * (c1 + (c1 >= 0.0f ? sq : -sq));
  float xi = c0 / (q != 0.0f ? q : 1e-30f);
  float quad = h / 2.0f + xi;
  bool ok = (disc >= 0.0f) && (fabsf(dd) > 1e-10f * h * h) && (quad >= 0.0f) && (quad <= h);
  return fminf(fmaxf(ok ? quad : lin, 0.0f), h);
}

// Geometry record, structure of arrays over the work set (m entries):
//   dtau  float [m]
//   meta  uint8 [m]   bits 0-5: crossing flags cp_x cm_x cp_y cm_y cp_z cm_z,
//                     bit 6: phi0 > 0, bit 7: phi0 < 0
//   dist  float [6m]  xp_x xm_x xp_y xm_y xp_z xm_z, read only where the flag is set
//   cfl   float       at geo_cfl_offset(m)
// A sweep streams 1 byte of geometry per node (the flags) and rebuilds dtau
// from the distances it reads anyway; dtau is stored for
// svie_reinit_geometry_unpack.
struct Geo {
  float* dtau;
  uint8_t* meta;
  float* dist;
  long long m;
};

// cfl of the geometry, stored after the arrays (16-byte aligned).
__host__ __device__ inline long long geo_cfl_offset(long long m) { return (29 * m + 15) & ~15LL; }
SVIE_DEV float geo_cfl(const void* base, long long m) {
  return __ldg(reinterpret_cast<const float*>(static_cast<const char*>(base) + geo_cfl_offset(m)));
}

SVIE_DEV Geo geo_view(void* base, long long m) {
  Geo g;
  char* b = (char*)base;
  g.dtau = (float*)b;
  g.dist = (float*)(b + 4 * m);
  g.meta = (uint8_t*)(b + 28 * m);
  g.m = m;
  return g;
}

__global__ void k_reinit_geometry(const float* __restrict__ f, const int32_t* __restrict__ idx, long long m,
                                  int sx, int sy, int sz, float h, float cfl, void* geo) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= m) return;
  Geo g = geo_view(geo, m);
  const int i = idx[t];
  const float* qp = f + i;
  const float c = __ldg(qp);
  float hmin = h;
  uint32_t flags = 0;
  const int st[3] = {sx, sy, sz};
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const int s = st[a];
    float m2 = __ldg(qp - 2 * s), m1 = __ldg(qp - s), p1 = __ldg(qp + s), p2 = __ldg(qp + 2 * s);
    float d_m1 = c - 2.0f * m1 + m2;
    float d_0 = p1 - 2.0f * c + m1;
    float d_p1 = p2 - 2.0f * p1 + c;
    bool cp = (c * p1) < 0.0f;
    bool cm = (c * m1) < 0.0f;
    float xp = interface_distance(c, p1, minmod(d_0, d_p1), h);
    float xm = interface_distance(c, m1, minmod(d_0, d_m1), h);
    hmin = fminf(hmin, cp ? xp : hmin);
    hmin = fminf(hmin, cm ? xm : hmin);
    flags |= (cp ? 1u : 0u) << (2 * a);
    flags |= (cm ? 1u : 0u) << (2 * a + 1);
    g.dist[(2 * a) * m + t] = fmaxf(xp, 1e-6f * h);
    g.dist[(2 * a + 1) * m + t] = fmaxf(xm, 1e-6f * h);
  }
  flags |= (c > 0.0f ? 1u : 0u) << 6;
  flags |= (c < 0.0f ? 1u : 0u) << 7;
  g.dtau[t] = cfl * fmaxf(hmin, 1e-3f * h);
  g.meta[t] = (uint8_t)flags;
  if (t == 0) *reinterpret_cast<float*>(static_cast<char*>(geo) + geo_cfl_offset(m)) = cfl;
}

SVIE_DEV float meta_sgn(uint32_t meta) { return (meta & 64u) ? 1.0f : ((meta & 128u) ? -1.0f : 0.0f); }

// reinit_rhs (kernels.py:363-379) at work-set entry t.  Divisions by h use
// the correctly rounded reciprocal rh (div_by); hh = RN(h * h).  Also returns
// hmin = min(h, stored distances of the flagged crossings), from which
// dtau = cfl * max(hmin, 1e-3 h) is rebuilt exactly as k_reinit_geometry
// computed it (a distance below 1e-6 h, stored clamped to 1e-6 h, gives the
// same 1e-3 h either way).
SVIE_DEV float reinit_rhs_at(const float* __restrict__ f, int i, long long t, const Geo& g, uint32_t flags, int sx,
                             int sy, int sz, float h, float rh, float hh, float& hmin) {
  const float* qp = f + i;
  const float c = __ldg(qp);
  const float sgn = meta_sgn(flags);
  const bool outside = sgn > 0.0f;
  float g2 = 0.0f;
  hmin = h;
  const int st[3] = {sx, sy, sz};
  float v3[3][4];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const int s = st[a];
    v3[a][0] = __ldg(qp - 2 * s);
    v3[a][1] = __ldg(qp - s);
    v3[a][2] = __ldg(qp + s);
    v3[a][3] = __ldg(qp + 2 * s);
  }
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const float m2 = v3[a][0], m1 = v3[a][1], p1 = v3[a][2], p2 = v3[a][3];
    const float mm_p = minmod(p1 - 2.0f * c + m1, p2 - 2.0f * p1 + c);
    const float mm_m = minmod(p1 - 2.0f * c + m1, c - 2.0f * m1 + m2);
    float Dp = div_by(p1 - c - 0.5f * mm_p, h, rh);
    float Dm = div_by(c - m1 + 0.5f * mm_m, h, rh);
    if ((flags >> (2 * a)) & 1u) {
      const float xp = g.dist[(2 * a) * g.m + t];
      Dp = -c / xp - 0.5f * xp * mm_p / hh;
      hmin = fminf(hmin, xp);
    }
    if ((flags >> (2 * a + 1)) & 1u) {
      const float xm = g.dist[(2 * a + 1) * g.m + t];
      Dm = c / xm + 0.5f * xm * mm_m / hh;
      hmin = fminf(hmin, xm);
    }
    const float a1 = outside ? fmaxf(Dm, 0.0f) : fminf(Dm, 0.0f);
    const float b1 = outside ? fminf(Dp, 0.0f) : fmaxf(Dp, 0.0f);
    g2 = g2 + fmaxf(a1 * a1, b1 * b1);
  }
  return -sgn * (sqrtf(g2) - 1.0f);
}

__global__ void __launch_bounds__(RI_THREADS, 8) k_reinit_sweep(const float* __restrict__ src, float* __restrict__ dst,
                                                             const int32_t* __restrict__ idx, long long m, int sx,
                                                             int sy, int sz, float h, float rh, void* geo,
                                                             int second) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= m) return;
  Geo g = geo_view(geo, m);
  const float cfl = geo_cfl(geo, m);
  const int i = idx[t];
  float hmin;
  const float r = reinit_rhs_at(src, i, t, g, g.meta[t], sx, sy, sz, h, rh, h * h, hmin);
  const float dtau = cfl * fmaxf(hmin, 1e-3f * h);
  if (!second) {
    dst[i] = src[i] + dtau * r;  // u0 + dtau rhs(A)
  } else {
    const float u0 = dst[i], u1 = src[i];
    dst[i] = 0.5f * (u0 + u1 + dtau * r);
  }
}

__global__ void k_reinit_rhs(const float* __restrict__ f, const int32_t* __restrict__ idx, long long m, int sx, int sy,
                             int sz, float h, float rh, void* geo, float* out) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= m) return;
  Geo g = geo_view(geo, m);
  float hmin;
  out[t] = reinit_rhs_at(f, idx[t], t, g, g.meta[t], sx, sy, sz, h, rh, h * h, hmin);
}

__global__ void k_geo_unpack(const void* geo, long long m, float* sgn, float* dtau, uint8_t* flags, float* dist6) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= m) return;
  Geo g = geo_view(const_cast<void*>(geo), m);
  const uint32_t meta = g.meta[t];
  sgn[t] = meta_sgn(meta);
  dtau[t] = g.dtau[t];
  for (int a = 0; a < 6; ++a) {
    flags[a * m + t] = (meta >> a) & 1u;
    dist6[a * m + t] = g.dist[a * m + t];
  }
}

__global__ void k_mark(const int32_t* __restrict__ band, long long m, uint8_t* __restrict__ mask) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < m) mask[band[t]] = 1;
}

// dst = src dilated by `r` cells along one axis (box, clipped at the borders);
// margin > 0 also clears the outer layers on every axis (last pass only).
__global__ void k_dilate_axis(const uint8_t* __restrict__ src, uint8_t* __restrict__ dst, int nx, int ny, int nz,
                              int axis, int r, int margin) {
  const long long syz = (long long)ny * nz;
  const int z = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y, x = blockIdx.z;
  if (z >= nz) return;
  {
    const long long e = (long long)x * syz + (long long)y * nz + z;
    const int c = axis == 0 ? x : (axis == 1 ? y : z);
    const int len = axis == 0 ? nx : (axis == 1 ? ny : nz);
    const long long st = axis == 0 ? syz : (axis == 1 ? nz : 1);
    uint8_t v = 0;
    const int lo = max(c - r, 0), hi = min(c + r, len - 1);
    for (int d = lo; d <= hi && !v; ++d) v = src[e + (long long)(d - c) * st];
    if (margin > 0 && (x < margin || y < margin || z < margin || x >= nx - margin || y >= ny - margin ||
                       z >= nz - margin))
      v = 0;
    dst[e] = v;
  }
}

// Box dilation by r <= DB_RMAX in one pass (the three axis passes of
// k_dilate_axis fused): a CTA owns a DB_X x DB_Y x DB_Z tile and reads its
// neighbourhood widened by r, one row (x, y) at a time as bit masks (three
// ballots of 32 z values, bit i <-> z = z0 - r + i); the box OR is then
// separable bit arithmetic: shifts along z, ORs of row masks along y and x.
// Nodes outside the grid count as 0; margin > 0 clears the outer layers.
constexpr int DB_X = 16, DB_Y = 16, DB_Z = 64, DB_RMAX = 8;
constexpr int DB_EMAX = DB_X + 2 * DB_RMAX;  // = DB_Y + 2 * DB_RMAX

__global__ void __launch_bounds__(256) k_dilate_box(const uint8_t* __restrict__ src, uint8_t* __restrict__ dst,
                                                    int nx, int ny, int nz, int r, int margin) {
  __shared__ uint32_t inm[DB_EMAX * DB_EMAX][3];
  __shared__ unsigned long long zm[DB_EMAX * DB_EMAX];
  __shared__ unsigned long long ym[DB_EMAX * DB_Y];
  __shared__ unsigned long long fm[DB_X * DB_Y];
  const int x0 = blockIdx.z * DB_X, y0 = blockIdx.y * DB_Y, z0 = blockIdx.x * DB_Z;
  const int EX = DB_X + 2 * r, EY = DB_Y + 2 * r, EZ = DB_Z + 2 * r;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  // four rows per warp step: twelve loads in flight before the ballots
  for (int row0 = warp; row0 < EX * EY; row0 += 32) {
    uint8_t v[4][3];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int row = row0 + 8 * u;
      const int ix = row / EY, iy = row - ix * EY;
      const int x = x0 - r + ix, y = y0 - r + iy;
      const bool rowok = row < EX * EY && x >= 0 && x < nx && y >= 0 && y < ny;
      const long long rb = rowok ? ((long long)x * ny + y) * nz : 0;
#pragma unroll
      for (int w = 0; w < 3; ++w) {
        const int i = 32 * w + lane, z = z0 - r + i;
        v[u][w] = (rowok && i < EZ && z >= 0 && z < nz) ? __ldg(src + rb + z) : 0;
      }
    }
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int row = row0 + 8 * u;
#pragma unroll
      for (int w = 0; w < 3; ++w) {
        const unsigned int b = __ballot_sync(0xffffffffu, v[u][w] != 0);
        if (lane == 0 && row < EX * EY) inm[row][w] = b;
      }
    }
  }
  __syncthreads();
  // z: output bit k (z = z0 + k) = OR of input bits k .. k + 2r
  for (int row = threadIdx.x; row < EX * EY; row += blockDim.x) {
    const unsigned long long lo = inm[row][0] | ((unsigned long long)inm[row][1] << 32);
    const unsigned long long hi = inm[row][2];
    unsigned long long acc = lo;
    for (int d = 1; d <= 2 * r; ++d) acc |= (lo >> d) | (hi << (64 - d));
    zm[row] = acc;
  }
  __syncthreads();
  // y: rows (ix, y) = OR over iy = y .. y + 2r
  for (int t = threadIdx.x; t < EX * DB_Y; t += blockDim.x) {
    const int ix = t / DB_Y, y = t - ix * DB_Y;
    unsigned long long acc = 0;
    for (int d = 0; d <= 2 * r; ++d) acc |= zm[ix * EY + y + d];
    ym[t] = acc;
  }
  __syncthreads();
  // x: rows (x, y) = OR over ix = x .. x + 2r
  for (int t = threadIdx.x; t < DB_X * DB_Y; t += blockDim.x) {
    const int x = t / DB_Y, y = t - x * DB_Y;
    unsigned long long acc = 0;
    for (int d = 0; d <= 2 * r; ++d) acc |= ym[(x + d) * DB_Y + y];
    fm[t] = acc;
  }
  __syncthreads();
  for (int row = warp; row < DB_X * DB_Y; row += 8) {
    const int x = x0 + row / DB_Y, y = y0 + row % DB_Y;
    if (x >= nx || y >= ny) continue;
    const bool rowclear = margin > 0 && (x < margin || y < margin || x >= nx - margin || y >= ny - margin);
    const unsigned long long mk = fm[row];
    uint8_t* drow = dst + ((long long)x * ny + y) * nz;
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int k = 32 * h + lane, z = z0 + k;
      if (z < nz) {
        const bool zclear = margin > 0 && (z < margin || z >= nz - margin);
        drow[z] = (!rowclear && !zclear && ((mk >> k) & 1ull)) ? 1 : 0;
      }
    }
  }
}

// dst = src dilated by the (2r+1)^3 box; tmp is a same-size scratch used
// only for r > DB_RMAX (three axis passes).
static void dilate_box(const uint8_t* src, uint8_t* dst, uint8_t* tmp, int nx, int ny, int nz, int r, int margin,
                       cudaStream_t s, int* launches) {
  if (r <= DB_RMAX) {
    const dim3 gd((nz + DB_Z - 1) / DB_Z, (ny + DB_Y - 1) / DB_Y, (nx + DB_X - 1) / DB_X);
    k_dilate_box<<<gd, 256, 0, s>>>(src, dst, nx, ny, nz, r, margin);
    *launches += 1;
    return;
  }
  const dim3 gd((nz + 127) / 128, ny, nx);
  k_dilate_axis<<<gd, 128, 0, s>>>(src, tmp, nx, ny, nz, 0, r, 0);
  k_dilate_axis<<<gd, 128, 0, s>>>(tmp, dst, nx, ny, nz, 1, r, 0);
  k_dilate_axis<<<gd, 128, 0, s>>>(dst, tmp, nx, ny, nz, 2, r, margin);
  cudaMemcpyAsync(dst, tmp, (size_t)nx * ny * nz, cudaMemcpyDeviceToDevice, s);
  *launches += 3;
}

inline size_t geo_bytes(long long m) { return (size_t)(m < 1 ? 1 : m) * 29 + 256; }

}  // namespace svie

using namespace svie;

extern "C" {

int svie_reinit_mask(const int32_t* band, int64_t m, int nx, int ny, int nz, int dilation, int margin, uint8_t* mask,
                     uint8_t* tmp, void* stream) {
  const long long n = (long long)nx * ny * nz;
  if (!mask || !tmp || n <= 0 || dilation < 0 || margin < 0 || m < 0) {
    set_error("svie_reinit_mask: bad arguments");
    return SVIE_ERR_ARG;
  }
  cudaStream_t s = (cudaStream_t)stream;
  // the band marked into tmp, then dilated into mask
  if (cudaMemsetAsync(tmp, 0, (size_t)n, s) != cudaSuccess) {
    set_error("svie_reinit_mask: memset failed");
    return SVIE_ERR_LAUNCH;
  }
  int launches = 0;
  if (m > 0) {
    k_mark<<<blocks_for(m, 256), 256, 0, s>>>(band, m, tmp);
    ++launches;
  }
  if (dilation <= DB_RMAX) {
    dilate_box(tmp, mask, nullptr, nx, ny, nz, dilation, margin, s, &launches);
  } else {
    // the three axis passes need a scratch distinct from source and target
    if (cudaMemcpyAsync(mask, tmp, (size_t)n, cudaMemcpyDeviceToDevice, s) != cudaSuccess) {
      set_error("svie_reinit_mask: copy failed");
      return SVIE_ERR_LAUNCH;
    }
    dilate_box(mask, mask, tmp, nx, ny, nz, dilation, margin, s, &launches);
  }
  return launch_status("svie_reinit_mask", launches);
}

size_t svie_reinit_geometry_bytes(int64_t m) { return geo_bytes(m); }

int svie_reinit_geometry(const float* phi, const int32_t* idx, int64_t m, int64_t sx, int64_t sy, int64_t sz,
                         float h, float cfl, void* geo, void* stream) {
  if (m < 0 || (m > 0 && (!phi || !idx || !geo))) {
    set_error("svie_reinit_geometry: bad arguments");
    return SVIE_ERR_ARG;
  }
  if (m == 0) return SVIE_OK;
  k_reinit_geometry<<<blocks_for(m, RI_THREADS), RI_THREADS, 0, (cudaStream_t)stream>>>(phi, idx, m, sx, sy, sz, h,
                                                                                        cfl, geo);
  return launch_status("svie_reinit_geometry");
}

int svie_reinit_iterate(float* phi, float* phi_tmp, int64_t n, const int32_t* idx, int64_t m, int64_t sx, int64_t sy,
                        int64_t sz, float h, const void* geo, int iterations, void* stream) {
  if (!phi || !phi_tmp || n <= 0 || m < 0 || iterations < 0) {
    set_error("svie_reinit_iterate: bad arguments");
    return SVIE_ERR_ARG;
  }
  if (m == 0 || iterations == 0) return SVIE_OK;
  cudaStream_t s = (cudaStream_t)stream;
  if (cudaMemcpyAsync(phi_tmp, phi, (size_t)n * sizeof(float), cudaMemcpyDeviceToDevice, s) != cudaSuccess) {
    set_error("svie_reinit_iterate: copy failed");
    return SVIE_ERR_LAUNCH;
  }
  const int nb = blocks_for(m, RI_THREADS);
  const float rh = rn_reciprocal(h);
  for (int it = 0; it < iterations; ++it) {
    k_reinit_sweep<<<nb, RI_THREADS, 0, s>>>(phi, phi_tmp, idx, m, sx, sy, sz, h, rh, const_cast<void*>(geo), 0);
    k_reinit_sweep<<<nb, RI_THREADS, 0, s>>>(phi_tmp, phi, idx, m, sx, sy, sz, h, rh, const_cast<void*>(geo), 1);
  }
  return launch_status("svie_reinit_iterate", 2 * iterations);
}

int svie_reinit_rhs(const float* phi, const int32_t* idx, int64_t m, int64_t sx, int64_t sy, int64_t sz, float h,
                    const void* geo, float* out, void* stream) {
  if (m <= 0) return m < 0 ? SVIE_ERR_ARG : SVIE_OK;
  k_reinit_rhs<<<blocks_for(m, RI_THREADS), RI_THREADS, 0, (cudaStream_t)stream>>>(
      phi, idx, m, sx, sy, sz, h, rn_reciprocal(h), const_cast<void*>(geo), out);
  return launch_status("svie_reinit_rhs");
}

int svie_reinit_geometry_unpack(const void* geo, int64_t m, float* sgn, float* dtau, uint8_t* flags, float* dist6,
                                void* stream) {
  if (m <= 0) return m < 0 ? SVIE_ERR_ARG : SVIE_OK;
  k_geo_unpack<<<blocks_for(m, 256), 256, 0, (cudaStream_t)stream>>>(geo, m, sgn, dtau, flags, dist6);
  return launch_status("svie_reinit_geometry_unpack");
}

}  // extern "C"

// levelset.dilate (levelset.py:25-34): out = mask dilated by the
// (2 steps + 1)^3 box, clipped at the borders; tmp is a same-size scratch grid.
extern "C" int svie_dilate(const uint8_t* mask, int nx, int ny, int nz, int steps, uint8_t* out, uint8_t* tmp,
                           void* stream) {
  const long long n = (long long)nx * ny * nz;
  if (!mask || !out || !tmp || n <= 0 || steps < 0) {
    svie::set_error("svie_dilate: bad arguments");
    return SVIE_ERR_ARG;
  }
  cudaStream_t s = (cudaStream_t)stream;
  if (mask == out && steps <= svie::DB_RMAX) {
    if (cudaMemcpyAsync(tmp, mask, (size_t)n, cudaMemcpyDeviceToDevice, s) != cudaSuccess) {
      svie::set_error("svie_dilate: copy failed");
      return SVIE_ERR_LAUNCH;
    }
    mask = tmp;
  }
  int launches = 0;
  svie::dilate_box(mask, out, tmp, nx, ny, nz, steps, 0, s, &launches);
  return svie::launch_status("svie_dilate", launches);
}
