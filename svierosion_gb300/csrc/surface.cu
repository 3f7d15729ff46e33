// Extraction of the zero level set as a triangle mesh (reference
// svierosion/surface.py:16-56): marching cubes on the cells whose lower corner
// is a band node, then one limited Newton step of every vertex on the tricubic
// interpolant of phi.
//
// The case table is generated from the method's definition (Lorensen and
// Cline 1987) rather than taken from a library: for each of the 256
// inside/outside corner patterns (inside = phi < 0) the crossed cell edges are
// joined face by face, on a face with four crossings so that the two inside
// corners are cut off (a choice made from the face alone, so neighbouring cells
// agree and the mesh is closed), and each resulting loop is fanned into
// triangles oriented from inside to outside.  One vertex per crossed grid edge,
// owned by the edge's lower node, is shared by the four cells around the edge.
//
// Three passes over the band (ascending order): counts per CTA; vertices
// (positions by linear interpolation, the owner's first vertex id and crossing
// bits stored in a dense grid-sized int32 array); faces.  Ids follow the band
// order, so the mesh is deterministic and equals the oracle's bit for bit.
#include <string.h>

#include <mutex>

#include "common.cuh"

namespace svie {

constexpr int SF_THREADS = 256;

__constant__ int8_t c_mc_tri[256][16];
__constant__ uint8_t c_mc_ntri[256];

// Cell corner v has offset (v & 1, (v >> 1) & 1, (v >> 2) & 1).  Edge e = 4 a +
// u + 2 w runs along axis a from corner ev0[e]; (u, w) are its coordinates on
// the other two axes in increasing axis order.
struct McGeometry {
  int eaxis[12], ev0[12], ev1[12];
  int fcorner[6][4], fedge[6][4];
  McGeometry() {
    for (int a = 0; a < 3; ++a) {
      const int o0 = a == 0 ? 1 : 0, o1 = a == 2 ? 1 : 2;
      for (int w = 0; w < 2; ++w)
        for (int u = 0; u < 2; ++u) {
          int c[3] = {0, 0, 0};
          c[o0] = u;
          c[o1] = w;
          const int e = 4 * a + u + 2 * w;
          eaxis[e] = a;
          ev0[e] = c[0] | (c[1] << 1) | (c[2] << 2);
          ev1[e] = ev0[e] | (1 << a);
        }
    }
    int f = 0;
    for (int a = 0; a < 3; ++a) {
      const int o0 = a == 0 ? 1 : 0, o1 = a == 2 ? 1 : 2;
      for (int s = 0; s < 2; ++s, ++f) {
        static const int uw[4][2] = {{0, 0}, {1, 0}, {1, 1}, {0, 1}};
        for (int k = 0; k < 4; ++k) {
          int c[3];
          c[a] = s;
          c[o0] = uw[k][0];
          c[o1] = uw[k][1];
          fcorner[f][k] = c[0] | (c[1] << 1) | (c[2] << 2);
        }
        for (int k = 0; k < 4; ++k) {
          const int p = fcorner[f][k], q = fcorner[f][(k + 1) & 3];
          for (int e = 0; e < 12; ++e)
            if ((ev0[e] == p && ev1[e] == q) || (ev0[e] == q && ev1[e] == p)) fedge[f][k] = e;
        }
      }
    }
  }
};

static void mc_case(const McGeometry& G, int cs, int8_t* out, int* ntri) {
  int inside[8];
  for (int v = 0; v < 8; ++v) inside[v] = (cs >> v) & 1;
  int adj[12][2], nadj[12] = {0};
  bool cross[12];
  for (int e = 0; e < 12; ++e) cross[e] = inside[G.ev0[e]] != inside[G.ev1[e]];
  auto join = [&](int p, int q) {
    adj[p][nadj[p]++] = q;
    adj[q][nadj[q]++] = p;
  };
  for (int f = 0; f < 6; ++f) {
    int cut[4], nc = 0;
    for (int k = 0; k < 4; ++k)
      if (inside[G.fcorner[f][k]] != inside[G.fcorner[f][(k + 1) & 3]]) cut[nc++] = k;
    if (nc == 2) {
      join(G.fedge[f][cut[0]], G.fedge[f][cut[1]]);
    } else if (nc == 4) {
      for (int k = 0; k < 4; ++k)
        if (inside[G.fcorner[f][k]]) join(G.fedge[f][(k + 3) & 3], G.fedge[f][k]);
    }
  }
  double mid[12][3], odir[12][3];
  for (int e = 0; e < 12; ++e)
    for (int d = 0; d < 3; ++d) {
      const int c0 = (G.ev0[e] >> d) & 1, c1 = (G.ev1[e] >> d) & 1;
      mid[e][d] = 0.5 * (c0 + c1);
      const int ci = inside[G.ev0[e]] ? c0 : c1, co = inside[G.ev0[e]] ? c1 : c0;
      odir[e][d] = co - ci;
    }
  bool seen[12] = {false};
  int n = 0;
  for (int start = 0; start < 12; ++start) {
    if (!cross[start] || seen[start]) continue;
    int loop[12], len = 0, prev = -1, cur = start;
    loop[len++] = start;
    seen[start] = true;
    for (;;) {
      const int q = (adj[cur][0] != prev) ? adj[cur][0] : adj[cur][1];
      if (q == start) break;
      loop[len++] = q;
      seen[q] = true;
      prev = cur;
      cur = q;
    }
    double area[3] = {0, 0, 0}, dir[3] = {0, 0, 0};
    for (int k = 1; k + 1 < len; ++k) {
      double u[3], v[3];
      for (int d = 0; d < 3; ++d) {
        u[d] = mid[loop[k]][d] - mid[loop[0]][d];
        v[d] = mid[loop[k + 1]][d] - mid[loop[0]][d];
      }
      area[0] += u[1] * v[2] - u[2] * v[1];
      area[1] += u[2] * v[0] - u[0] * v[2];
      area[2] += u[0] * v[1] - u[1] * v[0];
    }
    for (int k = 0; k < len; ++k)
      for (int d = 0; d < 3; ++d) dir[d] += odir[loop[k]][d];
    if (area[0] * dir[0] + area[1] * dir[1] + area[2] * dir[2] < 0) {
      for (int k = 0; k < len / 2; ++k) {
        const int t = loop[k];
        loop[k] = loop[len - 1 - k];
        loop[len - 1 - k] = t;
      }
    }
    for (int k = 1; k + 1 < len; ++k) {
      out[3 * n] = (int8_t)loop[0];
      out[3 * n + 1] = (int8_t)loop[k];
      out[3 * n + 2] = (int8_t)loop[k + 1];
      ++n;
    }
  }
  *ntri = n;
}

static void mc_tables(int8_t tri[256][16], uint8_t ntri[256]) {
  static const McGeometry G;
  for (int c = 0; c < 256; ++c) {
    int8_t row[16];
    for (int k = 0; k < 16; ++k) row[k] = -1;
    int n = 0;
    mc_case(G, c, row, &n);
    for (int k = 0; k < 16; ++k) tri[c][k] = row[k];
    ntri[c] = (uint8_t)n;
  }
}

static std::mutex g_mc_mutex;
static unsigned long long g_mc_loaded = 0;

static int mc_upload() {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev >= 64) {
    set_error("surface: no CUDA device");
    return SVIE_ERR_LAUNCH;
  }
  std::lock_guard<std::mutex> lock(g_mc_mutex);
  if ((g_mc_loaded >> dev) & 1ULL) return SVIE_OK;
  int8_t tri[256][16];
  uint8_t ntri[256];
  mc_tables(tri, ntri);
  if (cudaMemcpyToSymbol(c_mc_tri, tri, sizeof(tri)) != cudaSuccess ||
      cudaMemcpyToSymbol(c_mc_ntri, ntri, sizeof(ntri)) != cudaSuccess) {
    set_error("surface: table upload failed");
    return SVIE_ERR_LAUNCH;
  }
  g_mc_loaded |= 1ULL << dev;
  return SVIE_OK;
}

struct SfGrid {
  int nx, ny, nz;
  int sx, sy;
};

// case index of the cell with lower corner i, and the crossing bits of the
// three grid edges i -> i + e_a (bit a).
SVIE_DEV void cell_case(const float* __restrict__ f, int i, const SfGrid& G, int* cs, int* vbits) {
  int c = 0;
#pragma unroll
  for (int v = 0; v < 8; ++v) {
    const int off = (v & 1) * G.sx + ((v >> 1) & 1) * G.sy + ((v >> 2) & 1);
    c |= (__ldg(f + i + off) < 0.0f ? 1 : 0) << v;
  }
  const int in0 = c & 1;
  *vbits = ((((c >> 1) & 1) != in0) ? 1 : 0) | ((((c >> 2) & 1) != in0) ? 2 : 0) | ((((c >> 4) & 1) != in0) ? 4 : 0);
  *cs = c;
}

__global__ void __launch_bounds__(SF_THREADS) k_surf_count(const float* __restrict__ f,
                                                           const int32_t* __restrict__ band, long long m, SfGrid G,
                                                           int* counts) {
  __shared__ int sh[SF_THREADS / 32];
  const long long t = (long long)blockIdx.x * SF_THREADS + threadIdx.x;
  int nv = 0, nt = 0;
  if (t < m) {
    int cs, vb;
    cell_case(f, band[t], G, &cs, &vb);
    nv = __popc(vb);
    nt = c_mc_ntri[cs];
  }
  const int tv = block_reduce(nv, sh, OpSumI(), 0);
  const int tt = block_reduce(nt, sh, OpSumI(), 0);
  if (threadIdx.x == 0) {
    counts[blockIdx.x] = tv;
    counts[gridDim.x + blockIdx.x] = tt;
  }
}

// Exclusive prefix of one int per thread across the CTA.
SVIE_DEV int block_prefix(int v, int* sh) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  int x = v;
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  __syncthreads();
  if (lane == 31) sh[wid] = x;
  __syncthreads();
  if (threadIdx.x == 0) {
    int run = 0;
    for (int w = 0; w < nw; ++w) {
      const int c = sh[w];
      sh[w] = run;
      run += c;
    }
  }
  __syncthreads();
  return sh[wid] + x - v;
}

// Exclusive scan of the 2 nb block counts (vertices, then faces) in one CTA;
// totals -> totals[0], totals[1].
__global__ void __launch_bounds__(1024) k_surf_scan(int* counts, long long nb, long long* totals) {
  __shared__ int sh[32];
  for (int part = 0; part < 2; ++part) {
    int* c = counts + part * nb;
    const long long per = (nb + blockDim.x - 1) / blockDim.x;
    const long long s0 = (long long)threadIdx.x * per;
    const long long s1 = s0 + per < nb ? s0 + per : nb;
    long long local = 0;
    for (long long i = s0; i < s1; ++i) local += c[i];
    const int off = block_prefix((int)local, sh);
    long long run = off;
    for (long long i = s0; i < s1; ++i) {
      const int v = c[i];
      c[i] = (int)run;
      run += v;
    }
    if (threadIdx.x == blockDim.x - 1) totals[part] = run;
    __syncthreads();
  }
}

// Pass 2: vertices.  vinfo[i] = first vertex id of node i << 3 | crossing bits.
__global__ void __launch_bounds__(SF_THREADS) k_surf_vertices(const float* __restrict__ f,
                                                              const int32_t* __restrict__ band, long long m,
                                                              SfGrid G, const int* __restrict__ offsets,
                                                              int32_t* __restrict__ vinfo, float* __restrict__ verts,
                                                              long long nv_cap) {
  __shared__ int sh[32];
  const long long t = (long long)blockIdx.x * SF_THREADS + threadIdx.x;
  int i = 0, vb = 0;
  if (t < m) {
    int cs;
    i = band[t];
    cell_case(f, i, G, &cs, &vb);
  }
  const int v0 = offsets[blockIdx.x] + block_prefix(__popc(vb), sh);
  if (t >= m) return;
  vinfo[i] = (v0 << 3) | vb;
  if (!vb) return;
  const int x = i / G.sx, r = i - x * G.sx, y = r / G.sy, z = r - y * G.sy;
  const float p0 = __ldg(f + i);
  int v = v0;
  const int st[3] = {G.sx, G.sy, 1};
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    if (!((vb >> a) & 1)) continue;
    const float p1 = __ldg(f + i + st[a]);
    const float tt = p0 / (p0 - p1);
    float q[3] = {(float)x, (float)y, (float)z};
    q[a] = q[a] + tt;
    if (v < nv_cap) {
      verts[3LL * v] = q[0];
      verts[3LL * v + 1] = q[1];
      verts[3LL * v + 2] = q[2];
    }
    ++v;
  }
}

// Pass 3: faces (vertex ids of the three cell edges of every table triangle).
__global__ void __launch_bounds__(SF_THREADS) k_surf_faces(const float* __restrict__ f,
                                                           const int32_t* __restrict__ band, long long m, SfGrid G,
                                                           const int* __restrict__ offsets,
                                                           const int32_t* __restrict__ vinfo,
                                                           int32_t* __restrict__ faces, long long nt_cap) {
  __shared__ int sh[32];
  const long long t = (long long)blockIdx.x * SF_THREADS + threadIdx.x;
  int i = 0, cs = 0;
  if (t < m) {
    int vb;
    i = band[t];
    cell_case(f, i, G, &cs, &vb);
  }
  const int n = t < m ? (int)c_mc_ntri[cs] : 0;
  int o = offsets[blockIdx.x] + block_prefix(n, sh);
  if (!n) return;
  for (int k = 0; k < 3 * n; ++k) {
    const int e = c_mc_tri[cs][k];
    const int a = e >> 2, u = e & 1, w = (e >> 1) & 1;
    const int o0 = a == 0 ? 1 : 0, o1 = a == 2 ? 1 : 2;
    int d[3] = {0, 0, 0};
    d[o0] = u;
    d[o1] = w;
    const int owner = i + d[0] * G.sx + d[1] * G.sy + d[2];
    const int info = __ldg(vinfo + owner);
    const int rank = __popc(info & 7 & ((1 << a) - 1));
    const int j = k % 3;
    if (o < nt_cap) faces[3LL * o + j] = (info >> 3) + rank;
    if (j == 2) ++o;
  }
}

// One Newton step on the tricubic interpolant, limited to max_shift cells
// (surface.py:44-51).
__global__ void k_surf_project(const float* __restrict__ f, int ny, int nz, float* __restrict__ verts, long long nv,
                               float max_shift) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nv) return;
  const float3 p = make_float3(verts[3 * t], verts[3 * t + 1], verts[3 * t + 2]);
  float val, gx, gy, gz;
  tricubic_grad_at(f, ny, nz, p, &val, &gx, &gy, &gz);
  const float g2 = fmaxf(gx * gx + gy * gy + gz * gz, 1e-30f);
  const float s = val / g2;
  float sx = s * gx, sy = s * gy, sz = s * gz;
  const float nrm = sqrtf(sx * sx + sy * sy + sz * sz);
  const float scale = fminf(max_shift / fmaxf(nrm, max_shift), 1.0f);
  sx *= scale;
  sy *= scale;
  sz *= scale;
  verts[3 * t] = p.x - sx;
  verts[3 * t + 1] = p.y - sy;
  verts[3 * t + 2] = p.z - sz;
}

// Signed volume of the extracted mesh from its float32 index-coordinate
// vertices about (cx, cy, cz), accumulated in float64: only its sign is used
// (surface.py:54-55 flips the faces of a negative mesh).
__global__ void k_surf_volume(const float* __restrict__ v, const int32_t* __restrict__ f, long long T, double cx,
                              double cy, double cz, double* out) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  double s = 0.0;
  if (t < T) {
    double p[3][3];
    for (int a = 0; a < 3; ++a) {
      const long long vi = f[3 * t + a];
      p[a][0] = (double)v[3 * vi] - cx;
      p[a][1] = (double)v[3 * vi + 1] - cy;
      p[a][2] = (double)v[3 * vi + 2] - cz;
    }
    s = p[0][0] * (p[1][1] * p[2][2] - p[1][2] * p[2][1]) + p[0][1] * (p[1][2] * p[2][0] - p[1][0] * p[2][2]) +
        p[0][2] * (p[1][0] * p[2][1] - p[1][1] * p[2][0]);
  }
  s = warp_sum(s);
  if ((threadIdx.x & 31) == 0 && s != 0.0) atomicAdd(out, s / 6.0);
}

// World coordinates origin + h * v in float64, rounded after the product and
// after the sum as numpy rounds them (surface.py:56, grid.py:to_world).
__global__ void k_surf_world(const float* __restrict__ v, long long n3, double ox, double oy, double oz, double h,
                             double* __restrict__ out) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n3) return;
  const int a = (int)(i % 3);
  const double o = a == 0 ? ox : (a == 1 ? oy : oz);
  out[i] = __dadd_rn(o, __dmul_rn(h, (double)v[i]));
}

// Faces as int64, reversed (f2, f1, f0) when the signed volume is negative
// (surface.py:54-55); any negative index (a crossing met outside the band) is
// counted into *bad.
__global__ void k_surf_faces64(const int32_t* __restrict__ f, long long T, const double* __restrict__ vol,
                               int64_t* __restrict__ out, int* __restrict__ bad) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= T) return;
  const int a = f[3 * t], b = f[3 * t + 1], c = f[3 * t + 2];
  if ((a | b | c) < 0) atomicAdd(bad, 1);
  const bool flip = *vol < 0.0;
  out[3 * t] = flip ? c : a;
  out[3 * t + 1] = b;
  out[3 * t + 2] = flip ? a : c;
}

// float32((p - shift) / scale) of float64 points, as numpy's float64
// subtraction and division followed by the cast to float32; scale 1 is the
// plain shifted copy.
__global__ void k_points_f32(const double* __restrict__ p, long long n3, double sx, double sy, double sz,
                             double scale, float* __restrict__ out) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n3) return;
  const int a = (int)(i % 3);
  const double s = a == 0 ? sx : (a == 1 ? sy : sz);
  const double d = __dsub_rn(p[i], s);
  out[i] = __double2float_rn(scale == 1.0 ? d : __ddiv_rn(d, scale));
}

}  // namespace svie

using namespace svie;

extern "C" {

int svie_surface_table(int8_t* tri, uint8_t* ntri) {
  if (!tri || !ntri) {
    set_error("svie_surface_table: bad arguments");
    return SVIE_ERR_ARG;
  }
  int8_t t[256][16];
  uint8_t n[256];
  mc_tables(t, n);
  memcpy(tri, t, sizeof(t));
  memcpy(ntri, n, sizeof(n));
  return SVIE_OK;
}

size_t svie_surface_workspace_bytes(int64_t m) {
  const long long nb = (m + SF_THREADS - 1) / SF_THREADS;
  return (size_t)(2 * (nb < 1 ? 1 : nb)) * sizeof(int) + 256;
}

int svie_surface_scan(const float* phi, const int32_t* band, int64_t m, int nx, int ny, int nz, void* ws,
                      size_t ws_bytes, int64_t* totals, void* stream) {
  if (!phi || !totals || m < 0 || (m > 0 && !band) || (long long)nx * ny * nz >= (1LL << 31)) {
    set_error("svie_surface_scan: bad arguments");
    return SVIE_ERR_ARG;
  }
  if (!ws || ws_bytes < svie_surface_workspace_bytes(m)) {
    set_error("svie_surface_scan: workspace too small");
    return SVIE_ERR_WORKSPACE;
  }
  int st = mc_upload();
  if (st) return st;
  cudaStream_t s = (cudaStream_t)stream;
  if (m == 0) {
    if (cudaMemsetAsync(totals, 0, 2 * sizeof(int64_t), s) != cudaSuccess) return SVIE_ERR_LAUNCH;
    return SVIE_OK;
  }
  const long long nb = (m + SF_THREADS - 1) / SF_THREADS;
  const SfGrid G{nx, ny, nz, ny * nz, nz};
  k_surf_count<<<(unsigned)nb, SF_THREADS, 0, s>>>(phi, band, m, G, (int*)ws);
  k_surf_scan<<<1, 1024, 0, s>>>((int*)ws, nb, (long long*)totals);
  return launch_status("svie_surface_scan", 2);
}

int svie_surface_write(const float* phi, const int32_t* band, int64_t m, int nx, int ny, int nz, const void* ws,
                       size_t ws_bytes, int32_t* vinfo, float* verts, int64_t nv, int32_t* faces, int64_t nt,
                       void* stream) {
  if (!phi || !vinfo || m < 0 || (m > 0 && !band) || (nv > 0 && !verts) || (nt > 0 && !faces) ||
      nv >= (1LL << 28)) {
    set_error("svie_surface_write: bad arguments");
    return SVIE_ERR_ARG;
  }
  if (!ws || ws_bytes < svie_surface_workspace_bytes(m)) {
    set_error("svie_surface_write: workspace too small");
    return SVIE_ERR_WORKSPACE;
  }
  if (m == 0) return SVIE_OK;
  int st = mc_upload();
  if (st) return st;
  cudaStream_t s = (cudaStream_t)stream;
  const long long nb = (m + SF_THREADS - 1) / SF_THREADS;
  const SfGrid G{nx, ny, nz, ny * nz, nz};
  // owners outside the band (not expected for a distance-like phi) read as -1
  if (cudaMemsetAsync(vinfo, 0xFF, (size_t)nx * ny * nz * sizeof(int32_t), s) != cudaSuccess) {
    set_error("svie_surface_write: memset failed");
    return SVIE_ERR_LAUNCH;
  }
  k_surf_vertices<<<(unsigned)nb, SF_THREADS, 0, s>>>(phi, band, m, G, (const int*)ws, vinfo, verts, nv);
  k_surf_faces<<<(unsigned)nb, SF_THREADS, 0, s>>>(phi, band, m, G, (const int*)ws + nb, vinfo, faces, nt);
  return launch_status("svie_surface_write", 2);
}

int svie_surface_project(const float* phi, int ny, int nz, float* verts, int64_t nv, float max_shift, void* stream) {
  if (!phi || nv < 0 || (nv > 0 && !verts) || !(max_shift > 0)) {
    set_error("svie_surface_project: bad arguments");
    return SVIE_ERR_ARG;
  }
  if (nv == 0) return SVIE_OK;
  k_surf_project<<<blocks_for(nv, 256), 256, 0, (cudaStream_t)stream>>>(phi, ny, nz, verts, nv, max_shift);
  return launch_status("svie_surface_project");
}

int svie_surface_signed_volume(const float* verts, const int32_t* faces, int64_t nt, double cx, double cy, double cz,
                               double* out, void* stream) {
  if (nt < 0 || !out || (nt > 0 && (!verts || !faces))) {
    set_error("svie_surface_signed_volume: bad arguments");
    return SVIE_ERR_ARG;
  }
  cudaStream_t s = (cudaStream_t)stream;
  if (cudaMemsetAsync(out, 0, sizeof(double), s) != cudaSuccess) return SVIE_ERR_LAUNCH;
  if (nt == 0) return SVIE_OK;
  k_surf_volume<<<blocks_for(nt, 256), 256, 0, s>>>(verts, faces, nt, cx, cy, cz, out);
  return launch_status("svie_surface_signed_volume");
}

int svie_surface_finish(const float* verts, int64_t nv, const int32_t* faces, int64_t nt, const double* vol,
                        double ox, double oy, double oz, double h, double* world, int64_t* faces64, int* bad,
                        void* stream) {
  if (nv < 0 || nt < 0 || !vol || !bad || (nv > 0 && (!verts || !world)) || (nt > 0 && (!faces || !faces64))) {
    set_error("svie_surface_finish: bad arguments");
    return SVIE_ERR_ARG;
  }
  cudaStream_t s = (cudaStream_t)stream;
  if (cudaMemsetAsync(bad, 0, sizeof(int), s) != cudaSuccess) return SVIE_ERR_LAUNCH;
  int launches = 0;
  if (nv > 0) {
    k_surf_world<<<blocks_for(3 * nv, 256), 256, 0, s>>>(verts, 3 * nv, ox, oy, oz, h, world);
    ++launches;
  }
  if (nt > 0) {
    k_surf_faces64<<<blocks_for(nt, 256), 256, 0, s>>>(faces, nt, vol, faces64, bad);
    ++launches;
  }
  return launch_status("svie_surface_finish", launches);
}

int svie_points_f32(const double* points, int64_t n, double sx, double sy, double sz, double scale, float* out,
                    void* stream) {
  if (n < 0 || (n > 0 && (!points || !out)) || !(scale > 0.0)) {
    set_error("svie_points_f32: bad arguments");
    return SVIE_ERR_ARG;
  }
  if (n == 0) return SVIE_OK;
  k_points_f32<<<blocks_for(3 * n, 256), 256, 0, (cudaStream_t)stream>>>(points, 3 * n, sx, sy, sz, scale, out);
  return launch_status("svie_points_f32");
}

}  // extern "C"
