// Exact signed distance of a triangle mesh on the grid (reference
// svierosion/sdf.py:100-415), the one-time setup of every solve.
//
//  1. near field: one warp per triangle walks the nodes of its bounding box
//     dilated by `exact_band` cells and atomically minimises the packed key
//     (float bits of the distance << 32 | triangle id) per node;
//  2. closest-triangle propagation ring by ring over the 26-neighbourhood;
//  3. vertex-star refinement of nodes in (exact_band, band + 1];
//  4. sign by ray casting along grid lines: one warp per triangle rasterises
//     the lines that pierce it with the Simulation-of-Simplicity tie-break in
//     float64 (products and sums rounded exactly as in the reference, no FMA
//     contraction), then a prefix sum along the axis gives the winding number.
// Distances are evaluated in float32 index coordinates like the reference.
#include "common.cuh"

namespace svie {

SVIE_DEV float3 tri_v(const float* tri, long long t, int v) {
  const float* q = tri + 9 * t + 3 * v;
  return make_float3(q[0], q[1], q[2]);
}

SVIE_DEV float node_tri_dist(const float* tri, long long t, float px, float py, float pz) {
  return sqrtf(point_triangle_d2(make_float3(px, py, pz), tri_v(tri, t, 0), tri_v(tri, t, 1), tri_v(tri, t, 2)));
}

__global__ void k_keys_init(long long* keys, long long n) {
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x)
    keys[e] = 0x7fffffffffffffffLL;
}

// sdf.py:100-145; bbox from the float64 vertices, distances in float32.  A
// warp takes 32 triangles: each lane computes one triangle's node box in
// float64 (FP64 is slow on this part, so it runs once per triangle, not once
// per lane of a warp), then the warp walks the boxes one triangle after the
// other, a node per lane.
__global__ void k_near_field(const float* __restrict__ tri, const double* __restrict__ tri64, long long ntri, int nx,
                             int ny, int nz, double eb_cells, float eb_keep, unsigned long long* keys) {
  const long long t0 = (((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5) << 5;
  const int lane = threadIdx.x & 31;
  if (t0 >= ntri) return;  // whole warps
  const long long tl = t0 + lane;
  int lo[3] = {0, 0, 0}, dim[3] = {0, 0, 0};
  if (tl < ntri) {
    const double* q = tri64 + 9 * tl;
    const int shape[3] = {nx, ny, nz};
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      double mn = fmin(fmin(q[a], q[3 + a]), q[6 + a]);
      double mx = fmax(fmax(q[a], q[3 + a]), q[6 + a]);
      long long l = (long long)ceil(mn - eb_cells), h = (long long)floor(mx + eb_cells);
      l = l < 0 ? 0 : (l > shape[a] - 1 ? shape[a] - 1 : l);
      h = h < 0 ? 0 : (h > shape[a] - 1 ? shape[a] - 1 : h);
      lo[a] = (int)l;
      dim[a] = (int)(h - l + 1 > 0 ? h - l + 1 : 0);
    }
  }
  const long long syz = (long long)ny * nz;
  const int nt = (int)min(32LL, ntri - t0);
  // gridDim.y slices share the 32 triangles (big triangles: more warps per group)
  for (int k = blockIdx.y; k < nt; k += gridDim.y) {
    const int l0 = __shfl_sync(0xffffffffu, lo[0], k), l1 = __shfl_sync(0xffffffffu, lo[1], k),
              l2 = __shfl_sync(0xffffffffu, lo[2], k);
    const int d0 = __shfl_sync(0xffffffffu, dim[0], k), d1 = __shfl_sync(0xffffffffu, dim[1], k),
              d2 = __shfl_sync(0xffffffffu, dim[2], k);
    const long long t = t0 + k;
    const int d12 = d1 * d2, cnt = d0 * d12;  // below the grid size, < 2^31
    if (cnt == 0) continue;
    const float3 A = tri_v(tri, t, 0), B = tri_v(tri, t, 1), C = tri_v(tri, t, 2);
    for (int e = lane; e < cnt; e += 32) {
      const int ii = l0 + e / d12;
      const int rem = e - (e / d12) * d12;
      const int jj = l1 + rem / d2;
      const int kk = l2 + (rem - (rem / d2) * d2);
      const float d = sqrtf(point_triangle_d2(make_float3((float)ii, (float)jj, (float)kk), A, B, C));
      if (d <= eb_keep) {
        const unsigned long long key = ((unsigned long long)__float_as_uint(d) << 32) | (unsigned long long)t;
        atomicMin(keys + (ii * syz + (long long)jj * nz + kk), key);
      }
    }
  }
}

__global__ void k_unpack(const long long* __restrict__ keys, long long n, float* dist, int32_t* tid, uint8_t* known) {
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
    const long long k = keys[e];
    const bool found = k != 0x7fffffffffffffffLL;
    dist[e] = found ? __uint_as_float((unsigned int)(k >> 32)) : INFINITY;
    tid[e] = found ? (int32_t)(k & 0xffffffffLL) : -1;
    known[e] = found ? 1 : 0;
  }
}

__global__ void k_ring_mask(const uint8_t* __restrict__ known, int nx, int ny, int nz, uint8_t* ring) {
  const long long syz = (long long)ny * nz;
  const int z = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y, x = blockIdx.z;
  if (z >= nz) return;
  {
    const long long e = (long long)x * syz + (long long)y * nz + z;
    uint8_t r = 0;
    if (!known[e] && x > 0 && y > 0 && z > 0 && x < nx - 1 && y < ny - 1 && z < nz - 1) {
      for (int dx = -1; dx <= 1 && !r; ++dx)
        for (int dy = -1; dy <= 1 && !r; ++dy)
          for (int dz = -1; dz <= 1 && !r; ++dz)
            if (known[e + dx * syz + dy * nz + dz]) r = 1;
    }
    ring[e] = r;
  }
}

// The next ring from the last one: the unknown interior neighbours of the
// last ring's nodes.  Equal to k_ring_mask's set after the first ring: an
// unknown node next to an older known node would already be in a ring.
__global__ void k_ring_mark(const int32_t* __restrict__ last, long long m, const uint8_t* __restrict__ known, int nx,
                            int ny, int nz, uint8_t* ring) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= m) return;
  const long long syz = (long long)ny * nz;
  const long long u = last[t];
  const int x = (int)(u / syz), y = (int)((u / nz) % ny), z = (int)(u % nz);
  for (int dx = -1; dx <= 1; ++dx)
    for (int dy = -1; dy <= 1; ++dy)
      for (int dz = -1; dz <= 1; ++dz) {
        const int a = x + dx, b = y + dy, c = z + dz;
        if (a <= 0 || b <= 0 || c <= 0 || a >= nx - 1 || b >= ny - 1 || c >= nz - 1) continue;
        const long long e = (long long)a * syz + (long long)b * nz + c;
        if (!known[e]) ring[e] = 1;
      }
}

// The last K distinct triangle ids met by one thread, in registers (constant
// indices only).  A repeated candidate gives the same distance as its first
// visit, which can no longer be strictly smaller than the best (the best only
// decreases) nor change a minimum key, so it is skipped.
template <int K>
struct SeenTriangles {
  int v[K];
  int next = 0;
  SVIE_DEV SeenTriangles() {
#pragma unroll
    for (int k = 0; k < K; ++k) v[k] = -1;
  }
  // true if t (>= 0) is among the last K; otherwise records it in place of the oldest
  SVIE_DEV bool seen(int t) {
    bool hit = false;
#pragma unroll
    for (int k = 0; k < K; ++k) hit |= v[k] == t;
    if (hit) return true;
#pragma unroll
    for (int k = 0; k < K; ++k) v[k] = k == next ? t : v[k];
    next = next + 1 == K ? 0 : next + 1;
    return false;
  }
};

// sdf.py:183-200: best over the closest triangles of the 26 neighbours, in the
// reference's neighbour order (first strictly smaller distance wins).
__global__ void k_ring_update(const int32_t* __restrict__ upd, long long m, int nx, int ny, int nz,
                              const float* __restrict__ tri, const float* __restrict__ dist,
                              const int32_t* __restrict__ tid, float* new_dist, int32_t* new_tid) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= m) return;
  const long long n = (long long)nx * ny * nz;
  const long long syz = (long long)ny * nz;
  const long long u = upd[t];
  const float px = (float)(u / syz), py = (float)((u / nz) % ny), pz = (float)(u % nz);
  float best = dist[u];
  int32_t bt = tid[u];
  SeenTriangles<8> cache;
  for (int ox = -1; ox <= 1; ++ox)
    for (int oy = -1; oy <= 1; ++oy)
      for (int oz = -1; oz <= 1; ++oz) {
        if (ox == 0 && oy == 0 && oz == 0) continue;
        long long nb = u + ox * syz + oy * nz + oz;
        nb = nb < 0 ? 0 : (nb > n - 1 ? n - 1 : nb);
        const int32_t tt = tid[nb];
        if (tt < 0 || cache.seen(tt)) continue;
        const float d = node_tri_dist(tri, tt, px, py, pz);
        if (d < best) { best = d; bt = tt; }
      }
  new_dist[t] = best;
  new_tid[t] = bt;
}

__global__ void k_scatter(const int32_t* __restrict__ upd, long long m, const float* __restrict__ nd,
                          const int32_t* __restrict__ nt, float* dist, int32_t* tid, uint8_t* known) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= m) return;
  const long long u = upd[t];
  dist[u] = nd[t];
  tid[u] = nt[t];
  known[u] = 1;
}

__global__ void k_outer_mask(const float* __restrict__ dist, long long n, float lo, float hi, uint8_t* mask) {
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
    const float d = dist[e];
    mask[e] = (d > lo && d <= hi) ? 1 : 0;
  }
}

// sdf.py:211-265: minimum key over the vertex stars of the current triangle.
__global__ void k_star_pass(const int32_t* __restrict__ nodes, long long m, int ny, int nz, const float* __restrict__ tri,
                            const int32_t* __restrict__ vid, const int32_t* __restrict__ first,
                            const int32_t* __restrict__ deg, const int32_t* __restrict__ star, float* dist, int32_t* tid,
                            unsigned long long* changed) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  bool ch = false;
  if (t < m) {
    const long long u = nodes[t];
    const int32_t t0 = tid[u];
    if (t0 >= 0) {
      const long long syz = (long long)ny * nz;
      const float px = (float)(u / syz), py = (float)((u / nz) % ny), pz = (float)(u % nz);
      unsigned long long best = 0x7fffffffffffffffULL;
      SeenTriangles<8> cache;
      for (int v = 0; v < 3; ++v) {
        const int32_t vv = vid[3 * (long long)t0 + v];
        const int32_t f0 = first[vv], dg = deg[vv];
        for (int q = 0; q < dg; ++q) {
          const int32_t cand = star[f0 + q];
          if (cache.seen(cand)) continue;
          const float d = node_tri_dist(tri, cand, px, py, pz);
          const unsigned long long key = ((unsigned long long)__float_as_uint(d) << 32) | (unsigned int)cand;
          best = key < best ? key : best;
        }
      }
      const float bd = __uint_as_float((unsigned int)(best >> 32));
      if (bd < dist[u]) {
        dist[u] = bd;
        tid[u] = (int32_t)(best & 0xffffffffULL);
        ch = true;
      }
    }
  }
  const unsigned int c = __popc(__ballot_sync(0xffffffffu, ch));
  if ((threadIdx.x & 31) == 0 && c) atomicAdd(changed, (unsigned long long)c);
}

// _orient_sos (sdf.py:269-282): sign of x1*y2 - y1*x2 with the SoS tie-break.
SVIE_DEV int orient_sos(double x1, double y1, double x2, double y2, double* area) {
  const double a = __dsub_rn(__dmul_rn(x1, y2), __dmul_rn(y1, x2));
  *area = a;
  if (a > 0) return 1;
  if (a < 0) return -1;
  if (y2 > y1) return -1;
  if (y2 < y1) return 1;
  if (x1 > x2) return -1;
  if (x1 < x2) return 1;
  return 0;
}

// sdf.py:285-333 for one axis: a = axis, b = (a+1)%3, c = (a+2)%3; acc has
// (na+1) x nb x nc int32 counters.  A warp takes 32 triangles: each lane
// computes one triangle's range of grid lines (float64, once per triangle),
// then the warp walks the (triangle, line) pairs of all 32 triangles together,
// one pair per lane (a warp scan of the counts and a search for each pair's
// triangle), so the float64 crossing tests run with all lanes busy however
// few lines a triangle covers.
__global__ void k_crossings(const double* __restrict__ tri64, long long ntri, int na, int nb, int nc, int axis,
                            int signed_rule, int* acc) {
  const long long t0 = (((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5) << 5;
  const int lane = threadIdx.x & 31;
  if (t0 >= ntri) return;  // whole warps
  const long long tl = t0 + lane;
  const int a = axis, b = (axis + 1) % 3, c = (axis + 2) % 3;
  double U0 = 0, U1 = 0, U2 = 0, W0 = 0, W1 = 0, W2 = 0, Z0 = 0, Z1 = 0, Z2 = 0;
  int j0 = 0, k0 = 0, dk = 1, cnt = 0;
  if (tl < ntri) {
    const double* q = tri64 + 9 * tl;
    U0 = q[b]; U1 = q[3 + b]; U2 = q[6 + b];
    W0 = q[c]; W1 = q[3 + c]; W2 = q[6 + c];
    Z0 = q[a]; Z1 = q[3 + a]; Z2 = q[6 + a];
    const double j0d = ceil(fmin(fmin(U0, U1), U2)), j1d = floor(fmax(fmax(U0, U1), U2));
    const double k0d = ceil(fmin(fmin(W0, W1), W2)), k1d = floor(fmax(fmax(W0, W1), W2));
    const long long jl = (long long)fmin(fmax(j0d, 0.0), (double)nb), jh = (long long)fmin(fmax(j1d, -1.0), (double)(nb - 1));
    const long long kl = (long long)fmin(fmax(k0d, 0.0), (double)nc), kh = (long long)fmin(fmax(k1d, -1.0), (double)(nc - 1));
    const long long dj = jh - jl + 1 > 0 ? jh - jl + 1 : 0;
    const long long dkk = kh - kl + 1 > 0 ? kh - kl + 1 : 0;
    j0 = (int)jl;
    k0 = (int)kl;
    dk = dkk > 0 ? (int)dkk : 1;
    cnt = (int)(dj * dkk);  // lines of one triangle: below nb * nc < 2^31
  }
  long long incl = cnt;
  for (int o = 1; o < 32; o <<= 1) {
    const long long v = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += v;
  }
  const long long total = __shfl_sync(0xffffffffu, incl, 31);
  const long long excl = incl - cnt;
  // gridDim.y slices share the pairs (big triangles: more warps per group)
  for (long long base = 32LL * blockIdx.y; base < total; base += 32LL * gridDim.y) {
    const long long j = base + lane;
    // owner: the first lane whose inclusive count passes j (counts are non-decreasing)
    int own = 0;
    for (int step = 16; step; step >>= 1) {
      const long long v = __shfl_sync(0xffffffffu, incl, own + step - 1);
      if (v <= j) own += step;
    }
    const double u0 = __shfl_sync(0xffffffffu, U0, own), u1 = __shfl_sync(0xffffffffu, U1, own),
                 u2 = __shfl_sync(0xffffffffu, U2, own);
    const double w0 = __shfl_sync(0xffffffffu, W0, own), w1 = __shfl_sync(0xffffffffu, W1, own),
                 w2 = __shfl_sync(0xffffffffu, W2, own);
    const double z0 = __shfl_sync(0xffffffffu, Z0, own), z1 = __shfl_sync(0xffffffffu, Z1, own),
                 z2 = __shfl_sync(0xffffffffu, Z2, own);
    const int oj0 = __shfl_sync(0xffffffffu, j0, own), ok0 = __shfl_sync(0xffffffffu, k0, own),
              odk = __shfl_sync(0xffffffffu, dk, own);
    const long long oex = __shfl_sync(0xffffffffu, excl, own);
    if (j >= total) continue;
    const int e = (int)(j - oex);
    const int jj = oj0 + e / odk, kk = ok0 + (e - (e / odk) * odk);
    const double fj = (double)jj, fk = (double)kk;
    const double x1 = __dsub_rn(u0, fj), x2 = __dsub_rn(u1, fj), x3 = __dsub_rn(u2, fj);
    const double y1 = __dsub_rn(w0, fk), y2 = __dsub_rn(w1, fk), y3 = __dsub_rn(w2, fk);
    double A, B, C;
    const int sa = orient_sos(x2, y2, x3, y3, &A);
    const int sb = orient_sos(x3, y3, x1, y1, &B);
    const int sc = orient_sos(x1, y1, x2, y2, &C);
    if (!(sa != 0 && sb == sa && sc == sa)) continue;
    const double S = __dadd_rn(__dadd_rn(A, B), C);
    if (S == 0.0) continue;
    const double num = __dadd_rn(__dadd_rn(__dmul_rn(A, z0), __dmul_rn(B, z1)), __dmul_rn(C, z2));
    const double z = __ddiv_rn(num, S);
    long long i0 = (long long)floor(z) + 1;
    i0 = i0 < 0 ? 0 : (i0 > na ? na : i0);
    atomicAdd(acc + ((long long)i0 * nb + jj) * nc + kk, signed_rule ? -sa : 1);
  }
}

// Prefix sums along the axis; votes[x,y,z] += inside.
__global__ void k_inside(const int* __restrict__ acc, int nx, int ny, int nz, int axis, int signed_rule,
                         uint8_t* votes) {
  const int a = axis, b = (axis + 1) % 3, c = (axis + 2) % 3;
  const int shape[3] = {nx, ny, nz};
  const int na = shape[a], nb = shape[b], nc = shape[c];
  const long long lines = (long long)nb * nc;
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= lines) return;
  const int jj = (int)(t / nc), kk = (int)(t % nc);
  int run = 0;
  for (int i = 0; i < na; ++i) {
    run += acc[((long long)i * nb + jj) * nc + kk];
    const bool in = signed_rule ? (run != 0) : ((run & 1) != 0);
    int co[3];
    co[a] = i; co[b] = jj; co[c] = kk;
    if (in) votes[((long long)co[0] * ny + co[1]) * nz + co[2]] += 1;
  }
}

__global__ void k_sdf_finalize(const float* __restrict__ dist, const uint8_t* __restrict__ votes, long long n, int naxes,
                               float band, float h, float* phi) {
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
    const float d = __fmul_rn(fminf(dist[e], band), h);
    phi[e] = (2 * (int)votes[e] > naxes) ? -d : d;
  }
}

}  // namespace svie

using namespace svie;

extern "C" {

int svie_sdf_keys_init(int64_t* keys, int64_t n, void* stream) {
  if (!keys || n <= 0) {
    set_error("svie_sdf_keys_init: bad arguments");
    return SVIE_ERR_ARG;
  }
  k_keys_init<<<blocks_for(n, 256, 152 * 32), 256, 0, (cudaStream_t)stream>>>((long long*)keys, n);
  return launch_status("svie_sdf_keys_init");
}

int svie_sdf_near_field(const float* tri, const double* tri64, int64_t ntri, int nx, int ny, int nz,
                        double exact_band, float eb_keep, int slices, int64_t* keys, void* stream) {
  if (ntri < 0 || !keys || (ntri > 0 && (!tri || !tri64)) || ntri >= (1LL << 31) || slices < 1 || slices > 32) {
    set_error("svie_sdf_near_field: bad arguments");
    return SVIE_ERR_ARG;
  }
  if (ntri == 0) return SVIE_OK;
  // one warp per 32 triangles, times `slices`
  const dim3 grid(blocks_for(ntri, 256), slices);
  k_near_field<<<grid, 256, 0, (cudaStream_t)stream>>>(tri, tri64, ntri, nx, ny, nz, exact_band, eb_keep,
                                                        (unsigned long long*)keys);
  return launch_status("svie_sdf_near_field");
}

int svie_sdf_unpack(const int64_t* keys, int64_t n, float* dist, int32_t* tid, uint8_t* known, void* stream) {
  if (!keys || n <= 0) {
    set_error("svie_sdf_unpack: bad arguments");
    return SVIE_ERR_ARG;
  }
  k_unpack<<<blocks_for(n, 256, 152 * 32), 256, 0, (cudaStream_t)stream>>>((const long long*)keys, n, dist, tid, known);
  return launch_status("svie_sdf_unpack");
}

int svie_sdf_ring_mask(const uint8_t* known, int nx, int ny, int nz, uint8_t* ring, void* stream) {
  const long long n = (long long)nx * ny * nz;
  if (!known || !ring || n <= 0) {
    set_error("svie_sdf_ring_mask: bad arguments");
    return SVIE_ERR_ARG;
  }
  const dim3 gd((nz + 127) / 128, ny, nx);
  k_ring_mask<<<gd, 128, 0, (cudaStream_t)stream>>>(known, nx, ny, nz, ring);
  return launch_status("svie_sdf_ring_mask");
}

int svie_sdf_ring_mark(const int32_t* last, int64_t m, const uint8_t* known, int nx, int ny, int nz, uint8_t* ring,
                       void* stream) {
  if (m < 0 || !known || !ring || (m > 0 && !last) || nx < 1 || ny < 1 || nz < 1) {
    set_error("svie_sdf_ring_mark: bad arguments");
    return SVIE_ERR_ARG;
  }
  cudaStream_t s = (cudaStream_t)stream;
  if (cudaMemsetAsync(ring, 0, (size_t)nx * ny * nz, s) != cudaSuccess) {
    set_error("svie_sdf_ring_mark: memset failed");
    return SVIE_ERR_LAUNCH;
  }
  if (m == 0) return SVIE_OK;
  k_ring_mark<<<blocks_for(m, 256), 256, 0, s>>>(last, m, known, nx, ny, nz, ring);
  return launch_status("svie_sdf_ring_mark");
}

int svie_sdf_ring_update(const int32_t* upd, int64_t m, int nx, int ny, int nz, const float* tri, const float* dist,
                         const int32_t* tid, float* new_dist, int32_t* new_tid, void* stream) {
  if (m <= 0) return m < 0 ? SVIE_ERR_ARG : SVIE_OK;
  k_ring_update<<<blocks_for(m, 256), 256, 0, (cudaStream_t)stream>>>(upd, m, nx, ny, nz, tri, dist, tid, new_dist,
                                                                       new_tid);
  return launch_status("svie_sdf_ring_update");
}

int svie_sdf_scatter(const int32_t* upd, int64_t m, const float* new_dist, const int32_t* new_tid, float* dist,
                     int32_t* tid, uint8_t* known, void* stream) {
  if (m <= 0) return m < 0 ? SVIE_ERR_ARG : SVIE_OK;
  k_scatter<<<blocks_for(m, 256), 256, 0, (cudaStream_t)stream>>>(upd, m, new_dist, new_tid, dist, tid, known);
  return launch_status("svie_sdf_scatter");
}

int svie_sdf_outer_mask(const float* dist, int64_t n, float lo, float hi, uint8_t* mask, void* stream) {
  if (!dist || !mask || n <= 0) {
    set_error("svie_sdf_outer_mask: bad arguments");
    return SVIE_ERR_ARG;
  }
  k_outer_mask<<<blocks_for(n, 256, 152 * 32), 256, 0, (cudaStream_t)stream>>>(dist, n, lo, hi, mask);
  return launch_status("svie_sdf_outer_mask");
}

int svie_sdf_star_pass(const int32_t* nodes, int64_t m, int nx, int ny, int nz, const float* tri, const int32_t* vid,
                       const int32_t* first, const int32_t* deg, const int32_t* star, float* dist, int32_t* tid,
                       int64_t* changed, void* stream) {
  (void)nx;
  if (m <= 0) return m < 0 ? SVIE_ERR_ARG : SVIE_OK;
  k_star_pass<<<blocks_for(m, 256), 256, 0, (cudaStream_t)stream>>>(nodes, m, ny, nz, tri, vid, first, deg, star, dist,
                                                                     tid, (unsigned long long*)changed);
  return launch_status("svie_sdf_star_pass");
}

int svie_sdf_crossings(const double* tri64, int64_t ntri, int nx, int ny, int nz, int axis, int signed_rule,
                       int slices, int32_t* acc, void* stream) {
  if (ntri < 0 || axis < 0 || axis > 2 || !acc || ntri >= (1LL << 31) || slices < 1 || slices > 1024) {
    set_error("svie_sdf_crossings: bad arguments");
    return SVIE_ERR_ARG;
  }
  if (ntri == 0) return SVIE_OK;
  const int shape[3] = {nx, ny, nz};
  const int na = shape[axis], nb = shape[(axis + 1) % 3], nc = shape[(axis + 2) % 3];
  // one warp per 32 triangles, times `slices`
  const dim3 grid(blocks_for(ntri, 256), slices);
  k_crossings<<<grid, 256, 0, (cudaStream_t)stream>>>(tri64, ntri, na, nb, nc, axis, signed_rule, acc);
  return launch_status("svie_sdf_crossings");
}

int svie_sdf_inside(const int32_t* acc, int nx, int ny, int nz, int axis, int signed_rule, uint8_t* votes,
                    void* stream) {
  if (!acc || !votes || axis < 0 || axis > 2) {
    set_error("svie_sdf_inside: bad arguments");
    return SVIE_ERR_ARG;
  }
  const int shape[3] = {nx, ny, nz};
  const long long lines = (long long)shape[(axis + 1) % 3] * shape[(axis + 2) % 3];
  k_inside<<<blocks_for(lines, 128), 128, 0, (cudaStream_t)stream>>>(acc, nx, ny, nz, axis, signed_rule, votes);
  return launch_status("svie_sdf_inside");
}

int svie_sdf_finalize(const float* dist, const uint8_t* votes, int64_t n, int naxes, float band, float h, float* phi,
                      void* stream) {
  if (!dist || !votes || !phi || n <= 0 || naxes < 1) {
    set_error("svie_sdf_finalize: bad arguments");
    return SVIE_ERR_ARG;
  }
  k_sdf_finalize<<<blocks_for(n, 256, 152 * 32), 256, 0, (cudaStream_t)stream>>>(dist, votes, n, naxes, band, h, phi);
  return launch_status("svie_sdf_finalize");
}

}  // extern "C"
