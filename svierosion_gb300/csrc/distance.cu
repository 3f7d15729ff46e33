// Exact unsigned distance from points to a triangle soup (the vertex depth
// annotation, reference svierosion/api.py:104-168).
//
// The reference finds candidates with a k-d tree over the centroids of the
// (bisected) triangles.  Here the pieces are binned by centroid into a uniform
// cell grid (counting sort: counts, a scan, a fill), and every point walks
// Chebyshev shells of cells around its own cell, testing each piece with the
// squared-distance routine of the SDF.  Once shells 0..r are done, every
// unvisited centroid is farther than r * cs from the point, so every unvisited
// piece is farther than r * cs - rho (rho bounds centroid-to-piece distances);
// the walk stops when the best distance is within that bound, which makes the
// result the exact minimum over all pieces (the reference's exact=True).
#include "common.cuh"

namespace svie {

struct CellGrid {
  float ox, oy, oz, cs, inv_cs;
  int gx, gy, gz;
};

SVIE_DEV int cell_of(float v, float o, float inv_cs, int n) {
  const int c = (int)floorf((v - o) * inv_cs);
  return c < 0 ? 0 : (c >= n ? n - 1 : c);
}

SVIE_DEV float3 piece_vertex(const float* tri, long long t, int v) {
  const float* q = tri + 9 * t + 3 * v;
  return make_float3(q[0], q[1], q[2]);
}

SVIE_DEV int piece_cell(const float* tri, long long t, const CellGrid& G) {
  const float cx = (tri[9 * t] + tri[9 * t + 3] + tri[9 * t + 6]) * (1.0f / 3.0f);
  const float cy = (tri[9 * t + 1] + tri[9 * t + 4] + tri[9 * t + 7]) * (1.0f / 3.0f);
  const float cz = (tri[9 * t + 2] + tri[9 * t + 5] + tri[9 * t + 8]) * (1.0f / 3.0f);
  return (cell_of(cx, G.ox, G.inv_cs, G.gx) * G.gy + cell_of(cy, G.oy, G.inv_cs, G.gy)) * G.gz +
         cell_of(cz, G.oz, G.inv_cs, G.gz);
}

__global__ void k_piece_count(const float* __restrict__ tri, long long T, CellGrid G, int* __restrict__ count) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < T) atomicAdd(count + piece_cell(tri, t, G), 1);
}

// In-place exclusive scan of n ints: per-CTA scans of 1024 entries, then a
// single CTA over the CTA totals, then the offsets added back.
__global__ void __launch_bounds__(1024) k_scan_local(int* __restrict__ v, long long n, int* __restrict__ sums) {
  __shared__ int sh[32];
  const long long i = (long long)blockIdx.x * 1024 + threadIdx.x;
  const int x = i < n ? v[i] : 0;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  int s = x;
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, s, o);
    if (lane >= o) s += y;
  }
  if (lane == 31) sh[wid] = s;
  __syncthreads();
  if (wid == 0) {
    int w = sh[lane];
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += y;
    }
    sh[lane] = w;
  }
  __syncthreads();
  const int incl = s + (wid ? sh[wid - 1] : 0);
  if (i < n) v[i] = incl - x;
  if (threadIdx.x == 1023) sums[blockIdx.x] = incl;
}

__global__ void __launch_bounds__(1024) k_scan_sums(int* __restrict__ sums, long long nb) {
  __shared__ int sh[32];
  const long long per = (nb + 1023) / 1024;
  const long long s0 = (long long)threadIdx.x * per, s1 = s0 + per < nb ? s0 + per : nb;
  int local = 0;
  for (long long i = s0; i < s1; ++i) local += sums[i];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  int s = local;
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, s, o);
    if (lane >= o) s += y;
  }
  if (lane == 31) sh[wid] = s;
  __syncthreads();
  if (wid == 0) {
    int w = sh[lane];
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += y;
    }
    sh[lane] = w;
  }
  __syncthreads();
  int run = s - local + (wid ? sh[wid - 1] : 0);
  for (long long i = s0; i < s1; ++i) {
    const int c = sums[i];
    sums[i] = run;
    run += c;
  }
}

__global__ void k_scan_add(int* __restrict__ v, long long n, const int* __restrict__ sums) {
  const long long i = (long long)blockIdx.x * 1024 + threadIdx.x;
  if (i < n) v[i] += sums[blockIdx.x];
}

// In-place exclusive scan of n ints; sums: ceil(n / 1024) ints of scratch.
// Returns the number of kernels launched.
int scan_exclusive_i32(int* v, long long n, int* sums, cudaStream_t s) {
  if (n <= 0) return 0;
  const long long nb = (n + 1023) / 1024;
  k_scan_local<<<(unsigned)nb, 1024, 0, s>>>(v, n, sums);
  k_scan_sums<<<1, 1024, 0, s>>>(sums, nb);
  k_scan_add<<<(unsigned)nb, 1024, 0, s>>>(v, n, sums);
  return 3;
}

__global__ void k_piece_fill(const float* __restrict__ tri, long long T, CellGrid G, const int* __restrict__ start,
                             int* __restrict__ cursor, int* __restrict__ order) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= T) return;
  const int c = piece_cell(tri, t, G);
  order[start[c] + atomicAdd(cursor + c, 1)] = (int)t;
}

// distance from v to the interval [lo, lo + cs]
SVIE_DEV float box_gap(float v, float lo, float cs) { return fmaxf(fmaxf(lo - v, v - (lo + cs)), 0.0f); }

SVIE_DEV void visit_cell(const float* __restrict__ tri, const int* __restrict__ start, const int* __restrict__ order,
                         int c, float3 p, float* best) {
  const int e = start[c + 1];
  for (int k = start[c]; k < e; ++k) {
    const int t = order[k];
    const float d2 = point_triangle_d2(p, piece_vertex(tri, t, 0), piece_vertex(tri, t, 1), piece_vertex(tri, t, 2));
    *best = fminf(*best, d2);
  }
}

__global__ void k_point_distance(const float* __restrict__ pts, long long n, const float* __restrict__ tri,
                                 const int* __restrict__ start, const int* __restrict__ order, CellGrid G, float rho,
                                 float* __restrict__ out) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float3 p = make_float3(pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]);
  const int cx = cell_of(p.x, G.ox, G.inv_cs, G.gx), cy = cell_of(p.y, G.oy, G.inv_cs, G.gy),
            cz = cell_of(p.z, G.oz, G.inv_cs, G.gz);
  const int rmax = max(max(G.gx, G.gy), G.gz);
  float best = INFINITY;
  for (int r = 0; r <= rmax; ++r) {
    const int x0 = cx - r, x1 = cx + r, y0 = cy - r, y1 = cy + r, z0 = cz - r, z1 = cz + r;
    for (int x = max(x0, 0); x <= min(x1, G.gx - 1); ++x) {
      const float bx = box_gap(p.x, G.ox + x * G.cs, G.cs);
      for (int y = max(y0, 0); y <= min(y1, G.gy - 1); ++y) {
        const float by = box_gap(p.y, G.oy + y * G.cs, G.cs);
        const bool face = (x == x0 || x == x1 || y == y0 || y == y1);
        const int base = (x * G.gy + y) * G.gz;
        // on an x or y face of the shell every z; inside it only the two z faces
        const int zs = face ? max(z0, 0) : (z0 >= 0 ? z0 : z1);
        const int ze = min(z1, G.gz - 1);
        const int step = face ? 1 : (z1 - z0 > 0 ? z1 - z0 : 1);
        for (int z = zs; z <= ze; z += step) {
          // a cell whose box is farther than the best distance + rho holds no closer piece
          const float bz = box_gap(p.z, G.oz + z * G.cs, G.cs);
          const float gap = sqrtf(bx * bx + by * by + bz * bz) - rho;
          if (gap <= 0.0f || gap * gap <= best) visit_cell(tri, start, order, base + z, p, &best);
        }
      }
    }
    // unvisited centroids are farther than r cs (also for p outside the grid box,
    // whose cell is clamped: the bound only gets looser), unvisited pieces than r cs - rho
    const float reach = (float)r * G.cs - rho;
    if (reach > 0.0f && best <= reach * reach) break;
  }
  out[i] = sqrtf(best);
}

}  // namespace svie

using namespace svie;

extern "C" {

size_t svie_piece_grid_bytes(int64_t T, int gx, int gy, int gz) {
  const long long cells = (long long)gx * gy * gz;
  const long long nb = (cells + 1 + 1023) / 1024;
  return (size_t)(2 * (cells + 1) + T + nb) * sizeof(int) + 256;
}

int svie_piece_grid_build(const float* tri, int64_t T, float ox, float oy, float oz, float cs, int gx, int gy, int gz,
                          void* ws, size_t ws_bytes, void* stream) {
  const long long cells = (long long)gx * gy * gz;
  if (T < 0 || (T > 0 && !tri) || gx < 1 || gy < 1 || gz < 1 || !(cs > 0) || cells >= (1LL << 30) ||
      T >= (1LL << 31)) {
    set_error("svie_piece_grid_build: bad arguments");
    return SVIE_ERR_ARG;
  }
  if (!ws || ws_bytes < svie_piece_grid_bytes(T, gx, gy, gz)) {
    set_error("svie_piece_grid_build: workspace too small");
    return SVIE_ERR_WORKSPACE;
  }
  cudaStream_t s = (cudaStream_t)stream;
  int* start = (int*)ws;          // cells + 1
  int* cursor = start + cells + 1;  // cells + 1
  int* order = cursor + cells + 1;  // T
  int* sums = order + T;            // blocks of the scan
  if (cudaMemsetAsync(start, 0, (size_t)(2 * (cells + 1)) * sizeof(int), s) != cudaSuccess) {
    set_error("svie_piece_grid_build: memset failed");
    return SVIE_ERR_LAUNCH;
  }
  const CellGrid G{ox, oy, oz, cs, 1.0f / cs, gx, gy, gz};
  if (T > 0) k_piece_count<<<blocks_for(T, 256), 256, 0, s>>>(tri, T, G, start);
  scan_exclusive_i32(start, cells + 1, sums, s);
  if (T > 0) k_piece_fill<<<blocks_for(T, 256), 256, 0, s>>>(tri, T, G, start, cursor, order);
  return launch_status("svie_piece_grid_build", T > 0 ? 5 : 3);
}

int svie_point_mesh_distance(const float* pts, int64_t n, const float* tri, int64_t T, float ox, float oy, float oz,
                             float cs, int gx, int gy, int gz, const void* ws, size_t ws_bytes, float rho, float* out,
                             void* stream) {
  if (n < 0 || (n > 0 && (!pts || !out)) || (T > 0 && !tri) || !ws) {
    set_error("svie_point_mesh_distance: bad arguments");
    return SVIE_ERR_ARG;
  }
  if (ws_bytes < svie_piece_grid_bytes(T, gx, gy, gz)) {
    set_error("svie_point_mesh_distance: workspace too small");
    return SVIE_ERR_WORKSPACE;
  }
  if (n == 0) return SVIE_OK;
  const long long cells = (long long)gx * gy * gz;
  const int* start = (const int*)ws;
  const int* order = start + 2 * (cells + 1);
  const CellGrid G{ox, oy, oz, cs, 1.0f / cs, gx, gy, gz};
  k_point_distance<<<blocks_for(n, 128), 128, 0, (cudaStream_t)stream>>>(pts, n, tri, start, order, G, rho, out);
  return launch_status("svie_point_mesh_distance");
}

}  // extern "C"
