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

// Order-preserving unsigned keys of floats (sign bit set for non-negative
// values, all bits flipped for negative ones).
SVIE_DEV unsigned int fkey(float x) {
  const unsigned int b = __float_as_uint(x);
  return (b >> 31) ? ~b : (b | 0x80000000u);
}

SVIE_DEV float fkey_value(unsigned int k) { return __uint_as_float((k >> 31) ? (k & 0x7fffffffu) : ~k); }

// Bounding box of the pieces of every cell, as keys: box[6 c + a] = min, box[6 c + 3 + a] = max.
__global__ void k_piece_box(const float* __restrict__ tri, long long T, CellGrid G, unsigned int* __restrict__ box) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= T) return;
  const int c = piece_cell(tri, t, G);
  for (int a = 0; a < 3; ++a) {
    const float v0 = tri[9 * t + a], v1 = tri[9 * t + 3 + a], v2 = tri[9 * t + 6 + a];
    atomicMin(box + 6LL * c + a, fkey(fminf(fminf(v0, v1), v2)));
    atomicMax(box + 6LL * c + 3 + a, fkey(fmaxf(fmaxf(v0, v1), v2)));
  }
}

// Occupancy of the cells, one bit per cell (32 cells per word, a warp per word).
__global__ void k_piece_occupancy(const int* __restrict__ start, long long cells, unsigned int* __restrict__ bits) {
  const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const bool full = c < cells && start[c] < start[c + 1];
  const unsigned int w = __ballot_sync(0xffffffffu, full);
  if ((threadIdx.x & 31) == 0 && c < cells) bits[c >> 5] = w;
}

// Bounding sphere of every piece, in the order of the cell lists: sph[k] = (centroid,
// radius) of piece order[k]; the radius is widened by 1e-5 relative so that it bounds
// the float32 vertices despite rounding.
__global__ void k_piece_spheres(const float* __restrict__ tri, const int* __restrict__ order, long long T,
                                float4* __restrict__ sph) {
  const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= T) return;
  const int t = order[k];
  const float3 a = piece_vertex(tri, t, 0), b = piece_vertex(tri, t, 1), c = piece_vertex(tri, t, 2);
  const float3 m = make_float3((a.x + b.x + c.x) * (1.0f / 3.0f), (a.y + b.y + c.y) * (1.0f / 3.0f),
                               (a.z + b.z + c.z) * (1.0f / 3.0f));
  auto d2 = [&](float3 v) { return (v.x - m.x) * (v.x - m.x) + (v.y - m.y) * (v.y - m.y) + (v.z - m.z) * (v.z - m.z); };
  const float r = sqrtf(fmaxf(fmaxf(d2(a), d2(b)), d2(c)));
  sph[k] = make_float4(m.x, m.y, m.z, r * 1.00001f + 1e-30f);
}

// min keys start at the largest key, max keys at the smallest
__global__ void k_piece_box_init(unsigned int* __restrict__ box, long long n6) {
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e < n6) box[e] = (e % 6) < 3 ? 0xffffffffu : 0u;
}

// keys -> floats; an empty cell gets the box [+inf, -inf], at infinite distance from every point
__global__ void k_piece_box_finish(const int* __restrict__ start, long long cells, unsigned int* __restrict__ box) {
  const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= cells) return;
  float* f = reinterpret_cast<float*>(box + 6 * c);
  const bool empty = start[c] == start[c + 1];
  for (int a = 0; a < 3; ++a) {
    const unsigned int lo = box[6 * c + a], hi = box[6 * c + 3 + a];
    f[a] = empty ? INFINITY : fkey_value(lo);
    f[3 + a] = empty ? -INFINITY : fkey_value(hi);
  }
}

// distance from v to the interval [lo, hi] (infinite for an empty interval)
SVIE_DEV float span_gap(float v, float lo, float hi) { return fmaxf(fmaxf(lo - v, v - hi), 0.0f); }

// distance from v to the interval [lo, lo + cs]
SVIE_DEV float box_gap(float v, float lo, float cs) { return fmaxf(fmaxf(lo - v, v - (lo + cs)), 0.0f); }

// Cell (dx, dy, dz) number q of the Chebyshev shell of radius r: the two z
// faces ((2r+1)^2 cells each), the two y faces ((2r+1)(2r-1)), the two x faces
// ((2r-1)^2); 24 r^2 + 2 cells for r > 0, one for r = 0.
SVIE_DEV void shell_cell(int r, int q, int& dx, int& dy, int& dz) {
  if (r == 0) {
    dx = dy = dz = 0;
    return;
  }
  // u / w for 0 <= u < w * w and w < 2048 by a float reciprocal: (u + 0.5) / w is at
  // least 0.5 / w away from an integer, far more than the float rounding error
  auto divmod = [](int u, int w, float inv_w, int& quo, int& rem) {
    quo = w < 2000 ? (int)(((float)u + 0.5f) * inv_w) : u / w;
    rem = u - quo * w;
  };
  const int s = 2 * r + 1, t = 2 * r - 1;
  const float inv_s = 1.0f / (float)s, inv_t = 1.0f / (float)t;
  const int zf = s * s, yf = s * t;
  int a, b;
  if (q < 2 * zf) {
    dz = q < zf ? -r : r;
    divmod(q < zf ? q : q - zf, s, inv_s, a, b);
    dx = a - r;
    dy = b - r;
    return;
  }
  q -= 2 * zf;
  if (q < 2 * yf) {
    dy = q < yf ? -r : r;
    divmod(q < yf ? q : q - yf, t, inv_t, a, b);
    dx = a - r;
    dz = b - (r - 1);
    return;
  }
  q -= 2 * yf;
  const int xf = t * t;
  dx = q < xf ? -r : r;
  divmod(q < xf ? q : q - xf, t, inv_t, a, b);
  dy = a - (r - 1);
  dz = b - (r - 1);
}

// One warp per query point.  The lanes split the cells of each Chebyshev
// shell around the point's cell; a cell is a candidate while it is not farther
// than the best distance so far: first by its own box widened by rho (no memory
// access), then by its occupancy bit, then by the bounding box of its pieces.
// Each shell takes two passes: the first tests one piece of every candidate
// cell, which gives the warp a near-final bound; the second tests the other
// pieces of the cells that are still candidates, spread over all 32 lanes (a
// warp scan of the per-cell counts and a search for each piece's cell) so that
// a cell with many pieces does not leave the other lanes idle, each piece first
// against its bounding sphere.  After each shell the warp takes the minimum and
// stops once no unvisited piece can be closer (pieces are binned by centroid,
// so an unvisited one is farther than r cs - rho).  The result is the exact
// minimum over the pieces.
__global__ void __launch_bounds__(128, 8) k_point_distance(const float* __restrict__ pts, long long n,
                                                        const float* __restrict__ tri, const int* __restrict__ start,
                                                        const int* __restrict__ order, const float* __restrict__ box,
                                                        const unsigned int* __restrict__ occ,
                                                        const float4* __restrict__ sph, CellGrid G, float rho,
                                                        float* __restrict__ out) {
  const long long i = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (i >= n) return;  // whole warps
  const float3 p = make_float3(pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]);
  const int cx = cell_of(p.x, G.ox, G.inv_cs, G.gx), cy = cell_of(p.y, G.oy, G.inv_cs, G.gy),
            cz = cell_of(p.z, G.oz, G.inv_cs, G.gz);
  const int rmax = max(max(G.gx, G.gy), G.gz);
  // cell number q of shell r if it lies in the grid and is a candidate for `bound`, else -1;
  // the squared box distance is shrunk by 1e-5 so that rounding never drops a cell
  auto candidate = [&](int r, int q, float bound) -> int {
    int dx, dy, dz;
    shell_cell(r, q, dx, dy, dz);
    const int x = cx + dx, y = cy + dy, z = cz + dz;
    if (x < 0 || y < 0 || z < 0 || x >= G.gx || y >= G.gy || z >= G.gz) return -1;
    // the cell's own box, widened by rho, first (no memory access), then its occupancy bit
    const float ex = box_gap(p.x, G.ox + x * G.cs, G.cs), ey = box_gap(p.y, G.oy + y * G.cs, G.cs),
                ez = box_gap(p.z, G.oz + z * G.cs, G.cs);
    const float cgap = sqrtf(ex * ex + ey * ey + ez * ez) - rho;
    if (cgap > 0.0f && cgap * cgap * 0.99999f > bound) return -1;
    const int c = (x * G.gy + y) * G.gz + z;
    if (!((occ[c >> 5] >> (c & 31)) & 1u)) return -1;
    const float* b = box + 6LL * c;
    const float bx = span_gap(p.x, b[0], b[3]), by = span_gap(p.y, b[1], b[4]), bz = span_gap(p.z, b[2], b[5]);
    const float g2 = (bx * bx + by * by + bz * bz) * 0.99999f;
    return (g2 <= bound && g2 < INFINITY) ? c : -1;
  };
  auto piece_d2 = [&](int k) {
    const int t = order[k];
    return point_triangle_d2(p, piece_vertex(tri, t, 0), piece_vertex(tri, t, 1), piece_vertex(tri, t, 2));
  };
  float best = INFINITY;
  for (int r = 0; r <= rmax; ++r) {
    const int ncell = r ? 24 * r * r + 2 : 1;
    // pass 1: the first piece of every candidate cell.  Bit k of `was` records whether the
    // lane's k-th cell (q = lane + 32 k, k < 32) was a candidate: the bound only shrinks, so
    // pass 2 need not test the others again.
    unsigned int was = 0;
    for (int q = lane, k = 0; q < ncell; q += 32, ++k) {
      const int c = candidate(r, q, best);
      if (c >= 0) {
        if (k < 32) was |= 1u << k;
        const int k0 = start[c];
        if (k0 < start[c + 1]) best = fminf(best, piece_d2(k0));
      }
    }
    best = warp_min(best);
    // pass 2: the remaining pieces of the cells that are still candidates
    for (int q0 = 0, k = 0; q0 < ncell; q0 += 32, ++k) {
      const int q = q0 + lane;
      int k1 = 0, cnt = 0;
      if (q < ncell && (k >= 32 || ((was >> k) & 1u))) {
        const int c = candidate(r, q, best);
        if (c >= 0) {
          k1 = start[c] + 1;
          cnt = max(start[c + 1] - k1, 0);
        }
      }
      int incl = cnt;
      for (int o = 1; o < 32; o <<= 1) {
        const int v = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += v;
      }
      const int total = __shfl_sync(0xffffffffu, incl, 31);
      const int excl = incl - cnt;
      for (int base = 0; base < total; base += 32) {
        const int j = base + lane;
        // owner: the first lane whose inclusive count passes j (counts are non-decreasing)
        int lo = 0;
        for (int step = 16; step; step >>= 1) {
          const int v = __shfl_sync(0xffffffffu, incl, lo + step - 1);
          if (v <= j) lo += step;
        }
        const int ok1 = __shfl_sync(0xffffffffu, k1, lo), oex = __shfl_sync(0xffffffffu, excl, lo);
        if (j < total) {
          // the piece's bounding sphere first: skip it when even the sphere is farther than the best
          const int k = ok1 + (j - oex);
          const float4 b = __ldg(sph + k);
          const float ex = p.x - b.x, ey = p.y - b.y, ez = p.z - b.z;
          const float lb = sqrtf(ex * ex + ey * ey + ez * ez) - b.w;
          if (lb <= 0.0f || lb * lb * 0.99999f <= best) best = fminf(best, piece_d2(k));
        }
      }
    }
    best = warp_min(best);
    // unvisited centroids are farther than r cs (also for p outside the grid box,
    // whose cell is clamped: the bound only gets looser), unvisited pieces than r cs - rho
    const float reach = (float)r * G.cs - rho;
    if (reach > 0.0f && best <= reach * reach) break;
  }
  if (lane == 0) out[i] = sqrtf(best);
}

}  // namespace svie

using namespace svie;

extern "C" {

// Piece grid workspace: start (cells + 1), cursor (cells + 1), order (T), scan
// sums, then the per-cell piece boxes (6 floats per cell, 16-byte aligned).
static long long piece_box_offset(long long T, long long cells) {
  const long long nb = (cells + 1 + 1023) / 1024;
  return ((2 * (cells + 1) + T + nb) + 3) / 4 * 4;  // in ints
}

// then the occupancy bits (one per cell), then the piece spheres (float4 per piece, 16-byte aligned)
static long long piece_sphere_offset(long long T, long long cells) {
  return (piece_box_offset(T, cells) + 6 * cells + (cells + 31) / 32 + 3) / 4 * 4;  // in ints
}

size_t svie_piece_grid_bytes(int64_t T, int gx, int gy, int gz) {
  const long long cells = (long long)gx * gy * gz;
  return (size_t)(piece_sphere_offset(T, cells) + 4 * T) * sizeof(int) + 256;
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
  unsigned int* box = (unsigned int*)ws + piece_box_offset(T, cells);
  k_piece_box_init<<<blocks_for(6 * cells, 256), 256, 0, s>>>(box, 6 * cells);
  if (T > 0) k_piece_count<<<blocks_for(T, 256), 256, 0, s>>>(tri, T, G, start);
  scan_exclusive_i32(start, cells + 1, sums, s);
  if (T > 0) {
    k_piece_fill<<<blocks_for(T, 256), 256, 0, s>>>(tri, T, G, start, cursor, order);
    k_piece_box<<<blocks_for(T, 256), 256, 0, s>>>(tri, T, G, box);
    k_piece_spheres<<<blocks_for(T, 256), 256, 0, s>>>(tri, order, T,
                                                      (float4*)((int*)ws + piece_sphere_offset(T, cells)));
  }
  k_piece_box_finish<<<blocks_for(cells, 256), 256, 0, s>>>(start, cells, box);
  k_piece_occupancy<<<blocks_for(cells, 256), 256, 0, s>>>(start, cells, box + 6 * cells);
  return launch_status("svie_piece_grid_build", T > 0 ? 10 : 6);
}

int svie_point_mesh_distance(const float* pts, int64_t n, const float* tri, int64_t T, float ox, float oy, float oz,
                             float cs, int gx, int gy, int gz, const void* ws, size_t ws_bytes, float rho, float* out,
                             void* stream) {
  if (n < 0 || n >= (1LL << 31) || (n > 0 && (!pts || !out)) || (T > 0 && !tri) || !ws) {
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
  const float* box = (const float*)ws + piece_box_offset(T, cells);
  const unsigned int* occ = (const unsigned int*)(box + 6 * cells);
  const float4* sph = (const float4*)((const int*)ws + piece_sphere_offset(T, cells));
  const CellGrid G{ox, oy, oz, cs, 1.0f / cs, gx, gy, gz};
  k_point_distance<<<blocks_for(32 * n, 128), 128, 0, (cudaStream_t)stream>>>(pts, n, tri, start, order, box, occ,
                                                                               sph, G, rho, out);
  return launch_status("svie_point_mesh_distance");
}

}  // extern "C"
