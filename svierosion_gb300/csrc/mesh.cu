// Mesh preprocessing of the SDF on the GPU (the host-side numpy work of the
// reference's mesh_to_sdf / erode: svierosion/sdf.py:205-208,385,398-402 and
// svierosion/meshio.py:80-105).
//
//  * triangle soup in index coordinates (float64 and float32) and its longest
//    edge, so the caller knows whether split_long_triangles has any work;
//  * vertex welding: exactly coincident points get one id (np.unique on rows),
//    through an open-addressing hash table keyed by the coordinate bits;
//  * vertex stars as CSR (degree, first, triangle ids grouped by vertex);
//  * edge topology (boundary / non-manifold / misoriented edge counts) through
//    a hash table of undirected edges;
//  * the signed volume of the mesh in float64.
// Hash tables live in caller workspaces; every probe loop is bounded and
// reports SVIE_ERR_CAPACITY through a device flag instead of spinning.
#include <algorithm>

#include "common.cuh"

namespace svie {

SVIE_DEV unsigned long long mix64(unsigned long long x) {
  // splittable 64-bit finaliser (xor-shift-multiply)
  x ^= x >> 31;
  x *= 0x7fb5d329728ea185ULL;
  x ^= x >> 27;
  x *= 0x81dadef4bc2dd44dULL;
  x ^= x >> 33;
  return x;
}

SVIE_DEV unsigned long long dbits(double v) {
  return (unsigned long long)__double_as_longlong(v + 0.0);  // -0.0 and +0.0 weld together
}

__global__ void k_tri_index(const double* __restrict__ v, const int32_t* __restrict__ f, long long T, double ox,
                            double oy, double oz, double h, double* __restrict__ tri64, float* __restrict__ tri32,
                            unsigned int* max_edge_bits) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  float emax = 0.0f;
  if (t < T) {
    double p[3][3];
    for (int a = 0; a < 3; ++a) {
      const long long vi = f[3 * t + a];
      p[a][0] = (v[3 * vi] - ox) / h;
      p[a][1] = (v[3 * vi + 1] - oy) / h;
      p[a][2] = (v[3 * vi + 2] - oz) / h;
      for (int c = 0; c < 3; ++c) {
        tri64[9 * t + 3 * a + c] = p[a][c];
        tri32[9 * t + 3 * a + c] = (float)p[a][c];
      }
    }
    for (int a = 0; a < 3; ++a) {
      const int b = (a + 1) % 3;
      double dx = p[b][0] - p[a][0], dy = p[b][1] - p[a][1], dz = p[b][2] - p[a][2];
      emax = fmaxf(emax, (float)sqrt(dx * dx + dy * dy + dz * dz));
    }
  }
  emax = warp_max(emax);
  if ((threadIdx.x & 31) == 0 && emax > 0.0f) atomicMax(max_edge_bits, __float_as_uint(emax));
}

// ids[i] = representative of the points equal to point i (welding).
__global__ void k_weld(const double* __restrict__ pts, long long n, int* table, long long cap, int32_t* ids,
                       int* overflow) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double x = pts[3 * i], y = pts[3 * i + 1], z = pts[3 * i + 2];
  unsigned long long hsh = mix64(dbits(x) ^ mix64(dbits(y) ^ mix64(dbits(z))));
  long long s = (long long)(hsh % (unsigned long long)cap);
  for (long long probe = 0; probe < cap; ++probe) {
    int cur = table[s];
    if (cur < 0) {
      cur = atomicCAS(table + s, -1, (int)i);
      if (cur < 0) {
        ids[i] = (int32_t)i;
        return;
      }
    }
    if (pts[3 * (long long)cur] == x && pts[3 * (long long)cur + 1] == y && pts[3 * (long long)cur + 2] == z) {
      ids[i] = cur;
      return;
    }
    s = (s + 1 == cap) ? 0 : s + 1;
  }
  atomicExch(overflow, 1);
  ids[i] = (int32_t)i;
}

__global__ void k_gather_ids(const int32_t* __restrict__ faces, const int32_t* __restrict__ weld, long long n3,
                             int32_t* vid) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n3) vid[t] = weld ? weld[faces ? faces[t] : t] : faces[t];
}

__global__ void k_degree(const int32_t* __restrict__ vid, long long n3, int* deg) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n3) atomicAdd(deg + vid[t], 1);
}

// exclusive scan of deg into first (single CTA, sequential chunks per thread)
__global__ void __launch_bounds__(1024) k_scan_deg(const int* deg, long long nv, int* first) {
  __shared__ long long sh[1024];
  const long long per = (nv + blockDim.x - 1) / blockDim.x;
  const long long s0 = (long long)threadIdx.x * per;
  const long long s1 = min(s0 + per, nv);
  long long loc = 0;
  for (long long i = s0; i < s1; ++i) loc += deg[i];
  sh[threadIdx.x] = loc;
  __syncthreads();
  for (int o = 1; o < 1024; o <<= 1) {
    long long v = threadIdx.x >= o ? sh[threadIdx.x - o] : 0;
    __syncthreads();
    sh[threadIdx.x] += v;
    __syncthreads();
  }
  long long run = sh[threadIdx.x] - loc;
  for (long long i = s0; i < s1; ++i) {
    first[i] = (int)run;
    run += deg[i];
  }
}

__global__ void k_fill_star(const int32_t* __restrict__ vid, long long n3, const int* first, int* cursor,
                            int32_t* star) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n3) return;
  const int v = vid[t];
  star[first[v] + atomicAdd(cursor + v, 1)] = (int32_t)(t / 3);
}

// Undirected edges of the faces as given (meshio.py:88-105): count and
// direction sum (+1 for a < b, -1 otherwise) per edge.
__global__ void k_edges(const int32_t* __restrict__ f, long long T, unsigned long long* keys, int* count, int* dsum,
                        long long cap, int* overflow) {
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= 3 * T) return;
  const long long t = e / 3;
  const int j = (int)(e - 3 * t);
  const unsigned int a = (unsigned int)f[3 * t + j], b = (unsigned int)f[3 * t + (j + 1) % 3];
  const unsigned int lo = a < b ? a : b, hi = a < b ? b : a;
  const unsigned long long key = ((unsigned long long)lo << 32) | hi;
  long long s = (long long)(mix64(key) % (unsigned long long)cap);
  for (long long probe = 0; probe < cap; ++probe) {
    unsigned long long cur = keys[s];
    if (cur == ~0ULL) {
      cur = atomicCAS(keys + s, ~0ULL, key);
      if (cur == ~0ULL) cur = key;
    }
    if (cur == key) {
      atomicAdd(count + s, 1);
      atomicAdd(dsum + s, a < b ? 1 : -1);
      return;
    }
    s = (s + 1 == cap) ? 0 : s + 1;
  }
  atomicExch(overflow, 1);
}

__global__ void k_edge_stats(const unsigned long long* __restrict__ keys, const int* __restrict__ count,
                             const int* __restrict__ dsum, long long cap, unsigned long long* out) {
  const long long s = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= cap || keys[s] == ~0ULL) return;
  const int c = count[s];
  atomicAdd(out + 0, 1ULL);                             // edges
  if (c == 1) atomicAdd(out + 1, 1ULL);                 // boundary
  if (c > 2) atomicAdd(out + 2, 1ULL);                  // non-manifold
  if (c == 2 && dsum[s] != 0) atomicAdd(out + 3, 1ULL); // misoriented
}

// float64 signed volume (meshio.py:80-83) relative to the vertex mean `c`.
__global__ void k_signed_volume(const double* __restrict__ v, const int32_t* __restrict__ f, long long T, double cx,
                                double cy, double cz, double* out) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  double s = 0.0;
  if (t < T) {
    double p[3][3];
    for (int a = 0; a < 3; ++a) {
      const long long vi = f[3 * t + a];
      p[a][0] = v[3 * vi] - cx;
      p[a][1] = v[3 * vi + 1] - cy;
      p[a][2] = v[3 * vi + 2] - cz;
    }
    const double cxp = p[1][1] * p[2][2] - p[1][2] * p[2][1];
    const double cyp = p[1][2] * p[2][0] - p[1][0] * p[2][2];
    const double czp = p[1][0] * p[2][1] - p[1][1] * p[2][0];
    s = (p[0][0] * cxp + p[0][1] * cyp + p[0][2] * czp) / 6.0;
  }
  s = warp_sum(s);
  if ((threadIdx.x & 31) == 0 && s != 0.0) atomicAdd(out, s);
}

// Triangles of a device mesh as float32 coordinates relative to `shift`
// (T x 9), with the length of each first edge (v1 - v0, float32) and the
// largest edge length and centroid-to-vertex distance as float bits
// (maxbits[0], maxbits[1]; non-negative floats order like their bits).
__global__ void k_mesh_pieces(const double* __restrict__ v, const int32_t* __restrict__ f, long long T, double sx,
                              double sy, double sz, float* __restrict__ out, float* __restrict__ first,
                              unsigned int* maxbits) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  float edge = 0.0f, rad = 0.0f;
  if (t < T) {
    float q[3][3];
    for (int a = 0; a < 3; ++a) {
      const long long vi = f[3 * t + a];
      q[a][0] = (float)(v[3 * vi] - sx);
      q[a][1] = (float)(v[3 * vi + 1] - sy);
      q[a][2] = (float)(v[3 * vi + 2] - sz);
      for (int d = 0; d < 3; ++d) out[9 * t + 3 * a + d] = q[a][d];
    }
    float c[3];
    for (int d = 0; d < 3; ++d) c[d] = (q[0][d] + q[1][d] + q[2][d]) * (1.0f / 3.0f);
    for (int a = 0; a < 3; ++a) {
      const int b = (a + 1) % 3;
      float e2 = 0.0f, r2 = 0.0f;
      for (int d = 0; d < 3; ++d) {
        const float de = q[b][d] - q[a][d], dr = q[a][d] - c[d];
        e2 += de * de;
        r2 += dr * dr;
      }
      edge = fmaxf(edge, sqrtf(e2));
      rad = fmaxf(rad, sqrtf(r2));
      if (a == 0) first[t] = sqrtf(e2);
    }
  }
  edge = warp_max(edge);
  rad = warp_max(rad);
  if ((threadIdx.x & 31) == 0 && t - (threadIdx.x & 31) < T) {
    atomicMax(maxbits, __float_as_uint(edge));
    atomicMax(maxbits + 1, __float_as_uint(rad));
  }
}

// int64 faces -> int32, counting indices outside [0, V) into *bad
__global__ void k_faces_i32(const int64_t* __restrict__ src, long long n3, long long V, int32_t* __restrict__ dst,
                            int* bad) {
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n3) return;
  const long long v = src[e];
  const bool ok = v >= 0 && v < V;
  dst[e] = ok ? (int32_t)v : 0;
  if (!ok) atomicAdd(bad, 1);
}

// ------------------------------------------------------------ bounding box
// Order-preserving unsigned keys of IEEE values: the sign bit set for
// non-negative values, all bits flipped for negative ones.  min / max of keys
// are the min / max of the values (min and max are exact, so the box equals
// numpy's per-column min / max; -0.0 orders below +0.0, which compare equal).
SVIE_DEV unsigned long long order_key64(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}

SVIE_DEV double order_value64(unsigned long long k) {
  return __longlong_as_double((long long)((k >> 63) ? (k & 0x7fffffffffffffffull) : ~k));
}

SVIE_DEV unsigned int order_key32(float x) {
  const unsigned int b = __float_as_uint(x);
  return (b >> 31) ? ~b : (b | 0x80000000u);
}

SVIE_DEV float order_value32(unsigned int k) { return __uint_as_float((k >> 31) ? (k & 0x7fffffffu) : ~k); }

// keys[0..2] = min key per axis, keys[3..5] = max key per axis
__global__ void k_mesh_bounds(const double* __restrict__ v, long long n, unsigned long long* keys) {
  unsigned long long lo[3] = {~0ull, ~0ull, ~0ull}, hi[3] = {0ull, 0ull, 0ull};
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    for (int a = 0; a < 3; ++a) {
      const unsigned long long k = order_key64(v[3 * i + a]);
      lo[a] = k < lo[a] ? k : lo[a];
      hi[a] = k > hi[a] ? k : hi[a];
    }
  for (int a = 0; a < 3; ++a)
    for (int o = 16; o; o >>= 1) {
      const unsigned long long l = __shfl_xor_sync(0xffffffffu, lo[a], o), h = __shfl_xor_sync(0xffffffffu, hi[a], o);
      lo[a] = l < lo[a] ? l : lo[a];
      hi[a] = h > hi[a] ? h : hi[a];
    }
  if ((threadIdx.x & 31) == 0)
    for (int a = 0; a < 3; ++a) {
      atomicMin(keys + a, lo[a]);
      atomicMax(keys + 3 + a, hi[a]);
    }
}

__global__ void k_mesh_bounds_values(const unsigned long long* keys, double* out) {
  if (threadIdx.x < 6) out[threadIdx.x] = order_value64(keys[threadIdx.x]);
}

// ------------------------------------------------------ order statistics
// Exact k-th smallest values of a float array by a three-pass radix select
// over the order-preserving keys (digits of 11, 11 and 10 bits from the top).
// Two ranks are selected together (the two middle values of a median).  Each
// pass histograms the digit of the keys that match the selected prefix; one
// warp per rank then finds the digit that holds the rank.
constexpr int OS_BINS = 2048;
constexpr int OS_PASSES = 3;
__constant__ int c_os_shift[OS_PASSES] = {21, 10, 0};
__constant__ int c_os_width[OS_PASSES] = {11, 11, 10};

struct OrderState {
  unsigned int prefix[2];     // selected high bits of each rank's key
  long long rank[2];          // rank among the keys with that prefix
};

__global__ void __launch_bounds__(512) k_os_hist(const float* __restrict__ x, long long n, int pass,
                                                 const OrderState* __restrict__ st, unsigned int* __restrict__ hist) {
  __shared__ unsigned int h[2 * OS_BINS];
  for (int i = threadIdx.x; i < 2 * OS_BINS; i += blockDim.x) h[i] = 0;
  __syncthreads();
  const int shift = c_os_shift[pass], width = c_os_width[pass], top = shift + width;
  const unsigned int p0 = st->prefix[0], p1 = st->prefix[1], dmask = (1u << width) - 1u;
  const long long stride = (long long)gridDim.x * blockDim.x;
  const long long rounds = (n + stride - 1) / stride;  // the same for every lane: full-warp matches
  for (long long r = 0; r < rounds; ++r) {
    const long long i = r * stride + (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const unsigned int k = i < n ? order_key32(x[i]) : 0u;
    const unsigned int hi = top >= 32 ? 0u : (k >> top);
    const unsigned int d = (k >> shift) & dmask;
    for (int s = 0; s < 2; ++s) {
      const bool take = i < n && hi == (s ? p1 : p0);
      const unsigned int voters = __ballot_sync(0xffffffffu, take);
      if (take) {
        // lanes with the same digit add once, by their lowest lane
        const unsigned int peers = __match_any_sync(voters, d);
        if ((threadIdx.x & 31) == __ffs(peers) - 1) atomicAdd(&h[s * OS_BINS + d], __popc(peers));
      }
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < 2 * OS_BINS; i += blockDim.x)
    if (h[i]) atomicAdd(hist + i, h[i]);
}

__global__ void k_os_init(OrderState* st, long long k0, long long k1) {
  st->prefix[0] = st->prefix[1] = 0u;
  st->rank[0] = k0;
  st->rank[1] = k1;
}

// one warp per rank: the digit whose cumulative count passes the rank
__global__ void k_os_find(const unsigned int* __restrict__ hist, int pass, OrderState* st, float* out) {
  const int s = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int width = c_os_width[pass], bins = 1 << width, per = bins / 32;
  const unsigned int* hs = hist + s * OS_BINS;
  const long long rank = st->rank[s];
  long long local = 0;
  for (int j = 0; j < per; ++j) local += hs[lane * per + j];
  long long incl = local;
  for (int o = 1; o < 32; o <<= 1) {
    const long long v = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += v;
  }
  const long long excl = incl - local;
  const bool mine = excl <= rank && rank < incl;
  const unsigned int owner = __ballot_sync(0xffffffffu, mine);
  if (owner == 0) return;  // rank out of range: prevented by the host checks
  if (lane == __ffs(owner) - 1) {
    long long c = excl;
    int d = lane * per;
    while (c + hs[d] <= rank) c += hs[d++];
    const unsigned int prefix = (st->prefix[s] << width) | (unsigned int)d;
    st->prefix[s] = prefix;
    st->rank[s] = rank - c;
    if (pass == OS_PASSES - 1) out[s] = order_value32(prefix);
  }
}

}  // namespace svie

using namespace svie;

extern "C" {

int svie_mesh_tri_index(const double* vertices, const int32_t* faces, int64_t T, double ox, double oy, double oz,
                        double h, double* tri64, float* tri32, uint32_t* max_edge_bits, void* stream) {
  if (T < 0 || (T > 0 && (!vertices || !faces || !tri64 || !tri32 || !max_edge_bits)) || !(h > 0)) {
    set_error("svie_mesh_tri_index: bad arguments");
    return SVIE_ERR_ARG;
  }
  if (T == 0) return SVIE_OK;
  k_tri_index<<<blocks_for(T, 256), 256, 0, (cudaStream_t)stream>>>(vertices, faces, T, ox, oy, oz, h, tri64, tri32,
                                                                     (unsigned int*)max_edge_bits);
  return launch_status("svie_mesh_tri_index");
}

size_t svie_mesh_weld_table_bytes(int64_t n) { return (size_t)(2 * (n < 1 ? 1 : n) + 1) * sizeof(int); }

int svie_mesh_weld(const double* points, int64_t n, void* table, size_t table_bytes, int32_t* ids, int* overflow,
                   void* stream) {
  if (n < 0 || (n > 0 && (!points || !table || !ids || !overflow)) || n >= (1LL << 31)) {
    set_error("svie_mesh_weld: bad arguments");
    return SVIE_ERR_ARG;
  }
  if (n == 0) return SVIE_OK;
  const long long cap = (long long)(table_bytes / sizeof(int));
  if (cap < n + 1) {
    set_error("svie_mesh_weld: table too small");
    return SVIE_ERR_WORKSPACE;
  }
  cudaStream_t s = (cudaStream_t)stream;
  if (cudaMemsetAsync(table, 0xff, (size_t)cap * sizeof(int), s) != cudaSuccess) {
    set_error("svie_mesh_weld: memset failed");
    return SVIE_ERR_LAUNCH;
  }
  k_weld<<<blocks_for(n, 256), 256, 0, s>>>(points, n, (int*)table, cap, ids, overflow);
  return launch_status("svie_mesh_weld");
}

int svie_mesh_stars(const int32_t* faces, const int32_t* weld, int64_t T, int64_t nv, int32_t* vid, int32_t* deg,
                    int32_t* first, int32_t* cursor, int32_t* star, void* stream) {
  if (T < 0 || nv <= 0 || (T > 0 && (!vid || !deg || !first || !cursor || !star)) || 3 * T >= (1LL << 31) ||
      (!faces && !weld)) {
    set_error("svie_mesh_stars: bad arguments");
    return SVIE_ERR_ARG;
  }
  cudaStream_t s = (cudaStream_t)stream;
  if (cudaMemsetAsync(deg, 0, (size_t)nv * sizeof(int), s) != cudaSuccess ||
      cudaMemsetAsync(cursor, 0, (size_t)nv * sizeof(int), s) != cudaSuccess) {
    set_error("svie_mesh_stars: memset failed");
    return SVIE_ERR_LAUNCH;
  }
  if (T == 0) return SVIE_OK;
  const long long n3 = 3 * T;
  k_gather_ids<<<blocks_for(n3, 256), 256, 0, s>>>(faces, weld, n3, vid);
  k_degree<<<blocks_for(n3, 256), 256, 0, s>>>(vid, n3, deg);
  int scans = 1;
  if ((nv + 1023) / 1024 <= n3) {
    // multi-block scan, its block sums in `star` (written in full by k_fill_star afterwards)
    if (cudaMemcpyAsync(first, deg, (size_t)nv * sizeof(int), cudaMemcpyDeviceToDevice, s) != cudaSuccess) {
      set_error("svie_mesh_stars: copy failed");
      return SVIE_ERR_LAUNCH;
    }
    scans = scan_exclusive_i32(first, nv, star, s);
  } else {
    k_scan_deg<<<1, 1024, 0, s>>>(deg, nv, first);
  }
  k_fill_star<<<blocks_for(n3, 256), 256, 0, s>>>(vid, n3, first, cursor, star);
  return launch_status("svie_mesh_stars", 3 + scans);
}

size_t svie_mesh_edge_table_bytes(int64_t T) {
  const long long cap = 6 * (T < 1 ? 1 : T) + 1;
  return (size_t)cap * (sizeof(unsigned long long) + 2 * sizeof(int));
}

int svie_mesh_edge_topology(const int32_t* faces, int64_t T, void* table, size_t table_bytes, uint64_t* out4,
                            int* overflow, void* stream) {
  if (T < 0 || !out4 || !overflow || (T > 0 && (!faces || !table)) || 3 * T >= (1LL << 31)) {
    set_error("svie_mesh_edge_topology: bad arguments");
    return SVIE_ERR_ARG;
  }
  cudaStream_t s = (cudaStream_t)stream;
  if (cudaMemsetAsync(out4, 0, 4 * sizeof(uint64_t), s) != cudaSuccess) {
    set_error("svie_mesh_edge_topology: memset failed");
    return SVIE_ERR_LAUNCH;
  }
  if (T == 0) return SVIE_OK;
  const long long cap = (long long)(table_bytes / (sizeof(unsigned long long) + 2 * sizeof(int)));
  if (cap < 3 * T + 1) {
    set_error("svie_mesh_edge_topology: table too small");
    return SVIE_ERR_WORKSPACE;
  }
  unsigned long long* keys = (unsigned long long*)table;
  int* count = (int*)(keys + cap);
  int* dsum = count + cap;
  if (cudaMemsetAsync(keys, 0xff, (size_t)cap * sizeof(unsigned long long), s) != cudaSuccess ||
      cudaMemsetAsync(count, 0, 2 * (size_t)cap * sizeof(int), s) != cudaSuccess) {
    set_error("svie_mesh_edge_topology: memset failed");
    return SVIE_ERR_LAUNCH;
  }
  k_edges<<<blocks_for(3 * T, 256), 256, 0, s>>>(faces, T, keys, count, dsum, cap, overflow);
  k_edge_stats<<<blocks_for(cap, 256), 256, 0, s>>>(keys, count, dsum, cap, (unsigned long long*)out4);
  return launch_status("svie_mesh_edge_topology", 2);
}

int svie_mesh_faces_i32(const int64_t* faces64, int64_t T, int64_t V, int32_t* faces, int* bad, void* stream) {
  if (T < 0 || V < 0 || V >= (1LL << 31) || !bad || (T > 0 && (!faces64 || !faces))) {
    set_error("svie_mesh_faces_i32: bad arguments");
    return SVIE_ERR_ARG;
  }
  cudaStream_t s = (cudaStream_t)stream;
  if (cudaMemsetAsync(bad, 0, sizeof(int), s) != cudaSuccess) {
    set_error("svie_mesh_faces_i32: memset failed");
    return SVIE_ERR_LAUNCH;
  }
  if (T == 0) return SVIE_OK;
  k_faces_i32<<<blocks_for(3 * T, 256), 256, 0, s>>>(faces64, 3 * T, V, faces, bad);
  return launch_status("svie_mesh_faces_i32");
}

int svie_mesh_signed_volume(const double* vertices, const int32_t* faces, int64_t T, double cx, double cy, double cz,
                            double* out, void* stream) {
  if (T < 0 || !out || (T > 0 && (!vertices || !faces))) {
    set_error("svie_mesh_signed_volume: bad arguments");
    return SVIE_ERR_ARG;
  }
  cudaStream_t s = (cudaStream_t)stream;
  if (cudaMemsetAsync(out, 0, sizeof(double), s) != cudaSuccess) {
    set_error("svie_mesh_signed_volume: memset failed");
    return SVIE_ERR_LAUNCH;
  }
  if (T == 0) return SVIE_OK;
  k_signed_volume<<<blocks_for(T, 256), 256, 0, s>>>(vertices, faces, T, cx, cy, cz, out);
  return launch_status("svie_mesh_signed_volume");
}

int svie_mesh_pieces(const double* vertices, const int32_t* faces, int64_t T, double sx, double sy, double sz,
                     float* out, float* first_edge, uint32_t* maxbits, void* stream) {
  if (T < 0 || !maxbits || (T > 0 && (!vertices || !faces || !out || !first_edge))) {
    set_error("svie_mesh_pieces: bad arguments");
    return SVIE_ERR_ARG;
  }
  cudaStream_t s = (cudaStream_t)stream;
  if (cudaMemsetAsync(maxbits, 0, 2 * sizeof(uint32_t), s) != cudaSuccess) {
    set_error("svie_mesh_pieces: memset failed");
    return SVIE_ERR_LAUNCH;
  }
  if (T == 0) return SVIE_OK;
  k_mesh_pieces<<<blocks_for(T, 256), 256, 0, s>>>(vertices, faces, T, sx, sy, sz, out, first_edge, maxbits);
  return launch_status("svie_mesh_pieces");
}

int svie_mesh_bounds(const double* vertices, int64_t V, void* ws, size_t ws_bytes, double* out, void* stream) {
  if (V < 1 || !vertices || !out || !ws) {
    set_error("svie_mesh_bounds: bad arguments");
    return SVIE_ERR_ARG;
  }
  if (ws_bytes < 6 * sizeof(unsigned long long)) {
    set_error("svie_mesh_bounds: workspace too small");
    return SVIE_ERR_WORKSPACE;
  }
  cudaStream_t s = (cudaStream_t)stream;
  unsigned long long* keys = (unsigned long long*)ws;
  if (cudaMemsetAsync(keys, 0xff, 3 * sizeof(unsigned long long), s) != cudaSuccess ||
      cudaMemsetAsync(keys + 3, 0, 3 * sizeof(unsigned long long), s) != cudaSuccess) {
    set_error("svie_mesh_bounds: memset failed");
    return SVIE_ERR_LAUNCH;
  }
  int dev = 0, nsm = 152;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  const int blocks = (int)std::min<long long>(blocks_for(V, 256), 2LL * nsm);
  k_mesh_bounds<<<blocks, 256, 0, s>>>(vertices, V, keys);
  k_mesh_bounds_values<<<1, 32, 0, s>>>(keys, out);
  return launch_status("svie_mesh_bounds", 2);
}

size_t svie_order_stats_bytes(void) { return (size_t)OS_PASSES * 2 * OS_BINS * sizeof(unsigned int) + 64; }

int svie_order_stats_f32(const float* x, int64_t n, int64_t k0, int64_t k1, void* ws, size_t ws_bytes, float* out,
                         void* stream) {
  if (n < 1 || !x || !out || !ws || k0 < 0 || k1 < 0 || k0 >= n || k1 >= n) {
    set_error("svie_order_stats_f32: bad arguments");
    return SVIE_ERR_ARG;
  }
  if (ws_bytes < svie_order_stats_bytes()) {
    set_error("svie_order_stats_f32: workspace too small");
    return SVIE_ERR_WORKSPACE;
  }
  cudaStream_t s = (cudaStream_t)stream;
  unsigned int* hist = (unsigned int*)ws;
  OrderState* st = (OrderState*)(hist + OS_PASSES * 2 * OS_BINS);
  if (cudaMemsetAsync(ws, 0, svie_order_stats_bytes(), s) != cudaSuccess) {
    set_error("svie_order_stats_f32: memset failed");
    return SVIE_ERR_LAUNCH;
  }
  k_os_init<<<1, 1, 0, s>>>(st, k0, k1);
  int dev = 0, nsm = 152;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  const int blocks = (int)std::min<long long>(blocks_for(n, 512), 2LL * nsm);
  for (int p = 0; p < OS_PASSES; ++p) {
    k_os_hist<<<blocks, 512, 0, s>>>(x, n, p, st, hist + p * 2 * OS_BINS);
    k_os_find<<<1, 64, 0, s>>>(hist + p * 2 * OS_BINS, p, st, out);
  }
  return launch_status("svie_order_stats_f32", 1 + 2 * OS_PASSES);
}

}  // extern "C"
