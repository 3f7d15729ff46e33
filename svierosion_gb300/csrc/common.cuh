// Shared device helpers for the narrow-band level-set erosion kernels.
//
// Conventions (the same as the reference's kernels, svierosion/kernels.py:11-13):
//   * phi is a dense float32 grid in C order with axes (x, y, z); strides (ny*nz, nz, 1);
//   * band / node lists are sorted int32 flat indices (grids have < 2^31 nodes);
//   * points are in index (cell) coordinates.
// Every entry point returns an int status (0 = ok) and never allocates: scratch
// memory comes from a caller-provided workspace whose size a *_workspace_bytes()
// query reports.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <math.h>

#include <utility>

#include "../../include/svie.h"

#define SVIE_DEV __device__ __forceinline__

// threads of the one-CTA kernels that sum per-CTA partials
constexpr int SUM_THREADS = 256;

namespace svie {

// In-place exclusive scan of n ints on the stream; sums: ceil(n / 1024) ints
// of scratch.  Returns the number of kernels launched (distance.cu).
int scan_exclusive_i32(int* v, long long n, int* sums, cudaStream_t s);

// Records a message for svie_last_error(); defined in capi.cu.
void set_error(const char* fmt, ...);

// Counts kernel launches made through the C ABI (svie_launch_count).
void note_launches(int n);

// Status from the most recent launches on the calling thread; `n` is the number
// of kernels the entry point launched.
inline int launch_status(const char* what, int n = 1) {
  note_launches(n);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_error("%s: launch failed: %s", what, cudaGetErrorString(e));
    return SVIE_ERR_LAUNCH;
  }
  return SVIE_OK;
}

// ------------------------------------------- programmatic dependent launch
// Within one entry point's chain of kernels (the convolution passes, the
// reinitialisation half-steps, the volume sum), every kernel after the first
// is launched by launch_dependent: it may be scheduled while the previous
// kernel of the chain is still running (its blocks become resident as the
// previous grid's blocks retire) and it calls pdl_wait() before it touches
// memory.  pdl_wait() returns once the previous grid has completed and its
// writes are visible; in a kernel launched the ordinary way it returns at
// once.  pdl_release() lets the next dependent launch be scheduled (otherwise
// that happens when this grid ends).  The first kernel of a chain is launched
// the ordinary way, so whatever the caller queued before the call (kernels,
// copies, event waits, other libraries' work) completes before it starts.
SVIE_DEV void pdl_wait() { asm volatile("griddepcontrol.wait;\n" ::: "memory"); }
SVIE_DEV void pdl_release() { asm volatile("griddepcontrol.launch_dependents;\n" :::); }

// Whether launch_dependent uses the programmatic launch (SVIE_PDL=0 turns it off).
bool pdl_enabled();

// `chained`: the previous operation on the stream is the previous kernel of
// this entry point's own chain (false: an ordinary launch).
template <typename... KArgs, typename... Args>
inline cudaError_t launch_dependent(bool chained, void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem,
                                   cudaStream_t s, Args&&... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = chained && pdl_enabled() ? 1 : 0;
  return cudaLaunchKernelEx(&cfg, kernel, std::forward<Args>(args)...);
}

// launch_status for entry points whose launches went through launch_dependent
// (their first failure in `e`).
inline int dependent_status(cudaError_t e, const char* what, int n = 1) {
  if (e != cudaSuccess) {
    note_launches(n);
    set_error("%s: launch failed: %s", what, cudaGetErrorString(e));
    return SVIE_ERR_LAUNCH;
  }
  return launch_status(what, n);
}

inline int blocks_for(long long n, int threads, long long cap = 1LL << 30) {
  long long b = (n + threads - 1) / threads;
  if (b < 1) b = 1;
  if (b > cap) b = cap;
  return (int)b;
}

// ------------------------------------------------- division by a constant
// Correctly rounded float reciprocal of d (normal, positive), on the host:
// the double quotient rounded to float, then whichever float neighbour has
// the product with d closest to 1 (a product of two floats is exact in
// double, and so is 1 minus it).  1/d is never halfway between two floats
// unless it is exact.
inline float rn_reciprocal(float d) {
  float r = (float)(1.0 / (double)d);
  float best = r;
  double err = fabs(1.0 - (double)d * (double)r);
  const float cand[2] = {nextafterf(r, 0.0f), nextafterf(r, INFINITY)};
  for (float c : cand) {
    const double e = fabs(1.0 - (double)d * (double)c);
    if (e < err) { err = e; best = c; }
  }
  return best;
}

// Correctly rounded x / d given rd = RN(1/d): q = RN(x rd) is within one ulp
// of x / d, the remainder r = x - d q is exact in one fused multiply-add, and
// RN(q + r rd) is the correctly rounded quotient (P. Markstein, "Computation
// of elementary functions on the IBM RISC System/6000 processor", IBM J. Res.
// Dev. 34(1), 1990, Theorem 1), for normal x and d and a normal quotient.
// Three operations in place of a general division; a -0 quotient comes out +0.
SVIE_DEV float div_by(float x, float d, float rd) {
  const float q = __fmul_rn(x, rd);
  const float r = __fmaf_rn(-q, d, x);
  return __fmaf_rn(r, rd, q);
}

// -------------------------------------------------------------- float keys
// Monotone map float -> uint32 so that unsigned atomicMin/Max order floats.
SVIE_DEV unsigned int float_to_ordered(float f) {
  unsigned int u = __float_as_uint(f);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
SVIE_DEV float ordered_to_float(unsigned int u) {
  return __uint_as_float((u & 0x80000000u) ? (u & 0x7fffffffu) : ~u);
}

// ------------------------------------------------------- warp reductions
SVIE_DEV float warp_max(float v) {
  for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}
SVIE_DEV float warp_min(float v) {
  for (int o = 16; o > 0; o >>= 1) v = fminf(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}
SVIE_DEV double warp_sum(double v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
SVIE_DEV unsigned int warp_sum_u(unsigned int v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
SVIE_DEV int warp_min_i(int v) {
  for (int o = 16; o > 0; o >>= 1) v = min(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}
SVIE_DEV int warp_max_i(int v) {
  for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

// Warp sum of float values returned as a double in every lane.  The tree runs
// on (hi, lo) float pairs combined with Knuth's error-free TwoSum, so the warp
// total is exact to ~2^-46 relative while the FP64 pipe (slow on GB300) is used
// once per warp instead of five times per thread.
SVIE_DEV void two_sum(float a, float b, float& s, float& e) {
  s = a + b;
  const float bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}
SVIE_DEV double warp_sum_compensated(float v) {
  float hi = v, lo = 0.0f;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const float h2 = __shfl_xor_sync(0xffffffffu, hi, o);
    const float l2 = __shfl_xor_sync(0xffffffffu, lo, o);
    float s, e;
    two_sum(hi, h2, s, e);
    e += lo + l2;
    hi = s + e;
    lo = e - (hi - s);
  }
  return (double)hi + (double)lo;
}

// Double-float partial sums: a value hi + lo kept as two floats and added with
// TwoSum, about 2^-46 relative, in FP32 arithmetic throughout.  Per-CTA
// partials are stored in this form (8 bytes, the size of a double) and summed
// across CTAs without the FP64 pipe, whose rate on GB300 is 1/64 of FP32.
struct DF {
  float hi, lo;
};
SVIE_DEV DF df_add(DF a, DF b) {
  float s, e;
  two_sum(a.hi, b.hi, s, e);
  e += a.lo + b.lo;
  const float hi = s + e;
  return DF{hi, e - (hi - s)};
}
SVIE_DEV DF warp_sum_df(DF v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1)
    v = df_add(v, DF{__shfl_xor_sync(0xffffffffu, v.hi, o), __shfl_xor_sync(0xffffffffu, v.lo, o)});
  return v;
}
SVIE_DEV double df_value(DF v) { return (double)v.hi + (double)v.lo; }

// Sum of the n double-float partials p[0..n) by one CTA, in a fixed order
// (strided per thread, then a warp tree, then warp 0 over the warps); the
// result is valid in thread 0.  `scratch` holds blockDim.x / 32 entries.
SVIE_DEV DF block_sum_partials_df(const float2* __restrict__ p, long long n, DF* scratch) {
  DF v{0.0f, 0.0f};
  for (long long i = threadIdx.x; i < n; i += blockDim.x) {
    const float2 q = p[i];
    v = df_add(v, DF{q.x, q.y});
  }
  v = warp_sum_df(v);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  if (lane == 0) scratch[wid] = v;
  __syncthreads();
  if (wid == 0) {
    v = lane < nw ? scratch[lane] : DF{0.0f, 0.0f};
    v = warp_sum_df(v);
  }
  return v;
}

// Block sum of one float per thread as a double (compensated warp sums, FP64
// across the warps); the result is valid in thread 0.
SVIE_DEV DF block_sum_df(float v, DF* scratch) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  DF w = warp_sum_df(DF{v, 0.0f});
  __syncthreads();
  if (lane == 0) scratch[wid] = w;
  __syncthreads();
  if (threadIdx.x == 0)
    for (int i = 1; i < nw; ++i) w = df_add(w, scratch[i]);
  return w;
}

SVIE_DEV double block_sum_compensated(float v, double* scratch) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const double w = warp_sum_compensated(v);
  __syncthreads();
  if (lane == 0) scratch[wid] = w;
  __syncthreads();
  double r = 0.0;
  if (threadIdx.x == 0)
    for (int i = 0; i < nw; ++i) r += scratch[i];
  return r;
}

// Block-wide reduction through shared memory; every thread gets the result.
// `scratch` needs blockDim.x/32 entries; the block size is a multiple of 32.
template <typename T, typename Op>
SVIE_DEV T block_reduce(T v, T* scratch, Op op, T identity) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int o = 16; o > 0; o >>= 1) v = op(v, __shfl_xor_sync(0xffffffffu, v, o));
  __syncthreads();
  if (lane == 0) scratch[wid] = v;
  __syncthreads();
  T r = identity;
  for (int i = 0; i < nw; ++i) r = op(r, scratch[i]);
  return r;
}

struct OpMaxF { SVIE_DEV float operator()(float a, float b) const { return fmaxf(a, b); } };
struct OpMinF { SVIE_DEV float operator()(float a, float b) const { return fminf(a, b); } };
struct OpSumD { SVIE_DEV double operator()(double a, double b) const { return a + b; } };
struct OpSumU { SVIE_DEV unsigned int operator()(unsigned int a, unsigned int b) const { return a + b; } };
struct OpSumI { SVIE_DEV int operator()(int a, int b) const { return a + b; } };
struct OpSumLL { SVIE_DEV long long operator()(long long a, long long b) const { return a + b; } };
struct OpMinI { SVIE_DEV int operator()(int a, int b) const { return min(a, b); } };
struct OpMaxI { SVIE_DEV int operator()(int a, int b) const { return max(a, b); } };

// ----------------------------------------------------------- stencil maths
// Jiang-Peng WENO5 derivative from five differences (reference kernels.py:83-97).
// Divisions by constants are multiplications by their float reciprocals and
// the weights and the weighted mean use the hardware quotient: the result
// differs from the reference's division form by a few float32 ulps.
SVIE_DEV float weno5(float v1, float v2, float v3, float v4, float v5) {
  const float c1312 = (float)(13.0 / 12.0);
  const float r3 = (float)(1.0 / 3.0), r6 = (float)(1.0 / 6.0), c76 = (float)(7.0 / 6.0);
  const float c116 = (float)(11.0 / 6.0), c56 = (float)(5.0 / 6.0);
  float p1 = v1 * r3 - v2 * c76 + v3 * c116;
  float p2 = -v2 * r6 + v3 * c56 + v4 * r3;
  float p3 = v3 * r3 + v4 * c56 - v5 * r6;
  float e1 = v1 - 2.0f * v2 + v3, f1 = v1 - 4.0f * v2 + 3.0f * v3;
  float e2 = v2 - 2.0f * v3 + v4, f2 = v2 - v4;
  float e3 = v3 - 2.0f * v4 + v5, f3 = 3.0f * v3 - 4.0f * v4 + v5;
  float s1 = c1312 * (e1 * e1) + 0.25f * (f1 * f1);
  float s2 = c1312 * (e2 * e2) + 0.25f * (f2 * f2);
  float s3 = c1312 * (e3 * e3) + 0.25f * (f3 * f3);
  float vmax = fmaxf(fmaxf(fmaxf(v1 * v1, v2 * v2), fmaxf(v3 * v3, v4 * v4)), v5 * v5);
  float eps = 1e-6f * vmax + 1e-10f;
  float d1 = s1 + eps, d2 = s2 + eps, d3 = s3 + eps;
  // hardware quotients (at most 2 ulp; d^2 >= 1e-20 and the weights' sum stay far below 2^126, the
  // quotient's range): the weights and the result move by about 1e-7 relative, a fraction of the
  // instructions of the correctly rounded forms
  float a1 = __fdividef(0.1f, d1 * d1);
  float a2 = __fdividef(0.6f, d2 * d2);
  float a3 = __fdividef(0.3f, d3 * d3);
  return __fdividef(a1 * p1 + a2 * p2 + a3 * p3, a1 + a2 + a3);
}

// Godunov |grad phi| for inward motion at flat node i (reference kernels.py:146-169).
SVIE_DEV float godunov_at(const float* __restrict__ f, int i, int sx, int sy, int sz, float inv_h) {
  const float* q = f + i;
  const float c = __ldg(q);
  float g2 = 0.0f;
  const int st[3] = {sx, sy, sz};
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const int s = st[a];
    float m3 = __ldg(q - 3 * s), m2 = __ldg(q - 2 * s), m1 = __ldg(q - s);
    float p1 = __ldg(q + s), p2 = __ldg(q + 2 * s), p3 = __ldg(q + 3 * s);
    float d0 = (m2 - m3) * inv_h, d1 = (m1 - m2) * inv_h, d2 = (c - m1) * inv_h;
    float d3 = (p1 - c) * inv_h, d4 = (p2 - p1) * inv_h, d5 = (p3 - p2) * inv_h;
    float dm = weno5(d0, d1, d2, d3, d4);
    float dp = weno5(d5, d4, d3, d2, d1);
    float lo = fminf(dm, 0.0f), hi = fmaxf(dp, 0.0f);
    g2 = g2 + fmaxf(lo * lo, hi * hi);
  }
  return sqrtf(g2);
}

// Volume fraction of the unit cube below a plane (reference kernels.py:104-122):
// s = signed distance in cells, a >= b >= c >= 0 the sorted |normal| components.
SVIE_DEV float cube_plane_fraction(float s, float a, float b, float c) {
  float M = 0.5f * (a + b + c);
  float y = M - s;
  bool flip = y > M;
  y = flip ? 2.0f * M - y : y;
  y = fmaxf(y, 0.0f);
  const float tiny = 1e-12f;
  float bs = fmaxf(b, tiny), cs = fmaxf(c, tiny);
  float rb = __frcp_rn(bs), rc = __frcp_rn(cs), ra6 = __frcp_rn(6.0f * a);
  float q = 3.0f * y * y - 3.0f * y * c + c * c;
  float H;
  if (y <= c) {
    H = (y * y * y) * (rb * rc);
  } else if (y <= b) {
    H = q * rb;
  } else if (y <= b + c) {
    float u = fmaxf(y - b, 0.0f);
    H = (q - (u * u * u) * rc) * rb;
  } else {
    H = 3.0f * (2.0f * y - b - c);
  }
  float ua = fmaxf(y - a, 0.0f);
  float F = H * ra6 - (ua * ua * ua) * (ra6 * rb * rc);
  F = flip ? 1.0f - F : F;
  return fminf(fmaxf(F, 0.0f), 1.0f);
}

// Tangent-plane cell fraction at node i (reference kernels.py:173-181).
SVIE_DEV float cell_fraction_at(const float* __restrict__ f, int i, int sx, int sy, int sz) {
  const float* q = f + i;
  float c = __ldg(q);
  float gx = 0.5f * (__ldg(q + sx) - __ldg(q - sx));
  float gy = 0.5f * (__ldg(q + sy) - __ldg(q - sy));
  float gz = 0.5f * (__ldg(q + sz) - __ldg(q - sz));
  float gn = fmaxf(sqrtf(gx * gx + gy * gy + gz * gz), 1e-30f);
  float rg = __frcp_rn(gn);
  float x = fabsf(gx * rg), y = fabsf(gy * rg), z = fabsf(gz * rg);
  float hi = fmaxf(fmaxf(x, y), z);
  float lo = fminf(fminf(x, y), z);
  float mid = x + y + z - hi - lo;
  return cube_plane_fraction(c * rg, hi, mid, lo);
}

// Exact n / d for 0 <= n < 2^31 and 1 <= d < 2^31 by one multiply and a
// shift (T. Granlund and P. L. Montgomery, "Division by invariant integers
// using multiplication", PLDI 1994): with l = ceil(log2 d) and
// m = ceil(2^(31 + l) / d) < 2^32, n / d = (n m) >> (31 + l).
struct DivMagic {
  unsigned int m;
  int s;
};
inline DivMagic div_magic(int d) {
  int l = 0;
  while ((1LL << l) < d) ++l;
  const unsigned long long m = ((1ULL << (31 + l)) + (unsigned long long)d - 1) / (unsigned long long)d;
  return DivMagic{(unsigned int)m, 31 + l};
}
SVIE_DEV int div_exact(int n, DivMagic g) { return (int)(((unsigned long long)(unsigned int)n * g.m) >> g.s); }

// Grid constants of the closest-point projection: strides with their
// division constants, clamp bounds hi = (n - 3.001) rounded to float, the
// spacing and its correctly rounded reciprocal.
struct CpGeom {
  int sx, sy;
  DivMagic dsx, dsy;
  float hx, hy, hz, h, rh;
};
inline CpGeom cp_geom(int ny, int nz, float hx, float hy, float hz, float h) {
  CpGeom g;
  g.sx = ny * nz;
  g.sy = nz;
  g.dsx = div_magic(g.sx);
  g.dsy = div_magic(g.sy);
  g.hx = hx;
  g.hy = hy;
  g.hz = hz;
  g.h = h;
  g.rh = rn_reciprocal(h);
  return g;
}

// Float constants of a stage, rounded once on the host: the kernels then do no
// float64 work per node except the t - N difference of the SVI law.
struct StageConst {
  float h, inv_h, hx, hy, hz;  // spacing, 1/h, clamp bounds n - 3.001
  float n_cap, eps, cut_b, cut_scale;
  float t;  // the SVI law's t, rounded to float as the reference's float32 tensors see it
  // curvature laws: alpha, alpha - 1, alpha - 2 and delta rounded once; amode
  // 0: alpha = 1, 1: alpha < 1, 2: alpha > 1
  float alpha, am1, am2, delta;
  int amode;
  CpGeom cp;  // the closest-point projection's grid constants
};

// Band work of many level sets in one launch (svie_group_*): every member's
// band is cut into tiles of GROUP_TILE consecutive entries -- the CTAs of the
// one-level-set kernels -- and a launch takes a packed list of (member, tile)
// pairs.  A member's record holds its arrays, sizes and law; the tile bodies
// are the one-level-set kernels' own, so a member's results are bit-identical
// to solving it alone.
constexpr int GROUP_TILE = 256;

struct GroupInst {
  float* phi;
  const int32_t* band;
  float* field;       // SVI: the dense N field; curvature laws: interleaved (k1, k2)
  float* occ;
  float* u0;
  float* L[3];
  svie_stats* stats;  // stage statistics and the member's time step
  svie_stats* vstats; // volume statistics
  double* stage_part; // per-tile statistics partials
  double* vol_part;   // per-tile volume partials
  long long m;
  int nx, ny, nz, kind;  // kind 0: SVI law, 1: curvature law
  svie_law law;
  StageConst C;
};

// Group table layout: the member records, then the (member, tile) pairs, SVI
// members' tiles first.
__host__ __device__ inline size_t group_tiles_offset(int n) { return ((size_t)n * sizeof(GroupInst) + 15) & ~(size_t)15; }

// The CTA copies member k's record into shared memory (and waits for the copy).
SVIE_DEV void load_group_inst(GroupInst& dst, const GroupInst* src) {
  const int words = (int)(sizeof(GroupInst) / 4);
  for (int k = threadIdx.x; k < words; k += blockDim.x)
    reinterpret_cast<int*>(&dst)[k] = reinterpret_cast<const int*>(src)[k];
  __syncthreads();
}

// First Newton projection to the zero set (reference kernels.py:185-208).
// The division by h uses the correctly rounded reciprocal (div_by), the node
// coordinates the exact multiply-shift division: same results as the plain
// operations.
SVIE_DEV float3 closest_point_at(const float* __restrict__ f, int i, const CpGeom& G) {
  const int sx = G.sx, sy = G.sy;
  const float* q = f + i;
  float c = __ldg(q);
  float gx = 0.5f * (__ldg(q + sx) - __ldg(q - sx));
  float gy = 0.5f * (__ldg(q + sy) - __ldg(q - sy));
  float gz = 0.5f * (__ldg(q + 1) - __ldg(q - 1));
  float g2 = fmaxf(gx * gx + gy * gy + gz * gz, 1e-30f);
  float ac = fabsf(c);
  float length = ac / sqrtf(g2);
  float cap = div_by(1.25f * ac, G.h, G.rh) + 0.25f;
  float scale = (c / g2) * fminf(cap / fmaxf(length, 1e-30f), 1.0f);
  const int ii = div_exact(i, G.dsx), rem = i - ii * sx, jj = div_exact(rem, G.dsy);
  float fi = (float)ii;
  float fj = (float)jj;
  float fk = (float)(rem - jj * sy);
  float3 p;
  p.x = fminf(fmaxf(fi - scale * gx, 1.0f), G.hx);
  p.y = fminf(fmaxf(fj - scale * gy, 1.0f), G.hy);
  p.z = fminf(fmaxf(fk - scale * gz, 1.0f), G.hz);
  return p;
}

// Cubic Lagrange weights on nodes -1, 0, 1, 2 (reference kernels.py:134-136).
SVIE_DEV void cubic_w(float t, float w[4]) {
  const float r6 = (float)(1.0 / 6.0);
  w[0] = -t * (t - 1.0f) * (t - 2.0f) * r6;
  w[1] = (t + 1.0f) * (t - 1.0f) * (t - 2.0f) * 0.5f;
  w[2] = -(t + 1.0f) * t * (t - 2.0f) * 0.5f;
  w[3] = (t + 1.0f) * t * (t - 1.0f) * r6;
}
// Their derivatives (reference kernels.py:139-141).
SVIE_DEV void cubic_dw(float t, float w[4]) {
  w[0] = -(3.0f * t * t - 6.0f * t + 2.0f) / 6.0f;
  w[1] = (3.0f * t * t - 4.0f * t - 1.0f) / 2.0f;
  w[2] = -(3.0f * t * t - 2.0f * t - 2.0f) / 2.0f;
  w[3] = (3.0f * t * t - 1.0f) / 6.0f;
}

// tricubic_with_gradient (kernels.py:232-253): value and per-cell gradient at
// index coordinates p, accumulated tap by tap in the reference's order.
SVIE_DEV void tricubic_grad_at(const float* __restrict__ g, int ny, int nz, float3 p, float* val, float* gxo,
                               float* gyo, float* gzo) {
  const float fx = floorf(p.x), fy = floorf(p.y), fz = floorf(p.z);
  const float tx = p.x - fx, ty = p.y - fy, tz = p.z - fz;
  float wx[4], wy[4], wz[4], dx[4], dy[4], dz[4];
  cubic_w(tx, wx); cubic_w(ty, wy); cubic_w(tz, wz);
  cubic_dw(tx, dx); cubic_dw(ty, dy); cubic_dw(tz, dz);
  const long long syz = (long long)ny * nz;
  const long long b0 = ((long long)fx - 1) * syz + ((long long)fy - 1) * nz + ((long long)fz - 1);
  float v = 0.f, gx = 0.f, gy = 0.f, gz = 0.f;
  for (int a = 0; a < 4; ++a)
    for (int b = 0; b < 4; ++b)
      for (int c = 0; c < 4; ++c) {
        const float s = __ldg(g + b0 + a * syz + b * nz + c);
        v = v + wx[a] * wy[b] * wz[c] * s;
        gx = gx + dx[a] * wy[b] * wz[c] * s;
        gy = gy + wx[a] * dy[b] * wz[c] * s;
        gz = gz + wx[a] * wy[b] * dz[c] * s;
      }
  *val = v;
  *gxo = gx;
  *gyo = gy;
  *gzo = gz;
}

// Squared point-triangle distance with Ericson's region classification in the
// priority order of the reference (kernels.py:382-427).
// Every operation of the point-triangle distance is rounded on its own, in
// the reference's order (products first, then left-to-right sums, as its
// float32 tensor arithmetic evaluates them): no multiply-add is fused, so the
// distances, and the nearest-triangle ties they decide, are bit-identical.
SVIE_DEV float rmul(float x, float y) { return __fmul_rn(x, y); }
SVIE_DEV float radd(float x, float y) { return __fadd_rn(x, y); }
SVIE_DEV float rsub(float x, float y) { return __fsub_rn(x, y); }
SVIE_DEV float rdot3(float3 u, float3 v) { return radd(radd(rmul(u.x, v.x), rmul(u.y, v.y)), rmul(u.z, v.z)); }
SVIE_DEV float3 rsub3(float3 u, float3 v) { return make_float3(rsub(u.x, v.x), rsub(u.y, v.y), rsub(u.z, v.z)); }

SVIE_DEV float point_triangle_d2(float3 p, float3 a, float3 b, float3 c) {
  const float3 ab = rsub3(b, a), ac = rsub3(c, a);
  const float3 ap = rsub3(p, a), bp = rsub3(p, b), cp = rsub3(p, c);
  const float d1 = rdot3(ab, ap), d2 = rdot3(ac, ap);
  const float d3 = rdot3(ab, bp), d4 = rdot3(ac, bp);
  const float d5 = rdot3(ab, cp), d6 = rdot3(ac, cp);
  const float va = rsub(rmul(d3, d6), rmul(d5, d4));
  const float vb = rsub(rmul(d5, d2), rmul(d1, d6));
  const float vc = rsub(rmul(d1, d4), rmul(d3, d2));
  const float tiny = 1e-30f;
  float denom = radd(radd(va, vb), vc);
  denom = fabsf(denom) > tiny ? denom : tiny;
  float v = vb / denom, w = vc / denom;
  const float e1 = rsub(d4, d3), e2 = rsub(d5, d6);
  if (d1 <= 0.f && d2 <= 0.f) {                 // vertex a
    v = 0.f; w = 0.f;
  } else if (d3 >= 0.f && d4 <= d3) {           // vertex b
    v = 1.f; w = 0.f;
  } else if (vc <= 0.f && d1 >= 0.f && d3 <= 0.f) {  // edge ab
    v = d1 / fmaxf(rsub(d1, d3), tiny); w = 0.f;
  } else if (d6 >= 0.f && d5 <= d6) {           // vertex c
    v = 0.f; w = 1.f;
  } else if (vb <= 0.f && d2 >= 0.f && d6 <= 0.f) {  // edge ac
    v = 0.f; w = d2 / fmaxf(rsub(d2, d6), tiny);
  } else if (va <= 0.f && e1 >= 0.f && e2 >= 0.f) {  // edge bc
    const float wbc = e1 / fmaxf(radd(e1, e2), tiny);
    v = rsub(1.f, wbc); w = wbc;
  }
  // q = (a + v ab) + w ac, then |p - q|^2 as ((dx^2 + dy^2) + dz^2)
  const float3 q = make_float3(radd(radd(a.x, rmul(v, ab.x)), rmul(w, ac.x)),
                               radd(radd(a.y, rmul(v, ab.y)), rmul(w, ac.y)),
                               radd(radd(a.z, rmul(v, ab.z)), rmul(w, ac.z)));
  const float3 d = rsub3(p, q);
  return rdot3(d, d);
}

// Tricubic interpolation at index coordinates p (reference kernels.py:212-228),
// evaluated separably: a 4-tap sum along z per (x, y) row, then along y, then
// along x (84 multiply-adds in place of the 144 operations of the 64 products
// wx wy wz v).  Only the order of the float32 sums differs from the
// reference's 64-term sum: a few ulps of the result.
SVIE_DEV float tricubic_at(const float* __restrict__ g, int ny, int nz, float3 p) {
  float fx = floorf(p.x), fy = floorf(p.y), fz = floorf(p.z);
  float wx[4], wy[4], wz[4];
  cubic_w(p.x - fx, wx);
  cubic_w(p.y - fy, wy);
  cubic_w(p.z - fz, wz);
  const int syz = ny * nz;
  const float* b0 = g + (((int)fx - 1) * syz + ((int)fy - 1) * nz + ((int)fz - 1));
  float out = 0.0f;
#pragma unroll
  for (int a = 0; a < 4; ++a) {
    float ta = 0.0f;
#pragma unroll
    for (int b = 0; b < 4; ++b) {
      const float* row = b0 + (a * syz + b * nz);
      const float sz = fmaf(wz[3], __ldg(row + 3),
                            fmaf(wz[2], __ldg(row + 2), fmaf(wz[1], __ldg(row + 1), wz[0] * __ldg(row))));
      ta = fmaf(wy[b], sz, ta);
    }
    out = fmaf(wx[a], ta, out);
  }
  return out;
}

// Trilinear interpolation (reference kernels.py:257-270); `comp` selects a
// component of an interleaved field with `ncomp` floats per node.
SVIE_DEV float trilinear_at(const float* __restrict__ g, int ny, int nz, float3 p, int ncomp, int comp) {
  float fx = floorf(p.x), fy = floorf(p.y), fz = floorf(p.z);
  float tx = p.x - fx, ty = p.y - fy, tz = p.z - fz;
  const long long syz = (long long)ny * nz;
  const long long b0 = (long long)fx * syz + (long long)fy * nz + (long long)fz;  // 64-bit: ncomp * index may exceed 2^31
  float out = 0.0f;
#pragma unroll
  for (int a = 0; a < 2; ++a) {
    float wa = a ? tx : 1.0f - tx;
#pragma unroll
    for (int b = 0; b < 2; ++b) {
      float wb = wa * (b ? ty : 1.0f - ty);
#pragma unroll
      for (int c = 0; c < 2; ++c) {
        long long o = b0 + a * syz + b * nz + c;
        out = out + wb * (c ? tz : 1.0f - tz) * __ldg(g + o * ncomp + comp);
      }
    }
  }
  return out;
}

// trilinear_at of both components of an interleaved (k1, k2) field, one 8-byte
// load per corner; each component is accumulated in trilinear_at's order.
SVIE_DEV float2 trilinear2_at(const float2* __restrict__ g, int ny, int nz, float3 p) {
  float fx = floorf(p.x), fy = floorf(p.y), fz = floorf(p.z);
  float tx = p.x - fx, ty = p.y - fy, tz = p.z - fz;
  const long long syz = (long long)ny * nz;
  const long long b0 = (long long)fx * syz + (long long)fy * nz + (long long)fz;
  float2 out = make_float2(0.0f, 0.0f);
#pragma unroll
  for (int a = 0; a < 2; ++a) {
    float wa = a ? tx : 1.0f - tx;
#pragma unroll
    for (int b = 0; b < 2; ++b) {
      float wb = wa * (b ? ty : 1.0f - ty);
#pragma unroll
      for (int c = 0; c < 2; ++c) {
        const float2 v = __ldg(g + (b0 + a * syz + b * nz + c));
        const float w = wb * (c ? tz : 1.0f - tz);
        out.x = out.x + w * v.x;
        out.y = out.y + w * v.y;
      }
    }
  }
  return out;
}

// Principal curvatures k1 >= k2 of the level sets at node i (reference kernels.py:274-299).
SVIE_DEV float2 principal_curvatures_at(const float* __restrict__ f, int i, int sx, int sy, int sz, float h) {
  float c = __ldg(f + i);
  float xp = __ldg(f + i + sx), xm = __ldg(f + i - sx);
  float yp = __ldg(f + i + sy), ym = __ldg(f + i - sy);
  float zp = __ldg(f + i + sz), zm = __ldg(f + i - sz);
  // the divisions by the constants 2h, h^2 and 4h^2 through their correctly rounded reciprocals
  // (div_by): the same quotients as IEEE division, in three operations each
  float h2 = 2.0f * h, hh = h * h, h4 = 4.0f * h * h;
  const float r2 = __frcp_rn(h2), rhh = __frcp_rn(hh), r4 = __frcp_rn(h4);
  float px = div_by(xp - xm, h2, r2), py = div_by(yp - ym, h2, r2), pz = div_by(zp - zm, h2, r2);
  float pxx = div_by(xp - 2.0f * c + xm, hh, rhh);
  float pyy = div_by(yp - 2.0f * c + ym, hh, rhh);
  float pzz = div_by(zp - 2.0f * c + zm, hh, rhh);
  auto mixed = [&](int a, int b) {
    return div_by(__ldg(f + i + a + b) - __ldg(f + i + a - b) - __ldg(f + i - a + b) + __ldg(f + i - a - b), h4,
                  r4);
  };
  float pxy = mixed(sx, sy), pxz = mixed(sx, sz), pyz = mixed(sy, sz);
  float g2 = fmaxf(px * px + py * py + pz * pz, 1e-30f);
  float gn = sqrtf(g2);
  float ksum = ((pyy + pzz) * px * px + (pxx + pzz) * py * py + (pxx + pyy) * pz * pz -
                2.0f * (px * py * pxy + px * pz * pxz + py * pz * pyz)) / (g2 * gn);
  float K = (px * px * (pyy * pzz - pyz * pyz) + py * py * (pxx * pzz - pxz * pxz) +
             pz * pz * (pxx * pyy - pxy * pxy) + 2.0f * px * py * (pxz * pyz - pxy * pzz) +
             2.0f * py * pz * (pxy * pxz - pyz * pxx) + 2.0f * px * pz * (pxy * pyz - pxz * pyy)) /
            (g2 * g2);
  float H = 0.5f * ksum;
  float r = sqrtf(fmaxf(H * H - K, 0.0f));
  return make_float2(H + r, H - r);
}

}  // namespace svie
