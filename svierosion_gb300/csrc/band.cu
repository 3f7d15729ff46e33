// Narrow-band construction: order-preserving stream compaction.
//
// Replaces LevelSet.rebuild_band / _check_margin (reference
// svierosion/levelset.py:70-86) and the torch.nonzero calls on dense masks
// (levelset.py:173, evolve.py:100).  The output is the ascending list of flat
// indices, bit-identical to torch.nonzero given the same phi.
//
// Layout: each CTA owns a tile of TILE = THREADS * IPT consecutive nodes;
// warp w of the CTA owns IPT chunks of 32 consecutive nodes, chunk j being
// nodes tile0 + w * 32 * IPT + 32 j + lane, so every load and store is
// coalesced.  Pass 1 counts selected nodes per CTA; a one-CTA scan turns the
// counts into offsets (workspace: one int32 per CTA); pass 2 recomputes the
// predicate as one ballot per chunk, and popcounts of the ballots give each
// selected node its position, so the output keeps the flat order.  Both
// passes read the grid once (HBM-bound, 4 B/node each for phi).
#include <limits.h>

#include "common.cuh"

namespace svie {

constexpr int CMP_THREADS = 256;
constexpr int CMP_IPT = 16;
constexpr int CMP_TILE = CMP_THREADS * CMP_IPT;

inline long long cmp_blocks(long long n) { return (n + CMP_TILE - 1) / CMP_TILE; }

// Exclusive scan of one int per thread across the CTA; returns the prefix and
// writes the CTA total to *total.
SVIE_DEV int block_exclusive_scan(int v, int* sh, int* total) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  int x = v;
  for (int o = 1; o < 32; o <<= 1) {
    int y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) sh[wid] = x;
  __syncthreads();
  if (wid == 0) {
    int w = lane < nw ? sh[lane] : 0;
    int s = w;
    for (int o = 1; o < 32; o <<= 1) {
      int y = __shfl_up_sync(0xffffffffu, s, o);
      if (lane >= o) s += y;
    }
    if (lane < nw) sh[lane] = s - w;  // exclusive warp offsets
    if (lane == nw - 1) sh[32] = s;
  }
  __syncthreads();
  int r = sh[wid] + x - v;
  *total = sh[32];
  __syncthreads();
  return r;
}

// ------------------------------------------------------------ predicates
struct MaskPred {
  const uint8_t* mask;
  SVIE_DEV bool operator()(long long e) const { return mask[e] != 0; }
};

// First node of this warp's chunks.
SVIE_DEV long long warp_base() {
  return (long long)blockIdx.x * CMP_TILE + (long long)(threadIdx.x >> 5) * (32 * CMP_IPT);
}

// Exclusive offsets of the CTA's warps from their totals; CTA total -> *total.
SVIE_DEV int warp_offsets(int wt, int* sh, int* total) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  if (lane == 0) sh[wid] = wt;
  __syncthreads();
  if (threadIdx.x == 0) {
    int run = 0;
    for (int w = 0; w < nw; ++w) {
      const int c = sh[w];
      sh[w] = run;
      run += c;
    }
    sh[32] = run;
  }
  __syncthreads();
  const int r = sh[wid];
  *total = sh[32];
  __syncthreads();
  return r;
}

// Writes the selected nodes of the warp's chunks (ballots bal[j]) in order
// from position o; value(j) gives what to store for the lane's node of chunk j.
template <class Value>
SVIE_DEV void write_selected(const unsigned int* bal, long long o, int32_t* out, long long capacity, Value value) {
  const int lane = threadIdx.x & 31;
  const unsigned int lt = (1u << lane) - 1u;
#pragma unroll
  for (int j = 0; j < CMP_IPT; ++j) {
    if ((bal[j] >> lane) & 1u) {
      const long long pos = o + __popc(bal[j] & lt);
      if (pos < capacity) out[pos] = value(j);
    }
    o += __popc(bal[j]);
  }
}

template <class Pred>
__global__ void __launch_bounds__(CMP_THREADS) k_count(Pred pred, long long n, int* counts) {
  __shared__ int sh[CMP_THREADS / 32];
  const long long wb = warp_base() + (threadIdx.x & 31);
  int c = 0;
#pragma unroll 4
  for (int j = 0; j < CMP_IPT; ++j) {
    const long long e = wb + 32 * j;
    if (e < n && pred(e)) ++c;
  }
  int tot = block_reduce(c, sh, [](int a, int b) { return a + b; }, 0);
  if (threadIdx.x == 0) counts[blockIdx.x] = tot;
}

// Band count pass: clamp phi to [-cap, cap] in place (torch clamp_: NaN
// stays NaN) and count |phi| < thresh; all sixteen loads of a thread are
// issued before the conditional stores.
__global__ void __launch_bounds__(CMP_THREADS) k_band_count(float* __restrict__ phi, long long n, float cap,
                                                            float thresh, int* counts) {
  __shared__ int sh[CMP_THREADS / 32];
  const long long wb = warp_base() + (threadIdx.x & 31);
  float v[CMP_IPT];
#pragma unroll
  for (int j = 0; j < CMP_IPT; ++j) {
    const long long e = wb + 32 * j;
    v[j] = e < n ? phi[e] : 0.0f;
  }
  int c = 0;
#pragma unroll
  for (int j = 0; j < CMP_IPT; ++j) {
    const long long e = wb + 32 * j;
    if (e < n) {
      const float x = v[j];
      const float cl = (x != x) ? x : fminf(fmaxf(x, -cap), cap);
      if (cl != x && x == x) phi[e] = cl;
      c += fabsf(cl) < thresh ? 1 : 0;
    }
  }
  int tot = block_reduce(c, sh, [](int a, int b) { return a + b; }, 0);
  if (threadIdx.x == 0) counts[blockIdx.x] = tot;
}

// Single-CTA exclusive scan of nb block counts in place; total -> *total64.
__global__ void __launch_bounds__(1024) k_scan_counts(int* counts, long long nb, long long* total64) {
  __shared__ int sh[33];
  const long long per = (nb + blockDim.x - 1) / blockDim.x;
  const long long s0 = (long long)threadIdx.x * per;
  long long s1 = s0 + per;
  if (s1 > nb) s1 = nb;
  long long local = 0;
  for (long long i = s0; i < s1; ++i) local += counts[i];
  int tot;
  int off = block_exclusive_scan((int)local, sh, &tot);
  long long run = off;
  for (long long i = s0; i < s1; ++i) {
    int c = counts[i];
    counts[i] = (int)run;
    run += c;
  }
  if (threadIdx.x == 0) *total64 = tot;
}

template <class Pred>
__global__ void __launch_bounds__(CMP_THREADS) k_write(Pred pred, long long n, const int* offsets,
                                                       int32_t* out, long long capacity) {
  __shared__ int sh[33];
  const long long wb = warp_base() + (threadIdx.x & 31);
  unsigned int bal[CMP_IPT];
  int wt = 0;
#pragma unroll
  for (int j = 0; j < CMP_IPT; ++j) {
    const long long e = wb + 32 * j;
    bal[j] = __ballot_sync(0xffffffffu, e < n && pred(e));
    wt += __popc(bal[j]);
  }
  int tot;
  const long long o = (long long)offsets[blockIdx.x] + warp_offsets(wt, sh, &tot);
  write_selected(bal, o, out, capacity, [&](int j) { return (int32_t)(wb + 32 * j); });
}

// Band write pass: indices + dense occupancy + margin / static-count data.
__global__ void __launch_bounds__(CMP_THREADS) k_band_write(const float* __restrict__ phi, int nx, int ny,
                                                            int nz, float thresh, const int* offsets,
                                                            int32_t* out, long long capacity,
                                                            float* occ, svie_band_info* info) {
  __shared__ int sh[33];
  __shared__ long long shl[CMP_THREADS / 32];
  __shared__ int shi[CMP_THREADS / 32];
  const long long n = (long long)nx * ny * nz;
  const long long syz = (long long)ny * nz;
  const long long wb = warp_base() + (threadIdx.x & 31);
  unsigned int bal[CMP_IPT];
  int wt = 0;
  int inside_static = 0;
  int lo[3] = {INT_MAX, INT_MAX, INT_MAX}, hi[3] = {-1, -1, -1};
  int ilo[3] = {INT_MAX, INT_MAX, INT_MAX}, ihi[3] = {-1, -1, -1};
  // coordinates of the lane's first node, then advanced by 32 nodes per chunk
  int c[3] = {0, 0, 0};
  if (wb < n) {
    const int e0 = (int)wb, yz = e0 % (int)syz;
    c[0] = e0 / (int)syz;
    c[1] = yz / nz;
    c[2] = yz - c[1] * nz;
  }
  float pv[CMP_IPT];
#pragma unroll
  for (int j = 0; j < CMP_IPT; ++j) {
    const long long e = wb + 32 * j;
    pv[j] = e < n ? phi[e] : 0.0f;
  }
#pragma unroll
  for (int j = 0; j < CMP_IPT; ++j) {
    const long long e = wb + 32 * j;
    bool sel = false;
    if (e < n) {
      const float v = pv[j];
      sel = fabsf(v) < thresh;
      const bool neg = v < 0.0f;
      if (occ) occ[e] = neg ? 1.0f : 0.0f;
      if (sel) {
#pragma unroll
        for (int a = 0; a < 3; ++a) { lo[a] = min(lo[a], c[a]); hi[a] = max(hi[a], c[a]); }
      }
      if (neg) {
#pragma unroll
        for (int a = 0; a < 3; ++a) { ilo[a] = min(ilo[a], c[a]); ihi[a] = max(ihi[a], c[a]); }
        if (!sel) ++inside_static;
      }
    }
    bal[j] = __ballot_sync(0xffffffffu, sel);
    wt += __popc(bal[j]);
    c[2] += 32;
    while (c[2] >= nz) {
      c[2] -= nz;
      if (++c[1] == ny) { c[1] = 0; ++c[0]; }
    }
  }
  int tot;
  const long long o = (long long)offsets[blockIdx.x] + warp_offsets(wt, sh, &tot);
  write_selected(bal, o, out, capacity, [&](int j) { return (int32_t)(wb + 32 * j); });
  long long st = block_reduce((long long)inside_static, shl, OpSumLL(), 0LL);
  if (threadIdx.x == 0 && st) atomicAdd((unsigned long long*)&info->static_inside, (unsigned long long)st);
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    int v;
    v = block_reduce(lo[a], shi, OpMinI(), INT_MAX);
    if (threadIdx.x == 0 && v != INT_MAX) atomicMin(&info->lo[a], v);
    v = block_reduce(hi[a], shi, OpMaxI(), -1);
    if (threadIdx.x == 0 && v >= 0) atomicMax(&info->hi[a], v);
    v = block_reduce(ilo[a], shi, OpMinI(), INT_MAX);
    if (threadIdx.x == 0 && v != INT_MAX) atomicMin(&info->ilo[a], v);
    v = block_reduce(ihi[a], shi, OpMaxI(), -1);
    if (threadIdx.x == 0 && v >= 0) atomicMax(&info->ihi[a], v);
  }
}

__global__ void k_info_init(svie_band_info* info) {
  info->static_inside = 0;
  for (int a = 0; a < 3; ++a) {
    info->lo[a] = INT_MAX;
    info->hi[a] = -1;
    info->ilo[a] = INT_MAX;
    info->ihi[a] = -1;
  }
}

}  // namespace svie

using namespace svie;

extern "C" {

size_t svie_band_workspace_bytes(int64_t n) {
  long long nb = cmp_blocks(n < 1 ? 1 : n);
  return (size_t)(nb * sizeof(int) + 256);
}

int svie_band_scan(float* phi, int64_t n, float cap, float thresh, void* ws, size_t ws_bytes,
                   svie_band_info* info, void* stream) {
  if (!phi || !info || n <= 0 || n >= (1LL << 31)) {
    set_error("svie_band_scan: bad arguments (n=%lld)", (long long)n);
    return SVIE_ERR_ARG;
  }
  if (ws_bytes < svie_band_workspace_bytes(n) || !ws) {
    set_error("svie_band_scan: workspace too small");
    return SVIE_ERR_WORKSPACE;
  }
  cudaStream_t s = (cudaStream_t)stream;
  long long nb = cmp_blocks(n);
  k_band_count<<<(unsigned)nb, CMP_THREADS, 0, s>>>(phi, n, cap, thresh, (int*)ws);
  k_scan_counts<<<1, 1024, 0, s>>>((int*)ws, nb, (long long*)&info->count);
  k_info_init<<<1, 1, 0, s>>>(info);
  return launch_status("svie_band_scan", 3);
}

int svie_band_write(const float* phi, int nx, int ny, int nz, float thresh, const void* ws,
                    size_t ws_bytes, int32_t* band, int64_t capacity, float* occ,
                    svie_band_info* info, void* stream) {
  long long n = (long long)nx * ny * nz;
  if (!phi || !info || n <= 0 || n >= (1LL << 31) || (capacity > 0 && !band)) {
    set_error("svie_band_write: bad arguments");
    return SVIE_ERR_ARG;
  }
  if (ws_bytes < svie_band_workspace_bytes(n) || !ws) {
    set_error("svie_band_write: workspace too small");
    return SVIE_ERR_WORKSPACE;
  }
  long long nb = cmp_blocks(n);
  k_band_write<<<(unsigned)nb, CMP_THREADS, 0, (cudaStream_t)stream>>>(
      phi, nx, ny, nz, thresh, (const int*)ws, band, capacity, occ, info);
  return launch_status("svie_band_write");
}

int svie_mask_scan(const uint8_t* mask, int64_t n, void* ws, size_t ws_bytes, int64_t* count,
                   void* stream) {
  if (!mask || !count || n <= 0 || n >= (1LL << 31)) {
    set_error("svie_mask_scan: bad arguments");
    return SVIE_ERR_ARG;
  }
  if (ws_bytes < svie_band_workspace_bytes(n) || !ws) {
    set_error("svie_mask_scan: workspace too small");
    return SVIE_ERR_WORKSPACE;
  }
  cudaStream_t s = (cudaStream_t)stream;
  long long nb = cmp_blocks(n);
  MaskPred p{mask};
  k_count<<<(unsigned)nb, CMP_THREADS, 0, s>>>(p, n, (int*)ws);
  k_scan_counts<<<1, 1024, 0, s>>>((int*)ws, nb, (long long*)count);
  return launch_status("svie_mask_scan", 2);
}

int svie_mask_write(const uint8_t* mask, int64_t n, const void* ws, size_t ws_bytes, int32_t* out,
                    int64_t capacity, void* stream) {
  if (!mask || n <= 0 || n >= (1LL << 31) || (capacity > 0 && !out)) {
    set_error("svie_mask_write: bad arguments");
    return SVIE_ERR_ARG;
  }
  if (ws_bytes < svie_band_workspace_bytes(n) || !ws) {
    set_error("svie_mask_write: workspace too small");
    return SVIE_ERR_WORKSPACE;
  }
  long long nb = cmp_blocks(n);
  MaskPred p{mask};
  k_write<<<(unsigned)nb, CMP_THREADS, 0, (cudaStream_t)stream>>>(p, n, (const int*)ws, out, capacity);
  return launch_status("svie_mask_write");
}

}  // extern "C"

namespace svie {
// out[k] = vals[e] for the k-th e with mask[e] != 0 (order preserved).
__global__ void __launch_bounds__(CMP_THREADS) k_select(const uint8_t* __restrict__ mask, const int32_t* __restrict__ vals,
                                                        long long n, const int* offsets, int32_t* out,
                                                        long long capacity) {
  __shared__ int sh[33];
  const long long wb = warp_base() + (threadIdx.x & 31);
  unsigned int bal[CMP_IPT];
  int wt = 0;
#pragma unroll
  for (int j = 0; j < CMP_IPT; ++j) {
    const long long e = wb + 32 * j;
    bal[j] = __ballot_sync(0xffffffffu, e < n && mask[e]);
    wt += __popc(bal[j]);
  }
  int tot;
  const long long o = (long long)offsets[blockIdx.x] + warp_offsets(wt, sh, &tot);
  write_selected(bal, o, out, capacity, [&](int j) { return vals[wb + 32 * j]; });
}
}  // namespace svie

extern "C" int svie_mask_select(const uint8_t* mask, const int32_t* vals, int64_t n, const void* ws, size_t ws_bytes,
                                int32_t* out, int64_t capacity, void* stream) {
  if (!mask || !vals || n <= 0 || n >= (1LL << 31) || (capacity > 0 && !out)) {
    svie::set_error("svie_mask_select: bad arguments");
    return SVIE_ERR_ARG;
  }
  if (ws_bytes < svie_band_workspace_bytes(n) || !ws) {
    svie::set_error("svie_mask_select: workspace too small");
    return SVIE_ERR_WORKSPACE;
  }
  long long nb = svie::cmp_blocks(n);
  svie::k_select<<<(unsigned)nb, svie::CMP_THREADS, 0, (cudaStream_t)stream>>>(mask, vals, n, (const int*)ws, out,
                                                                              capacity);
  return svie::launch_status("svie_mask_select");
}

// ------------------------------------------------- brick-ordered compaction
// The same selections (mask[i] != 0, or |phi[i]| < thresh) listed brick by
// brick: bricks of 4 x 4 x 16 nodes in x-major brick order, inside a brick the
// 16 rows (x, y) in order and z fastest.  A CTA of the stencil kernels then
// covers one or two bricks, so the x/y taps of its warps land on rows that
// neighbouring warps of the same CTA load, instead of on new cache lines.
// Node lists in this order drive the RK stages and the reinitialisation
// sweeps; the sorted list stays the API's `band`.
namespace svie {

constexpr int BRX = 4, BRY = 4, BRZ = 16;
constexpr int BRICK = BRX * BRY * BRZ;  // 256 = CMP_TILE / CMP_IPT rows of 16

struct BrickGeom {
  int nx, ny, nz, nbx, nby, nbz;
  __host__ __device__ long long bricks() const { return (long long)nbx * nby * nbz; }
};

// A warp covers 32 rows of 16 nodes = two bricks; in chunk j its lanes hold
// rows 2j and 2j + 1 of the pair (half-warp per row, z fastest), so the
// ballot bits follow the list order.  Node of the lane in chunk j, or -1.
struct BrickWalk {
  long long base[2];  // node (x0, y0, z0 + lane % 16) of each brick
  int x0[2], y0[2], z0[2];
  int xm[2], ym[2];   // rows of each brick inside the grid along x and y (0 where this lane's z is outside)
  int syz, nz, hl;    // strides; hl = lane / 16, the half-warp
  SVIE_DEV BrickWalk(const BrickGeom& G) {
    const long long b0 = ((long long)blockIdx.x * CMP_THREADS + (threadIdx.x & ~31)) >> 4;
    const int zl = threadIdx.x & 15;
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const long long b = b0 + h;
      const bool ok = b < G.bricks();
      const int bz = ok ? (int)(b % G.nbz) : 0;
      const long long bxy = ok ? b / G.nbz : 0;
      x0[h] = (int)(bxy / G.nby) * BRX;
      y0[h] = (int)(bxy % G.nby) * BRY;
      z0[h] = bz * BRZ;
      const bool zin = ok && z0[h] + zl < G.nz;
      xm[h] = zin ? min(BRX, G.nx - x0[h]) : 0;
      ym[h] = zin ? min(BRY, G.ny - y0[h]) : 0;
      base[h] = ((long long)x0[h] * G.ny + y0[h]) * G.nz + z0[h] + zl;
    }
    syz = G.ny * G.nz;
    nz = G.nz;
    hl = (threadIdx.x >> 4) & 1;
  }
  // Chunk j: brick j / 8, row (2j % 16) + hl of it, i.e. x offset (2j % 16) / 4
  // (the same for both half-warps: 2j % 16 is even) and y offset 2j % 4 + hl.
  SVIE_DEV bool valid(int j) const {
    const int h = j >> 3;
    return ((2 * j) & 15) / 4 < xm[h] && ((2 * j) & 3) + hl < ym[h];
  }
  SVIE_DEV long long offset(int j) const {
    return base[j >> 3] + (long long)(((2 * j) & 15) / 4 * syz + (((2 * j) & 3) + hl) * nz);
  }
  // Node of chunk j, or -1 outside the grid.
  SVIE_DEV long long node(const BrickGeom&, int j) const { return valid(j) ? offset(j) : -1; }
};

// The CTA's static-inside count and band / inside bounding boxes into the
// band info: warp reductions, then one barrier and warp 0 across the warps,
// one atomic per quantity (exact and order independent).  Ends the caller.
SVIE_DEV void band_info_commit(int inside_static, const int* lo, const int* hi, const int* ilo, const int* ihi,
                               svie_band_info* info) {
  constexpr int NW = CMP_THREADS / 32;
  int r[13] = {inside_static, lo[0], lo[1], lo[2], -hi[0], -hi[1], -hi[2],
               ilo[0], ilo[1], ilo[2], -ihi[0], -ihi[1], -ihi[2]};
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    r[0] += __shfl_xor_sync(0xffffffffu, r[0], o);
#pragma unroll
    for (int k = 1; k < 13; ++k) r[k] = min(r[k], __shfl_xor_sync(0xffffffffu, r[k], o));
  }
  __shared__ int shr[13][NW];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) {
#pragma unroll
    for (int k = 0; k < 13; ++k) shr[k][wid] = r[k];
  }
  __syncthreads();
  if (wid != 0) return;
#pragma unroll
  for (int k = 0; k < 13; ++k) r[k] = lane < NW ? shr[k][lane] : (k == 0 ? 0 : INT_MAX);
#pragma unroll
  for (int o = NW / 2; o > 0; o >>= 1) {
    r[0] += __shfl_xor_sync(0xffffffffu, r[0], o);
#pragma unroll
    for (int k = 1; k < 13; ++k) r[k] = min(r[k], __shfl_xor_sync(0xffffffffu, r[k], o));
  }
  if (lane != 0) return;
  if (r[0]) atomicAdd((unsigned long long*)&info->static_inside, (unsigned long long)r[0]);
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    if (r[1 + a] != INT_MAX) atomicMin(&info->lo[a], r[1 + a]);
    if (-r[4 + a] >= 0) atomicMax(&info->hi[a], -r[4 + a]);
    if (r[7 + a] != INT_MAX) atomicMin(&info->ilo[a], r[7 + a]);
    if (-r[10 + a] >= 0) atomicMax(&info->ihi[a], -r[10 + a]);
  }
}

// LevelSet.rebuild_band (levelset.py:70-77) in brick order, pass 1: clamp phi
// to [-cap, cap] in place (NaN stays NaN) and count |phi| < thresh per CTA.
__global__ void __launch_bounds__(CMP_THREADS) k_brick_band_count(float* __restrict__ phi, BrickGeom G, float cap,
                                                                  float thresh, int* counts) {
  __shared__ int sh[CMP_THREADS / 32];
  const BrickWalk W(G);
  float v[CMP_IPT];
#pragma unroll
  for (int j = 0; j < CMP_IPT; ++j) v[j] = W.valid(j) ? phi[W.offset(j)] : 0.0f;
  int c = 0;
#pragma unroll
  for (int j = 0; j < CMP_IPT; ++j) {
    if (W.valid(j)) {
      const float x = v[j];
      const float cl = (x != x) ? x : fminf(fmaxf(x, -cap), cap);
      if (cl != x && x == x) phi[W.offset(j)] = cl;
      c += fabsf(cl) < thresh ? 1 : 0;
    }
  }
  int tot = block_reduce(c, sh, [](int a, int b) { return a + b; }, 0);
  if (threadIdx.x == 0) counts[blockIdx.x] = tot;
}

// Pass 2: brick-ordered band indices, dense occupancy (phi < 0) and the band
// info (static inside count, band and inside bounding boxes).
__global__ void __launch_bounds__(CMP_THREADS) k_brick_band_write(const float* __restrict__ phi, BrickGeom G,
                                                                  float thresh, const int* offsets, int32_t* out,
                                                                  long long capacity, float* occ,
                                                                  svie_band_info* info) {
  __shared__ int sh[33];
  const BrickWalk W(G);
  float pv[CMP_IPT];
#pragma unroll
  for (int j = 0; j < CMP_IPT; ++j) pv[j] = W.valid(j) ? phi[W.offset(j)] : 0.0f;
  unsigned int bal[CMP_IPT];
  int wt = 0, inside_static = 0;
  unsigned int selm = 0, negm = 0;  // chunks where this lane holds a band / an inside node
#pragma unroll
  for (int j = 0; j < CMP_IPT; ++j) {
    const bool valid = W.valid(j);
    const float v = pv[j];
    const bool sel = valid && fabsf(v) < thresh;
    const bool neg = valid && v < 0.0f;
    if (valid && occ) occ[W.offset(j)] = neg ? 1.0f : 0.0f;
    bal[j] = __ballot_sync(0xffffffffu, sel);
    wt += __popc(bal[j]);
    selm |= (sel ? 1u : 0u) << j;
    negm |= (neg ? 1u : 0u) << j;
    inside_static += (neg && !sel) ? 1 : 0;
  }
  // bounding boxes of this lane's nodes: chunk k of brick h sits at x offset
  // k / 2, y offset 2 (k % 2) + hl and the lane's z
  int lo[3] = {INT_MAX, INT_MAX, INT_MAX}, hi[3] = {-1, -1, -1};
  int ilo[3] = {INT_MAX, INT_MAX, INT_MAX}, ihi[3] = {-1, -1, -1};
  auto box = [&](unsigned int M, int h, int* l, int* u) {
    if (!M) return;
    const int z = W.z0[h] + (threadIdx.x & 15);
    l[0] = min(l[0], W.x0[h] + ((__ffs(M) - 1) >> 1));
    u[0] = max(u[0], W.x0[h] + ((31 - __clz(M)) >> 1));
    l[1] = min(l[1], W.y0[h] + ((M & 0x55u) ? W.hl : 2 + W.hl));
    u[1] = max(u[1], W.y0[h] + ((M & 0xAAu) ? 2 + W.hl : W.hl));
    l[2] = min(l[2], z);
    u[2] = max(u[2], z);
  };
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    box((selm >> (8 * h)) & 0xffu, h, lo, hi);
    box((negm >> (8 * h)) & 0xffu, h, ilo, ihi);
  }
  int tot;
  const long long o = (long long)offsets[blockIdx.x] + warp_offsets(wt, sh, &tot);
  write_selected(bal, o, out, capacity, [&](int j) { return (int32_t)W.node(G, j); });
  band_info_commit(inside_static, lo, hi, ilo, ihi, info);
}

// ---------------------------------------------- rebuild over a node list
// LevelSet.rebuild_band restricted to a node list: the reinitialisation work
// set (the band dilated, in brick order).  Off the list phi has not changed
// since the last rebuild, where it was clamped to +-cap, so the new band
// (|phi| < thresh < cap) lies in the list and comes out in brick order, the
// same list a full rebuild makes.  The list entries of a warp's chunks are
// the warp's 32 x CMP_IPT consecutive entries (coalesced index loads).
__global__ void __launch_bounds__(CMP_THREADS) k_list_band_count(float* __restrict__ phi,
                                                                 const int32_t* __restrict__ idx, long long m,
                                                                 float cap, float thresh, int* counts) {
  __shared__ int sh[CMP_THREADS / 32];
  const long long wb = warp_base() + (threadIdx.x & 31);
  int iv[CMP_IPT];
  float v[CMP_IPT];
#pragma unroll
  for (int j = 0; j < CMP_IPT; ++j) iv[j] = wb + 32 * j < m ? __ldg(idx + wb + 32 * j) : -1;
#pragma unroll
  for (int j = 0; j < CMP_IPT; ++j) v[j] = iv[j] >= 0 ? phi[iv[j]] : 0.0f;
  int c = 0;
#pragma unroll
  for (int j = 0; j < CMP_IPT; ++j) {
    if (iv[j] >= 0) {
      const float x = v[j];
      const float cl = (x != x) ? x : fminf(fmaxf(x, -cap), cap);
      if (cl != x && x == x) phi[iv[j]] = cl;
      c += fabsf(cl) < thresh ? 1 : 0;
    }
  }
  int tot = block_reduce(c, sh, [](int a, int b) { return a + b; }, 0);
  if (threadIdx.x == 0) counts[blockIdx.x] = tot;
}

// Pass 2: the band entries in list order, occupancy (phi < 0) of every listed
// node, the band and inside boxes of the listed nodes, and the number of
// listed inside nodes off the band (info->static_inside).
__global__ void __launch_bounds__(CMP_THREADS) k_list_band_write(const float* __restrict__ phi,
                                                                 const int32_t* __restrict__ idx, long long m,
                                                                 float thresh, const int* offsets, int32_t* out,
                                                                 long long capacity, float* occ, int syz, int nz,
                                                                 DivMagic dsyz, DivMagic dnz, svie_band_info* info) {
  __shared__ int sh[33];
  const long long wb = warp_base() + (threadIdx.x & 31);
  int iv[CMP_IPT];
  float v[CMP_IPT];
#pragma unroll
  for (int j = 0; j < CMP_IPT; ++j) iv[j] = wb + 32 * j < m ? __ldg(idx + wb + 32 * j) : -1;
#pragma unroll
  for (int j = 0; j < CMP_IPT; ++j) v[j] = iv[j] >= 0 ? phi[iv[j]] : 0.0f;
  unsigned int bal[CMP_IPT];
  int wt = 0, inside_static = 0;
  int lo[3] = {INT_MAX, INT_MAX, INT_MAX}, hi[3] = {-1, -1, -1};
  int ilo[3] = {INT_MAX, INT_MAX, INT_MAX}, ihi[3] = {-1, -1, -1};
#pragma unroll
  for (int j = 0; j < CMP_IPT; ++j) {
    const bool valid = iv[j] >= 0;
    const bool sel = valid && fabsf(v[j]) < thresh;
    const bool neg = valid && v[j] < 0.0f;
    if (valid && occ) occ[iv[j]] = neg ? 1.0f : 0.0f;
    bal[j] = __ballot_sync(0xffffffffu, sel);
    wt += __popc(bal[j]);
    if (sel || neg) {
      const int i = iv[j], x = div_exact(i, dsyz), r = i - x * syz, y = div_exact(r, dnz), z = r - y * nz;
      const int c[3] = {x, y, z};
#pragma unroll
      for (int a = 0; a < 3; ++a) {
        if (sel) { lo[a] = min(lo[a], c[a]); hi[a] = max(hi[a], c[a]); }
        if (neg) { ilo[a] = min(ilo[a], c[a]); ihi[a] = max(ihi[a], c[a]); }
      }
      inside_static += (neg && !sel) ? 1 : 0;
    }
  }
  int tot;
  const long long o = (long long)offsets[blockIdx.x] + warp_offsets(wt, sh, &tot);
  write_selected(bal, o, out, capacity, [&](int j) { return (int32_t)iv[j]; });
  band_info_commit(inside_static, lo, hi, ilo, ihi, info);
}

// Listed nodes with phi < 0 whose bit in `marked` (the bit layout of
// svie_reinit_bits) is clear, added to *count.
__global__ void __launch_bounds__(CMP_THREADS) k_list_inside_off_mask(const float* __restrict__ phi,
                                                                      const int32_t* __restrict__ idx, long long m,
                                                                      const uint32_t* __restrict__ marked, int nz,
                                                                      int nzw, DivMagic dnz,
                                                                      unsigned long long* count) {
  __shared__ int sh[CMP_THREADS / 32];
  const long long wb = warp_base() + (threadIdx.x & 31);
  int c = 0;
#pragma unroll 4
  for (int j = 0; j < CMP_IPT; ++j) {
    const long long e = wb + 32 * j;
    if (e < m) {
      const int i = __ldg(idx + e);
      if (__ldg(phi + i) < 0.0f) {
        const int row = div_exact(i, dnz), z = i - row * nz;
        c += ((__ldg(marked + (long long)row * nzw + (z >> 5)) >> (z & 31)) & 1u) ? 0 : 1;
      }
    }
  }
  const int tot = block_reduce(c, sh, [](int a, int b) { return a + b; }, 0);
  if (threadIdx.x == 0 && tot) atomicAdd(count, (unsigned long long)tot);
}

template <class Pred>
__global__ void __launch_bounds__(CMP_THREADS) k_brick_count(Pred pred, BrickGeom G, int* counts) {
  __shared__ int sh[CMP_THREADS / 32];
  const BrickWalk W(G);
  int c = 0;
#pragma unroll
  for (int j = 0; j < CMP_IPT; ++j) {
    const long long e = W.node(G, j);
    if (e >= 0 && pred(e)) ++c;
  }
  int tot = block_reduce(c, sh, [](int a, int b) { return a + b; }, 0);
  if (threadIdx.x == 0) counts[blockIdx.x] = tot;
}

template <class Pred>
__global__ void __launch_bounds__(CMP_THREADS) k_brick_write(Pred pred, BrickGeom G, const int* offsets, int32_t* out,
                                                             long long capacity) {
  __shared__ int sh[33];
  const BrickWalk W(G);
  unsigned int bal[CMP_IPT];
  int wt = 0;
#pragma unroll
  for (int j = 0; j < CMP_IPT; ++j) {
    const long long e = W.node(G, j);
    bal[j] = __ballot_sync(0xffffffffu, e >= 0 && pred(e));
    wt += __popc(bal[j]);
  }
  int tot;
  const long long o = (long long)offsets[blockIdx.x] + warp_offsets(wt, sh, &tot);
  write_selected(bal, o, out, capacity, [&](int j) { return (int32_t)W.node(G, j); });
}

// The reinitialisation work mask as bits (svie_reinit_bits: rows (x, y) of
// nzw words, bit z % 32 of word z / 32, nothing set past nz).  One lane per
// brick row of 16 nodes: thread t of CTA k takes row t % 16 of brick
// 16 k + t / 16, i.e. the same 4096 nodes per CTA and the same order (brick,
// row, z) as the node-per-lane brick kernels.  Returns the row's 16 bits.
SVIE_DEV unsigned int brick_row_bits(const uint32_t* __restrict__ bits, int nzw, const BrickGeom& G, long long* e0) {
  const long long r = (long long)blockIdx.x * CMP_THREADS + threadIdx.x;
  const long long b = r >> 4;
  *e0 = -1;
  if (b >= G.bricks()) return 0u;
  const int bz = (int)(b % G.nbz);
  const long long bxy = b / G.nbz;
  const int lr = (int)(r & 15);
  const int x = (int)(bxy / G.nby) * BRX + (lr >> 2), y = (int)(bxy % G.nby) * BRY + (lr & 3), z0 = bz * BRZ;
  if (x >= G.nx || y >= G.ny) return 0u;
  *e0 = ((long long)x * G.ny + y) * G.nz + z0;
  return (__ldg(bits + ((long long)x * G.ny + y) * nzw + (z0 >> 5)) >> (z0 & 31)) & 0xffffu;
}

__global__ void __launch_bounds__(CMP_THREADS) k_brick_bits_count(const uint32_t* __restrict__ bits, int nzw,
                                                                  BrickGeom G, int* counts) {
  __shared__ int sh[CMP_THREADS / 32];
  long long e0;
  const int c = __popc(brick_row_bits(bits, nzw, G, &e0));
  int tot = block_reduce(c, sh, [](int a, int b) { return a + b; }, 0);
  if (threadIdx.x == 0) counts[blockIdx.x] = tot;
}

__global__ void __launch_bounds__(CMP_THREADS) k_brick_bits_write(const uint32_t* __restrict__ bits, int nzw,
                                                                  BrickGeom G, const int* offsets, int32_t* out,
                                                                  long long capacity) {
  __shared__ int sh[CMP_THREADS / 32];
  long long e0;
  unsigned int rb = brick_row_bits(bits, nzw, G, &e0);
  const int c = __popc(rb);
  // exclusive prefix of the row counts over the CTA (lane order = list order)
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  int s = c;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, s, o);
    if (lane >= o) s += y;
  }
  if (lane == 31) sh[wid] = s;
  __syncthreads();
  int before = 0;
  for (int w = 0; w < wid; ++w) before += sh[w];
  long long o = (long long)offsets[blockIdx.x] + before + s - c;
  while (rb) {
    const int k = __ffs(rb) - 1;
    rb &= rb - 1u;
    if (o < capacity) out[o] = (int32_t)(e0 + k);
    ++o;
  }
}

struct AbsLessPred {
  const float* phi;
  float thresh;
  SVIE_DEV bool operator()(long long e) const { return fabsf(phi[e]) < thresh; }
};

static BrickGeom brick_geom(int nx, int ny, int nz) {
  return BrickGeom{nx, ny, nz, (nx + BRX - 1) / BRX, (ny + BRY - 1) / BRY, (nz + BRZ - 1) / BRZ};
}

static long long brick_blocks(const BrickGeom& G) {
  const long long rows = G.bricks() * (BRICK / CMP_IPT);
  return (rows + CMP_THREADS - 1) / CMP_THREADS;
}

}  // namespace svie

extern "C" {

size_t svie_brick_workspace_bytes(int nx, int ny, int nz) {
  return (size_t)svie::brick_blocks(svie::brick_geom(nx, ny, nz)) * sizeof(int) + 256;
}

int svie_brick_scan(int kind, const void* src, int nx, int ny, int nz, float thresh, void* ws, size_t ws_bytes,
                    int64_t* count, void* stream) {
  using namespace svie;
  const long long n = (long long)nx * ny * nz;
  if (!src || !count || n <= 0 || n >= (1LL << 31) || kind < 0 || kind > 2) {
    set_error("svie_brick_scan: bad arguments");
    return SVIE_ERR_ARG;
  }
  if (!ws || ws_bytes < svie_brick_workspace_bytes(nx, ny, nz)) {
    set_error("svie_brick_scan: workspace too small");
    return SVIE_ERR_WORKSPACE;
  }
  cudaStream_t s = (cudaStream_t)stream;
  const BrickGeom G = brick_geom(nx, ny, nz);
  const long long nb = brick_blocks(G);
  if (kind == 0) k_brick_count<<<(unsigned)nb, CMP_THREADS, 0, s>>>(MaskPred{(const uint8_t*)src}, G, (int*)ws);
  else if (kind == 1) k_brick_count<<<(unsigned)nb, CMP_THREADS, 0, s>>>(AbsLessPred{(const float*)src, thresh}, G, (int*)ws);
  else k_brick_bits_count<<<(unsigned)nb, CMP_THREADS, 0, s>>>((const uint32_t*)src, (nz + 31) / 32, G, (int*)ws);
  k_scan_counts<<<1, 1024, 0, s>>>((int*)ws, nb, (long long*)count);
  return launch_status("svie_brick_scan", 2);
}

int svie_brick_write(int kind, const void* src, int nx, int ny, int nz, float thresh, const void* ws, size_t ws_bytes,
                     int32_t* out, int64_t capacity, void* stream) {
  using namespace svie;
  const long long n = (long long)nx * ny * nz;
  if (!src || n <= 0 || n >= (1LL << 31) || kind < 0 || kind > 2 || (capacity > 0 && !out)) {
    set_error("svie_brick_write: bad arguments");
    return SVIE_ERR_ARG;
  }
  if (!ws || ws_bytes < svie_brick_workspace_bytes(nx, ny, nz)) {
    set_error("svie_brick_write: workspace too small");
    return SVIE_ERR_WORKSPACE;
  }
  cudaStream_t s = (cudaStream_t)stream;
  const BrickGeom G = brick_geom(nx, ny, nz);
  const long long nb = brick_blocks(G);
  if (kind == 0)
    k_brick_write<<<(unsigned)nb, CMP_THREADS, 0, s>>>(MaskPred{(const uint8_t*)src}, G, (const int*)ws, out, capacity);
  else if (kind == 1)
    k_brick_write<<<(unsigned)nb, CMP_THREADS, 0, s>>>(AbsLessPred{(const float*)src, thresh}, G, (const int*)ws, out,
                                                       capacity);
  else
    k_brick_bits_write<<<(unsigned)nb, CMP_THREADS, 0, s>>>((const uint32_t*)src, (nz + 31) / 32, G, (const int*)ws,
                                                            out, capacity);
  return launch_status("svie_brick_write");
}

int svie_brick_band_scan(float* phi, int nx, int ny, int nz, float cap, float thresh, void* ws, size_t ws_bytes,
                         svie_band_info* info, void* stream) {
  using namespace svie;
  const long long n = (long long)nx * ny * nz;
  if (!phi || !info || n <= 0 || n >= (1LL << 31)) {
    set_error("svie_brick_band_scan: bad arguments");
    return SVIE_ERR_ARG;
  }
  if (!ws || ws_bytes < svie_brick_workspace_bytes(nx, ny, nz)) {
    set_error("svie_brick_band_scan: workspace too small");
    return SVIE_ERR_WORKSPACE;
  }
  cudaStream_t s = (cudaStream_t)stream;
  const BrickGeom G = brick_geom(nx, ny, nz);
  const long long nb = brick_blocks(G);
  k_brick_band_count<<<(unsigned)nb, CMP_THREADS, 0, s>>>(phi, G, cap, thresh, (int*)ws);
  k_scan_counts<<<1, 1024, 0, s>>>((int*)ws, nb, (long long*)&info->count);
  k_info_init<<<1, 1, 0, s>>>(info);
  return launch_status("svie_brick_band_scan", 3);
}

int svie_brick_band_write(const float* phi, int nx, int ny, int nz, float thresh, const void* ws, size_t ws_bytes,
                          int32_t* out, int64_t capacity, float* occ, svie_band_info* info, void* stream) {
  using namespace svie;
  const long long n = (long long)nx * ny * nz;
  if (!phi || !info || n <= 0 || n >= (1LL << 31) || (capacity > 0 && !out)) {
    set_error("svie_brick_band_write: bad arguments");
    return SVIE_ERR_ARG;
  }
  if (!ws || ws_bytes < svie_brick_workspace_bytes(nx, ny, nz)) {
    set_error("svie_brick_band_write: workspace too small");
    return SVIE_ERR_WORKSPACE;
  }
  const BrickGeom G = brick_geom(nx, ny, nz);
  const long long nb = brick_blocks(G);
  k_brick_band_write<<<(unsigned)nb, CMP_THREADS, 0, (cudaStream_t)stream>>>(phi, G, thresh, (const int*)ws, out,
                                                                             capacity, occ, info);
  return launch_status("svie_brick_band_write");
}

size_t svie_list_workspace_bytes(int64_t m) {
  return (size_t)((m + svie::CMP_TILE - 1) / svie::CMP_TILE + 1) * sizeof(int) + 256;
}

int svie_list_band_scan(float* phi, const int32_t* idx, int64_t m, float cap, float thresh, void* ws, size_t ws_bytes,
                        svie_band_info* info, void* stream) {
  using namespace svie;
  if (!phi || !info || m < 0 || (m > 0 && !idx)) {
    set_error("svie_list_band_scan: bad arguments");
    return SVIE_ERR_ARG;
  }
  if (!ws || ws_bytes < svie_list_workspace_bytes(m)) {
    set_error("svie_list_band_scan: workspace too small");
    return SVIE_ERR_WORKSPACE;
  }
  cudaStream_t s = (cudaStream_t)stream;
  const long long nb = (m + CMP_TILE - 1) / CMP_TILE;
  if (nb > 0) k_list_band_count<<<(unsigned)nb, CMP_THREADS, 0, s>>>(phi, idx, m, cap, thresh, (int*)ws);
  k_scan_counts<<<1, 1024, 0, s>>>((int*)ws, nb, (long long*)&info->count);
  k_info_init<<<1, 1, 0, s>>>(info);
  return launch_status("svie_list_band_scan", nb > 0 ? 3 : 2);
}

int svie_list_band_write(const float* phi, const int32_t* idx, int64_t m, int nx, int ny, int nz, float thresh,
                         const void* ws, size_t ws_bytes, int32_t* out, int64_t capacity, float* occ,
                         svie_band_info* info, void* stream) {
  using namespace svie;
  if (!phi || !info || m < 0 || (m > 0 && !idx) || (capacity > 0 && !out) || nx <= 0 || ny <= 0 || nz <= 0 ||
      (long long)nx * ny * nz >= (1LL << 31)) {
    set_error("svie_list_band_write: bad arguments");
    return SVIE_ERR_ARG;
  }
  if (!ws || ws_bytes < svie_list_workspace_bytes(m)) {
    set_error("svie_list_band_write: workspace too small");
    return SVIE_ERR_WORKSPACE;
  }
  const long long nb = (m + CMP_TILE - 1) / CMP_TILE;
  if (nb == 0) return SVIE_OK;
  const int syz = ny * nz;
  k_list_band_write<<<(unsigned)nb, CMP_THREADS, 0, (cudaStream_t)stream>>>(
      phi, idx, m, thresh, (const int*)ws, out, capacity, occ, syz, nz, div_magic(syz), div_magic(nz), info);
  return launch_status("svie_list_band_write");
}

int svie_list_inside_off_mask(const float* phi, const int32_t* idx, int64_t m, const uint32_t* marked, int nx, int ny,
                              int nz, uint64_t* count, void* stream) {
  using namespace svie;
  if (!phi || !marked || !count || m < 0 || (m > 0 && !idx) || nz <= 0) {
    set_error("svie_list_inside_off_mask: bad arguments");
    return SVIE_ERR_ARG;
  }
  cudaStream_t s = (cudaStream_t)stream;
  if (cudaMemsetAsync(count, 0, sizeof(uint64_t), s) != cudaSuccess) {
    set_error("svie_list_inside_off_mask: memset failed");
    return SVIE_ERR_LAUNCH;
  }
  const long long nb = (m + CMP_TILE - 1) / CMP_TILE;
  if (nb == 0) return SVIE_OK;
  k_list_inside_off_mask<<<(unsigned)nb, CMP_THREADS, 0, s>>>(phi, idx, m, marked, nz, (nz + 31) / 32, div_magic(nz),
                                                               (unsigned long long*)count);
  return launch_status("svie_list_inside_off_mask");
}

}  // extern "C"
