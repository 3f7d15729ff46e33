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
#include <algorithm>

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

// Geometry record over the m work-set nodes (byte offsets in GeoLayout; the
// local pseudo-time step is not stored: the sweeps rebuild it from the
// distances they read):
//   meta  uint8 [m]     bits 0-5: crossing flags cp_x cm_x cp_y cm_y cp_z cm_z,
//                       bit 6: phi0 > 0, bit 7: phi0 < 0
//   wbase int32 [W + 1] per warp of 32 entries (W = ceil(m / 32)): index of
//                       its first distance in `dist`; wbase[W] = the count
//   dist  float [<= 6m] the subcell distances of the flagged crossings only,
//                       in work-set order and flag-bit order within a node
//   wx    int32 [W + 1] per warp: index of its first general entry in xlist
//   xlist int32 [<= m]  the general entries (work-set order): those with a
//                       flagged crossing or without a sign (phi0 zero or NaN),
//                       by grid index
//   xoff  int32 [<= m]  the index of each one's first distance in dist
//   plist int32 [<= m]  the plain entries (every other one, work-set order) as
//                       their grid index, complemented (~i) where phi0 < 0
//   xmeta uint8 [<= m]  the meta byte of each general entry
//   cfl   float, then np int32: the number of plain entries
//   sums  int32         scratch of the scan that makes wbase
// A sweep streams 4 bytes of list per plain node (index and sign in one word,
// every lane of a warp busy) and reads distances only at crossings, from an
// array a few per cent of the work set long: the sweep's whole footprint (the
// band part of the two grids, the lists and distances) then stays in L2
// across the 40 sweeps of a call.
struct GeoLayout {
  long long m, W, meta, wbase, dist, wx, xlist, xoff, plist, xmeta, cfl, sums, nsums, total;
};

__host__ __device__ inline long long align16ll(long long b) { return (b + 15) & ~15LL; }

__host__ __device__ inline GeoLayout geo_layout(long long m) {
  GeoLayout L;
  L.m = m;
  L.W = (m + 31) / 32;
  L.meta = 0;
  L.wbase = align16ll(m);
  L.dist = align16ll(L.wbase + 4 * (L.W + 1));
  L.wx = align16ll(L.dist + 24 * m);
  L.xlist = align16ll(L.wx + 4 * (L.W + 1));
  L.xoff = align16ll(L.xlist + 4 * m);
  L.plist = align16ll(L.xoff + 4 * m);
  L.xmeta = align16ll(L.plist + 4 * m);
  L.cfl = align16ll(L.xmeta + m);
  L.sums = L.cfl + 16;
  L.nsums = (L.W + 1 + 1023) / 1024;
  L.total = L.sums + 4 * L.nsums + 256;
  return L;
}

struct Geo {
  uint8_t* meta;
  int* wbase;
  float* dist;
  int* wx;     // per warp: index of its first crossing node in xlist; wx[W] = the count
  int* xlist;      // the general work-set entries (crossing or no sign) by grid index, in work-set order
  int* xoff;       // for each of them, the index of its first distance in dist
  int* plist;      // the plain entries' grid indices, ~i where phi0 < 0
  uint8_t* xmeta;  // the general entries' meta bytes
  float* cfl;
  int* np;         // the number of plain entries
  long long m, W;
};

// The same view built on the host (the sweeps take it as a kernel argument
// instead of deriving the offsets from m in every thread).
inline Geo geo_view_host(void* base, long long m) {
  const GeoLayout L = geo_layout(m);
  char* b = (char*)base;
  Geo g;
  g.meta = (uint8_t*)(b + L.meta);
  g.wbase = (int*)(b + L.wbase);
  g.dist = (float*)(b + L.dist);
  g.wx = (int*)(b + L.wx);
  g.xlist = (int*)(b + L.xlist);
  g.xoff = (int*)(b + L.xoff);
  g.plist = (int*)(b + L.plist);
  g.xmeta = (uint8_t*)(b + L.xmeta);
  g.cfl = (float*)(b + L.cfl);
  g.np = (int*)(b + L.cfl + 4);
  g.m = m;
  g.W = L.W;
  return g;
}

SVIE_DEV Geo geo_view(void* base, long long m) {
  const GeoLayout L = geo_layout(m);
  char* b = (char*)base;
  Geo g;
  g.meta = (uint8_t*)(b + L.meta);
  g.wbase = (int*)(b + L.wbase);
  g.dist = (float*)(b + L.dist);
  g.wx = (int*)(b + L.wx);
  g.xlist = (int*)(b + L.xlist);
  g.xoff = (int*)(b + L.xoff);
  g.plist = (int*)(b + L.plist);
  g.xmeta = (uint8_t*)(b + L.xmeta);
  g.cfl = (float*)(b + L.cfl);
  g.np = (int*)(b + L.cfl + 4);
  g.m = m;
  g.W = L.W;
  return g;
}

// Crossing flags and sign bits of node i alone (the flags of geometry_at).
SVIE_DEV uint32_t crossing_flags(const float* __restrict__ f, int i, int sx, int sy, int sz) {
  const float* qp = f + i;
  const float c = __ldg(qp);
  uint32_t flags = 0;
  const int st[3] = {sx, sy, sz};
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const float m1 = __ldg(qp - st[a]), p1 = __ldg(qp + st[a]);
    flags |= ((c * p1) < 0.0f ? 1u : 0u) << (2 * a);
    flags |= ((c * m1) < 0.0f ? 1u : 0u) << (2 * a + 1);
  }
  flags |= (c > 0.0f ? 1u : 0u) << 6;
  flags |= (c < 0.0f ? 1u : 0u) << 7;
  return flags;
}

// Crossing geometry at node i (kernels.py:335-359): flag bits 2a (cp) and
// 2a + 1 (cm), distances d[2a] = xp, d[2a + 1] = xm clamped below to 1e-6 h,
// and dtau = cfl max(hmin, 1e-3 h) with hmin from the unclamped distances.
SVIE_DEV uint32_t geometry_at(const float* __restrict__ f, int i, int sx, int sy, int sz, float h, float cfl,
                              float d[6], float& dtau) {
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
    d[2 * a] = fmaxf(xp, 1e-6f * h);
    d[2 * a + 1] = fmaxf(xm, 1e-6f * h);
  }
  flags |= (c > 0.0f ? 1u : 0u) << 6;
  flags |= (c < 0.0f ? 1u : 0u) << 7;
  dtau = cfl * fmaxf(hmin, 1e-3f * h);
  return flags;
}

// A work-set entry with meta byte `meta` takes the general path (the compact
// list xlist) when it has a flagged crossing or no sign bit; every other entry
// is plain: no subcell branch and dtau = cfl max(h, 1e-3 h).
SVIE_DEV bool general_entry(uint32_t meta) { return (meta & 63u) != 0u || (meta & 192u) == 0u; }

// Exclusive prefix of v over the lanes of the warp (all lanes take part).
SVIE_DEV int warp_exclusive(int v) {
  const int lane = threadIdx.x & 31;
  int s = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, s, o);
    if (lane >= o) s += y;
  }
  return s - v;
}

// Pass 1: flags and sign bits from the 7-point stencil; per-warp counts of
// the flagged distances (wbase) and of the general entries (wx).
__global__ void k_reinit_count(const float* __restrict__ f, const int32_t* __restrict__ idx, long long m, int sx,
                               int sy, int sz, float cfl, void* geo) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  Geo g = geo_view(geo, m);
  uint32_t flags = 0;
  if (t < m) {
    flags = crossing_flags(f, idx[t], sx, sy, sz);
    g.meta[t] = (uint8_t)flags;
  }
  const int cnt = __reduce_add_sync(0xffffffffu, __popc(flags & 63u));
  const int cx = __reduce_add_sync(0xffffffffu, (t < m && general_entry(flags)) ? 1 : 0);
  const long long w = t >> 5;
  if ((threadIdx.x & 31) == 0 && w < g.W) {
    g.wbase[w] = cnt;
    g.wx[w] = cx;
  }
  if (t == 0) {
    g.wbase[g.W] = 0;
    g.wx[g.W] = 0;
    *g.cfl = cfl;
  }
}

// Pass 3 (after the exclusive scans of wbase and wx): the plain and general
// lists, with each general entry's flags and first distance.  The flags come
// from pass 1.  The warps before warp w are full, so 32 w - wx[w] plain
// entries precede it.
__global__ void k_reinit_lists(const int32_t* __restrict__ idx, long long m, void* geo) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  Geo g = geo_view(geo, m);
  const bool act = t < m;
  const uint32_t meta = act ? g.meta[t] : 0u;
  const uint32_t flags = meta & 63u;
  const bool gen = act && general_entry(meta);
  const long long w = t >> 5;
  if (t == 0) *g.np = (int)(m - g.wx[g.W]);
  const int po = warp_exclusive(act && !gen ? 1 : 0);
  if (act && !gen) {
    const int i = idx[t];
    g.plist[32 * w - g.wx[w] + po] = (meta & 64u) ? i : ~i;
  }
  if (!__ballot_sync(0xffffffffu, gen)) return;
  const int off = warp_exclusive(__popc(flags));
  const int xo = warp_exclusive(gen ? 1 : 0);
  if (!gen) return;
  const int k = g.wx[w] + xo;
  g.xlist[k] = idx[t];
  g.xmeta[k] = (uint8_t)meta;
  g.xoff[k] = g.wbase[w] + off;
}

// Pass 4: the subcell distances of the flagged crossings, over the general
// list (grid-stride; every lane of a warp holds a general entry).
__global__ void k_reinit_dist(const float* __restrict__ f, long long m, int sx, int sy, int sz, float h, float cfl,
                              void* geo) {
  Geo g = geo_view(geo, m);
  const int X = g.wx[g.W];
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < X; k += gridDim.x * blockDim.x) {
    const uint32_t flags = g.xmeta[k] & 63u;
    if (!flags) continue;
    float d[6], dtau;
    geometry_at(f, g.xlist[k], sx, sy, sz, h, cfl, d, dtau);
    float* out = g.dist + g.xoff[k];
    int r = 0;
#pragma unroll
    for (int b = 0; b < 6; ++b)
      if ((flags >> b) & 1u) out[r++] = d[b];
  }
}

// Array form of the geometry for kernels.reinit_geometry: every node's
// distances (also where no crossing is flagged), flags one byte per axis side.
__global__ void k_reinit_geometry_full(const float* __restrict__ f, const int32_t* __restrict__ idx, long long m,
                                       int sx, int sy, int sz, float h, float cfl, float* sgn, float* dtau_out,
                                       uint8_t* flags6, float* dist6) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= m) return;
  float d[6], dtau;
  const uint32_t flags = geometry_at(f, idx[t], sx, sy, sz, h, cfl, d, dtau);
  sgn[t] = (flags & 64u) ? 1.0f : ((flags & 128u) ? -1.0f : 0.0f);
  dtau_out[t] = dtau;
  for (int a = 0; a < 6; ++a) {
    flags6[a * m + t] = (flags >> a) & 1u;
    dist6[a * m + t] = d[a];
  }
}

// Packed form from the 14 arrays (kernels.reinit_rhs takes them from the
// caller): pass 1 counts, pass 2 (after the scan) writes the distances.  The
// grid indices are not known here: both sweep lists stay empty (svie_reinit_rhs
// reads the entries by position).  dtau is not kept: the RHS does not use it.
__global__ void k_reinit_pack(const float* __restrict__ sgn, const uint8_t* __restrict__ flags6,
                              const float* __restrict__ dist6, long long m, void* geo, int pass) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  Geo g = geo_view(geo, m);
  uint32_t flags = 0;
  if (t < m)
    for (int a = 0; a < 6; ++a) flags |= (flags6[a * m + t] ? 1u : 0u) << a;
  if (pass == 0) {
    const int cnt = __reduce_add_sync(0xffffffffu, __popc(flags));
    const long long w = t >> 5;
    if ((threadIdx.x & 31) == 0 && w < g.W) {
      g.wbase[w] = cnt;
      g.wx[w] = 0;
    }
    if (t == 0) {
      g.wbase[g.W] = 0;
      g.wx[g.W] = 0;
      *g.cfl = 0.0f;
      *g.np = 0;
    }
    if (t < m) {
      const float s = sgn[t];
      g.meta[t] = (uint8_t)(flags | (s > 0.0f ? 64u : 0u) | (s < 0.0f ? 128u : 0u));
    }
    return;
  }
  const int off = warp_exclusive(__popc(flags));
  if (t >= m) return;
  const int doff = g.wbase[t >> 5] + off;
  float* out = g.dist + doff;
  int r = 0;
  for (int b = 0; b < 6; ++b)
    if ((flags >> b) & 1u) out[r++] = dist6[b * m + t];
}

SVIE_DEV float meta_sgn(uint32_t meta) { return (meta & 64u) ? 1.0f : ((meta & 128u) ? -1.0f : 0.0f); }

// Index of entry t's first distance in g.dist; every lane of the warp calls
// it (lanes past m with flags 0).  Warps without any crossing skip the scan.
SVIE_DEV int dist_offset(const Geo& g, long long t, uint32_t flags) {
  const uint32_t f6 = flags & 63u;
  if (!__ballot_sync(0xffffffffu, f6 != 0u)) return 0;
  const int off = warp_exclusive(__popc(f6));
  return f6 ? __ldg(g.wbase + (t >> 5)) + off : 0;
}

// reinit_rhs (kernels.py:363-379) at work-set entry t.  Divisions by h and by
// hh = RN(h * h) use the correctly rounded reciprocals rh and rhh (div_by).  Also returns
// hmin = min(h, stored distances of the flagged crossings), from which
// dtau = cfl * max(hmin, 1e-3 h) is rebuilt exactly as geometry_at computed
// it (a distance below 1e-6 h, stored clamped to 1e-6 h, gives the same
// 1e-3 h either way).  `off`: the node's first distance (dist_offset).
// CROSS = false: a node without flagged crossings (the subcell branches
// compiled out, hmin = h).
template <bool CROSS = true>
SVIE_DEV float reinit_rhs_at(const float* __restrict__ f, int i, const Geo& g, int off, uint32_t flags, int sx,
                             int sy, int sz, float h, float rh, float hh, float rhh, float& hmin) {
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
  const float* dn = g.dist + off;
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const float m2 = v3[a][0], m1 = v3[a][1], p1 = v3[a][2], p2 = v3[a][3];
    const float mm_p = minmod(p1 - 2.0f * c + m1, p2 - 2.0f * p1 + c);
    const float mm_m = minmod(p1 - 2.0f * c + m1, c - 2.0f * m1 + m2);
    float Dp = div_by(p1 - c - 0.5f * mm_p, h, rh);
    float Dm = div_by(c - m1 + 0.5f * mm_m, h, rh);
    if (CROSS && ((flags >> (2 * a)) & 1u)) {
      const float xp = __ldg(dn + __popc(flags & ((1u << (2 * a)) - 1u)));
      Dp = -c / xp - div_by(0.5f * xp * mm_p, hh, rhh);
      hmin = fminf(hmin, xp);
    }
    if (CROSS && ((flags >> (2 * a + 1)) & 1u)) {
      const float xm = __ldg(dn + __popc(flags & ((1u << (2 * a + 1)) - 1u)));
      Dm = c / xm + div_by(0.5f * xm * mm_m, hh, rhh);
      hmin = fminf(hmin, xm);
    }
    const float a1 = outside ? fmaxf(Dm, 0.0f) : fminf(Dm, 0.0f);
    const float b1 = outside ? fminf(Dp, 0.0f) : fmaxf(Dp, 0.0f);
    g2 = g2 + fmaxf(a1 * a1, b1 * b1);
  }
  return -sgn * (sqrtf(g2) - 1.0f);
}

// One Jacobi half-step of the TVD-RK2 pseudo-time iteration at work-set
// entry t: first = u0 + dtau rhs(A) into B, second = (u0 + B + dtau rhs(B)) / 2
// into A (u0 is A's value, still in dst).
SVIE_DEV void sweep_update(const float* __restrict__ src, float* __restrict__ dst, int i, float r, float dtau,
                           int second) {
  if (!second) {
    dst[i] = src[i] + dtau * r;
  } else {
    const float u0 = dst[i], u1 = src[i];
    dst[i] = 0.5f * (u0 + u1 + dtau * r);
  }
}

// One launch per half-step.  Blocks [0, nbm) take the plain entries (about
// nine in ten) from the plain list, whose word holds the grid index and the
// sign: no subcell branch, no distance reads, dtau = cfl max(h, 1e-3 h), and
// every lane of a warp busy.  The blocks after them take the general entries
// from their compact list (count wx[W]), grid-stride, so that no warp runs the
// subcell branch for a few lanes; they are scheduled last and fill the tail of
// the first part.
__global__ void __launch_bounds__(RI_THREADS, 8) k_reinit_sweep(const float* __restrict__ src, float* __restrict__ dst,
                                                             int sx, int sy, int sz, float h, float rh, float rhh,
                                                             Geo g, int second, int nbm) {
  pdl_wait();  // the previous half-step's writes (and the geometry) are visible from here on
  pdl_release();
  const float cfl = __ldg(g.cfl);
  if ((int)blockIdx.x < nbm) {
    // a contiguous run of the brick-ordered plain list per block: the bricks that follow one
    // another along z are swept by the same SM, whose L1 still holds their shared rows
    const long long P = __ldg(g.np);
    const long long per = ((P + nbm - 1) / nbm + blockDim.x - 1) / blockDim.x * blockDim.x;
    const long long k0 = (long long)blockIdx.x * per, k1 = min(k0 + per, P);
    for (long long k = k0 + threadIdx.x; k < k1; k += blockDim.x) {
      const int e = __ldg(g.plist + k);
      const int i = e >= 0 ? e : ~e;
      float hmin;
      // z stride 1 (C order) as a constant: the z neighbours become immediate offsets
      const float r = reinit_rhs_at<false>(src, i, g, 0, e >= 0 ? 64u : 128u, sx, sy, 1, h, rh, h * h, rhh, hmin);
      sweep_update(src, dst, i, r, cfl * fmaxf(hmin, 1e-3f * h), second);
    }
    return;
  }
  const int X = __ldg(g.wx + g.W);
  const int stride = (gridDim.x - nbm) * blockDim.x;
  for (int k = (blockIdx.x - nbm) * blockDim.x + threadIdx.x; k < X; k += stride) {
    const int i = __ldg(g.xlist + k);
    const uint32_t flags = __ldg(g.xmeta + k);
    float hmin;
    const float r = reinit_rhs_at<true>(src, i, g, __ldg(g.xoff + k), flags, sx, sy, 1, h, rh, h * h, rhh, hmin);
    sweep_update(src, dst, i, r, cfl * fmaxf(hmin, 1e-3f * h), second);
  }
}

__global__ void k_reinit_rhs(const float* __restrict__ f, const int32_t* __restrict__ idx, long long m, int sx, int sy,
                             int sz, float h, float rh, float rhh, Geo g, float* out) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const bool act = t < m;
  const uint32_t flags = act ? g.meta[t] : 0u;
  const int off = dist_offset(g, t, flags);
  if (!act) return;
  float hmin;
  out[t] = reinit_rhs_at(f, idx[t], g, off, flags, sx, sy, sz, h, rh, h * h, rhh, hmin);
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

// ------------------------------------------------- bit-packed work mask
// The reinitialisation work mask as bits: rows (x, y) of nzw = ceil(nz / 32)
// words, bit z % 32 of word z / 32 (4.6 MB on the 448 x 336 x 245 grid
// instead of 37 MB of bytes).  The band is marked with atomicOr, then the
// box dilation runs as three separable word passes (z by shifts across the
// neighbouring words, then y and x as ORs of neighbouring rows), the last of
// which also clears the margin layers and the bits past nz.
__global__ void k_mark_bits(const int32_t* __restrict__ band, long long m, int nz, int nzw, uint32_t* bits) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= m) return;
  const int i = band[t];
  const int row = i / nz, z = i - row * nz;
  atomicOr(bits + (long long)row * nzw + (z >> 5), 1u << (z & 31));
}

__global__ void k_dilate_bits_z(const uint32_t* __restrict__ in, uint32_t* __restrict__ out, long long nwords,
                                int nzw, int r) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nwords) return;
  const int w = (int)(t % nzw);
  const uint32_t cur = in[t];
  const uint32_t prev = w > 0 ? in[t - 1] : 0u, next = w + 1 < nzw ? in[t + 1] : 0u;
  uint32_t acc = cur;
  for (int d = 1; d <= r; ++d) acc |= (cur << d) | (prev >> (32 - d)) | (cur >> d) | (next << (32 - d));
  out[t] = acc;
}

// axis 1: OR over rows y - r .. y + r; axis 0: over x - r .. x + r, then the
// margin and the bits past nz are cleared.
__global__ void k_dilate_bits_rows(const uint32_t* __restrict__ in, uint32_t* __restrict__ out, int nx, int ny,
                                   int nz, int nzw, int axis, int r, int margin) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long nwords = (long long)nx * ny * nzw;
  if (t >= nwords) return;
  const int w = (int)(t % nzw);
  const long long row = t / nzw;
  const int x = (int)(row / ny), y = (int)(row - (long long)x * ny);
  const int c = axis == 0 ? x : y, len = axis == 0 ? nx : ny;
  const long long step = axis == 0 ? (long long)ny * nzw : nzw;
  uint32_t acc = 0;
  const int lo = max(c - r, 0), hi = min(c + r, len - 1);
  for (int d = lo; d <= hi; ++d) acc |= in[t + (long long)(d - c) * step];
  if (axis == 0) {
    // valid z: margin <= z < nz - margin (margin 0: z < nz)
    if (x < margin || y < margin || x >= nx - margin || y >= ny - margin) acc = 0;
    const int zlo = margin - 32 * w, zhi = nz - margin - 32 * w;  // bit range [zlo, zhi)
    const uint32_t below = zlo <= 0 ? 0u : (zlo >= 32 ? 0xffffffffu : ((1u << zlo) - 1u));
    const uint32_t upto = zhi >= 32 ? 0xffffffffu : (zhi <= 0 ? 0u : ((1u << zhi) - 1u));
    acc &= upto & ~below;
  }
  out[t] = acc;
}

inline size_t geo_bytes(long long m) { return (size_t)geo_layout(m < 1 ? 1 : m).total; }

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

size_t svie_reinit_bits_bytes(int nx, int ny, int nz) {
  return (size_t)nx * ny * ((nz + 31) / 32) * sizeof(uint32_t);
}

int svie_reinit_bits(const int32_t* band, int64_t m, int nx, int ny, int nz, int dilation, int margin, uint32_t* bits,
                     uint32_t* tmp, uint32_t* marked, void* stream) {
  if (!bits || !tmp || nx <= 0 || ny <= 0 || nz <= 0 || (long long)nx * ny * nz >= (1LL << 31) || dilation < 0 ||
      dilation > 31 || margin < 0 || m < 0 || (m > 0 && !band)) {
    set_error("svie_reinit_bits: bad arguments (dilation <= 31)");
    return SVIE_ERR_ARG;
  }
  cudaStream_t s = (cudaStream_t)stream;
  const int nzw = (nz + 31) / 32;
  const long long nwords = (long long)nx * ny * nzw;
  // the band's own bits go to `marked` when given (kept for the caller), else to tmp
  uint32_t* mk = marked ? marked : tmp;
  if (cudaMemsetAsync(mk, 0, (size_t)nwords * sizeof(uint32_t), s) != cudaSuccess) {
    set_error("svie_reinit_bits: memset failed");
    return SVIE_ERR_LAUNCH;
  }
  int launches = 3;
  if (m > 0) {
    k_mark_bits<<<blocks_for(m, 256), 256, 0, s>>>(band, m, nz, nzw, mk);
    ++launches;
  }
  const int nb = blocks_for(nwords, 256);
  k_dilate_bits_z<<<nb, 256, 0, s>>>(mk, bits, nwords, nzw, dilation);
  k_dilate_bits_rows<<<nb, 256, 0, s>>>(bits, tmp, nx, ny, nz, nzw, 1, dilation, 0);
  k_dilate_bits_rows<<<nb, 256, 0, s>>>(tmp, bits, nx, ny, nz, nzw, 0, dilation, margin);
  return launch_status("svie_reinit_bits", launches);
}

size_t svie_reinit_geometry_bytes(int64_t m) { return geo_bytes(m); }

int svie_reinit_geometry(const float* phi, const int32_t* idx, int64_t m, int64_t sx, int64_t sy, int64_t sz,
                         float h, float cfl, void* geo, void* stream) {
  if (m < 0 || (m > 0 && (!phi || !idx || !geo)) || ((uintptr_t)geo & 15)) {
    set_error("svie_reinit_geometry: bad arguments (geo must be 16-byte aligned)");
    return SVIE_ERR_ARG;
  }
  if (m == 0) return SVIE_OK;
  cudaStream_t s = (cudaStream_t)stream;
  const GeoLayout L = geo_layout(m);
  const int nb = blocks_for(m, RI_THREADS);
  k_reinit_count<<<nb, RI_THREADS, 0, s>>>(phi, idx, m, sx, sy, sz, cfl, geo);
  char* b = (char*)geo;
  int ns = scan_exclusive_i32((int*)(b + L.wbase), L.W + 1, (int*)(b + L.sums), s);
  ns += scan_exclusive_i32((int*)(b + L.wx), L.W + 1, (int*)(b + L.sums), s);
  k_reinit_lists<<<nb, RI_THREADS, 0, s>>>(idx, m, geo);
  int dev = 0, nsm = 1;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  const int nd = (int)std::min<long long>((long long)nb, 8LL * nsm);
  k_reinit_dist<<<nd, RI_THREADS, 0, s>>>(phi, m, sx, sy, sz, h, cfl, geo);
  return launch_status("svie_reinit_geometry", 3 + ns);
}

int svie_reinit_iterate(float* phi, float* phi_tmp, int64_t n, const int32_t* idx, int64_t m, int64_t sx, int64_t sy,
                        int64_t sz, float h, const void* geo, int iterations, void* stream) {
  if (!phi || !phi_tmp || n <= 0 || m < 0 || iterations < 0 || sz != 1) {
    set_error("svie_reinit_iterate: bad arguments (C-order grid: sz == 1)");
    return SVIE_ERR_ARG;
  }
  if (m == 0 || iterations == 0) return SVIE_OK;
  cudaStream_t s = (cudaStream_t)stream;
  if (cudaMemcpyAsync(phi_tmp, phi, (size_t)n * sizeof(float), cudaMemcpyDeviceToDevice, s) != cudaSuccess) {
    set_error("svie_reinit_iterate: copy failed");
    return SVIE_ERR_LAUNCH;
  }
  const float rh = rn_reciprocal(h), rhh = rn_reciprocal(h * h);
  const Geo g = geo_view_host(const_cast<void*>(geo), m);
  int dev = 0, nsm = 1;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  // main blocks: one resident wave (8 per SM), each over a contiguous run of the list
  const int nb = (int)std::min<long long>((long long)blocks_for(m, RI_THREADS), 8LL * nsm);
  const int nbx = (int)std::min<long long>((long long)blocks_for(m, RI_THREADS), 8LL * nsm);
  // every half-step after the first is a dependent launch: its blocks are scheduled while the
  // previous half-step drains and wait in the kernel for its completion
  const dim3 grid(nb + nbx), block(RI_THREADS);
  cudaError_t e = cudaSuccess;
  for (int it = 0; it < iterations && e == cudaSuccess; ++it) {
    e = launch_dependent(it > 0, k_reinit_sweep, grid, block, 0, s, (const float*)phi, phi_tmp, (int)sx, (int)sy,
                         (int)sz, h, rh, rhh, g, 0, nb);
    if (e == cudaSuccess)
      e = launch_dependent(true, k_reinit_sweep, grid, block, 0, s, (const float*)phi_tmp, phi, (int)sx, (int)sy,
                           (int)sz, h, rh, rhh, g, 1, nb);
  }
  if (e != cudaSuccess) {
    set_error("svie_reinit_iterate: launch failed: %s", cudaGetErrorString(e));
    return SVIE_ERR_LAUNCH;
  }
  return launch_status("svie_reinit_iterate", 2 * iterations);
}

int svie_reinit_rhs(const float* phi, const int32_t* idx, int64_t m, int64_t sx, int64_t sy, int64_t sz, float h,
                    const void* geo, float* out, void* stream) {
  if (m <= 0) return m < 0 ? SVIE_ERR_ARG : SVIE_OK;
  k_reinit_rhs<<<blocks_for(m, RI_THREADS), RI_THREADS, 0, (cudaStream_t)stream>>>(
      phi, idx, m, sx, sy, sz, h, rn_reciprocal(h), rn_reciprocal(h * h), geo_view_host(const_cast<void*>(geo), m),
      out);
  return launch_status("svie_reinit_rhs");
}

int svie_reinit_geometry_arrays(const float* phi, const int32_t* idx, int64_t m, int64_t sx, int64_t sy, int64_t sz,
                                float h, float cfl, float* sgn, float* dtau, uint8_t* flags, float* dist6,
                                void* stream) {
  if (m < 0 || (m > 0 && (!phi || !idx || !sgn || !dtau || !flags || !dist6))) {
    set_error("svie_reinit_geometry_arrays: bad arguments");
    return SVIE_ERR_ARG;
  }
  if (m == 0) return SVIE_OK;
  k_reinit_geometry_full<<<blocks_for(m, 256), 256, 0, (cudaStream_t)stream>>>(phi, idx, m, sx, sy, sz, h, cfl,
                                                                             sgn, dtau, flags, dist6);
  return launch_status("svie_reinit_geometry_arrays");
}

int svie_reinit_geometry_pack(const float* sgn, const float* dtau, const uint8_t* flags, const float* dist6, int64_t m,
                              void* geo, void* stream) {
  if (m < 0 || (m > 0 && (!sgn || !flags || !dist6 || !geo)) || ((uintptr_t)geo & 15)) {
    set_error("svie_reinit_geometry_pack: bad arguments (geo must be 16-byte aligned)");
    return SVIE_ERR_ARG;
  }
  if (m == 0) return SVIE_OK;
  cudaStream_t s = (cudaStream_t)stream;
  const GeoLayout L = geo_layout(m);
  const int nb = blocks_for(m, 256);
  k_reinit_pack<<<nb, 256, 0, s>>>(sgn, flags, dist6, m, geo, 0);
  char* b = (char*)geo;
  int ns = scan_exclusive_i32((int*)(b + L.wbase), L.W + 1, (int*)(b + L.sums), s);
  ns += scan_exclusive_i32((int*)(b + L.wx), L.W + 1, (int*)(b + L.sums), s);
  k_reinit_pack<<<nb, 256, 0, s>>>(sgn, flags, dist6, m, geo, 1);
  return launch_status("svie_reinit_geometry_pack", 2 + ns);
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
