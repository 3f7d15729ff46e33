// Ball-convolution evaluation of N_r (reference svierosion/svi.py:24-93).
//
// The grid sizes are 2^a 3^b 5^c 7^d (Grid.around rounds up to them,
// svierosion/grid.py:18-28), so every axis FFT is a mixed-radix Stockham
// transform with radices 8, 7, 6, 5, 4, 3, 2 computed on lines staged in shared
// memory.  The 3-D real transform runs as five HBM passes over the complex64
// half spectrum S[x][y][kz] (kz = 0..nz/2, the rfftn layout):
//
//   1. z  R2C: two real lines packed into one complex line per FFT;
//   2. y  C2C forward on [ny x W] tiles of consecutive kz;
//   3. x  C2C forward, multiply by the real kernel spectrum K^, C2C inverse, all
//      while the lines are in shared memory;
//   4. y  C2C inverse;
//   5. z  C2R with the epilogue out = beta + alpha * value fused in.
//
// The ball weights w are even in each axis, so K^ is real and even in each
// frequency; it is computed once in float64 directly from w (three separable
// cosine sums) and stored for kx <= nx/2, ky <= ny/2, kz <= nz/2 only.
// Inverse transforms use conj(FFT(conj(x))).  All arithmetic is float32 with
// float64-accurate twiddle tables.
#include <math.h>
#include <string.h>

#include <cuda.h>  // CUtensorMap (the tensor-map encoder is reached through the runtime's driver entry point)

#include <map>
#include <mutex>

#include "common.cuh"
#include "fft_dev.cuh"
#include "fft_jit.h"

namespace svie {

// FFT_T, AxisPlan, the radix butterflies, the tile stages and the pass epilogues are in fft_dev.cuh,
// shared with the pass kernels compiled at run time for one axis length.

// Radix order: the largest odd radix first, then the even radices
// (descending), then the other odd ones.  With an odd first radix no stage of
// the 8-line tiles writes at an even stride from p = 1 (see tile_stage).
static bool factor_axis(int n, AxisPlan* p) {
  if (n < 1 || n > FFT_MAXN) return false;
  static const int rs[] = {8, 7, 6, 5, 4, 3, 2};
  int m = n, cnt = 0, fac[FFT_MAXST + 1];
  for (int r : rs) {
    while (m % r == 0) {
      if (cnt >= FFT_MAXST) return false;
      fac[cnt++] = r;
      m /= r;
    }
  }
  if (m != 1) return false;
  int order[FFT_MAXST], st = 0, first_odd = -1;
  for (int i = 0; i < cnt; ++i)
    if (fac[i] & 1) { first_odd = i; break; }
  if (first_odd >= 0) order[st++] = fac[first_odd];
  for (int i = 0; i < cnt; ++i)
    if (!(fac[i] & 1)) order[st++] = fac[i];
  for (int i = 0; i < cnt; ++i)
    if ((fac[i] & 1) && i != first_odd) order[st++] = fac[i];
  unsigned long long packed = 0, rpacked = 0;
  for (int i = 0; i < st; ++i) {
    packed |= (unsigned long long)order[i] << (4 * i);
    rpacked |= (unsigned long long)order[st - 1 - i] << (4 * i);
  }
  p->n = n;
  p->nst = st;
  p->radices = packed;
  p->rradices = rpacked;
  p->rstw = nullptr;
  return true;
}

// ------------------------------------------------ TMA tile loads (mbarrier)
// A tile of the 8-line passes is one box or a few boxes of a 3-D tensor map
// over the padded half spectrum (floats: 2 nzp x ny x nx), copied by the
// tensor memory accelerator into shared memory; one thread issues the copies
// and the CTA waits on an mbarrier for their bytes.  The wait is bounded:
// after TMA_WAIT_LIMIT polls the CTA records a timeout in g_tma_timeouts,
// polls once more as long for the copies in flight, and skips its tile.
__device__ unsigned int g_tma_timeouts = 0;
constexpr long long TMA_WAIT_LIMIT = 1LL << 22;

SVIE_DEV unsigned int smem_u32(const void* p) { return (unsigned int)__cvta_generic_to_shared(p); }
SVIE_DEV void mbar_init(uint64_t* bar, unsigned int count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
// the initialised barrier visible to the asynchronous proxy (the TMA unit)
SVIE_DEV void fence_barrier_init() { asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory"); }
SVIE_DEV void mbar_expect_tx(uint64_t* bar, unsigned int bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}
SVIE_DEV void tma_load_3d(void* dst, const CUtensorMap* map, int x, int y, int z, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
      "[%5];\n" ::"r"(smem_u32(dst)),
      "l"(map), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
      : "memory");
}
SVIE_DEV bool mbar_try_wait(uint64_t* bar, unsigned int phase) {
  unsigned int ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(phase)
      : "memory");
  return ok != 0;
}
// true when the phase completed within the limit
SVIE_DEV bool mbar_wait_bounded(uint64_t* bar, unsigned int phase) {
  for (long long i = 0; i < TMA_WAIT_LIMIT; ++i)
    if (mbar_try_wait(bar, phase)) return true;
  return false;
}

// ----------------------------------------------------------------- z passes
// The bodies are z_r2c_body / z_c2r_body in fft_dev.cuh.
template <int LW, int PS>
__global__ void __launch_bounds__(FFT_T) k_fft_z_r2c(const float* __restrict__ in, float2* __restrict__ out,
                                                     AxisPlan P, long long nlines, int nzp,
                                                     const uint8_t* __restrict__ lineflag) {
  pdl_wait();
  pdl_release();
  z_r2c_body<LW, PS>(in, out, P, nlines, nzp, lineflag, PlanStages<LW, PS>{P});
}

template <int LW, int PS>
__global__ void __launch_bounds__(FFT_T) k_fft_z_c2r(const float2* __restrict__ in, float* __restrict__ out,
                                                     AxisPlan P, long long nlines, int nzp, float alpha, float beta,
                                                     const uint8_t* __restrict__ lineflag) {
  pdl_wait();
  pdl_release();
  z_c2r_body<LW, PS>(in, out, P, nlines, nzp, alpha, beta, lineflag, PlanStages<LW, PS>{P});
}

// ------------------------------------------------------------ strided passes
// Lines along an axis with element stride `stride`; a CTA takes LW
// consecutive lines (LW = 8: one aligned 64-byte row segment of the padded
// spectrum) of one outer slab: base = data + blockIdx.y * outer_stride +
// blockIdx.x * LW.  The tile is stored like the spectrum (position-major,
// PS = LW), so thread t loads line t % LW of rows t / LW, + FFT_T / LW, ...
// mode 0 = forward, 1 = inverse, 2 = forward * K^ then inverse (x axis only;
// the outer index is y and the line index kz).

// Slab skipping: when `slabflag` is given, a CTA returns at once for an outer
// slab whose flag lacks `need` (bit 0: the forward data of the slab is zero,
// bit 1: no N value of the slab is read afterwards).
// MINB: CTAs per SM the register budget is sized for (the y passes fit four
// in shared memory, the x pass three).
template <int LW, int MINB>
__global__ void __launch_bounds__(FFT_T, MINB) k_fft_strided(float2* __restrict__ data, AxisPlan P, long long stride,
                                                       int ninner, long long outer_stride, int mode, KGeom K,
                                                       const uint8_t* __restrict__ slabflag, int need,
                                                       const __grid_constant__ CUtensorMap tmap, int tma_rows,
                                                       int tma_axis) {
  pdl_wait();
  pdl_release();
  if (slabflag && !(__ldg(slabflag + blockIdx.y) & need)) return;
  extern __shared__ __align__(128) float2 sm[];
  constexpr int KS = FFT_T / LW;  // rows per sweep of the CTA
  const int n = P.n;
  float2* sa = sm;
  float2* sb = sm + LW * n;
  const int c0 = blockIdx.x * LW;
  const int nl = min(LW, ninner - c0);
  float2* base = data + (long long)blockIdx.y * outer_stride + c0;
  // the whole tile in flight at once (LW = 8: whole 64-byte segments of the
  // padded rows, the columns past ninner included and never stored; LW = 1: one
  // value per row).  With a tensor map (tma_rows > 0, LW = 8) thread 0 issues
  // n / tma_rows TMA boxes of tma_rows rows into the tile (rows along tensor
  // dimension 1 for tma_axis 0, dimension 2 for tma_axis 1); otherwise every
  // thread issues cp.async copies.
  uint64_t* bar = reinterpret_cast<uint64_t*>(sm + (2 * LW + 2) * n);
  const bool tma = LW == 8 && tma_rows > 0;
  if (tma) {
    if (threadIdx.x == 0) {
      mbar_init(bar, 1);
      fence_barrier_init();
      mbar_expect_tx(bar, (unsigned int)n * LW * (unsigned int)sizeof(float2));
      for (int r0 = 0; r0 < n; r0 += tma_rows) {
        if (tma_axis == 0) tma_load_3d(sa + r0 * LW, &tmap, 2 * c0, r0, (int)blockIdx.y, bar);
        else tma_load_3d(sa + r0 * LW, &tmap, 2 * c0, (int)blockIdx.y, r0, bar);
      }
    }
  } else if (LW == 8) {
    for (int e = threadIdx.x; e < 4 * n; e += FFT_T) {
      const int row = e >> 2, part = 2 * (e & 3);
      cp_async16(sa + row * LW + part, base + row * stride + part);
    }
  } else {
    for (int row = threadIdx.x; row < n; row += FFT_T) cp_async8(sa + row, base + row * stride);
  }
  cp_async_commit();
  const float2* stw = stage_twiddles_to_smem(sm, LW, P);
  if (mode == 2)
    for (int e = threadIdx.x; e < n - 1; e += FFT_T) sm[2 * LW * n + n + e] = __ldg(P.rstw + e);
  const int c = threadIdx.x % LW, k0 = threadIdx.x / LW;
  const bool col = c < nl;
  const long long rstep = KS * stride;
  cp_async_wait<0>();
  if (tma) {
    __syncthreads();  // the barrier was initialised by thread 0 before any thread polls it
    // every thread observes the copies' completion itself; the CTA decides together
    if (!__syncthreads_and(mbar_wait_bounded(bar, 0))) {
      if (threadIdx.x == 0) atomicAdd(&g_tma_timeouts, 1u);
      mbar_wait_bounded(bar, 0);  // the copies in flight, once more within the limit
      return;
    }
  }
  __syncthreads();
  const int nst = P.nst;
  int p = 1;
  float2* r = run_stages<LW, LW, FFT_T>(sa, sb, n, P.radices, 0, nst - 1, stw, mode == 1, p);
  const int Rl = radix_of(P.radices, nst - 1);
  if (mode != 2) {
    run_last<LW, LW, FFT_T>(r, n, Rl, stw, mode == 1 && nst == 1, StoreEpi{base, stride, nl, mode != 0});
    return;
  }
  // forward, then K^ and the first inverse stage in one pass, then the rest
  // of the inverse in reverse radix order (its twiddles follow the forward's)
  const float2* rstw = stw + n;
  const int nyh = K.ny / 2 + 1;
  const int y = blockIdx.y, yr = min(y, K.ny - y);
  float2* o = (r == sa) ? sb : sa;
  run_last<LW, LW, FFT_T>(r, n, Rl, stw, false,
                          KEpi<LW>{o, K.kred + (long long)yr * K.nzh + c0, (long long)nyh * K.nzh, n, nl});
  __syncthreads();
  if (nst == 1) {  // that stage was the whole transform both ways
    if (col) {
      float2* g = base + (long long)k0 * stride + c;
      for (int k = k0; k < n; k += KS, g += rstep) {
        const float2 v = o[k * LW + c];
        *g = make_float2(v.x, -v.y);
      }
    }
    return;
  }
  int p2 = Rl;
  float2* r2 = run_stages<LW, LW, FFT_T>(o, r, n, P.rradices, 1, nst - 1, rstw, false, p2);
  run_last<LW, LW, FFT_T>(r2, n, radix_of(P.rradices, nst - 1), rstw, false, StoreEpi{base, stride, nl, true});
}

// Persistent form of the 8-line strided pass: each CTA walks the tiles
// t = blockIdx.x, + gridDim.x, ... (tile t: column block t % ncb of outer slab
// t / ncb) and copies the next tile into a third shared buffer with cp.async
// while it transforms the current one, so the loads of one tile overlap the
// butterflies of the previous.  The copies take whole 64-byte row segments:
// the spectrum rows are padded to multiples of 8 complex values (the columns
// past ninner are copied and transformed but never stored).  Modes 0 and 1
// and the slab skipping of k_fft_strided (the y passes); with KX also mode 2,
// the x pass with the K^ product fused (the reverse-order stage twiddles
// follow the forward ones in shared memory).  Every line goes through the
// same stage functions as in k_fft_strided, so both forms give the same bits.
template <int NT, int MINB, bool KX>
__global__ void __launch_bounds__(NT, MINB) k_fft_tiles(float2* __restrict__ data, AxisPlan P, long long stride,
                                                     int ninner, long long outer_stride, int nouter, int mode,
                                                     KGeom K, const uint8_t* __restrict__ slabflag, int need) {
  pdl_wait();
  pdl_release();
  constexpr int LW = 8;
  extern __shared__ __align__(16) float2 sm[];
  const int n = P.n, tile = LW * n, nst = P.nst;
  const int ncb = (ninner + LW - 1) / LW;
  const long long ntiles = (long long)ncb * nouter;
  float2* stw = sm + 3 * tile;
  for (int e = threadIdx.x; e < n - 1; e += NT) stw[e] = __ldg(P.stw + e);
  const float2* rstw = stw + n;
  if (KX && mode == 2)
    for (int e = threadIdx.x; e < n - 1; e += NT) stw[n + e] = __ldg(P.rstw + e);
  auto next = [&](long long t) {
    if (slabflag)
      while (t < ntiles && !(__ldg(slabflag + t / ncb) & need)) t += gridDim.x;
    return t;
  };
  auto issue = [&](long long t, float2* dst) {
    const long long outer = t / ncb;
    const float2* src = data + outer * outer_stride + (t - outer * ncb) * LW;
    for (int e = threadIdx.x; e < 4 * n; e += NT) {
      const int row = e >> 2, part = 2 * (e & 3);
      cp_async16(dst + row * LW + part, src + row * stride + part);
    }
  };
  float2* bi = sm;         // the tile being transformed
  float2* bq = sm + tile;  // its ping-pong partner
  float2* bf = sm + 2 * tile;  // the next tile, in flight
  long long t = next(blockIdx.x);
  if (t < ntiles) issue(t, bi);
  cp_async_commit();
  const int Rl = radix_of(P.radices, nst - 1);
  while (t < ntiles) {
    const long long tn = next(t + gridDim.x);
    if (tn < ntiles) issue(tn, bf);
    cp_async_commit();
    cp_async_wait<1>();  // every group but the newest (the prefetch) has landed
    __syncthreads();
    const long long outer = t / ncb;
    const int c0 = (int)(t - outer * ncb) * LW;
    const int nl = min(LW, ninner - c0);
    float2* base = data + outer * outer_stride + c0;
    int p = 1;
    float2* r = run_stages<LW, LW, NT>(bi, bq, n, P.radices, 0, nst - 1, stw, mode == 1, p);
    if (!KX || mode != 2) {
      run_last<LW, LW, NT>(r, n, Rl, stw, mode == 1 && nst == 1, StoreEpi{base, stride, nl, mode == 1});
    } else {
      // forward, K^ and the first inverse stage, then the rest of the inverse (as k_fft_strided)
      const int y = (int)outer, yr = min(y, K.ny - y);
      float2* o = (r == bi) ? bq : bi;
      run_last<LW, LW, NT>(r, n, Rl, stw, false,
                           KEpi<LW>{o, K.kred + (long long)yr * K.nzh + c0, (long long)(K.ny / 2 + 1) * K.nzh, n,
                                    nl});
      __syncthreads();
      if (nst == 1) {
        for (int e = threadIdx.x; e < tile; e += NT) {
          const int k = e / LW, c = e % LW;
          if (c < nl) {
            const float2 v = o[e];
            base[(long long)k * stride + c] = make_float2(v.x, -v.y);
          }
        }
      } else {
        int p2 = Rl;
        float2* r2 = run_stages<LW, LW, NT>(o, r, n, P.rradices, 1, nst - 1, rstw, false, p2);
        run_last<LW, LW, NT>(r2, n, radix_of(P.rradices, nst - 1), rstw, false, StoreEpi{base, stride, nl, true});
      }
    }
    __syncthreads();  // bi and bq are free: the next tile is bf, the one after goes to bq
    float2* tmp = bi;
    bi = bf;
    bf = bq;
    bq = tmp;
    t = tn;
  }
  cp_async_wait<0>();
}

// ------------------------------------------------------ plan construction
__global__ void k_twiddles(float2* tw, int n) {
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  double s, c;
  sincospi(2.0 * (double)k / (double)n, &s, &c);
  tw[k] = make_float2((float)c, (float)(-s));
}

// Stage twiddle table from the axis table: entry p - 1 + k (R - 1) + (q - 1)
// of the stage with span p and radix R is tw[q k n / (p R)] (k < p, 1 <= q < R).
__global__ void k_stage_twiddles(AxisPlan P, float2* stw) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= P.n - 1) return;
  int p = 1;
  for (int st = 0; st < P.nst; ++st) {
    const int R = (int)((P.radices >> (4 * st)) & 15ULL);
    if (e < p * R - 1) {
      const int r = e - (p - 1), k = r / (R - 1), q = r % (R - 1) + 1;
      stw[e] = P.tw[q * k * (P.n / (p * R))];
      return;
    }
    p *= R;
  }
}

struct GL32 {
  double x[64], w[64];
};

// Ball/cell overlap fractions (reference svi.py:24-55) in float64, one block
// per (x, y) column of cells.  Cells entirely inside the ball weigh 1, cells
// outside 0; for a cut cell the z-extent of the ball is integrated exactly and
// the (x, y) integral by quad x quad Gauss-Legendre points.  The half-height
// zr(X, Y) of the ball at a quadrature point is the same for every cell of the
// column, so the block computes the quad^2 square roots once (shared memory)
// and reuses them for each cut cell; the cell's sum is a block reduction.
__global__ void __launch_bounds__(256) k_ball_weights(double R, int m, int quad, GL32 gl, double* __restrict__ w) {
  extern __shared__ double zr[];  // quad * quad square roots, then one class byte per cell of the column
  __shared__ double gx[64], gw[64], red[8];
  const int side = 2 * m + 1;
  const int q2 = quad * quad;
  unsigned char* cls = reinterpret_cast<unsigned char*>(zr + q2);
  const int i = (int)(blockIdx.x / side) - m, j = (int)(blockIdx.x % side) - m;
  const double ci = i, cj = j;
  double* col = w + ((long long)(i + m) * side + (j + m)) * side;
  if (threadIdx.x < quad) {
    gx[threadIdx.x] = gl.x[threadIdx.x];
    gw[threadIdx.x] = gl.w[threadIdx.x];
  }
  // each cell of the column classified once: 1 inside, 0 outside, 2 cut
  auto nr = [](double c) { const double v = fabs(c) - 0.5; return v > 0 ? v : 0.0; };
  const double a0 = nr(ci), a1 = nr(cj), b0 = fabs(ci) + 0.5, b1 = fabs(cj) + 0.5;
  bool any_cut = false;
  for (int kk = threadIdx.x; kk < side; kk += blockDim.x) {
    const double ck = kk - m;
    const double a2 = nr(ck), b2 = fabs(ck) + 0.5;
    const double near = sqrt(a0 * a0 + a1 * a1 + a2 * a2);  // squares of half-integers: exact sums
    const double far = sqrt(b0 * b0 + b1 * b1 + b2 * b2);
    const unsigned char c = far <= R ? 1 : ((near < R && far > R) ? 2 : 0);
    cls[kk] = c;
    if (c != 2) col[kk] = c == 1 ? 1.0 : 0.0;
    any_cut |= c == 2;
  }
  if (!__syncthreads_or(any_cut)) return;
  for (int p = threadIdx.x; p < q2; p += blockDim.x) {
    const double X = ci + gx[p / quad], Y = cj + gx[p % quad];
    const double r2 = R * R - X * X - Y * Y;
    zr[p] = sqrt(r2 > 0 ? r2 : 0.0);
  }
  __syncthreads();
  for (int kk = 0; kk < side; ++kk) {
    if (cls[kk] != 2) continue;
    const double ck = kk - m;
    const double lo = ck - 0.5, hi = ck + 0.5;
    double acc = 0.0;
    for (int p = threadIdx.x; p < q2; p += blockDim.x) {
      const double z = zr[p];
      double L = fmin(hi, z) - fmax(lo, -z);
      if (L < 0) L = 0;
      acc += L * gw[p / quad] * gw[p % quad];
    }
    for (int o = 16; o; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
      double t = 0.0;
      for (int k = 0; k < (int)(blockDim.x >> 5); ++k) t += red[k];
      col[kk] = t;
    }
    __syncthreads();
  }
}

// K^ step A: A[(i,j)][kz] = sum_k w[i][j][k] cos(2 pi kz k / nz), i, j in [-m, m].
__global__ void k_khat_a(const double* __restrict__ w, int m, int nz, int nzh, double* __restrict__ A) {
  extern __shared__ double ctab[];
  for (int t = threadIdx.x; t < nz; t += blockDim.x) ctab[t] = cospi(2.0 * t / nz);
  __syncthreads();
  const int side = 2 * m + 1;
  const long long tot = (long long)side * side * nzh;
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < tot; t += (long long)gridDim.x * blockDim.x) {
    const long long ij = t / nzh;
    const int kz = (int)(t - ij * nzh);
    const double* row = w + ij * side;
    double acc = 0.0;
    // phase (kz k) mod nz, stepped by kz from k = -m (no division in the loop)
    int ph = (int)(((long long)kz * (nz - m % nz)) % nz);
    for (int k = -m; k <= m; ++k) {
      acc += row[k + m] * ctab[ph];
      ph += kz;
      if (ph >= nz) ph -= nz;
    }
    A[t] = acc;
  }
}

// step B: Bq[i][ky][kz] = sum_j A[i][j][kz] cos(2 pi ky j / ny), ky <= ny/2.
__global__ void k_khat_b(const double* __restrict__ A, int m, int ny, int nzh, double* __restrict__ Bq) {
  extern __shared__ double ctab[];
  for (int t = threadIdx.x; t < ny; t += blockDim.x) ctab[t] = cospi(2.0 * t / ny);
  __syncthreads();
  const int side = 2 * m + 1, nyh = ny / 2 + 1;
  const long long tot = (long long)side * nyh * nzh;
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < tot; t += (long long)gridDim.x * blockDim.x) {
    const int kz = (int)(t % nzh);
    const int ky = (int)((t / nzh) % nyh);
    const int i = (int)(t / ((long long)nzh * nyh));
    double acc = 0.0;
    int ph = (int)(((long long)ky * (ny - m % ny)) % ny);
    for (int j = -m; j <= m; ++j) {
      acc += A[((long long)i * side + (j + m)) * nzh + kz] * ctab[ph];
      ph += ky;
      if (ph >= ny) ph -= ny;
    }
    Bq[t] = acc;
  }
}

// step C: K[kx][ky][kz] = sum_i Bq[i][ky][kz] cos(2 pi kx i / nx), kx <= nx/2 -> float.
__global__ void k_khat_c(const double* __restrict__ Bq, int m, int nx, int ny, int nzh, float* __restrict__ K) {
  extern __shared__ double ctab[];
  for (int t = threadIdx.x; t < nx; t += blockDim.x) ctab[t] = cospi(2.0 * t / nx);
  __syncthreads();
  const int nxh = nx / 2 + 1, nyh = ny / 2 + 1;
  const long long plane = (long long)nyh * nzh;
  const long long tot = (long long)nxh * plane;
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < tot; t += (long long)gridDim.x * blockDim.x) {
    const int kx = (int)(t / plane);
    const long long r = t - (long long)kx * plane;
    double acc = 0.0;
    int ph = (int)(((long long)kx * (nx - m % nx)) % nx);
    for (int i = -m; i <= m; ++i) {
      acc += Bq[(long long)(i + m) * plane + r] * ctab[ph];
      ph += kx;
      if (ph >= nx) ph -= nx;
    }
    K[t] = (float)acc;
  }
}

// Line flags for the masked convolution: bit 0 on (x, y) lines holding band
// nodes (all solid lines: the padding keeps the grid boundary outside), then
// bit 1 on those lines dilated by `dil` lines in x and y (every tricubic
// stencil at a closest point of a band node).
__global__ void k_mark_lines(const int32_t* __restrict__ band, long long m, int nz, uint8_t* flags) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < m) flags[band[t] / nz] = 1;
}

// tmp[x, y] = any band line within dil lines along x.
__global__ void k_dilate_lines_x(const uint8_t* __restrict__ flags, uint8_t* __restrict__ tmp, int nx, int ny,
                                 int dil) {
  const int y = blockIdx.x * blockDim.x + threadIdx.x, x = blockIdx.y;
  if (y >= ny) return;
  uint8_t v = 0;
  for (int d = max(x - dil, 0); d <= min(x + dil, nx - 1) && !v; ++d) v = flags[d * ny + y] & 1;
  tmp[x * ny + y] = v;
}

// flags[x, y] |= 2 if tmp has a line within dil lines along y (bit 0 kept).
__global__ void k_dilate_lines_y(const uint8_t* __restrict__ tmp, uint8_t* __restrict__ flags, int nx, int ny,
                                 int dil) {
  const int y = blockIdx.x * blockDim.x + threadIdx.x, x = blockIdx.y;
  if (y >= ny) return;
  uint8_t v = 0;
  for (int d = max(y - dil, 0); d <= min(y + dil, ny - 1) && !v; ++d) v = tmp[x * ny + d];
  if (v) flags[x * ny + y] |= 2;
}

__global__ void k_slab_flags(const uint8_t* __restrict__ lines, int nx, int ny, uint8_t* slabs) {
  const int x = blockIdx.x;
  uint8_t v = 0;
  for (int y = threadIdx.x; y < ny; y += blockDim.x) v |= lines[x * ny + y];
  // OR-reduce the two flag bits across the CTA
  const int b0 = __syncthreads_or(v & 1), b1 = __syncthreads_or(v & 2);
  if (threadIdx.x == 0) slabs[x] = (uint8_t)((b0 ? 1 : 0) | (b1 ? 2 : 0));
}

// Full complex64 half spectrum from the reduced real one.
__global__ void k_khat_expand(const float* __restrict__ K, int nx, int ny, int nzh, float2* __restrict__ out) {
  const long long tot = (long long)nx * ny * nzh;
  const int nyh = ny / 2 + 1;
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < tot; t += (long long)gridDim.x * blockDim.x) {
    const int kz = (int)(t % nzh);
    const int y = (int)((t / nzh) % ny);
    const int x = (int)(t / ((long long)nzh * ny));
    const int xr = min(x, nx - x), yr = min(y, ny - y);
    out[t] = make_float2(K[((long long)xr * nyh + yr) * nzh + kz], 0.0f);
  }
}

// ------------------------------------------------------------ plan layout
inline size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }

struct PlanLayout {
  size_t tw_x, tw_y, tw_z, stw_x, stw_y, stw_z, rstw_x, kred, total;
};

static PlanLayout plan_layout(int nx, int ny, int nz) {
  PlanLayout L;
  size_t off = 0;
  L.tw_x = off; off += align256((size_t)nx * sizeof(float2));
  L.tw_y = off; off += align256((size_t)ny * sizeof(float2));
  L.tw_z = off; off += align256((size_t)nz * sizeof(float2));
  L.stw_x = off; off += align256((size_t)nx * sizeof(float2));
  L.stw_y = off; off += align256((size_t)ny * sizeof(float2));
  L.stw_z = off; off += align256((size_t)nz * sizeof(float2));
  L.rstw_x = off; off += align256((size_t)nx * sizeof(float2));
  L.kred = off; off += align256((size_t)(nx / 2 + 1) * (ny / 2 + 1) * (nz / 2 + 1) * sizeof(float));
  L.total = off;
  return L;
}

// Tile shapes: z passes 16 complex lines (PS = 17) and strided passes 8 lines
// when the two buffers and the twiddles fit in shared memory, else one line
// per tile (axes longer than about 830 for z and 1700 for x and y).
// ------------------------------------------------- pass variants and choice
// Each axis pass has a few launch forms that differ in how lines are grouped
// into CTAs (lines per tile, CTAs per SM, persistent or one tile per CTA).
// Every line goes through the same radix stages with the same twiddles.  The
// forms of one code family give the same bits: the z forms; the 8-line forms
// of y and x (0 and 1); the one-line forms of y and x (2), which are compiled
// apart from the 8-line ones and so may differ from them in the last bit
// wherever the compiler fuses a multiply and an add differently.  The tuner
// only chooses within the family the fixed rule picks for the shape, so that
// results never depend on a timing:
//   z: 0 = 16 line pairs per CTA (3 CTAs/SM at nz ~ 250), 1 = 8 pairs,
//      2 = one pair (axes too long for the others);
//   y: 0 = persistent 8-line tiles with the next tile prefetched, 1 = one
//      8-line tile per CTA, 2 = one line per CTA;
//   x: 0 = one 8-line tile per CTA, 1 = persistent 8-line tiles, 2 = one line.
// The fixed rule takes z 0, y 1 and x 0 where they fit: the fastest forms on
// every grid from 100 x 75 x 60 to 448 x 336 x 245 that was timed on a GB300
// (the persistent forms lose there: y by 3-10%, x by 3-12%).  The radix order
// is not a choice: it changes the rounding, and results must not depend on a
// timing.
constexpr int FFT_NCHOICE = 3;

static size_t z_smem(int c, int n) { return tile_smem(c == 0 ? 17 : (c == 1 ? 9 : 1), n); }
// the strided passes also hold the reverse-order twiddles of the fused x pass
// (and the mbarrier of the TMA tile load)
static size_t strided_smem(int lw, int n) { return tile_smem(lw, n) + (size_t)n * sizeof(float2) + 16; }
// the persistent passes hold three tiles and the twiddles (the x pass both orders)
static size_t tiles_smem(int n, bool kx) { return (3 * 8 + (kx ? 2 : 1)) * (size_t)n * sizeof(float2); }
static size_t y_smem(int c, int n) { return c == 0 ? tiles_smem(n, false) : strided_smem(c == 1 ? 8 : 1, n); }
static size_t x_smem(int c, int n) { return c == 1 ? tiles_smem(n, true) : strided_smem(c == 0 ? 8 : 1, n); }
static bool fits(size_t b) { return b <= TILE_SMEM_MAX; }

struct FftChoice {
  int z, y, x;
  int jit = 0;   // the 8-line y and x forms run as passes compiled for the axis lengths (svie_conv_jit)
  int kept = 0;  // the forms were tuned or set (svie_conv_tune, svie_conv_set_choice)
};

// the fixed rule (above)
static FftChoice default_choice(int nx, int ny, int nz) {
  FftChoice c;
  c.z = fits(z_smem(0, nz)) ? 0 : 2;
  c.y = fits(y_smem(1, ny)) ? 1 : 2;
  c.x = fits(x_smem(0, nx)) ? 0 : 2;
  return c;
}

// Forms the tuner may choose for an axis: those that fit and share the fixed
// rule's code family (the one-line y and x forms only where no 8-line form fits).
static bool tunable_z(int c, int nz) { return fits(z_smem(c, nz)); }
static bool tunable_y(int c, int ny) { return fits(y_smem(c, ny)) && (c < 2) == fits(y_smem(1, ny)); }
static bool tunable_x(int c, int nx) { return fits(x_smem(c, nx)) && (c < 2) == fits(x_smem(0, nx)); }

static bool choice_fits(const FftChoice& c, int nx, int ny, int nz) {
  return c.z >= 0 && c.z < FFT_NCHOICE && c.y >= 0 && c.y < FFT_NCHOICE && c.x >= 0 && c.x < FFT_NCHOICE &&
         fits(z_smem(c.z, nz)) && fits(y_smem(c.y, ny)) && fits(x_smem(c.x, nx));
}

// Chosen forms per (device, grid shape): set by svie_conv_tune or svie_conv_set_choice.
struct GridKey {
  int dev, nx, ny, nz;
  bool operator<(const GridKey& o) const {
    if (dev != o.dev) return dev < o.dev;
    if (nx != o.nx) return nx < o.nx;
    if (ny != o.ny) return ny < o.ny;
    return nz < o.nz;
  }
};
static std::mutex g_choice_mu;
static std::map<GridKey, FftChoice> g_choice;

static GridKey grid_key(int nx, int ny, int nz) {
  int dev = 0;
  cudaGetDevice(&dev);
  return GridKey{dev, nx, ny, nz};
}

static FftChoice choice_for(int nx, int ny, int nz, bool* tuned = nullptr) {
  const GridKey k = grid_key(nx, ny, nz);
  std::lock_guard<std::mutex> lock(g_choice_mu);
  auto it = g_choice.find(k);
  if (tuned) *tuned = it != g_choice.end() && it->second.kept;
  return it != g_choice.end() ? it->second : default_choice(nx, ny, nz);
}

// Grid of a persistent kernel: as many CTAs as are resident at once, at most one per tile.
static unsigned persistent_grid(const void* fn, int threads, size_t smem, long long ntiles) {
  int dev = 0, nsm = 1, per = 1;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, fn, threads, smem) != cudaSuccess || per < 1) per = 1;
  const long long g = (long long)per * nsm;
  return (unsigned)(ntiles < g ? ntiles : g);
}

static int ensure_smem_attr() {
  static unsigned long long done = 0;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return SVIE_ERR_LAUNCH;
  if (dev < 64 && (done >> dev) & 1ULL) return SVIE_OK;
  const int bytes = 227 * 1024;
  const void* fns[] = {(const void*)k_fft_z_r2c<16, 17>, (const void*)k_fft_z_r2c<8, 9>,
                       (const void*)k_fft_z_r2c<1, 1>,   (const void*)k_fft_z_c2r<16, 17>,
                       (const void*)k_fft_z_c2r<8, 9>,   (const void*)k_fft_z_c2r<1, 1>,
                       (const void*)k_fft_strided<8, 4>, (const void*)k_fft_strided<8, 3>,
                       (const void*)k_fft_strided<1, 1>, (const void*)k_fft_tiles<256, 3, false>,
                       (const void*)k_fft_tiles<256, 2, true>};
  cudaError_t e1 = cudaSuccess;
  for (const void* f : fns)
    if (e1 == cudaSuccess) e1 = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  if (e1 != cudaSuccess) {
    set_error("fft: cudaFuncSetAttribute failed");
    return SVIE_ERR_LAUNCH;
  }
  if (dev < 64) done |= 1ULL << dev;
  return SVIE_OK;
}

struct Plans {
  AxisPlan x, y, z;
  const float* kred;
};

static int make_plans(const void* plan, int nx, int ny, int nz, Plans* P) {
  if (!plan) {
    set_error("fft: null plan");
    return SVIE_ERR_ARG;
  }
  PlanLayout L = plan_layout(nx, ny, nz);
  const char* b = (const char*)plan;
  if (!factor_axis(nx, &P->x) || !factor_axis(ny, &P->y) || !factor_axis(nz, &P->z)) {
    set_error("fft: axis sizes %d x %d x %d must be 2^a 3^b 5^c 7^d and <= %d", nx, ny, nz, FFT_MAXN);
    return SVIE_ERR_UNSUPPORTED;
  }
  P->x.tw = (const float2*)(b + L.tw_x);
  P->y.tw = (const float2*)(b + L.tw_y);
  P->z.tw = (const float2*)(b + L.tw_z);
  P->x.stw = (const float2*)(b + L.stw_x);
  P->y.stw = (const float2*)(b + L.stw_y);
  P->z.stw = (const float2*)(b + L.stw_z);
  P->x.rstw = (const float2*)(b + L.rstw_x);
  P->kred = (const float*)(b + L.kred);
  return SVIE_OK;
}

// ------------------------------------------------------ TMA tensor maps
typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static EncodeTiledFn encode_tiled() {
  static std::once_flag once;
  static EncodeTiledFn fn = nullptr;
  std::call_once(once, [] {
    const char* v = getenv("SVIE_TMA");
    if (v && v[0] == '0') return;
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = (EncodeTiledFn)f;
  });
  return fn;
}

// Rows per TMA box for an axis of n positions: the largest even divisor of n
// up to 256 (a box dimension is at most 256, and an even row count keeps every
// box's shared-memory address a multiple of 128 bytes); 0 when n is odd.
static int tma_box_rows(int n) {
  if (n & 1) return 0;
  for (int r = 256; r >= 2; r -= 2)
    if (n % r == 0) return r;
  return 0;
}

// Tensor map over the padded half spectrum as floats (2 nzp, ny, nx), boxes of
// 16 floats (8 complex columns) by `rows` positions along y (axis 0) or x
// (axis 1).  Returns the rows per box, or 0 when no map could be made (then
// the pass loads its tiles with cp.async).
static int spectrum_map(CUtensorMap* map, float2* spec, int nx, int ny, int nzp, int n, int axis) {
  memset(map, 0, sizeof(*map));
  const int rows = tma_box_rows(n);
  EncodeTiledFn fn = encode_tiled();
  if (!fn || rows == 0 || ((uintptr_t)spec & 15)) return 0;
  const cuuint64_t dims[3] = {(cuuint64_t)2 * nzp, (cuuint64_t)ny, (cuuint64_t)nx};
  const cuuint64_t strides[2] = {(cuuint64_t)nzp * sizeof(float2), (cuuint64_t)ny * nzp * sizeof(float2)};
  const cuuint32_t box[3] = {16, axis == 0 ? (cuuint32_t)rows : 1u, axis == 0 ? 1u : (cuuint32_t)rows};
  const cuuint32_t estr[3] = {1, 1, 1};
  const CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, spec, dims, strides, box, estr,
                        CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                        CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? rows : 0;
}

template <int LW, int PS>
static void launch_z_as(const Plans& P, long long nlines, int nzp, const float* f, float2* spec, float* out,
                        bool fwd, float alpha, float beta, cudaStream_t s, const uint8_t* lineflag, bool chained) {
  const size_t smem = tile_smem(PS, P.z.n);
  const dim3 grid((unsigned)((nlines + 2 * LW - 1) / (2 * LW))), block(FFT_T);
  // a failed launch is reported by the caller's launch_status (cudaGetLastError)
  if (fwd) launch_dependent(chained, k_fft_z_r2c<LW, PS>, grid, block, smem, s, f, spec, P.z, nlines, nzp, lineflag);
  else launch_dependent(chained, k_fft_z_c2r<LW, PS>, grid, block, smem, s, (const float2*)spec, out, P.z, nlines, nzp,
                        alpha, beta, lineflag);
}

static void launch_z(const Plans& P, int nx, int ny, int nz, const float* f, float2* spec, float* out, bool fwd,
                     float alpha, float beta, cudaStream_t s, const uint8_t* lineflag, int c, bool chained,
                     bool jit = false) {
  const long long nlines = (long long)nx * ny;
  const int nzp = padded_nzh(nz);
  CUfunction r2c = nullptr, c2r = nullptr;
  if (c == 0 && jit && jit_z(nz, P.z.radices, P.z.nst, &r2c, &c2r) == SVIE_OK) {
    const dim3 grid((unsigned)((nlines + 31) / 32)), block(FFT_T);
    AxisPlan az = P.z;
    long long nl = nlines;
    int nzp_ = nzp;
    float a = alpha, b = beta;
    const float* fin = f;
    const float2* spec_in = spec;
    void* fargs[] = {&fin, &spec, &az, &nl, &nzp_, &lineflag};
    void* iargs[] = {&spec_in, &out, &az, &nl, &nzp_, &a, &b, &lineflag};
    if (jit_launch(fwd ? r2c : c2r, grid, block, tile_smem(17, nz), s, chained, fwd ? fargs : iargs)) return;
  }
  if (c == 0) launch_z_as<16, 17>(P, nlines, nzp, f, spec, out, fwd, alpha, beta, s, lineflag, chained);
  else if (c == 1) launch_z_as<8, 9>(P, nlines, nzp, f, spec, out, fwd, alpha, beta, s, lineflag, chained);
  else launch_z_as<1, 1>(P, nlines, nzp, f, spec, out, fwd, alpha, beta, s, lineflag, chained);
}

// y lines: outer index x, line index kz, element stride nzp.
static void launch_y(const Plans& P, int nx, int ny, int nz, float2* spec, int mode, cudaStream_t s,
                     const uint8_t* slabflag, int c, bool chained, bool jit = false) {
  const int nzh = nz / 2 + 1, nzp = padded_nzh(nz);
  const KGeom K{nullptr, ny, nzh};
  const int need = mode == 1 ? 2 : 1;
  const long long ostr = (long long)ny * nzp;
  const size_t smem = y_smem(c, ny);
  if (c == 0) {
    const long long ntiles = (long long)((nzh + 7) / 8) * nx;
    const void* fn = (const void*)k_fft_tiles<256, 3, false>;
    launch_dependent(chained, k_fft_tiles<256, 3, false>, dim3(persistent_grid(fn, 256, smem, ntiles)), dim3(256), smem, s,
                     spec, P.y, (long long)nzp, nzh, ostr, nx, mode, K, slabflag, need);
  } else if (c == 1) {
    const dim3 g((unsigned)((nzh + 7) / 8), (unsigned)nx);
    CUfunction jf = nullptr;
    if (jit && jit_strided(ny, JIT_Y_MINB, P.y.radices, P.y.nst, &jf) == SVIE_OK) {
      long long stride = nzp, ostr_ = ostr;
      int ninner = nzh, mode_ = mode, need_ = need;
      AxisPlan ax = P.y;
      KGeom kg = K;
      void* args[] = {&spec, &ax, &stride, &ninner, &ostr_, &mode_, &kg, &slabflag, &need_};
      // the two tile buffers only: this pass reads its stage twiddles from the plan
      const size_t jsmem = 2 * 8 * (size_t)ny * sizeof(float2);
      if (jit_launch(jf, g, dim3(FFT_T), jsmem, s, chained, args)) return;
    }
    CUtensorMap map;
    const int rows = spectrum_map(&map, spec, nx, ny, nzp, ny, 0);
    launch_dependent(chained, k_fft_strided<8, 4>, g, dim3(FFT_T), smem, s, spec, P.y, (long long)nzp, nzh, ostr, mode, K,
                     slabflag, need, map, rows, 0);
  } else {
    const dim3 g((unsigned)nzh, (unsigned)nx);
    CUtensorMap none;
    memset(&none, 0, sizeof(none));
    launch_dependent(chained, k_fft_strided<1, 1>, g, dim3(FFT_T), smem, s, spec, P.y, (long long)nzp, nzh, ostr, mode, K,
                     slabflag, need, none, 0, 0);
  }
}

// x lines: outer index y, line index kz, element stride ny * nzp.
static void launch_x(const Plans& P, int nx, int ny, int nz, float2* spec, int mode, cudaStream_t s, int c,
                     bool chained, bool jit = false) {
  const int nzh = nz / 2 + 1, nzp = padded_nzh(nz);
  const KGeom K{P.kred, ny, nzh};
  const long long lstr = (long long)ny * nzp;
  const size_t smem = x_smem(c, nx);
  const uint8_t* none = nullptr;
  if (c == 1) {
    const long long ntiles = (long long)((nzh + 7) / 8) * ny;
    const void* fn = (const void*)k_fft_tiles<256, 2, true>;
    launch_dependent(chained, k_fft_tiles<256, 2, true>, dim3(persistent_grid(fn, 256, smem, ntiles)), dim3(256), smem, s,
                     spec, P.x, lstr, nzh, (long long)nzp, ny, mode, K, none, 0);
  } else if (c == 0) {
    const dim3 g((unsigned)((nzh + 7) / 8), (unsigned)ny);
    CUfunction jf = nullptr;
    if (jit && jit_strided(nx, JIT_X_MINB, P.x.radices, P.x.nst, &jf) == SVIE_OK) {
      long long stride = lstr, ostr_ = nzp;
      int ninner = nzh, mode_ = mode, need_ = 0;
      AxisPlan ax = P.x;
      KGeom kg = K;
      void* args[] = {&spec, &ax, &stride, &ninner, &ostr_, &mode_, &kg, &none, &need_};
      if (jit_launch(jf, g, dim3(FFT_T), smem, s, chained, args)) return;
    }
    CUtensorMap map;
    const int rows = spectrum_map(&map, spec, nx, ny, nzp, nx, 1);
    launch_dependent(chained, k_fft_strided<8, 3>, g, dim3(FFT_T), smem, s, spec, P.x, lstr, nzh, (long long)nzp, mode, K, none,
                     0, map, rows, 1);
  } else {
    const dim3 g((unsigned)nzh, (unsigned)ny);
    CUtensorMap zero;
    memset(&zero, 0, sizeof(zero));
    launch_dependent(chained, k_fft_strided<1, 1>, g, dim3(FFT_T), smem, s, spec, P.x, lstr, nzh, (long long)nzp, mode, K, none,
                     0, zero, 0, 0);
  }
}

// Times one pass form: `reps` launches of `fn` after one untimed launch, the
// shortest kept (ms; a negative value when a launch failed).
template <class F>
static float time_form(F fn, int reps, cudaStream_t s, cudaEvent_t e0, cudaEvent_t e1) {
  fn();
  float best = -1.0f;
  for (int r = 0; r < reps; ++r) {
    cudaEventRecord(e0, s);
    fn();
    cudaEventRecord(e1, s);
    if (cudaEventSynchronize(e1) != cudaSuccess) return -1.0f;
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (best < 0.0f || ms < best) best = ms;
  }
  return cudaGetLastError() == cudaSuccess ? best : -1.0f;
}

static void gauss_legendre(int n, double* x, double* w) {
  // Newton iteration on the Legendre polynomial P_n from the Chebyshev-like
  // initial guesses cos(pi (i - 1/4) / (n + 1/2)); nodes returned ascending,
  // scaled to [-1/2, 1/2] with weights summing to 1.
  for (int i = 0; i < n; ++i) {
    double z = cos(M_PI * (i + 0.75) / (n + 0.5)), pp = 1.0;
    for (int it = 0; it < 100; ++it) {
      double p1 = 1.0, p2 = 0.0;
      for (int j = 1; j <= n; ++j) {
        double p3 = p2;
        p2 = p1;
        p1 = ((2.0 * j - 1.0) * z * p2 - (j - 1.0) * p3) / j;
      }
      pp = n * (z * p1 - p2) / (z * z - 1.0);
      double z1 = z;
      z = z1 - p1 / pp;
      if (fabs(z - z1) < 1e-16) break;
    }
    x[n - 1 - i] = 0.5 * z;
    w[n - 1 - i] = 0.5 * 2.0 / ((1.0 - z * z) * pp * pp);
  }
}

}  // namespace svie

using namespace svie;

extern "C" {

int svie_ball_half_width(double radius, double spacing) {
  if (!(radius > 0) || !(spacing > 0)) return -1;
  double R = radius / spacing;
  return (int)floor(R + 0.5) + 1;
}

int svie_ball_weights(double radius, double spacing, int quad, double* w, void* stream) {
  int m = svie_ball_half_width(radius, spacing);
  if (m < 1 || !w || quad < 1 || quad > 64) {
    set_error("svie_ball_weights: bad arguments");
    return SVIE_ERR_ARG;
  }
  GL32 gl;
  memset(&gl, 0, sizeof(gl));
  gauss_legendre(quad, gl.x, gl.w);
  const long long side = 2 * m + 1;
  const size_t smem = (size_t)quad * quad * sizeof(double) + (size_t)side;
  if (smem > 48 * 1024) {
    set_error("svie_ball_weights: ball too large for one column per block (radius/spacing %g)", radius / spacing);
    return SVIE_ERR_UNSUPPORTED;
  }
  k_ball_weights<<<(unsigned)(side * side), 256, smem, (cudaStream_t)stream>>>(radius / spacing, m, quad, gl, w);
  return launch_status("svie_ball_weights");
}

int svie_conv_supported(int n) {
  AxisPlan p;
  return factor_axis(n, &p) ? 1 : 0;
}

size_t svie_conv_plan_bytes(int nx, int ny, int nz) { return plan_layout(nx, ny, nz).total; }

size_t svie_conv_workspace_bytes(int nx, int ny, int nz) {
  return align256((size_t)nx * ny * padded_nzh(nz) * sizeof(float2));
}

int svie_conv_spectrum_row(int nz) { return padded_nzh(nz); }

size_t svie_conv_init_workspace_bytes(int nx, int ny, int nz, int m) {
  const size_t side = 2 * (size_t)m + 1, nzh = nz / 2 + 1, nyh = ny / 2 + 1;
  (void)nx;
  return align256(side * side * nzh * sizeof(double)) + align256(side * nyh * nzh * sizeof(double));
}

int svie_conv_plan_init(void* plan, int nx, int ny, int nz, const double* w, int m, void* ws, size_t ws_bytes,
                           void* stream) {
  if (!plan || !w || m < 1 || 2 * m + 1 > nx || 2 * m + 1 > ny || 2 * m + 1 > nz) {
    set_error("svie_conv_plan_init: ball kernel larger than the grid or bad arguments");
    return SVIE_ERR_ARG;
  }
  if (!ws || ws_bytes < svie_conv_init_workspace_bytes(nx, ny, nz, m)) {
    set_error("svie_conv_plan_init: workspace too small");
    return SVIE_ERR_WORKSPACE;
  }
  Plans P;
  int st = make_plans(plan, nx, ny, nz, &P);
  if (st) return st;
  cudaStream_t s = (cudaStream_t)stream;
  PlanLayout L = plan_layout(nx, ny, nz);
  char* b = (char*)plan;
  k_twiddles<<<blocks_for(nx, 256), 256, 0, s>>>((float2*)(b + L.tw_x), nx);
  k_twiddles<<<blocks_for(ny, 256), 256, 0, s>>>((float2*)(b + L.tw_y), ny);
  k_twiddles<<<blocks_for(nz, 256), 256, 0, s>>>((float2*)(b + L.tw_z), nz);
  k_stage_twiddles<<<blocks_for(nx, 256), 256, 0, s>>>(P.x, (float2*)(b + L.stw_x));
  k_stage_twiddles<<<blocks_for(ny, 256), 256, 0, s>>>(P.y, (float2*)(b + L.stw_y));
  k_stage_twiddles<<<blocks_for(nz, 256), 256, 0, s>>>(P.z, (float2*)(b + L.stw_z));
  AxisPlan xr = P.x;  // the x axis in reverse radix order: the inverse half of the fused x pass
  xr.radices = P.x.rradices;
  k_stage_twiddles<<<blocks_for(nx, 256), 256, 0, s>>>(xr, (float2*)(b + L.rstw_x));
  const int side = 2 * m + 1, nzh = nz / 2 + 1, nyh = ny / 2 + 1, nxh = nx / 2 + 1;
  double* A = (double*)ws;
  double* Bq = (double*)((char*)ws + align256((size_t)side * side * nzh * sizeof(double)));
  const int TB = 256;
  k_khat_a<<<blocks_for((long long)side * side * nzh, TB, 4096), TB, nz * sizeof(double), s>>>(w, m, nz, nzh, A);
  k_khat_b<<<blocks_for((long long)side * nyh * nzh, TB, 4096), TB, ny * sizeof(double), s>>>(A, m, ny, nzh, Bq);
  k_khat_c<<<blocks_for((long long)nxh * nyh * nzh, TB, 8192), TB, nx * sizeof(double), s>>>(
      Bq, m, nx, ny, nzh, (float*)(b + L.kred));
  return launch_status("svie_conv_plan_init", 10);
}

int svie_conv_apply(const void* plan, int nx, int ny, int nz, const float* f, float* out, double alpha,
                    double beta, void* ws, size_t ws_bytes, void* stream) {
  Plans P;
  int st = make_plans(plan, nx, ny, nz, &P);
  if (st) return st;
  if (!f || !out) {
    set_error("svie_conv_apply: null input/output");
    return SVIE_ERR_ARG;
  }
  if (!ws || ws_bytes < svie_conv_workspace_bytes(nx, ny, nz) || ((uintptr_t)ws & 15)) {
    set_error("svie_conv_apply: workspace too small or not 16-byte aligned");
    return SVIE_ERR_WORKSPACE;
  }
  if ((st = ensure_smem_attr())) return st;
  cudaStream_t s = (cudaStream_t)stream;
  float2* spec = (float2*)ws;
  const FftChoice c = choice_for(nx, ny, nz);
  launch_z(P, nx, ny, nz, f, spec, nullptr, true, 0.f, 0.f, s, nullptr, c.z, false, c.jit);
  launch_y(P, nx, ny, nz, spec, 0, s, nullptr, c.y, true, c.jit);
  launch_x(P, nx, ny, nz, spec, 2, s, c.x, true, c.jit);
  launch_y(P, nx, ny, nz, spec, 1, s, nullptr, c.y, true, c.jit);
  launch_z(P, nx, ny, nz, nullptr, spec, out, false, (float)alpha, (float)beta, s, nullptr, c.z, true, c.jit);
  return launch_status("svie_conv_apply", 5);
}

int svie_conv_apply_masked(const void* plan, int nx, int ny, int nz, const float* f, float* out, double alpha,
                           double beta, void* ws, size_t ws_bytes, const uint8_t* lineflag, const uint8_t* slabflag,
                           void* const* events, void* stream) {
  Plans P;
  int st = make_plans(plan, nx, ny, nz, &P);
  if (st) return st;
  if (!f || !out || (!lineflag) != (!slabflag)) {
    set_error("svie_conv_apply_masked: null input/output, or only one of the two flag arrays");
    return SVIE_ERR_ARG;
  }
  if (!ws || ws_bytes < svie_conv_workspace_bytes(nx, ny, nz) || ((uintptr_t)ws & 15)) {
    set_error("svie_conv_apply_masked: workspace too small or not 16-byte aligned");
    return SVIE_ERR_WORKSPACE;
  }
  if ((st = ensure_smem_attr())) return st;
  cudaStream_t s = (cudaStream_t)stream;
  float2* spec = (float2*)ws;
  cudaEvent_t* ev = (cudaEvent_t*)events;
  const FftChoice c = choice_for(nx, ny, nz);
  // with timing events between the passes every pass is an ordinary launch
  const bool ch = ev == nullptr;
  if (ev) cudaEventRecord(ev[0], s);
  launch_z(P, nx, ny, nz, f, spec, nullptr, true, 0.f, 0.f, s, lineflag, c.z, false, c.jit);
  if (ev) cudaEventRecord(ev[1], s);
  launch_y(P, nx, ny, nz, spec, 0, s, slabflag, c.y, ch, c.jit);
  if (ev) cudaEventRecord(ev[2], s);
  launch_x(P, nx, ny, nz, spec, 2, s, c.x, ch, c.jit);
  if (ev) cudaEventRecord(ev[3], s);
  launch_y(P, nx, ny, nz, spec, 1, s, slabflag, c.y, ch, c.jit);
  if (ev) cudaEventRecord(ev[4], s);
  launch_z(P, nx, ny, nz, nullptr, spec, out, false, (float)alpha, (float)beta, s, lineflag, c.z, ch, c.jit);
  if (ev) cudaEventRecord(ev[5], s);
  return launch_status("svie_conv_apply_masked", 5);
}

unsigned int svie_conv_tma_timeouts(void) {
  unsigned int v = 0;
  if (cudaMemcpyFromSymbol(&v, g_tma_timeouts, sizeof(v)) != cudaSuccess) return 0xFFFFFFFFu;
  return v;
}

int svie_conv_get_choice(int nx, int ny, int nz, int* z, int* y, int* x) {
  bool tuned = false;
  const FftChoice c = choice_for(nx, ny, nz, &tuned);
  if (z) *z = c.z;
  if (y) *y = c.y;
  if (x) *x = c.x;
  return tuned ? 1 : 0;
}

int svie_conv_set_choice(int nx, int ny, int nz, int z, int y, int x) {
  const GridKey k = grid_key(nx, ny, nz);
  if (z < 0 || y < 0 || x < 0) {
    std::lock_guard<std::mutex> lock(g_choice_mu);
    g_choice.erase(k);
    return SVIE_OK;
  }
  FftChoice c{z, y, x};
  c.kept = 1;
  if (!choice_fits(c, nx, ny, nz)) {
    set_error("svie_conv_set_choice: forms (%d, %d, %d) do not exist or do not fit shared memory for %d x %d x %d",
              z, y, x, nx, ny, nz);
    return SVIE_ERR_ARG;
  }
  std::lock_guard<std::mutex> lock(g_choice_mu);
  auto it = g_choice.find(k);
  if (it != g_choice.end()) c.jit = it->second.jit;
  g_choice[k] = c;
  return SVIE_OK;
}

int svie_conv_jit(int nx, int ny, int nz) {
  AxisPlan ax, ay, az;
  if (!factor_axis(nx, &ax) || !factor_axis(ny, &ay) || !factor_axis(nz, &az)) {
    set_error("svie_conv_jit: axis sizes %d x %d x %d are not supported", nx, ny, nz);
    return SVIE_ERR_UNSUPPORTED;
  }
  if (!fits(y_smem(1, ny)) || !fits(x_smem(0, nx))) {
    set_error("svie_conv_jit: the 8-line passes do not fit shared memory on %d x %d x %d", nx, ny, nz);
    return SVIE_ERR_UNSUPPORTED;
  }
  if (!jit_available()) {
    set_error("svie_conv_jit: NVRTC or the CUDA driver functions were not found");
    return SVIE_ERR_UNSUPPORTED;
  }
  // request the three passes (their compilations start on background threads)
  CUfunction fy = nullptr, fx = nullptr, zf = nullptr, zi = nullptr;
  jit_strided(ny, JIT_Y_MINB, ay.radices, ay.nst, &fy);
  jit_strided(nx, JIT_X_MINB, ax.radices, ax.nst, &fx);
  if (fits(z_smem(0, nz))) jit_z(nz, az.radices, az.nst, &zf, &zi);
  const GridKey k = grid_key(nx, ny, nz);
  std::lock_guard<std::mutex> lock(g_choice_mu);
  auto it = g_choice.find(k);
  FftChoice c = it != g_choice.end() ? it->second : default_choice(nx, ny, nz);
  c.jit = 1;
  g_choice[k] = c;
  return SVIE_OK;
}

int svie_conv_jit_enabled(int nx, int ny, int nz) { return choice_for(nx, ny, nz).jit ? 1 : 0; }

int svie_conv_jit_ready(int nx, int ny, int nz) {
  AxisPlan ax, ay, az;
  if (!factor_axis(nx, &ax) || !factor_axis(ny, &ay) || !factor_axis(nz, &az) || !jit_available()) return 0;
  CUfunction f = nullptr, g = nullptr;
  if (jit_strided(ny, JIT_Y_MINB, ay.radices, ay.nst, &f) != SVIE_OK ||
      jit_strided(nx, JIT_X_MINB, ax.radices, ax.nst, &f) != SVIE_OK)
    return 0;
  return !fits(z_smem(0, nz)) || jit_z(nz, az.radices, az.nst, &f, &g) == SVIE_OK;
}

int svie_conv_jit_stop(void) {
  jit_stop();
  return SVIE_OK;
}

int svie_conv_jit_wait(int timeout_ms) {
  if (timeout_ms < 0) {
    set_error("svie_conv_jit_wait: negative timeout");
    return SVIE_ERR_ARG;
  }
  const int st = jit_wait(timeout_ms);
  if (st) set_error("svie_conv_jit_wait: compilations still running after %d ms", timeout_ms);
  return st;
}

int svie_conv_jit_source(int n, int minb, char* buf, size_t buf_bytes) {
  AxisPlan a;
  if (!factor_axis(n, &a) || minb < 0 || minb > 8 || !buf) {
    set_error("svie_conv_jit_source: bad arguments");
    return SVIE_ERR_ARG;
  }
  const std::string src = minb ? jit_strided_source_for_test(n, minb, a.radices, a.nst)
                               : jit_z_source_for_test(n, a.radices, a.nst);
  if (src.size() + 1 > buf_bytes) {
    set_error("svie_conv_jit_source: %zu bytes needed", src.size() + 1);
    return SVIE_ERR_CAPACITY;
  }
  memcpy(buf, src.c_str(), src.size() + 1);
  return SVIE_OK;
}

int svie_conv_tune(const void* plan, int nx, int ny, int nz, const float* f, float* out, void* ws, size_t ws_bytes,
                   int reps, void* stream) {
  Plans P;
  int st = make_plans(plan, nx, ny, nz, &P);
  if (st) return st;
  if (!f || !out || reps < 1 || reps > 100) {
    set_error("svie_conv_tune: null input/output or reps outside 1..100");
    return SVIE_ERR_ARG;
  }
  if (!ws || ws_bytes < svie_conv_workspace_bytes(nx, ny, nz) || ((uintptr_t)ws & 15)) {
    set_error("svie_conv_tune: workspace too small or not 16-byte aligned");
    return SVIE_ERR_WORKSPACE;
  }
  cudaStream_t s = (cudaStream_t)stream;
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(s, &cap) != cudaSuccess || cap != cudaStreamCaptureStatusNone) {
    set_error("svie_conv_tune: the stream is being captured (tuning synchronises it)");
    return SVIE_ERR_ARG;
  }
  if ((st = ensure_smem_attr())) return st;
  float2* spec = (float2*)ws;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) {
    if (e0) cudaEventDestroy(e0);
    set_error("svie_conv_tune: cudaEventCreate failed");
    return SVIE_ERR_LAUNCH;
  }
  FftChoice best = default_choice(nx, ny, nz);
  best.jit = choice_for(nx, ny, nz).jit;  // the compiled passes, when the shape has them, are what is timed
  float tz = -1.f, ty = -1.f, tx = -1.f;
  bool failed = false;
  int launched = 1;
  // the spectrum of f in the workspace first, so that every form transforms real data
  const FftChoice d = best;
  launch_z(P, nx, ny, nz, f, spec, nullptr, true, 0.f, 0.f, s, nullptr, d.z, false);
  for (int c = 0; c < FFT_NCHOICE && !failed; ++c) {
    if (tunable_z(c, nz)) {  // forward and inverse z
      const float t = time_form([&] {
        launch_z(P, nx, ny, nz, f, spec, nullptr, true, 0.f, 0.f, s, nullptr, c, false, d.jit);
        launch_z(P, nx, ny, nz, nullptr, spec, out, false, 1.f, 0.f, s, nullptr, c, false, d.jit);
        launched += 2;
      }, reps, s, e0, e1);
      if (t < 0.f) failed = true;
      else if (tz < 0.f || t < tz) { tz = t; best.z = c; }
    }
    if (!failed && tunable_y(c, ny)) {  // forward and inverse y
      const float t = time_form([&] {
        launch_y(P, nx, ny, nz, spec, 0, s, nullptr, c, false, d.jit);
        launch_y(P, nx, ny, nz, spec, 1, s, nullptr, c, false, d.jit);
        launched += 2;
      }, reps, s, e0, e1);
      if (t < 0.f) failed = true;
      else if (ty < 0.f || t < ty) { ty = t; best.y = c; }
    }
    if (!failed && tunable_x(c, nx)) {  // the fused x pass
      const float t = time_form([&] {
        launch_x(P, nx, ny, nz, spec, 2, s, c, false, d.jit);
        launched += 1;
      }, reps, s, e0, e1);
      if (t < 0.f) failed = true;
      else if (tx < 0.f || t < tx) { tx = t; best.x = c; }
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (failed) return launch_status("svie_conv_tune", launched);
  best.kept = 1;
  {
    std::lock_guard<std::mutex> lock(g_choice_mu);
    g_choice[grid_key(nx, ny, nz)] = best;
  }
  return launch_status("svie_conv_tune", launched);
}

int svie_conv_line_flags(const int32_t* band, int64_t m, int nx, int ny, int nz, int dilation, uint8_t* lineflag,
                         uint8_t* slabflag, uint8_t* tmp, void* stream) {
  if (!lineflag || !slabflag || !tmp || m < 0 || (m > 0 && !band) || dilation < 0) {
    set_error("svie_conv_line_flags: bad arguments");
    return SVIE_ERR_ARG;
  }
  cudaStream_t s = (cudaStream_t)stream;
  if (cudaMemsetAsync(lineflag, 0, (size_t)nx * ny, s) != cudaSuccess) {
    set_error("svie_conv_line_flags: memset failed");
    return SVIE_ERR_LAUNCH;
  }
  if (m > 0) k_mark_lines<<<blocks_for(m, 256), 256, 0, s>>>(band, m, nz, lineflag);
  const dim3 g((ny + 127) / 128, nx);
  k_dilate_lines_x<<<g, 128, 0, s>>>(lineflag, tmp, nx, ny, dilation);
  k_dilate_lines_y<<<g, 128, 0, s>>>(tmp, lineflag, nx, ny, dilation);
  k_slab_flags<<<nx, 256, 0, s>>>(lineflag, nx, ny, slabflag);
  return launch_status("svie_conv_line_flags", m > 0 ? 4 : 3);
}

int svie_conv_kernel_hat(const void* plan, int nx, int ny, int nz, void* out_c64, void* stream) {
  Plans P;
  int st = make_plans(plan, nx, ny, nz, &P);
  if (st) return st;
  const long long tot = (long long)nx * ny * (nz / 2 + 1);
  k_khat_expand<<<blocks_for(tot, 256, 8192), 256, 0, (cudaStream_t)stream>>>(P.kred, nx, ny, nz / 2 + 1,
                                                                             (float2*)out_c64);
  return launch_status("svie_conv_kernel_hat");
}

int svie_rfft3(const void* plan, int nx, int ny, int nz, const float* f, void* spec, void* stream) {
  Plans P;
  int st = make_plans(plan, nx, ny, nz, &P);
  if (st) return st;
  if (!f || !spec || ((uintptr_t)spec & 15)) {
    set_error("svie_rfft3: null input, or spectrum not 16-byte aligned");
    return SVIE_ERR_ARG;
  }
  if ((st = ensure_smem_attr())) return st;
  cudaStream_t s = (cudaStream_t)stream;
  const FftChoice c = choice_for(nx, ny, nz);
  launch_z(P, nx, ny, nz, f, (float2*)spec, nullptr, true, 0.f, 0.f, s, nullptr, c.z, false, c.jit);
  launch_y(P, nx, ny, nz, (float2*)spec, 0, s, nullptr, c.y, true, c.jit);
  launch_x(P, nx, ny, nz, (float2*)spec, 0, s, c.x, true, c.jit);
  return launch_status("svie_rfft3", 3);
}

int svie_irfft3(const void* plan, int nx, int ny, int nz, void* spec, float* out, double alpha, double beta,
                void* stream) {
  Plans P;
  int st = make_plans(plan, nx, ny, nz, &P);
  if (st) return st;
  if (!spec || !out || ((uintptr_t)spec & 15)) {
    set_error("svie_irfft3: null input, or spectrum not 16-byte aligned");
    return SVIE_ERR_ARG;
  }
  if ((st = ensure_smem_attr())) return st;
  cudaStream_t s = (cudaStream_t)stream;
  const FftChoice c = choice_for(nx, ny, nz);
  launch_x(P, nx, ny, nz, (float2*)spec, 1, s, c.x, false, c.jit);
  launch_y(P, nx, ny, nz, (float2*)spec, 1, s, nullptr, c.y, true, c.jit);
  launch_z(P, nx, ny, nz, nullptr, (float2*)spec, out, false, (float)alpha, (float)beta, s, nullptr, c.z, true,
           c.jit);
  return launch_status("svie_irfft3", 3);
}

}  // extern "C"
