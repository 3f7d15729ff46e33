// Device building blocks of the convolution passes: the axis plan, the radix
// butterflies, the Stockham tile stages and the pass epilogues.  Included by
// fft.cu (the passes compiled with the library) and by the source of the pass
// kernels compiled at run time for one axis length (fft_jit.cu), so that both
// run the same arithmetic.  Device code only; under NVRTC (__CUDACC_RTC__) the
// few definitions that otherwise come from common.cuh are made here.
#pragma once

#ifdef __CUDACC_RTC__
typedef unsigned char uint8_t;
typedef int int32_t;
typedef unsigned int uint32_t;
typedef unsigned long long uint64_t;
#define SVIE_DEV __device__ __forceinline__
namespace svie {
SVIE_DEV void pdl_wait() { asm volatile("griddepcontrol.wait;\n" ::: "memory"); }
SVIE_DEV void pdl_release() { asm volatile("griddepcontrol.launch_dependents;\n" :::); }
}  // namespace svie
#endif

namespace svie {

constexpr int FFT_T = 256;      // threads per CTA
constexpr int FFT_MAXST = 14;   // radix stages per axis
constexpr int FFT_MAXN = 7168;  // longest supported axis (its one-line pass fits shared memory)

struct AxisPlan {
  int n;
  int nst;
  unsigned long long radices;  // radix of stage s in bits [4s, 4s+4) (no arrays: no local-memory copy)
  const float2* tw;            // tw[k] = exp(-2 pi i k / n), k < n
  const float2* stw;           // per-stage twiddles: stage with span p at p - 1 + k (R - 1) + q - 1 (n - 1 entries)
  unsigned long long rradices; // the radices in reverse order (the inverse of the fused x pass)
  const float2* rstw;          // stage twiddles of the reverse order (x axis only)
};

SVIE_DEV float2 cmul(float2 a, float2 b) { return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); }
SVIE_DEV float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
SVIE_DEV float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
SVIE_DEV float2 cconj(float2 a) { return make_float2(a.x, -a.y); }
SVIE_DEV float2 mul_mi(float2 a) { return make_float2(a.y, -a.x); }  // -i * a

// cos / sin of 2 pi t / R for the odd radices (values of the trigonometric
// functions at rational multiples of pi, to float precision).
__constant__ float c_cos3[3] = {1.0f, -0.5f, -0.5f};
__constant__ float c_sin3[3] = {0.0f, 0.86602540378443865f, -0.86602540378443865f};
__constant__ float c_cos5[5] = {1.0f, 0.30901699437494742f, -0.80901699437494742f, -0.80901699437494742f,
                                0.30901699437494742f};
__constant__ float c_sin5[5] = {0.0f, 0.95105651629515357f, 0.58778525229247313f, -0.58778525229247313f,
                                -0.95105651629515357f};
__constant__ float c_cos7[7] = {1.0f, 0.62348980185873353f, -0.22252093395631440f, -0.90096886790241913f,
                                -0.90096886790241913f, -0.22252093395631440f, 0.62348980185873353f};
__constant__ float c_sin7[7] = {0.0f, 0.78183148246802981f, 0.97492791218182361f, 0.43388373911755812f,
                                -0.43388373911755812f, -0.97492791218182361f, -0.78183148246802981f};

// Forward DFT of R points in place: y_p = sum_q x_q exp(-2 pi i p q / R).
template <int R>
SVIE_DEV void dft(float2* x);

template <>
SVIE_DEV void dft<2>(float2* x) {
  float2 a = x[0], b = x[1];
  x[0] = cadd(a, b);
  x[1] = csub(a, b);
}

template <>
SVIE_DEV void dft<4>(float2* x) {
  float2 t0 = cadd(x[0], x[2]), t1 = csub(x[0], x[2]);
  float2 t2 = cadd(x[1], x[3]), t3 = csub(x[1], x[3]);
  x[0] = cadd(t0, t2);
  x[2] = csub(t0, t2);
  x[1] = cadd(t1, mul_mi(t3));
  x[3] = csub(t1, mul_mi(t3));
}

template <>
SVIE_DEV void dft<8>(float2* x) {
  float2 e[4] = {x[0], x[2], x[4], x[6]};
  float2 o[4] = {x[1], x[3], x[5], x[7]};
  dft<4>(e);
  dft<4>(o);
  const float r = 0.70710678118654752f;
  float2 w1 = make_float2(r * (o[1].x + o[1].y), r * (o[1].y - o[1].x));    // o1 * (r - ir)
  float2 w2 = mul_mi(o[2]);                                                  // o2 * (-i)
  float2 w3 = make_float2(r * (o[3].y - o[3].x), -r * (o[3].x + o[3].y));   // o3 * (-r - ir)
  x[0] = cadd(e[0], o[0]);
  x[4] = csub(e[0], o[0]);
  x[1] = cadd(e[1], w1);
  x[5] = csub(e[1], w1);
  x[2] = cadd(e[2], w2);
  x[6] = csub(e[2], w2);
  x[3] = cadd(e[3], w3);
  x[7] = csub(e[3], w3);
}

// Odd radix with the symmetric pairing of q and R-q.
template <int R>
SVIE_DEV void dft_odd(float2* x, const float* C, const float* S) {
  constexpr int H = (R - 1) / 2;
  float2 a[H], b[H];
#pragma unroll
  for (int q = 1; q <= H; ++q) {
    a[q - 1] = cadd(x[q], x[R - q]);
    b[q - 1] = csub(x[q], x[R - q]);
  }
  float2 x0 = x[0];
  float2 y0 = x0;
#pragma unroll
  for (int q = 0; q < H; ++q) y0 = cadd(y0, a[q]);
#pragma unroll
  for (int p = 1; p <= H; ++p) {
    float2 re = x0, im = make_float2(0.f, 0.f);
#pragma unroll
    for (int q = 1; q <= H; ++q) {
      const int t = (p * q) % R;
      re.x += a[q - 1].x * C[t];
      re.y += a[q - 1].y * C[t];
      im.x += b[q - 1].x * S[t];
      im.y += b[q - 1].y * S[t];
    }
    // y_p = re - i*im ; y_{R-p} = re + i*im
    x[p] = make_float2(re.x + im.y, re.y - im.x);
    x[R - p] = make_float2(re.x - im.y, re.y + im.x);
  }
  x[0] = y0;
}

template <>
SVIE_DEV void dft<3>(float2* x) { dft_odd<3>(x, c_cos3, c_sin3); }
template <>
SVIE_DEV void dft<5>(float2* x) { dft_odd<5>(x, c_cos5, c_sin5); }
template <>
SVIE_DEV void dft<7>(float2* x) { dft_odd<7>(x, c_cos7, c_sin7); }

// 6 = 2 x 3: two 3-point DFTs on the even / odd samples, then twiddles
// w6^k = exp(-2 pi i k / 6) and a final radix-2 combination.
template <>
SVIE_DEV void dft<6>(float2* x) {
  float2 e[3] = {x[0], x[2], x[4]};
  float2 o[3] = {x[1], x[3], x[5]};
  dft<3>(e);
  dft<3>(o);
  const float h = 0.86602540378443865f;
  const float2 o1 = make_float2(0.5f * o[1].x + h * o[1].y, 0.5f * o[1].y - h * o[1].x);    // o1 * (1/2 - i h)
  const float2 o2 = make_float2(-0.5f * o[2].x + h * o[2].y, -0.5f * o[2].y - h * o[2].x);  // o2 * (-1/2 - i h)
  x[0] = cadd(e[0], o[0]);
  x[3] = csub(e[0], o[0]);
  x[1] = cadd(e[1], o1);
  x[4] = csub(e[1], o1);
  x[2] = cadd(e[2], o2);
  x[5] = csub(e[2], o2);
}

// ------------------------------------------------------------ tile layout
// A tile holds LW lines of length n in shared memory, element (line l,
// position x) at x * PS + l.  Butterfly j of a stage takes line j % LW and
// column b = j / LW, so the 16 lanes of a half-warp (one wavefront of 8-byte
// shared accesses) touch LW lines at 16 / LW consecutive columns:
//  - LW = 16: every stage access is 16 consecutive slots, free of bank
//    conflicts for any PS (the z passes use PS = 17 so that their loads and
//    stores, lanes along a line, are conflict-free too);
//  - LW = 8 (PS = 8): the two columns b, b + 1 (b even) land on different
//    halves of the bank row whenever their positions differ in parity, which
//    fails only where a run of k = b mod p wraps inside the pair (p odd, R
//    even) and in a first stage of even radix; factor_axis puts one odd radix
//    first so that only the wrap case remains (measured: about 1.5% extra
//    wavefronts);
//  - LW = 1 (PS = 1): one line per tile, for axes too long for the others.
// Each stage is one Stockham radix-R pass from src to dst (ping-pong).
template <int R, int LW, int PS, int NT = FFT_T>
SVIE_DEV void tile_stage(const float2* __restrict__ src, float2* __restrict__ dst, int n, int p, unsigned int pmagic,
                         const float2* __restrict__ stw, bool conj_in) {
  const int m = n / R;
  const int total = LW * m;
  for (int j = threadIdx.x; j < total; j += NT) {
    const int l = j % LW, b = j / LW;
    // k = b mod p; umulhi(b, ceil(2^32 / p)) = b / p exactly for b * p < 2^32
    const int k = (p == 1) ? 0 : b - (int)__umulhi((unsigned)b, pmagic) * p;
    const float2* s = src + b * PS + l;
    float2 v[R];
#pragma unroll
    for (int q = 0; q < R; ++q) v[q] = s[q * m * PS];
    if (conj_in) {
#pragma unroll
      for (int q = 0; q < R; ++q) v[q].y = -v[q].y;
    }
    if (k) {
      const float2* tk = stw + k * (R - 1);  // the stage's twiddles w^(q k n / (p R)), q = 1..R-1
#pragma unroll
      for (int q = 1; q < R; ++q) v[q] = cmul(v[q], tk[q - 1]);
    }
    dft<R>(v);
    float2* d = dst + ((b - k) * R + k) * PS + l;
#pragma unroll
    for (int q = 0; q < R; ++q) d[q * p * PS] = v[q];
  }
  __syncthreads();
}

SVIE_DEV int radix_of(unsigned long long rad, int st) { return (int)((rad >> (4 * st)) & 15ULL); }

// Stages [s0, s1) of the radix sequence `rad` (4 bits per stage) from a to b
// and back; p is the span before stage s0 and is advanced past s1.  Returns
// the buffer holding the result.  `stw` is the stage-twiddle table of that
// sequence staged in shared memory; the stage with span p starts at entry
// p - 1 (the earlier stages hold p - 1 entries).  conj_first: stage s0 reads
// conj(a) (inverse transforms as conj(FFT(conj(x)))).
template <int LW, int PS, int NT>
SVIE_DEV float2* run_stages(float2* a, float2* b, int n, unsigned long long rad, int s0, int s1, const float2* stw,
                            bool conj_first, int& p) {
  for (int st = s0; st < s1; ++st) {
    const int R = radix_of(rad, st);
    const unsigned int mg = p > 1 ? 0xFFFFFFFFu / (unsigned)p + 1u : 0u;
    const float2* sw = stw + (p - 1);
    const bool cj = conj_first && st == s0;
    switch (R) {
      case 8: tile_stage<8, LW, PS, NT>(a, b, n, p, mg, sw, cj); break;
      case 7: tile_stage<7, LW, PS, NT>(a, b, n, p, mg, sw, cj); break;
      case 6: tile_stage<6, LW, PS, NT>(a, b, n, p, mg, sw, cj); break;
      case 5: tile_stage<5, LW, PS, NT>(a, b, n, p, mg, sw, cj); break;
      case 4: tile_stage<4, LW, PS, NT>(a, b, n, p, mg, sw, cj); break;
      case 3: tile_stage<3, LW, PS, NT>(a, b, n, p, mg, sw, cj); break;
      default: tile_stage<2, LW, PS, NT>(a, b, n, p, mg, sw, cj); break;
    }
    float2* t = a; a = b; b = t;
    p *= R;
  }
  return a;
}

template <int LW, int PS, int NT = FFT_T>
SVIE_DEV float2* run_tile_fft(float2* a, float2* b, const AxisPlan& P, const float2* stw, bool conj_first = false) {
  int p = 1;
  return run_stages<LW, PS, NT>(a, b, P.n, P.radices, 0, P.nst, stw, conj_first, p);
}

// The last stage of a transform (span p = m = n / R, so k = b): butterfly
// (line l, column b) reads and writes the positions b + q m of line l, and its
// outputs go to epi.apply(v, b, l, m) instead of back to shared memory.
template <int R, int LW, int PS, int NT, class Epi>
SVIE_DEV void last_stage(const float2* __restrict__ src, int n, const float2* __restrict__ stw, bool conj_in,
                         const Epi& epi) {
  const int m = n / R;
  const int total = LW * m;
  for (int j = threadIdx.x; j < total; j += NT) {
    const int l = j % LW, b = j / LW;
    const float2* s = src + b * PS + l;
    float2 v[R];
#pragma unroll
    for (int q = 0; q < R; ++q) v[q] = s[q * m * PS];
    if (conj_in) {
#pragma unroll
      for (int q = 0; q < R; ++q) v[q].y = -v[q].y;
    }
    if (b) {
      const float2* tk = stw + (m - 1) + b * (R - 1);
#pragma unroll
      for (int q = 1; q < R; ++q) v[q] = cmul(v[q], tk[q - 1]);
    }
    dft<R>(v);
    epi.template apply<R>(v, b, l, m);
  }
}

template <int LW, int PS, int NT, class Epi>
SVIE_DEV void run_last(const float2* src, int n, int R, const float2* stw, bool conj_in, const Epi& epi) {
  const float2* sw = stw;
  switch (R) {
    case 8: last_stage<8, LW, PS, NT>(src, n, sw, conj_in, epi); break;
    case 7: last_stage<7, LW, PS, NT>(src, n, sw, conj_in, epi); break;
    case 6: last_stage<6, LW, PS, NT>(src, n, sw, conj_in, epi); break;
    case 5: last_stage<5, LW, PS, NT>(src, n, sw, conj_in, epi); break;
    case 4: last_stage<4, LW, PS, NT>(src, n, sw, conj_in, epi); break;
    case 3: last_stage<3, LW, PS, NT>(src, n, sw, conj_in, epi); break;
    default: last_stage<2, LW, PS, NT>(src, n, sw, conj_in, epi); break;
  }
}

// Epilogue: store line l's outputs at base + l + position * stride (lines
// l < nl only), conjugated for inverse transforms.
struct StoreEpi {
  float2* base;
  long long stride;
  int nl;
  bool conj;
  template <int R>
  SVIE_DEV void apply(float2 (&v)[R], int b, int l, int m) const {
    if (l >= nl) return;
    float2* g = base + l + (long long)b * stride;
    const long long ms = (long long)m * stride;
#pragma unroll
    for (int q = 0; q < R; ++q) {
      float2 w = v[q];
      if (conj) w.y = -w.y;
      g[q * ms] = w;
    }
  }
};

// Epilogue of the x pass: multiply the forward outputs by K^ (real, even in
// kx) and conjugate, then run the first stage of the inverse, whose radix
// order is the forward's reversed: its first radix is this stage's R and it
// reads exactly the positions b + q m this butterfly holds (span 1, no
// twiddles); the results go to dst at positions b R + q.
template <int PS>
struct KEpi {
  float2* dst;
  const float* krow;  // K^ row of this slab and column block: + l + kr * kst
  long long kst;
  int n, nl;
  template <int R>
  SVIE_DEV void apply(float2 (&v)[R], int b, int l, int m) const {
#pragma unroll
    for (int q = 0; q < R; ++q) {
      const int pos = b + q * m, kr = min(pos, n - pos);
      const float kv = l < nl ? __ldg(krow + l + kr * kst) : 0.0f;
      v[q] = make_float2(v[q].x * kv, -(v[q].y * kv));
    }
    dft<R>(v);
    float2* d = dst + b * R * PS + l;
#pragma unroll
    for (int q = 0; q < R; ++q) d[q * PS] = v[q];
  }
};

__host__ __device__ inline int padded_nzh(int nz) { return ((nz / 2 + 1) + 7) & ~7; }  // 64-byte rows
// shared memory of a tile: two buffers of n positions and the stage-twiddle table (n entries)
__host__ __device__ inline size_t tile_smem(int PS, int n) { return (2 * (size_t)PS + 1) * (size_t)n * sizeof(float2); }
constexpr size_t TILE_SMEM_MAX = 227 * 1024;

// Copy the axis' stage twiddles (n - 1 entries) into shared memory after the buffers.
SVIE_DEV float2* stage_twiddles_to_smem(float2* sm, int PS, const AxisPlan& P) {
  float2* stw = sm + 2 * PS * P.n;
  for (int e = threadIdx.x; e < P.n - 1; e += blockDim.x) stw[e] = __ldg(P.stw + e);
  return stw;
}

// 16-byte asynchronous global -> shared copies (L2 only), completed by groups.
SVIE_DEV void cp_async16(void* smem, const void* gmem) {
  const unsigned int sa = (unsigned int)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(gmem) : "memory");
}
// 8- and 4-byte forms (cached in L1 as well: the only forms for these sizes).
SVIE_DEV void cp_async8(void* smem, const void* gmem) {
  const unsigned int sa = (unsigned int)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(sa), "l"(gmem) : "memory");
}
SVIE_DEV void cp_async4(void* smem, const void* gmem) {
  const unsigned int sa = (unsigned int)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(sa), "l"(gmem) : "memory");
}
SVIE_DEV void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
SVIE_DEV void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

struct KGeom {
  const float* kred;  // [(nx/2+1)][(ny/2+1)][nzh]
  int ny, nzh;
};

// ----------------------------------------------------------------- z passes
// The stages of a whole tile transform, from buffer a, ping-ponging with b;
// the buffer holding the result is returned.  PlanStages runs the plan's radix
// sequence at run time (the z pass kernels of fft.cu); the z passes compiled
// for one axis length pass a functor with the stages unrolled.
template <int LW, int PS>
struct PlanStages {
  const AxisPlan& P;
  SVIE_DEV float2* operator()(float2* a, float2* b, const float2* stw) const { return run_tile_fft<LW, PS>(a, b, P, stw); }
};

// Forward: real lines [nlines][n] -> half spectra at out[line * nzp + k].
// A CTA takes 2 LW real lines, packed in pairs into LW complex lines (one
// contiguous chunk of the input); a warp loads one pair, lanes along z.
// `lineflag` (optional): lines whose flag lacks bit 0 hold no solid, so their
// input is zero; a tile without any such line only writes zeros.
template <int LW, int PS, class Stages>
SVIE_DEV void z_r2c_body(const float* __restrict__ in, float2* __restrict__ out, const AxisPlan& P, long long nlines,
                         int nzp, const uint8_t* __restrict__ lineflag, const Stages& stages) {
  extern __shared__ float2 sm[];
  const int n = P.n, nh = n / 2 + 1;
  float2* sa = sm;
  float2* sb = sm + PS * n;
  const long long line0 = (long long)blockIdx.x * 2 * LW;
  const int nl = (int)min((long long)2 * LW, nlines - line0);
  const float* src = in + line0 * n;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  constexpr int NW = FFT_T / 32;
  if (lineflag) {
    const int any = __syncthreads_or(threadIdx.x < nl ? (__ldg(lineflag + line0 + threadIdx.x) & 1) : 0);
    if (!any) {
      float2* dst = out + line0 * nzp;
      for (int l = warp; l < nl; l += NW)
        for (int k = lane; k < nh; k += 32) dst[(long long)l * nzp + k] = make_float2(0.f, 0.f);
      return;
    }
  }
  // the whole tile in flight at once: 4-byte asynchronous copies straight into
  // the paired layout, lanes along (z, line of the pair) so that both the
  // global reads (two 64-byte runs) and the shared writes are contiguous
  float* sf = reinterpret_cast<float*>(sa);
  for (int w = warp; w < LW; w += NW) {
    const int par = lane & 1, l = 2 * w + par;
    const bool ok = l < nl && (!lineflag || (__ldg(lineflag + line0 + l) & 1));
    const float* g = src + (long long)l * n;
    for (int z = lane >> 1; z < n; z += 16) {
      float* d = sf + 2 * (z * PS + w) + par;
      if (ok) cp_async4(d, g + z);
      else *d = 0.0f;
    }
  }
  cp_async_commit();
  const float2* stw = stage_twiddles_to_smem(sm, PS, P);
  cp_async_wait<0>();
  __syncthreads();
  const float2* r = stages(sa, sb, stw);
  // untangle the two real spectra of each pair: X1 = (C_k + conj C_{n-k}) / 2,
  // X2 = (C_k - conj C_{n-k}) / (2 i)
  float2* dst = out + line0 * nzp;
  for (int w = warp; 2 * w < nl; w += NW) {
    const bool has2 = 2 * w + 1 < nl;
    float2* d0 = dst + (long long)(2 * w) * nzp;
    for (int k = lane; k < nh; k += 32) {
      const float2 a = r[k * PS + w];
      const float2 b = r[(k == 0 ? 0 : n - k) * PS + w];
      d0[k] = make_float2(0.5f * (a.x + b.x), 0.5f * (a.y - b.y));
      if (has2) d0[nzp + k] = make_float2(0.5f * (a.y + b.y), -0.5f * (a.x - b.x));
    }
  }
}

// Real lines 2w (real parts) and 2w + 1 (imaginary parts, negated: the
// inverse-by-forward transform) of the tile to dst = out + line0 * n,
// out = beta + alpha * value; with `lineflag`, only lines with bit 1.
template <int LW, int PS>
SVIE_DEV void c2r_store(const float2* __restrict__ r, float* __restrict__ dst, int n, int nl, long long line0,
                        float alpha, float beta, const uint8_t* __restrict__ lineflag) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  constexpr int NW = FFT_T / 32;
  for (int w = warp; 2 * w < nl; w += NW) {
    const int l0 = 2 * w, l1 = 2 * w + 1;
    const bool w0 = !lineflag || (__ldg(lineflag + line0 + l0) & 2);
    const bool w1 = l1 < nl && (!lineflag || (__ldg(lineflag + line0 + l1) & 2));
    if (!w0 && !w1) continue;
    float* d0 = dst + (long long)l0 * n;
    for (int z = lane; z < n; z += 32) {
      const float2 v = r[z * PS + w];
      if (w0) d0[z] = beta + alpha * v.x;
      if (w1) d0[n + z] = beta + alpha * (-v.y);
    }
  }
}

// Inverse: half spectra -> real lines, out = beta + alpha * irfft_unnormalised.
// `lineflag` (optional): only lines with bit 1 set are written (the others
// are never read); a tile without such lines returns at once.
template <int LW, int PS, class Stages>
SVIE_DEV void z_c2r_body(const float2* __restrict__ in, float* __restrict__ out, const AxisPlan& P, long long nlines,
                         int nzp, float alpha, float beta, const uint8_t* __restrict__ lineflag, const Stages& stages) {
  extern __shared__ float2 sm[];
  const int n = P.n;
  float2* sa = sm;
  float2* sb = sm + PS * n;
  const long long line0 = (long long)blockIdx.x * 2 * LW;
  const int nl = (int)min((long long)2 * LW, nlines - line0);
  if (lineflag) {
    const int any = __syncthreads_or(threadIdx.x < nl ? (__ldg(lineflag + line0 + threadIdx.x) & 2) : 0);
    if (!any) return;
  }
  const float2* src = in + line0 * nzp;
  const bool even = (n & 1) == 0;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nzh = n / 2 + 1;
  constexpr int NW = FFT_T / 32;
  // C_k = X1_k + i X2_k over k = 0..n-1 (X_{n-k} = conj X_k), stored
  // conjugated for the inverse-by-forward transform
  auto combine = [&](float2 a, float2 b, int k, int kk) {
    if (kk == 0 || (even && kk == n / 2)) { a.y = 0.f; b.y = 0.f; }
    if (k > n / 2) { a.y = -a.y; b.y = -b.y; }
    return make_float2(a.x - b.y, -(a.y + b.x));
  };
  if (2 * LW * nzh <= PS * n) {
    // the 2 LW half spectra land in the idle second buffer with 8-byte
    // asynchronous copies (all in flight at once), then C is built from there
    for (int l = warp; l < 2 * LW; l += NW) {
      float2* d = sb + l * nzh;
      const float2* g = src + (long long)l * nzp;
      for (int k = lane; k < nzh; k += 32) {
        if (l < nl) cp_async8(d + k, g + k);
        else d[k] = make_float2(0.f, 0.f);
      }
    }
    cp_async_commit();
    const float2* stw = stage_twiddles_to_smem(sm, PS, P);
    cp_async_wait<0>();
    __syncthreads();
    for (int w = warp; w < LW; w += NW) {
      const float2* x1 = sb + (2 * w) * nzh;
      const float2* x2 = x1 + nzh;
      for (int k = lane; k < n; k += 32) {
        const int kk = k > n / 2 ? n - k : k;
        sa[k * PS + w] = combine(x1[kk], x2[kk], k, kk);
      }
    }
    __syncthreads();
    const float2* r = stages(sa, sb, stw);
    c2r_store<LW, PS>(r, out + line0 * n, n, nl, line0, alpha, beta, lineflag);
    return;
  }
  const float2* stw = stage_twiddles_to_smem(sm, PS, P);
  for (int w = warp; w < LW; w += NW) {
    const bool has1 = 2 * w < nl, has2 = 2 * w + 1 < nl;
    const float2* s1 = src + (long long)(2 * w) * nzp;
    const float2* s2 = s1 + nzp;
    // four positions of both half spectra in flight per thread before the stores
    for (int k0 = lane; k0 < n; k0 += 4 * 32) {
      float2 x1[4], x2[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int k = k0 + 32 * u;
        const int kk = k > n / 2 ? n - k : k;
        x1[u] = (has1 && k < n) ? __ldg(s1 + kk) : make_float2(0.f, 0.f);
        x2[u] = (has2 && k < n) ? __ldg(s2 + kk) : make_float2(0.f, 0.f);
      }
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int k = k0 + 32 * u;
        if (k >= n) break;
        const int kk = k > n / 2 ? n - k : k;
        sa[k * PS + w] = combine(x1[u], x2[u], k, kk);
      }
    }
  }
  __syncthreads();
  const float2* r = stages(sa, sb, stw);
  c2r_store<LW, PS>(r, out + line0 * n, n, nl, line0, alpha, beta, lineflag);
}

// ------------------------------------------- stages with compile-time shape
// tile_stage and last_stage with the radix R, the butterfly columns M = n / R
// and the span P as constants (the pass kernels compiled for one axis length):
// every shared-memory access of a butterfly is an immediate offset from one
// base address, and b mod P is a constant division.  Each butterfly performs
// the same operations as in tile_stage / last_stage.
template <int R, int M, int P, int LW, int PS, int NT>
SVIE_DEV void tile_stage_c(const float2* __restrict__ src, float2* __restrict__ dst, const float2* __restrict__ stw,
                           bool conj_in) {
  constexpr int total = LW * M;
  for (int j = threadIdx.x; j < total; j += NT) {
    const int l = j % LW, b = j / LW;
    const int k = (P == 1) ? 0 : b % P;
    const float2* s = src + b * PS + l;
    float2 v[R];
#pragma unroll
    for (int q = 0; q < R; ++q) v[q] = s[q * M * PS];
    if (conj_in) {
#pragma unroll
      for (int q = 0; q < R; ++q) v[q].y = -v[q].y;
    }
    if (k) {
      const float2* tk = stw + (P - 1) + k * (R - 1);
#pragma unroll
      for (int q = 1; q < R; ++q) v[q] = cmul(v[q], tk[q - 1]);
    }
    dft<R>(v);
    float2* d = dst + ((b - k) * R + k) * PS + l;
#pragma unroll
    for (int q = 0; q < R; ++q) d[q * P * PS] = v[q];
  }
  __syncthreads();
}

template <int R, int M, int LW, int PS, int NT, class Epi>
SVIE_DEV void last_stage_c(const float2* __restrict__ src, const float2* __restrict__ stw, bool conj_in,
                           const Epi& epi) {
  constexpr int total = LW * M;
  for (int j = threadIdx.x; j < total; j += NT) {
    const int l = j % LW, b = j / LW;
    const float2* s = src + b * PS + l;
    float2 v[R];
#pragma unroll
    for (int q = 0; q < R; ++q) v[q] = s[q * M * PS];
    if (conj_in) {
#pragma unroll
      for (int q = 0; q < R; ++q) v[q].y = -v[q].y;
    }
    if (b) {
      const float2* tk = stw + (M - 1) + b * (R - 1);
#pragma unroll
      for (int q = 1; q < R; ++q) v[q] = cmul(v[q], tk[q - 1]);
    }
    dft<R>(v);
    epi.template apply<R>(v, b, l, M);
  }
}

}  // namespace svie
