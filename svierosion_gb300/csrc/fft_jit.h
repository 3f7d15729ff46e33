// Convolution pass kernels compiled at run time for one axis length (fft_jit.cu).
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>

#include <string>

namespace svie {

// The 8-line strided pass (k_fft_strided<8, minb>) compiled for an axis of n
// positions with the given radix sequence (4 bits per stage), in the current
// context.  SVIE_OK and *fn once it is loaded; until then (its compilation
// starts on a background thread at the first request) and when it cannot be
// made, an error status with *fn = null.
int jit_strided(int n, int minb, unsigned long long radices, int nst, CUfunction* fn);

// CTAs per SM of the compiled y and x passes.  From 4 up a compiled pass reads
// its stage twiddles from the plan instead of shared memory (its tiles need 16 n
// float2 only): five y tiles of n = 336 then fit.  The x passes keep theirs in
// shared memory at three CTAs per SM (four, with the twiddles from the plan,
// measured no faster).
constexpr int JIT_Y_MINB = 5, JIT_X_MINB = 3;

// The z passes (16 line pairs per CTA) compiled for an axis of n positions:
// the forward (R2C) and inverse (C2R) kernels of one module.
int jit_z(int n, unsigned long long radices, int nst, CUfunction* r2c, CUfunction* c2r);

// NVRTC and the driver functions were found.
bool jit_available();

// Waits up to timeout_ms for every compilation started so far (SVIE_OK when
// none is still running).
int jit_wait(int timeout_ms);

// Drops the queued compilations, waits (at most 10 s) for the one in progress
// and joins the worker; later requests are refused.  For a host's exit path.
void jit_stop();

// Launches a compiled pass on `s` (a dependent launch when `chained`); false
// when the launch failed (the caller then launches the library's pass).
bool jit_launch(CUfunction fn, dim3 grid, dim3 block, size_t smem, cudaStream_t s, bool chained, void** args);

// The generated source (for the CPU test that compiles it).
std::string jit_strided_source_for_test(int n, int minb, unsigned long long radices, int nst);
std::string jit_z_source_for_test(int n, unsigned long long radices, int nst);

}  // namespace svie
