"""The convolution passes compiled at run time for one axis length: the generated sources of the
strided and z passes for a range of axis lengths (one to four radix stages, odd and even) compile
with NVRTC for sm_103a.
No device is needed; skipped when NVRTC cannot be loaded."""

import ctypes
from pathlib import Path

import pytest

from svierosion_gb300 import _native

CSRC = Path(_native.__file__).resolve().parent / "csrc"


def _nvrtc():
    for name in ("libnvrtc.so.13", "libnvrtc.so", "/usr/local/cuda/lib64/libnvrtc.so"):
        try:
            return ctypes.CDLL(name)
        except OSError:
            continue
    pytest.skip("NVRTC not available")


def _compile(nv, src: bytes):
    prog = ctypes.c_void_p()
    assert nv.nvrtcCreateProgram(ctypes.byref(prog), src, b"svie_jit_strided.cu", 0, None, None) == 0
    opts = [b"-arch=sm_103a", b"-std=c++17", b"-I" + str(CSRC).encode()]
    rc = nv.nvrtcCompileProgram(prog, len(opts), (ctypes.c_char_p * len(opts))(*opts))
    size = ctypes.c_size_t()
    nv.nvrtcGetProgramLogSize(prog, ctypes.byref(size))
    log = ctypes.create_string_buffer(size.value)
    nv.nvrtcGetProgramLog(prog, log)
    cubin = ctypes.c_size_t()
    if rc == 0:
        nv.nvrtcGetCUBINSize(prog, ctypes.byref(cubin))
    nv.nvrtcDestroyProgram(ctypes.byref(prog))
    return rc, log.value.decode(errors="replace"), cubin.value


# minb 0: the z passes (forward and inverse); else the 8-line strided pass for that many CTAs per SM
# (from 4 CTAs per SM the strided pass reads its stage twiddles from the plan)
@pytest.mark.parametrize("n,minb", [(336, 4), (336, 5), (448, 3), (448, 4), (245, 4), (90, 4), (7, 3), (1792, 3),
                                    (245, 0), (175, 0), (128, 0), (7, 0)])
def test_generated_pass_compiles(n, minb):
    lib = _native.lib()
    buf = ctypes.create_string_buffer(1 << 16)
    assert lib.svie_conv_jit_source(n, minb, buf, len(buf)) == 0
    src = buf.value
    assert (b"svie_jit_z_r2c" in src if minb == 0 else b"svie_jit_strided" in src) and b"_stage_c<" in src
    nv = _nvrtc()
    rc, log, cubin = _compile(nv, src)
    assert rc == 0 and cubin > 0, log[:2000]


def test_source_refuses_bad_lengths():
    lib = _native.lib()
    buf = ctypes.create_string_buffer(1 << 16)
    assert lib.svie_conv_jit_source(11, 4, buf, len(buf)) != 0       # not 2^a 3^b 5^c 7^d
    assert lib.svie_conv_jit_source(336, 4, buf, 16) != 0             # buffer too small
