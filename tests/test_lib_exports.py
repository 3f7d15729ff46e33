"""CPU checks of the C ABI: the library builds, loads and exports every symbol
that include/svie.h declares (no compute calls without a GPU)."""

import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


@pytest.fixture(scope="module")
def lib():
    from svierosion_gb300 import _native, build

    if not _native.LIB_PATH.exists():
        build.build()
    return _native.load()


def declared_functions():
    text = (ROOT / "include" / "svie.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(svie_\w+)\s*\(", text)))


def test_header_declares_the_boundary():
    names = declared_functions()
    assert "svie_stage_svi" in names and "svie_conv_apply" in names and "svie_band_scan" in names
    assert len(names) >= 50


def test_every_declared_symbol_is_exported(lib):
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_binding_table_matches_header(lib):
    from svierosion_gb300 import _native

    declared = set(declared_functions())
    bound = set(_native.exported_names())
    assert bound <= declared, bound - declared


def test_size_queries_without_gpu(lib):
    assert lib.svie_version() == 1
    assert lib.svie_conv_spectrum_row(245) == 128
    assert lib.svie_conv_supported(448) == 1 and lib.svie_conv_supported(11) == 0
    assert lib.svie_ball_half_width(0.1, 1 / 64) == 7
    assert lib.svie_conv_workspace_bytes(448, 336, 245) >= 448 * 336 * 123 * 8
    assert lib.svie_band_workspace_bytes(1 << 20) > 0
    assert lib.svie_conv_supported(7168) == 1 and lib.svie_conv_supported(7200) == 0


def test_fft_form_table_without_gpu(lib):
    """The per-shape table of pass forms (host only, no launch): the fixed rule, set, refuse, clear."""
    import ctypes
    z, y, x = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    get = lambda *s: (lib.svie_conv_get_choice(*s, ctypes.byref(z), ctypes.byref(y), ctypes.byref(x)),
                      z.value, y.value, x.value)
    assert get(448, 336, 245) == (0, 0, 1, 0)
    # an x axis too long for 8-line tiles and a z axis too long for 16 line pairs: one-line forms
    assert get(7168, 336, 7168) == (0, 2, 1, 2)
    assert lib.svie_conv_set_choice(448, 336, 245, 1, 2, 1) == 0
    assert get(448, 336, 245) == (1, 1, 2, 1)
    assert lib.svie_conv_set_choice(448, 336, 245, 0, 3, 0) != 0
    assert lib.svie_conv_set_choice(7168, 336, 245, 0, 0, 0) != 0   # 8-line x tiles do not fit
    assert lib.svie_conv_set_choice(448, 336, 245, -1, 0, 0) == 0
    assert get(448, 336, 245) == (0, 0, 1, 0)


def test_compile_worker_stop_without_gpu(lib):
    """Stopping the compile worker when none was started returns at once (the interpreter-exit hook
    runs it in every process that loaded the library), and may be repeated.  In a child process:
    a stopped worker refuses later compilations for the rest of its process."""
    import subprocess
    import sys
    code = ("import sys, time; sys.path.insert(0, sys.argv[1]); from svierosion_gb300 import _native as n; "
            "l = n.load(); t0 = time.time(); assert l.svie_conv_jit_stop() == 0 and l.svie_conv_jit_stop() == 0; "
            "assert time.time() - t0 < 1.0")
    r = subprocess.run([sys.executable, "-c", code, str(ROOT)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr[-2000:]


def test_no_cpu_fallback():
    import torch
    import svierosion_gb300 as S
    from svierosion_gb300 import kernels as K

    flat = torch.zeros(1000)
    with pytest.raises((ValueError, RuntimeError)):
        K.godunov_inward(flat, torch.arange(10), 100, 10, 1, 1.0)
    if not torch.cuda.is_available():
        with pytest.raises(RuntimeError):
            S.get_device()


def test_status_codes_match_header():
    import re

    from svierosion_gb300 import _native as nat

    text = (ROOT / "include" / "svie.h").read_text()
    codes = dict(re.findall(r"#define (SVIE_(?:OK|ERR_[A-Z]+)) (\d+)", text))
    assert len(codes) == 7
    for name, value in codes.items():
        assert getattr(nat, name) == int(value), name
