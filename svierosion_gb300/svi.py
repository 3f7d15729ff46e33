"""Spherical volume invariant N_r by FFT convolution (reference svierosion/svi.py).

``N_r(x) = 1 - h^3 (w * f)(x) / |B_r|`` with ``w`` the exact ball/cell overlap
fractions (float64, computed on the GPU) and ``f`` the cell occupancy.  The
convolution is the package's own mixed-radix R2C/C2R FFT with the kernel
spectrum multiply fused into the x pass (csrc/fft.cu).
"""

from __future__ import annotations

import json
import math
import os
from collections import OrderedDict
from pathlib import Path

import numpy as np
import torch

from . import _native as nat
from .grid import Grid, get_device


def ball_cell_weights(radius: float, spacing: float, quad: int = 32) -> np.ndarray:
    """Exact fractions |B_r(0) cap cell(i,j,k)| / h^3 for |i|,|j|,|k| <= m (svi.py:24-55)."""
    w = _ball_weights_device(radius, spacing, quad, get_device())
    return w.cpu().numpy()


_WEIGHTS_CACHE: "OrderedDict[tuple, tuple]" = OrderedDict()
_WEIGHTS_CACHE_SIZE = 16


def _ball_weights_device(radius, spacing, quad, device) -> torch.Tensor:
    """Device ball weights, computed once per (radius, spacing, quad, device) and kept read-only.

    Solids of one served stream share the same few radii and spacings; the
    cache entry carries an event so that a reader on another stream waits
    for the producing kernel."""
    key = (float(radius), float(spacing), int(quad), torch.device(device).index)
    hit = _WEIGHTS_CACHE.get(key)
    if hit is not None:
        _WEIGHTS_CACHE.move_to_end(key)
        w, ev = hit
        torch.cuda.current_stream(w.device).wait_event(ev)
        return w
    m = nat.lib().svie_ball_half_width(float(radius), float(spacing))
    if m < 1:
        raise ValueError("radius and spacing must be positive")
    side = 2 * m + 1
    w = torch.empty((side, side, side), dtype=torch.float64, device=device)
    nat.call("svie_ball_weights", float(radius), float(spacing), int(quad), nat.ptr(w), nat.stream())
    ev = torch.cuda.Event()
    ev.record(torch.cuda.current_stream(w.device))
    _WEIGHTS_CACHE[key] = (w, ev)
    while len(_WEIGHTS_CACHE) > _WEIGHTS_CACHE_SIZE:
        _WEIGHTS_CACHE.popitem(last=False)
    return w


# grid shapes whose pass forms were timed in this process, per device (svie_conv_tune)
_TUNED: set = set()
TUNE_REPS = 2
# Tuning costs a few milliseconds once per shape (8.6 ms at 448 x 336 x 245, about 1 ms at
# 160 x 120 x 90): by default only grids of at least this many nodes are tuned, where that is
# a small part of one solve; smaller ones keep the fixed rule.
TUNE_MIN_NODES = 1 << 23


def autotune_enabled(nodes: int | None = None) -> bool:
    """Whether a grid of `nodes` nodes is tuned at its first convolution: SVIE_FFT_TUNE=0 never,
    =all always, otherwise (default) from TUNE_MIN_NODES nodes up."""
    mode = os.environ.get("SVIE_FFT_TUNE", "1")
    if mode == "0":
        return False
    return mode == "all" or nodes is None or nodes >= TUNE_MIN_NODES


def jit_enabled(nodes: int | None = None) -> bool:
    """Whether a grid of `nodes` nodes gets its y and x passes compiled for its axis lengths at its
    first convolution (svie_conv_jit): SVIE_FFT_JIT=0 never, =all always, otherwise (default) from
    TUNE_MIN_NODES nodes up (a compilation takes about a second per axis length)."""
    mode = os.environ.get("SVIE_FFT_JIT", "1")
    if mode == "0":
        return False
    return mode == "all" or nodes is None or nodes >= TUNE_MIN_NODES


def _cache_path():
    """SVIE_FFT_TUNE_CACHE: a JSON file of tuned pass forms kept across processes (unset: none)."""
    p = os.environ.get("SVIE_FFT_TUNE_CACHE")
    return Path(p) if p else None


def _cache_key(device, shape) -> str:
    return f"{torch.cuda.get_device_name(device)}|{'x'.join(str(int(n)) for n in shape)}"


def load_tuned_forms(device, shape) -> bool:
    """Set the forms of `shape` from the tuning cache file when it holds them for this GPU model."""
    path = _cache_path()
    if path is None or not path.exists():
        return False
    try:
        forms = json.loads(path.read_text()).get(_cache_key(device, shape))
    except (OSError, ValueError):
        return False
    if not forms:
        return False
    try:
        set_fft_choice(shape, forms["z"], forms["y"], forms["x"], device)
    except (nat.SvieError, KeyError, TypeError):
        return False
    return True


def save_tuned_forms(device, shape) -> None:
    """Record the forms the tuner kept for `shape` in the tuning cache file (when one is set)."""
    path = _cache_path()
    if path is None:
        return
    try:
        table = json.loads(path.read_text()) if path.exists() else {}
    except (OSError, ValueError):
        table = {}
    c = fft_choice(shape)
    table[_cache_key(device, shape)] = {"z": c["z"], "y": c["y"], "x": c["x"]}
    tmp = path.with_name(path.name + ".tmp")
    tmp.write_text(json.dumps(table, indent=1, sort_keys=True) + "\n")
    tmp.replace(path)


def fft_choice(shape) -> dict:
    """The launch forms the convolution passes use on `shape` (indices as in svie_conv_get_choice)
    and whether they were tuned or set."""
    z, y, x = (nat.ctypes.c_int() for _ in range(3))
    tuned = nat.lib().svie_conv_get_choice(*(int(n) for n in shape), nat.ctypes.byref(z), nat.ctypes.byref(y),
                                           nat.ctypes.byref(x))
    return {"z": z.value, "y": y.value, "x": x.value, "tuned": bool(tuned)}


def set_fft_choice(shape, z: int, y: int, x: int, device=None) -> None:
    """Force the pass forms on `shape` (negative values return to tuning at the next first use)."""
    nat.call("svie_conv_set_choice", *(int(n) for n in shape), int(z), int(y), int(x))
    key = (torch.device(get_device(device)).index, tuple(int(n) for n in shape))
    if z < 0 or y < 0 or x < 0:
        _TUNED.discard(key)
    else:
        _TUNED.add(key)


class BallConvolution:
    """Cached kernel spectrum on a grid; evaluates interior ball volumes (svi.py:58-93)."""

    def __init__(self, grid: Grid, radius: float, device=None, quad: int = 32, scratch=None):
        self.grid = grid
        self.radius = float(radius)
        self.device = get_device(device)
        w = _ball_weights_device(radius, grid.spacing, quad, self.device)
        self.m = (w.shape[0] - 1) // 2
        self.ball_volume = 4.0 / 3.0 * math.pi * radius ** 3
        self.quadrature_volume = float(w.sum()) * grid.spacing ** 3
        if any(2 * self.m + 1 > n for n in grid.shape):
            raise ValueError("ball kernel larger than the grid")
        L = nat.lib()
        if not all(L.svie_conv_supported(int(n)) for n in grid.shape):
            raise ValueError(f"grid {grid.shape}: every dimension must be 2^a 3^b 5^c 7^d and <= 7168 "
                             "(use Grid.around(..., fast=True))")
        nx, ny, nz = grid.shape
        self.plan = torch.empty(L.svie_conv_plan_bytes(nx, ny, nz), dtype=torch.uint8, device=self.device)
        init_ws = torch.empty(L.svie_conv_init_workspace_bytes(nx, ny, nz, self.m), dtype=torch.uint8,
                              device=self.device)
        nat.call("svie_conv_plan_init", nat.ptr(self.plan), nx, ny, nz, nat.ptr(w), self.m, nat.ptr(init_ws),
                 init_ws.numel(), nat.stream())
        del init_ws
        self.workspace_bytes = L.svie_conv_workspace_bytes(nx, ny, nz)
        self.scratch = scratch if scratch is not None else nat.Scratch(self.device)
        self._khat = None

    @property
    def kernel_hat(self) -> torch.Tensor:
        """complex64 [nx, ny, nz/2+1] spectrum of the wrapped kernel (svi.py:76-81)."""
        if self._khat is None:
            nx, ny, nz = self.grid.shape
            k = torch.empty((nx, ny, nz // 2 + 1), dtype=torch.complex64, device=self.device)
            nat.call("svie_conv_kernel_hat", nat.ptr(self.plan), nx, ny, nz, nat.ptr(k), nat.stream())
            self._khat = k
        return self._khat

    def apply_into(self, f: torch.Tensor, out: torch.Tensor, alpha: float, beta: float, events=None,
                   flags=None) -> torch.Tensor:
        """out = beta + alpha * G * (w (*) f), G = number of nodes (unnormalised FFT pair).

        ``events``: optional six timing events recorded around the five passes;
        ``flags``: optional (lineflag, slabflag) from svie_conv_line_flags -- then
        only the N values that stencils at band closest points read are valid."""
        nx, ny, nz = self.grid.shape
        f = f.reshape(-1)
        if f.dtype != torch.float32 or not f.is_contiguous():
            f = f.to(torch.float32).contiguous()
        ws = self.scratch.get("conv", self.workspace_bytes)
        self._tune(f, out, ws)
        if events is None and flags is None:
            nat.call("svie_conv_apply", nat.ptr(self.plan), nx, ny, nz, nat.ptr(f), nat.ptr(out.view(-1)),
                     float(alpha), float(beta), nat.ptr(ws), ws.numel(), nat.stream())
        else:
            from .profiling import KernelTimer
            lf, sf = flags if flags is not None else (None, None)
            ev = KernelTimer.handles(events) if events is not None else None
            nat.call("svie_conv_apply_masked", nat.ptr(self.plan), nx, ny, nz, nat.ptr(f), nat.ptr(out.view(-1)),
                     float(alpha), float(beta), nat.ptr(ws), ws.numel(), nat.ptr(lf), nat.ptr(sf), ev, nat.stream())
        return out

    def _tune(self, f, out, ws) -> None:
        """Once per grid shape and process (not while a graph is captured): compile the passes for
        the shape's axis lengths (jit_enabled) and keep the fixed rule's forms, the ones those
        passes serve; without them, time the pass forms, or take them from the tuning cache file
        (SVIE_FFT_TUNE_CACHE) when it holds this GPU model and shape; newly tuned forms are added
        to that file."""
        key = (self.device.index, tuple(self.grid.shape))
        if key in _TUNED or torch.cuda.is_current_stream_capturing():
            return
        nx, ny, nz = self.grid.shape
        lib = nat.lib()
        if jit_enabled(self.grid.size):
            if not lib.svie_conv_jit_enabled(nx, ny, nz):
                # the passes compiled for these axis lengths; on failure the library's own passes stay
                lib.svie_conv_jit(nx, ny, nz)
            if lib.svie_conv_jit_enabled(nx, ny, nz) and not lib.svie_conv_get_choice(nx, ny, nz, None, None, None):
                # timing now would measure the library's passes (the compiled ones are still being
                # built) and could pick a form that has no compiled pass, a fifth slower
                _TUNED.add(key)
                return
        if not autotune_enabled(self.grid.size):
            _TUNED.add(key)
            return
        if load_tuned_forms(self.device, self.grid.shape):
            return
        nat.call("svie_conv_tune", nat.ptr(self.plan), nx, ny, nz, nat.ptr(f), nat.ptr(out.view(-1)), nat.ptr(ws),
                 ws.numel(), TUNE_REPS, nat.stream())
        _TUNED.add(key)
        save_tuned_forms(self.device, self.grid.shape)

    def interior_volume(self, fractions: torch.Tensor) -> torch.Tensor:
        """Dense |B_r(x) cap Omega| (svi.py:84-88)."""
        out = torch.empty(self.grid.shape, dtype=torch.float32, device=self.device)
        return self.apply_into(fractions, out, self.grid.spacing ** 3 / self.grid.size, 0.0)

    def exterior_fraction(self, fractions: torch.Tensor) -> torch.Tensor:
        """Dense N_r(x) = 1 - |B_r(x) cap Omega| / |B_r| (svi.py:90-93)."""
        out = torch.empty(self.grid.shape, dtype=torch.float32, device=self.device)
        return self.exterior_fraction_into(fractions, out)

    def exterior_fraction_into(self, fractions: torch.Tensor, out: torch.Tensor, events=None,
                               flags=None) -> torch.Tensor:
        a = -self.grid.spacing ** 3 / (self.ball_volume * self.grid.size)
        return self.apply_into(fractions, out, a, 1.0, events=events, flags=flags)


def sphere_exterior_fraction(radius_ball: float, radius_sphere: float) -> float:
    """Exact N_r at a point of a sphere of radius R (svi.py:96-101)."""
    r, R = radius_ball, radius_sphere
    if r > 2 * R:
        return 1.0 - (R / r) ** 3
    return 0.5 + 3.0 * r / (16.0 * R)


def rfftn(f: torch.Tensor, conv: BallConvolution) -> torch.Tensor:
    """Forward 3-D real FFT with the package's kernels; complex64 [nx, ny, nz/2+1]."""
    nx, ny, nz = conv.grid.shape
    row = nat.lib().svie_conv_spectrum_row(nz)
    spec = torch.empty((nx, ny, row), dtype=torch.complex64, device=conv.device)
    f = f.reshape(-1).to(torch.float32).contiguous()
    nat.call("svie_rfft3", nat.ptr(conv.plan), nx, ny, nz, nat.ptr(f), nat.ptr(spec), nat.stream())
    return spec[:, :, : nz // 2 + 1]


def irfftn(spec: torch.Tensor, conv: BallConvolution) -> torch.Tensor:
    """Inverse of :func:`rfftn` (normalised like torch.fft.irfftn)."""
    nx, ny, nz = conv.grid.shape
    row = nat.lib().svie_conv_spectrum_row(nz)
    buf = torch.zeros((nx, ny, row), dtype=torch.complex64, device=conv.device)
    buf[:, :, : nz // 2 + 1] = spec
    out = torch.empty(conv.grid.shape, dtype=torch.float32, device=conv.device)
    nat.call("svie_irfft3", nat.ptr(conv.plan), nx, ny, nz, nat.ptr(buf), nat.ptr(out), 1.0 / conv.grid.size, 0.0,
             nat.stream())
    return out
