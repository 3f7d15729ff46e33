"""Narrow-band level set on a CUDA device (reference svierosion/levelset.py).

``phi`` is a dense float32 CUDA tensor (negative inside), the band is the
ascending list of flat indices with ``|phi| < width * h`` (clamped to
``+-width * h`` elsewhere), at least :data:`MARGIN` cells from the boundary.
Besides the reference's state the level set keeps, for the fused stages:

* ``band32`` -- the band as int32 (``band`` is the int64 view of the API);
* ``work32`` -- the same nodes in brick order (4 x 4 x 16 bricks), the order
  in which the stencil kernels visit them;
* ``occ``    -- the dense occupancy ``(phi < 0)`` with the band's cell
  fractions, maintained incrementally: off the band phi only changes at a
  band rebuild, so only band entries are rewritten between rebuilds;
* ``static_inside`` -- the number of nodes off the band with ``phi < 0``,
  which turns the solid volume into a band-only float64 reduction.
"""

from __future__ import annotations

import numpy as np
import torch

from . import _native as nat
from .grid import Grid, get_device

MARGIN = 4  # cells between any band node and the grid boundary (levelset.py:22)


def dilate(mask: torch.Tensor, steps: int = 1) -> torch.Tensor:
    """Binary dilation by the (2 steps + 1)^3 box (levelset.py:25-34)."""
    m = mask.to(torch.uint8).contiguous()
    out = torch.empty_like(m)
    tmp = torch.empty_like(m)
    nx, ny, nz = m.shape
    nat.call("svie_dilate", nat.ptr(m), nx, ny, nz, int(steps), nat.ptr(out), nat.ptr(tmp), nat.stream())
    return out.view(torch.bool)


def cube_plane_fraction(s, a, b, c):
    """Volume fraction of the unit cube below a plane (levelset.py:37-48)."""
    from .kernels import cube_plane_fraction as f
    return f(s, a, b, c)


def _read(t: torch.Tensor, dtype: np.dtype):
    return np.frombuffer(t.cpu().numpy().tobytes(), dtype=dtype)[0]


class LevelSet:
    """A level set function with an explicitly stored narrow band (levelset.py:51-183)."""

    def __init__(self, phi: torch.Tensor, grid: Grid, width: float = 6.0, scratch: nat.Scratch | None = None):
        if tuple(phi.shape) != tuple(grid.shape):
            raise ValueError("phi shape does not match grid")
        if grid.size >= 2 ** 31:
            raise ValueError("grids are limited to 2^31 nodes (int32 node indices)")
        self.grid = grid
        self.h = float(grid.spacing)
        self.width = float(width)
        dev = phi.device if phi.is_cuda else get_device()
        self.phi = phi.to(device=dev, dtype=torch.float32).contiguous()
        self.device = self.phi.device
        # workspaces of this level set (and of the simulation that evolves it):
        # one set per instance, so that solids on different streams never share
        self.scratch = scratch if scratch is not None else nat.Scratch(self.device)
        self.strides = tuple(int(s) for s in grid.strides)
        self.occ = torch.empty(grid.size, dtype=torch.float32, device=self.device)
        self.occ_current = False
        self._info = torch.zeros(nat.BAND_INFO_BYTES, dtype=torch.uint8, device=self.device)
        self._vstats = torch.zeros(nat.STATS_BYTES, dtype=torch.uint8, device=self.device)
        self._band64 = None
        self._band32 = None
        self.last_flags = (1, 1)
        self.rebuild_band()

    # ------------------------------------------------------------ band
    @property
    def flat(self) -> torch.Tensor:
        return self.phi.view(-1)

    @property
    def work32(self) -> torch.Tensor:
        """The band in brick order (int32), the list the stencil kernels visit."""
        return self._work32

    @work32.setter
    def work32(self, idx: torch.Tensor) -> None:
        self._work32 = idx
        # counts the band's replacements: a rebuilt list may reuse the old one's memory and
        # size, so users key cached per-band data on this instead of the pointer alone
        self.band_generation = getattr(self, "band_generation", 0) + 1

    @property
    def band32(self) -> torch.Tensor:
        """The band in ascending flat order (int32), listed on first use after a rebuild."""
        if self._band32 is None:
            self._band32 = self._ascending_band()
        return self._band32

    @band32.setter
    def band32(self, idx: torch.Tensor) -> None:
        self._band32 = idx

    @property
    def band(self) -> torch.Tensor:
        """Band as int64 flat indices (the reference's dtype)."""
        if self._band64 is None:
            self._band64 = self.band32.to(torch.int64)
        return self._band64

    @band.setter
    def band(self, idx: torch.Tensor) -> None:
        self.band32 = idx.to(device=self.device, dtype=torch.int32).contiguous()
        self.work32 = self.band32
        self._band64 = None
        self.occ_current = False

    def _thresh(self):
        cap = self.width * self.h
        return nat.f32(cap), nat.f32(cap * (1 - 1e-5))

    def rebuild_band(self) -> None:
        """Clamp phi to +-width*h and list |phi| < width*h (1 - 1e-5) (levelset.py:70-77).

        The stencil kernels take the brick-ordered list ``work32``; the
        ascending list of the API (``band32`` / ``band``) is made on demand."""
        cap, thresh = self._thresh()
        nx, ny, nz = self.grid.shape
        sc = self.scratch
        bws = sc.get("brick", nat.lib().svie_brick_workspace_bytes(nx, ny, nz))
        nat.call("svie_brick_band_scan", nat.ptr(self.flat), nx, ny, nz, cap, thresh, nat.ptr(bws), bws.numel(),
                 nat.ptr(self._info), nat.stream())
        count = int(_read(self._info, nat.BAND_INFO_DTYPE)["count"])
        work = torch.empty(count, dtype=torch.int32, device=self.device)
        nat.call("svie_brick_band_write", nat.ptr(self.flat), nx, ny, nz, thresh, nat.ptr(bws), bws.numel(),
                 nat.ptr(work), count, nat.ptr(self.occ), nat.ptr(self._info), nat.stream())
        info = _read(self._info, nat.BAND_INFO_DTYPE)
        self.work32 = work
        self._band32 = None
        self._band64 = None
        self.static_inside = int(info["static_inside"])
        self.band_lo = tuple(int(v) for v in info["lo"])
        self.band_hi = tuple(int(v) for v in info["hi"])
        self.inside_lo = tuple(int(v) for v in info["ilo"])
        self.inside_hi = tuple(int(v) for v in info["ihi"])
        self.occ_current = False
        if count:
            shape = self.grid.shape
            for ax in range(3):
                if self.band_lo[ax] < MARGIN or self.band_hi[ax] > shape[ax] - 1 - MARGIN:
                    raise RuntimeError("narrow band reaches the grid boundary; enlarge the padding")

    def _ascending_band(self) -> torch.Tensor:
        """The nodes of ``work32`` (the band of the last rebuild) in ascending flat order."""
        n = self.grid.size
        nx, ny, nz = self.grid.shape
        m = self.work32.numel()
        if m == 0:
            return torch.empty(0, dtype=torch.int32, device=self.device)
        sc = self.scratch
        mask = sc.get("reinit_mask", n)
        tmp = sc.get("reinit_tmp", n)
        nat.call("svie_reinit_mask", nat.ptr(self.work32), m, nx, ny, nz, 0, 0, nat.ptr(mask), nat.ptr(tmp),
                 nat.stream())
        ws = sc.get("band", nat.lib().svie_band_workspace_bytes(n))
        cnt = sc.get("band_count", 8)
        nat.call("svie_mask_scan", nat.ptr(mask), n, nat.ptr(ws), ws.numel(), nat.ptr(cnt), nat.stream())
        band = torch.empty(m, dtype=torch.int32, device=self.device)
        nat.call("svie_mask_write", nat.ptr(mask), n, nat.ptr(ws), ws.numel(), nat.ptr(band), m, nat.stream())
        return band

    def interface_nodes(self, idx: torch.Tensor | None = None) -> torch.Tensor:
        """Band nodes having a 6-neighbour of the opposite sign (levelset.py:88-91)."""
        from .kernels import interface_mask
        idx32 = self.band32 if idx is None else idx.to(torch.int32).contiguous()
        m = idx32.numel()
        if m == 0:
            return torch.empty(0, dtype=torch.int64, device=self.device)
        mask = interface_mask(self.flat, idx32, *self.strides).view(torch.uint8)
        sc = self.scratch
        ws = sc.get("select", nat.lib().svie_band_workspace_bytes(m))
        cnt = sc.get("select_count", 8)
        nat.call("svie_mask_scan", nat.ptr(mask), m, nat.ptr(ws), ws.numel(), nat.ptr(cnt), nat.stream())
        k = int(cnt[:8].cpu().view(torch.int64)[0])
        out = torch.empty(k, dtype=torch.int32, device=self.device)
        nat.call("svie_mask_select", nat.ptr(mask), nat.ptr(idx32), m, nat.ptr(ws), ws.numel(), nat.ptr(out), k,
                 nat.stream())
        return out.to(torch.int64)

    def _volume_kernel(self, write_occ: bool):
        sc = self.scratch
        m = self.work32.numel()
        ws = sc.get("volume", nat.lib().svie_volume_workspace_bytes(m))
        nat.call("svie_band_volume", nat.ptr(self.flat), nat.ptr(self.work32), m, *self.strides,
                 nat.ptr(self.occ) if write_occ else None, nat.ptr(ws), ws.numel(), nat.ptr(self._vstats),
                 nat.stream())
        if write_occ:
            self.occ_current = True

    def has_interface(self) -> bool:
        """Band has both signs (levelset.py:93-95)."""
        self._volume_kernel(False)
        st = _read(self._vstats, nat.STATS_DTYPE)
        return bool(st["any_neg"]) and bool(st["any_pos"])

    # ---------------------------------------------------- derivatives
    def central_gradient(self, idx: torch.Tensor) -> torch.Tensor:
        """Second-order central gradient in phi per cell, (m, 3) (levelset.py:98-101)."""
        i = idx.to(torch.int32).contiguous()
        out = torch.empty((i.numel(), 3), dtype=torch.float32, device=self.device)
        nat.call("svie_central_gradient", nat.ptr(self.flat), nat.ptr(i), i.numel(), *self.strides, nat.ptr(out),
                 nat.stream())
        return out

    def godunov_norm_inward(self, idx: torch.Tensor) -> torch.Tensor:
        from .kernels import godunov_inward
        return godunov_inward(self.flat, idx, *self.strides, 1.0 / self.h)

    def principal_curvatures(self, idx: torch.Tensor):
        from .kernels import principal_curvatures
        return principal_curvatures(self.flat, idx, *self.strides, self.h)

    # ------------------------------------------------- volume fractions
    def cell_fractions(self, idx: torch.Tensor | None = None) -> torch.Tensor:
        from .kernels import cell_fractions
        return cell_fractions(self.flat, self.band32 if idx is None else idx, *self.strides)

    def dense_fractions(self) -> torch.Tensor:
        """Dense occupancy field (levelset.py:117-121), recomputed from phi."""
        f = torch.empty(self.grid.size, dtype=torch.float32, device=self.device)
        nat.call("svie_dense_occupancy", nat.ptr(self.flat), self.grid.size, nat.ptr(f), nat.stream())
        nat.call("svie_scatter_fractions", nat.ptr(self.flat), nat.ptr(self.work32), self.work32.numel(),
                 *self.strides, nat.ptr(f), nat.stream())
        return f.view(self.grid.shape)

    def refresh_occupancy(self) -> None:
        """Bring the maintained occupancy up to date with the band values."""
        if not self.occ_current:
            nat.call("svie_scatter_fractions", nat.ptr(self.flat), nat.ptr(self.work32), self.work32.numel(),
                     *self.strides, nat.ptr(self.occ), nat.stream())
            self.occ_current = True

    def volume_async(self) -> None:
        """Launch the band volume reduction (result in the volume stats)."""
        self._volume_kernel(True)

    def volume_from_stats(self, st) -> float:
        return (self.static_inside + float(st["fsum"])) * self.h ** 3

    def band_values(self) -> torch.Tensor:
        """phi at the band nodes in ascending order (the reference's ``flat[band]``)."""
        b = self.band32
        out = torch.empty(b.numel(), dtype=torch.float32, device=self.device)
        nat.call("svie_gather", nat.ptr(self.flat), nat.ptr(b), b.numel(), nat.ptr(out), nat.stream())
        return out

    def volume(self) -> float:
        """Solid volume (levelset.py:123-126): off-band inside count + float64 sum of band fractions."""
        self._volume_kernel(True)
        st = _read(self._vstats, nat.STATS_DTYPE)
        self.last_flags = (int(st["any_neg"]), int(st["any_pos"]))
        return self.volume_from_stats(st)

    # ----------------------------------------------------- projection
    def closest_points(self, idx: torch.Tensor, newton_steps: int = 1) -> torch.Tensor:
        """Projection of nodes onto the zero level set, index coordinates (levelset.py:129-146)."""
        nx, ny, nz = self.grid.shape
        i = idx.to(torch.int32).contiguous()
        out = torch.empty((i.numel(), 3), dtype=torch.float32, device=self.device)
        nat.call("svie_closest_points_newton", nat.ptr(self.flat), nat.ptr(i), i.numel(), ny, nz, nx - 3.001,
                 ny - 3.001, nz - 3.001, self.h, int(newton_steps), nat.ptr(out), nat.stream())
        return out

    # --------------------------------------------------- reinitialisation
    def reinitialize(self, iterations: int = 12, cfl: float = 0.45, dilation: int = 3, timer=None,
                     work_set_rebuild: bool = False) -> None:
        """Subcell-fixed PDE reinitialisation (Min 2010) on the dilated band (levelset.py:154-183).

        ``timer`` (optional profiling.KernelTimer): events around the sweeps
        ("reinit_sweep", 2 iterations launches) and the work-set size.

        ``work_set_rebuild``: rebuild the band over the work set only, for a phi
        that changed only on the band since the last rebuild (the evolution
        loop's case).  Off the work set phi is then unchanged and clamped, so
        the band, its order, phi, the occupancy and ``static_inside`` equal the
        full rebuild's; the inside box becomes the old box joined with the work
        set's inside nodes (a box that contains the exact one)."""
        n = self.grid.size
        nx, ny, nz = self.grid.shape
        sc = self.scratch
        lib = nat.lib()
        fast = work_set_rebuild and dilation <= 31
        # the work mask (band dilated, margin cleared) as bits, listed in brick order
        marked = None
        if dilation <= 31:
            kind, nbytes = 2, lib.svie_reinit_bits_bytes(nx, ny, nz)
            mask, tmp = sc.get("reinit_mask", nbytes), sc.get("reinit_tmp", nbytes)
            if fast:
                marked = sc.get("reinit_marked", nbytes)  # the band's own bits, kept
            nat.call("svie_reinit_bits", nat.ptr(self.work32), self.work32.numel(), nx, ny, nz, int(dilation), MARGIN,
                     nat.ptr(mask), nat.ptr(tmp), nat.ptr(marked), nat.stream())
        else:
            kind = 0
            mask, tmp = sc.get("reinit_mask", n), sc.get("reinit_tmp", n)
            nat.call("svie_reinit_mask", nat.ptr(self.work32), self.work32.numel(), nx, ny, nz, int(dilation), MARGIN,
                     nat.ptr(mask), nat.ptr(tmp), nat.stream())
        ws = sc.get("brick", lib.svie_brick_workspace_bytes(nx, ny, nz))
        cnt = sc.get("reinit_count", 8)
        nat.call("svie_brick_scan", kind, nat.ptr(mask), nx, ny, nz, 0.0, nat.ptr(ws), ws.numel(), nat.ptr(cnt),
                 nat.stream())
        m = int(cnt[:8].cpu().view(torch.int64)[0])
        idx = sc.get("reinit_idx", 4 * max(m, 1))[:4 * m].view(torch.int32)
        nat.call("svie_brick_write", kind, nat.ptr(mask), nx, ny, nz, 0.0, nat.ptr(ws), ws.numel(), nat.ptr(idx), m,
                 nat.stream())
        geo = sc.get("reinit_geo", lib.svie_reinit_geometry_bytes(m))
        nat.call("svie_reinit_geometry", nat.ptr(self.flat), nat.ptr(idx), m, *self.strides, self.h, cfl,
                 nat.ptr(geo), nat.stream())
        off_inside = None
        if fast:
            # inside work-set nodes off the old band, before the sweeps
            off_inside = sc.get("reinit_off_inside", 8)
            nat.call("svie_list_inside_off_mask", nat.ptr(self.flat), nat.ptr(idx), m, nat.ptr(marked), nx, ny, nz,
                     nat.ptr(off_inside), nat.stream())
        phi_tmp = sc.get("reinit_phi", 4 * n)
        timed = timer is not None and timer.wants("reinit_sweep") and m > 0 and iterations > 0
        if timed:
            ev = timer.take(2)
            ev[0].record()
        nat.call("svie_reinit_iterate", nat.ptr(self.flat), nat.ptr(phi_tmp), n, nat.ptr(idx), m, *self.strides,
                 self.h, nat.ptr(geo), int(iterations), nat.stream())
        if timed:
            ev[1].record()
            timer.add(["reinit_sweep"], ev, [2 * int(iterations)])
            timer.note("reinit_work", m)
        if fast:
            self.rebuild_band_on(idx, off_inside)
        else:
            self.rebuild_band()

    def rebuild_band_on(self, idx: torch.Tensor, off_inside: torch.Tensor) -> None:
        """rebuild_band over the node list ``idx`` (the work set), valid when phi
        changed only on it since the last rebuild; ``off_inside`` (device int64)
        holds the listed nodes that were inside and off the old band before phi
        changed, so that ``static_inside`` stays exact."""
        cap, thresh = self._thresh()
        nx, ny, nz = self.grid.shape
        m = idx.numel()
        lib = nat.lib()
        ws = self.scratch.get("list", lib.svie_list_workspace_bytes(m))
        nat.call("svie_list_band_scan", nat.ptr(self.flat), nat.ptr(idx), m, cap, thresh, nat.ptr(ws), ws.numel(),
                 nat.ptr(self._info), nat.stream())
        # the band is part of the list: a list-sized buffer takes it without
        # reading the count first (one host sync for count and info together)
        buf = torch.empty(max(m, 1), dtype=torch.int32, device=self.device)
        nat.call("svie_list_band_write", nat.ptr(self.flat), nat.ptr(idx), m, nx, ny, nz, thresh, nat.ptr(ws),
                 ws.numel(), nat.ptr(buf), m, nat.ptr(self.occ), nat.ptr(self._info), nat.stream())
        info = _read(self._info, nat.BAND_INFO_DTYPE)
        count = int(info["count"])
        work = buf[:count]
        before = int(off_inside[:8].cpu().view(torch.int64)[0])
        self.static_inside = self.static_inside - before + int(info["static_inside"])
        self.work32 = work
        self._band32 = None
        self._band64 = None
        self.band_lo = tuple(int(v) for v in info["lo"])
        self.band_hi = tuple(int(v) for v in info["hi"])
        ilo, ihi = [int(v) for v in info["ilo"]], [int(v) for v in info["ihi"]]
        if self.inside_hi[0] >= 0:
            ilo = [min(a, b) for a, b in zip(ilo, self.inside_lo)]
            ihi = [max(a, b) for a, b in zip(ihi, self.inside_hi)]
        self.inside_lo, self.inside_hi = tuple(ilo), tuple(ihi)
        self.occ_current = False
        if count:
            shape = self.grid.shape
            for ax in range(3):
                if self.band_lo[ax] < MARGIN or self.band_hi[ax] > shape[ax] - 1 - MARGIN:
                    raise RuntimeError("narrow band reaches the grid boundary; enlarge the padding")


# ------------------------------------------------------------- interpolation
def tricubic(flat: torch.Tensor, shape, p: torch.Tensor) -> torch.Tensor:
    from . import kernels as K
    return K.tricubic(flat, int(shape[1]), int(shape[2]), p)


def tricubic_with_gradient(flat: torch.Tensor, shape, p: torch.Tensor):
    from . import kernels as K
    return K.tricubic_with_gradient(flat, int(shape[1]), int(shape[2]), p)


def trilinear(flat: torch.Tensor, shape, p: torch.Tensor) -> torch.Tensor:
    from . import kernels as K
    return K.trilinear(flat, int(shape[1]), int(shape[2]), p)
