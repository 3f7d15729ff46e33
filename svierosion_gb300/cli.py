"""Command line interface: ``python -m svierosion_gb300 <command> ...`` (reference svierosion/cli.py).

Commands
--------
erode     erode a PLY mesh under an SVI or curvature law until a volume fraction
compare   run several laws on one mesh to the same volume fraction
distance  vertex-wise distance from one mesh to another
shapes    write the built-in solids as PLY files
info      print basic statistics of a mesh

The commands, options and defaults are the reference's, so its scripts run unchanged; the work runs
on the GPU through :func:`~svierosion_gb300.api.erode`, and the result files are those of
:func:`~svierosion_gb300.api.write_result`.  ``--render`` (a PNG made with matplotlib in the
reference) is accepted and reported as unavailable: no plotting library is part of this build.
``--no-compile`` is accepted and has no effect (nothing is compiled at run time).
"""

from __future__ import annotations

import argparse
import sys
import time
from pathlib import Path

import numpy as np

# option tables: (flags, keyword arguments of add_argument)
LAW_OPTIONS = [
    (("--law",), dict(choices=["svi", "mean", "gauss"], default="svi",
                      help="speed law: svi = N^k/(t-N)^s, mean = (H_+)^alpha, gauss = (k1_+ k2_+)^alpha")),
    (("--radius", "-r"), dict(type=float, help="SVI ball radius r (mesh units)")),
    (("--radius-rel",), dict(type=float, help="SVI radius as a fraction of the largest bounding-box side")),
    (("-k",), dict(type=int, default=1, help="SVI exponent k (default 1)")),
    (("-s",), dict(type=int, default=0, choices=[0, 1], help="SVI geometric term switch s")),
    (("-t",), dict(type=float, help="SVI singularity location t (needed for s=1)")),
    (("--eps",), dict(type=float, default=0.0, help="additive constant speed (grassfire)")),
    (("--alpha",), dict(type=float, default=1.0, help="curvature-law exponent")),
    (("--delta",), dict(type=float, default=None,
                        help="regularisation of x^alpha near 0 for alpha < 1 (default: automatic)")),
    (("--max-speed-ratio",), dict(type=float, default=100.0,
                                  help="cap of the s=1 SVI speed relative to the flat-surface speed")),
]
NUMERICS_OPTIONS = [
    (("--target",), dict(type=float, default=0.9, help="final volume fraction (default 0.9)")),
    (("--snapshots",), dict(type=float, nargs="*", default=[],
                            help="additional volume fractions at which meshes are written")),
    (("--spacing",), dict(type=float, help="grid spacing h (mesh units)")),
    (("--resolution",), dict(type=int, default=200,
                             help="cells across the largest bounding-box side (if --spacing not given)")),
    (("--band",), dict(type=float, default=6.0, help="narrow band half width (cells)")),
    (("--cfl",), dict(type=float, default=0.5)),
    (("--device",), dict(default=None, help="CUDA device (the GPU path has no CPU fallback)")),
    (("--no-compile",), dict(action="store_true", help="accepted for compatibility; no effect")),
    (("--no-project",), dict(action="store_true",
                             help="do not project marching-cubes vertices onto the tricubic zero set")),
]


def _options(parser, table, title=None):
    group = parser.add_argument_group(title) if title else parser
    for flags, kw in table:
        group.add_argument(*flags, **kw)


def _params(args, mesh):
    """ErosionParams from the parsed options (cli.py:55-68): an SVI radius given absolutely or
    relative to the largest side of the bounding box."""
    from .api import ErosionParams
    radius = args.radius
    if args.law == "svi" and radius is None:
        if args.radius_rel is None:
            raise SystemExit("error: the SVI law needs --radius or --radius-rel")
        lo, hi = mesh.bounds
        radius = args.radius_rel * float((hi - lo).max())
    return ErosionParams(law=args.law, radius=radius, k=args.k, s=args.s, t=args.t, eps=args.eps,
                         max_speed_ratio=args.max_speed_ratio, alpha=args.alpha, delta=args.delta,
                         target_fraction=args.target, snapshots=tuple(args.snapshots), spacing=args.spacing,
                         resolution=args.resolution, band=args.band, cfl=args.cfl, device=args.device,
                         project_vertices=not args.no_project)


def _progress(verbose):
    """A step callback that prints a progress line on the first step and then every 2 s."""
    last = [time.time()]

    def report(sim, rec):
        if not verbose:
            return
        now = time.time()
        if rec.step != 1 and now - last[0] <= 2.0:
            return
        last[0] = now
        rng = (f" N=[{rec.qmin:.3f},{rec.qmax:.3f}]" if sim.law.requires_svi
               else f" H=[{rec.qmin:.3g},{rec.qmax:.3g}]")
        capped = f" capped={rec.capped}" if rec.capped else ""
        print(f"  step {rec.step:6d}  t={rec.time:.5g}  dt={rec.dt:.2e}  V/V0={rec.fraction:.5f}  "
              f"vmax={rec.vmax:.3g}{rng}{capped}", flush=True)
    return report


def _no_render(path, quiet):
    if path and not quiet:
        print(f"[svierosion] --render {path}: not written (no plotting library in this build)", file=sys.stderr)


# ------------------------------------------------------------------ commands
def cmd_erode(args) -> int:
    from .api import erode, volume_fraction_report, write_result
    from .meshio import read_ply
    mesh = read_ply(args.input)
    params = _params(args, mesh)
    src = Path(args.input)
    out = Path(args.output) if args.output else src.with_name(src.stem + "_eroded.ply")
    talk = not args.quiet
    if talk:
        print(f"[svierosion] {args.input}: {len(mesh.vertices)} vertices, {len(mesh.faces)} triangles, "
              f"volume {mesh.volume():.6g}, watertight {mesh.is_watertight()}")
    res = erode(mesh, params, callback=_progress(talk), verbose=talk)
    written = write_result(res, out, args.quality)
    if talk:
        print("[svierosion] " + res.summary())
        print("[svierosion] " + volume_fraction_report(res))
        for f in written:
            print(f"[svierosion] wrote {f}")
    _no_render(args.render, args.quiet)
    return 0 if res.stop_reason == "target_volume" else 2


def cmd_compare(args) -> int:
    from .compare import default_comparison_laws, run_comparison
    from .meshio import read_ply
    mesh = read_ply(args.input)
    lo, hi = mesh.bounds
    radius = args.radius if args.radius is not None else (args.radius_rel or 0.15) * float((hi - lo).max())
    run_comparison(mesh, default_comparison_laws(radius, t=args.t), Path(args.output), target=args.target,
                   resolution=args.resolution, spacing=args.spacing, device=args.device, verbose=not args.quiet)
    return 0


def cmd_distance(args) -> int:
    from .api import point_mesh_distance
    from .meshio import read_ply, write_ply
    a, b = read_ply(args.mesh_a), read_ply(args.mesh_b)
    ab = point_mesh_distance(a.vertices, b, device=args.device, exact=True)
    ba = point_mesh_distance(b.vertices, a, device=args.device, exact=True)
    for name, d in (("A->B", ab), ("B->A", ba)):
        print(f"{name}: mean {d.mean():.6g}  rms {np.sqrt((d ** 2).mean()):.6g}  max {d.max():.6g}")
    print(f"Hausdorff {max(ab.max(), ba.max()):.6g}")
    if args.output:
        write_ply(args.output, a, vertex_data={"quality": ab.astype(np.float32)})
        print(f"wrote {args.output} (vertex quality = distance to {args.mesh_b})")
    return 0


def cmd_shapes(args) -> int:
    from . import shapes
    from .meshio import write_ply
    out = Path(args.output)
    out.mkdir(parents=True, exist_ok=True)
    for name, make in shapes.SHAPES.items():
        m = make()
        path = out / f"{name}.ply"
        write_ply(path, m)
        print(f"{name:14s} {len(m.faces):7d} triangles  volume {m.volume():.5f}  -> {path}")
    return 0


def cmd_info(args) -> int:
    from .meshio import read_ply
    m = read_ply(args.input)
    lo, hi = m.bounds
    topo = m.edge_topology()
    print(f"vertices {len(m.vertices)}, triangles {len(m.faces)}")
    print(f"bounding box {lo} .. {hi} (extent {hi - lo})")
    print(f"area {m.area():.6g}, signed volume {m.signed_volume():.6g}")
    print(f"edges {topo['edges']}, boundary {topo['boundary_edges']}, non-manifold "
          f"{topo['nonmanifold_edges']}, misoriented {topo['misoriented_edges']}")
    print(f"vertex properties: {sorted(m.vertex_data)}")
    return 0


COMMANDS = {
    "erode": (cmd_erode, "erode a mesh", [
        (("input",), {}),
        (("-o", "--output"), dict(help="output PLY (default: <input>_eroded.ply)")),
        "law", "numerics",
        (("--quality",), dict(default="depth",
                              help="vertex scalar duplicated as 'quality' (MeshLab colour map): depth, N, speed, H")),
        (("--render",), dict(help="PNG of the initial and eroded meshes (unavailable in this build)")),
        (("--quiet",), dict(action="store_true")),
    ]),
    "compare": (cmd_compare, "compare SVI and curvature flows on one mesh", [
        (("input",), {}),
        (("-o", "--output"), dict(required=True, help="output directory")),
        (("--radius", "-r"), dict(type=float)),
        (("--radius-rel",), dict(type=float, help="radius / largest bounding-box side (default 0.15)")),
        (("-t",), dict(type=float, default=0.93, help="t for the s=1 SVI laws")),
        (("--target",), dict(type=float, default=0.9)),
        (("--spacing",), dict(type=float)),
        (("--resolution",), dict(type=int, default=160)),
        (("--device",), dict(default=None)),
        (("--no-compile",), dict(action="store_true")),
        (("--quiet",), dict(action="store_true")),
    ]),
    "distance": (cmd_distance, "distances between two meshes", [
        (("mesh_a",), {}), (("mesh_b",), {}),
        (("-o", "--output"), dict(help="write mesh A with per-vertex distance as quality")),
        (("--device",), dict(default=None)),
    ]),
    "shapes": (cmd_shapes, "write the built-in solids", [(("output",), {})]),
    "info": (cmd_info, "mesh statistics", [(("input",), {})]),
}


def build_parser() -> argparse.ArgumentParser:
    ap = argparse.ArgumentParser(prog="svierosion_gb300", description=__doc__,
                                 formatter_class=argparse.RawDescriptionHelpFormatter)
    sub = ap.add_subparsers(dest="command", required=True)
    for name, (fn, text, spec) in COMMANDS.items():
        p = sub.add_parser(name, help=text)
        for item in spec:
            if item == "law":
                _options(p, LAW_OPTIONS, "flow")
            elif item == "numerics":
                _options(p, NUMERICS_OPTIONS, "numerics")
            else:
                p.add_argument(*item[0], **item[1])
        p.set_defaults(func=fn)
    return ap


def main(argv=None) -> int:
    args = build_parser().parse_args(argv)
    return args.func(args)


if __name__ == "__main__":
    sys.exit(main())
