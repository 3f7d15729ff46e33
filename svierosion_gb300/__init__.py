"""svierosion_gb300: the SVIErosion narrow-band level-set erosion step on GB300.

A drop-in for the reference's erosion path (``erode``/``ErosionParams`` and the
``svi``/``kernels``/``levelset``/``sdf`` modules, same names and argument
orders): a Python host holding PyTorch tensors calls hand-written sm_103a CUDA
kernels in ``libsvie.so`` through a C ABI (include/svie.h).  There is no CPU
path: on a machine without the built library or a CUDA device every call
raises.
"""

from .api import ErosionParams, ErosionResult, erode, make_grid, point_mesh_distance, write_result
from .evolve import ErosionSimulation, RunResult, StepRecord
from .flows import GaussCurvatureLaw, MeanCurvatureLaw, SVIPowerLaw, make_law
from .grid import Grid, get_device
from .levelset import LevelSet
from .meshio import TriMesh, read_ply, write_ply
from .sdf import mesh_to_sdf
from .surface import extract_surface
from .svi import BallConvolution

__version__ = "0.1.0"

__all__ = ["ErosionParams", "ErosionResult", "erode", "make_grid", "point_mesh_distance", "write_result",
           "ErosionSimulation", "RunResult", "StepRecord", "GaussCurvatureLaw", "MeanCurvatureLaw", "SVIPowerLaw",
           "make_law", "Grid", "get_device", "LevelSet", "TriMesh", "read_ply", "write_ply", "mesh_to_sdf",
           "extract_surface", "BallConvolution"]
