"""Full-float64 variant of the oracle (test infrastructure only).

The same restatement of the reference algorithm as ``reference_np`` with every
float32 quantity computed in float64 and the spectra in complex128: a second
instance of the module whose ``F32`` / ``C64`` type constants are float64 /
complex128.  It is the "full-FP64 run" against which the float32 path's error
is stated (N_r, volume trajectory, stopping step, final surface); the
reference itself is float32 throughout (svierosion/levelset.py:60,
svierosion/svi.py:76).
"""

from __future__ import annotations

import importlib.util
import sys
from pathlib import Path

import numpy as np


def _load():
    spec = importlib.util.spec_from_file_location("oracle._reference_fp64",
                                                  Path(__file__).with_name("reference_np.py"))
    mod = importlib.util.module_from_spec(spec)
    sys.modules[spec.name] = mod
    spec.loader.exec_module(mod)
    mod.F32 = np.float64
    mod.C64 = np.complex128
    return mod


fp64 = _load()
