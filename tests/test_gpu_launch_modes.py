"""Launch modes change timing only: the same solve with dependent launches off (SVIE_PDL=0), with every
grid shape's convolution forms tuned (SVIE_FFT_TUNE=all), with the TMA tile loads of the convolution
passes replaced by cp.async (SVIE_TMA=0) and with the y and x passes compiled for every shape's axis
lengths (SVIE_FFT_JIT=all) gives the default run's results bit for bit.  Each mode runs in
its own process, because the switches are read once per process."""

import json
import os
import subprocess
import sys
import time
from pathlib import Path

import pytest

pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parents[1]

SCRIPT = r"""
import hashlib, json, sys
import numpy as np
sys.path.insert(0, sys.argv[1])
import svierosion_gb300 as S
from svierosion_gb300 import shapes
frag = shapes.fragment(3, seed=5)
L = float((frag.bounds[1] - frag.bounds[0]).max())
from svierosion_gb300 import _native as nat
out = {}
for law, kw in (("svi", dict(radius=0.08 * L, k=1, s=0, max_steps=12)), ("mean", dict(alpha=1.0, max_steps=30))):
    runs = []
    for _ in range(2):  # the second solve finds the compiled passes loaded (SVIE_FFT_JIT=all)
        res = S.erode(frag, S.ErosionParams(law=law, resolution=40, target_fraction=0.1, **kw),
                      extract_meshes=False, keep_state=True)
        phi = res.level_set.phi.cpu().numpy()
        runs.append({"fractions": [r.fraction for r in res.history], "dt": [r.dt for r in res.history],
                     "phi": hashlib.sha256(phi.tobytes()).hexdigest()})
        nat.lib().svie_conv_jit_wait(120000)
    assert runs[0] == runs[1]
    out[law] = runs[1]
out["tma_timeouts"] = int(nat.lib().svie_conv_tma_timeouts())
print(json.dumps(out))
"""


def _run(env_extra):
    env = dict(os.environ, **env_extra)
    r = subprocess.run([sys.executable, "-c", SCRIPT, str(ROOT)], env=env, capture_output=True, text=True,
                       timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    return json.loads(r.stdout.strip().splitlines()[-1])


def test_dependent_launches_and_tuning_change_no_bits():
    base = _run({"SVIE_PDL": "1", "SVIE_FFT_TUNE": "1"})
    assert len(base["svi"]["fractions"]) == 12 and len(base["mean"]["fractions"]) == 30
    assert base["tma_timeouts"] == 0
    for extra in ({"SVIE_PDL": "0"}, {"SVIE_FFT_TUNE": "all"}, {"SVIE_TMA": "0"}, {"SVIE_FFT_JIT": "all"}):
        assert _run(extra) == base, extra


EXIT_SCRIPT = r"""
import sys, time
sys.path.insert(0, sys.argv[1])
import torch
from svierosion_gb300 import _native as nat
torch.cuda.init()
torch.zeros(1, device="cuda")
lib = nat.lib()
mode = sys.argv[2]
assert lib.svie_conv_jit(448, 336, 245) == 0
if mode in ("idle", "gone"):
    assert lib.svie_conv_jit_wait(120000) == 0 and lib.svie_conv_jit_ready(448, 336, 245)
if mode == "gone":
    time.sleep(0.5)
print("exiting", mode, flush=True)
"""


@pytest.mark.parametrize("mode", ["compiling", "idle", "gone"])
def test_process_exits_cleanly_around_the_compile_worker(mode):
    """A process that requested the passes compiled for a shape exits with status 0, whether its
    background worker is still compiling (the exit waits for that compilation and joins the
    worker), idle in its loop, or already gone."""
    t0 = time.time()
    r = subprocess.run([sys.executable, "-c", EXIT_SCRIPT, str(ROOT), mode], capture_output=True, text=True,
                       timeout=240)
    assert r.returncode == 0, (r.returncode, r.stderr[-2000:])
    assert "exiting " + mode in r.stdout
    assert time.time() - t0 < 200
