"""CPU oracle for the narrow-band level-set erosion path.

TEST INFRASTRUCTURE ONLY.  This package restates, in numpy, the reference
SVIErosion algorithm for the erosion step (svierosion/kernels.py, levelset.py,
svi.py, flows.py, evolve.py, sdf.py, grid.py).  It is the checker: the tests,
``__graft_entry__.smoke()`` and the CPU-baseline legs of ``bench.py`` may call
it; the product package ``svierosion_gb300`` never imports it.

Parity is pinned: ``tests/golden/make_golden.py`` ran the reference itself
(imported from its source tree) on seeded inputs and committed the results as
fixtures under ``tests/golden/``; ``tests/test_oracle_golden.py`` checks this
oracle against every fixture.
"""

from .reference_np import *  # noqa: F401,F403
