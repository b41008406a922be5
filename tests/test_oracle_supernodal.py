"""The CPU oracle's supernodal factorisation (dense BLAS-3 kernels from
scipy, the method of CHOLMOD's supernodal factorisation; used for the timed
CPU baseline) against its block factorisation on the same systems: steps
agree to round-off (1e-12 relative)."""
import os
import subprocess
import sys

import pytest

from _systems import RATE_PARAMS, STRESS_PARAMS


@pytest.mark.parametrize("params,n,vf,seed", [(RATE_PARAMS, 300, 0.5, 21), (STRESS_PARAMS, 400, 0.52, 22)],
                         ids=["rate", "stress"])
def test_supernodal_matches_block_factorisation(params, n, vf, seed):
    # a fresh process: the BLAS kernels, once set, are used by every later
    # factorisation of that process
    here = os.path.dirname(os.path.abspath(__file__))
    root = os.path.dirname(here)
    paths = [root, os.path.join(root, "oracle"), here]
    code = f"""
import sys, numpy as np
sys.path[:0] = {paths!r}
import pyoracle
from _systems import RATE_PARAMS, STRESS_PARAMS, make_packing
params = {params!r}
p = make_packing({n}, {vf}, {seed})
res = []
for blas in (False, True):
    if blas:
        assert pyoracle.use_blas()
    o = pyoracle.OracleSim(params, p.position, p.radius, p.lx, p.ly, p.lz)
    o.first_time()
    for k in range(3):
        o.step(calc_stress=(k == 2))
    res.append((o.particles()["vel"], o.scalars()["total_stress"]))
(v0, s0), (v1, s1) = res
print(np.abs(v0 - v1).max() / np.abs(v0).max(), np.abs(s0 - s1).max() / np.abs(s0).max())
"""
    pytest.importorskip("scipy")
    out = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, cwd=here)
    assert out.returncode == 0, out.stderr[-2000:]
    ev, es = map(float, out.stdout.split())
    assert ev <= 1e-12 and es <= 1e-12, (ev, es)
