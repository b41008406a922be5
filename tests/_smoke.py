"""Smoke check used by __graft_entry__.smoke(): one predictor-corrector step of
a 200-particle stress-controlled suspension on cuda:0, against the CPU oracle."""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def run_smoke():
    for p in (ROOT, os.path.join(ROOT, "oracle"), os.path.join(ROOT, "tests")):
        if p not in sys.path:
            sys.path.insert(0, p)
    import lf_dem_gb300 as E
    import pyoracle
    from _systems import STRESS_PARAMS, make_packing
    from lf_dem_gb300 import build as B
    B.build()
    pyoracle.build()
    rc, name, cc, nsm = E.device_info(0)
    if rc != E.LFG_OK:
        raise RuntimeError(f"no sm_103 device on cuda:0 ({name}, cc {cc})")
    p = make_packing(200, 0.5, 7)
    o = pyoracle.OracleSim(STRESS_PARAMS, p.position, p.radius, p.lx, p.ly, p.lz)
    o.first_time()
    g = E.Sim(STRESS_PARAMS, p.position, p.radius, p.lx, p.ly, p.lz)
    o.step(calc_stress=True)
    g.step(calc_stress=True)
    vo, vg = o.particles()["vel"], g.particles()["vel"]
    err = np.abs(vo - vg).max() / np.abs(vo).max()
    if not err <= 1e-10:
        raise AssertionError(f"GPU step differs from the oracle: rel err {err:.3e}")
    so, sg = o.scalars(), g.scalars()
    serr = np.abs(so["total_stress"] - sg["total_stress"]).max() / np.abs(so["total_stress"]).max()
    if not serr <= 1e-10:
        raise AssertionError(f"GPU stress differs from the oracle: rel err {serr:.3e}")
    print(f"smoke ok: {name}, velocity rel err {err:.2e}, stress rel err {serr:.2e}")
