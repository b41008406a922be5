"""The in-plane (3 unknowns per particle) form of 2D runs against LF_DEM's
6x6 blocks.  In a monolayer (all particles at y = 0, shear in the x-z plane)
every pair's normal has n_y = 0, so the 6x6 resistance blocks couple x, z
translation and y rotation only among themselves (System.cpp:478-491 keeps
the 6x6 layout of StokesSolver.cpp:87-100 anyway).  The engine's default for
2D runs factors those three unknowns alone; these tests hold it to the 6x6
form (the reference's own 2D fixture rate_2d_n200 is replayed through the
default in tests/test_gpu_golden.py).  Tolerances: 1e-10 relative in FP64,
1e-8 with the FP32 factor and FP64 refinement."""
import numpy as np
import pytest

from _systems import RATE_PARAMS, STRESS_PARAMS
from lf_dem_gb300 import packing as PK

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return float(np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(np.asarray(b)).max(), 1e-300))


def test_planar_solver_matches_six_unknowns(oracle, engine):
    """lfg_solver with dof 3 against dof 6 on the R_FU of a 2D packing."""
    p = PK.generate(600, 0.75, seed=71, twodim=True)
    o = oracle.OracleSim(RATE_PARAMS, p.position, p.radius, p.lx, p.ly, p.lz)
    o.first_time()
    d15, r, c, o18 = o.assemble()
    n = len(p.radius)
    rng = np.random.default_rng(71)
    b = rng.standard_normal((2, n, 6))
    b[:, :, [1, 3, 5]] = 0.0          # a monolayer's forces: in-plane, torque about y
    b = b.reshape(2, 6 * n)
    x_ref = o.solve_assembled(b)
    for prec, tol in ((engine.PREC_FP64, 1e-10), (engine.PREC_FP32_REFINE, 1e-8)):
        xs = {}
        for dof in (6, 3):
            s = engine.Solver(n, prec, dof=dof)
            s.set_blocks(d15, r, c, o18, True, positions=p.position)
            s.factorize()
            xs[dof] = s.solve(b)
            st = s.stats()
            s.close()
            if dof == 3:
                assert st["n_blocks"] == n
        assert _rel(xs[3], x_ref) <= tol, (prec, _rel(xs[3], x_ref))
        assert _rel(xs[3], xs[6]) <= tol
        x3 = xs[3].reshape(2, n, 6)
        assert not x3[:, :, [1, 3, 5]].any()   # out-of-plane components are exactly 0


@pytest.mark.parametrize("params,vf,seed", [(RATE_PARAMS, 0.72, 72), (STRESS_PARAMS, 0.76, 73)],
                         ids=["rate", "stress"])
@pytest.mark.parametrize("precision,tol", [(0, 1e-10), (1, 1e-8)], ids=["fp64", "fp32_refine"])
def test_planar_steps_match_six_unknowns(engine, params, vf, seed, precision, tol):
    """Four predictor-corrector steps of the same 2D suspension with 3 and with
    6 unknowns per particle: positions, velocities, stresses and the pair and
    contact lists agree."""
    p = PK.generate(500, vf, seed=seed, twodim=True)
    sims = {dof: engine.Sim(params, p.position, p.radius, p.lx, p.ly, p.lz, precision=precision, dof_2d=dof)
            for dof in (3, 6)}
    for k in range(4):
        for g in sims.values():
            g.step(calc_stress=(k == 3))
        a, b = sims[3], sims[6]
        pa, pb = a.particles(), b.particles()
        for key in ("pos", "vel", "ang", "na_vel"):
            assert _rel(pa[key], pb[key]) <= tol, (k, key, _rel(pa[key], pb[key]))
        qa, qb = a.pairs(), b.pairs()
        assert np.array_equal(np.stack([qa["p0"], qa["p1"]], 1), np.stack([qb["p0"], qb["p1"]], 1))
        assert np.array_equal(qa["contact_active"], qb["contact_active"])
        sa, sb = a.scalars(), b.scalars()
        assert _rel(sa["total_stress"], sb["total_stress"]) <= tol
        assert abs(sa["shear_rate"] - sb["shear_rate"]) <= tol * abs(sb["shear_rate"])
    ta, tb = sims[3].timing(), sims[6].timing()
    # the in-plane system has half the unknowns: about an eighth of the flops
    assert ta["factor_flops"] < 0.2 * tb["factor_flops"]
    for g in sims.values():
        g.close()
