"""GPU parity of the resistance solve (lfg_solver_*) against the CPU oracle on
the R_FU that the oracle assembles for seeded packings."""
import numpy as np
import pytest

from _systems import RATE_PARAMS, make_packing

pytestmark = pytest.mark.gpu


def _assembled(oracle, n, vf, seed):
    p = make_packing(n, vf, seed)
    o = oracle.OracleSim(RATE_PARAMS, p.position, p.radius, p.lx, p.ly, p.lz)
    o.first_time()
    d15, r, c, o18 = o.assemble()
    return p, o, d15, r, c, o18


@pytest.mark.parametrize("n,vf,seed", [(200, 0.45, 11), (500, 0.5, 12)])
def test_fp64_solve_matches_oracle(oracle, engine, n, vf, seed):
    p, o, d15, r, c, o18 = _assembled(oracle, n, vf, seed)
    rng = np.random.default_rng(seed)
    b = rng.standard_normal((3, 6 * n))
    x_ref = o.solve_assembled(b)
    s = engine.Solver(n, engine.PREC_FP64)
    s.set_blocks(d15, r, c, o18, True, positions=p.position)
    s.factorize()
    x = s.solve(b)
    rel = np.abs(x - x_ref).max() / np.abs(x_ref).max()
    assert rel < 1e-10, rel
    # reuse of the analysis with new values: scale the matrix by 2
    s.set_blocks(2 * d15, r, c, 2 * o18, False)
    s.factorize()
    x2 = s.solve(b)
    assert np.abs(2 * x2 - x_ref).max() / np.abs(x_ref).max() < 1e-10


@pytest.mark.parametrize("n,vf,seed", [(500, 0.5, 13)])
def test_fp32_refine_matches_oracle(oracle, engine, n, vf, seed):
    p, o, d15, r, c, o18 = _assembled(oracle, n, vf, seed)
    rng = np.random.default_rng(seed)
    b = rng.standard_normal((4, 6 * n))
    x_ref = o.solve_assembled(b)
    s = engine.Solver(n, engine.PREC_FP32_REFINE)
    s.set_blocks(d15, r, c, o18, True, positions=p.position)
    s.factorize()
    x = s.solve(b)
    rel = np.abs(x - x_ref).max() / np.abs(x_ref).max()
    assert rel < 1e-10, rel
    assert s.last.refine_iters >= 1


def test_not_spd_reported(oracle, engine):
    p, o, d15, r, c, o18 = _assembled(oracle, 200, 0.45, 14)
    bad = d15.copy()
    bad[37, 0] = -1e6  # a strongly negative translational diagonal entry
    s = engine.Solver(200, engine.PREC_FP64)
    s.set_blocks(bad, r, c, o18, True, positions=p.position)
    with pytest.raises(engine.LFGError) as ei:
        s.factorize()
    assert ei.value.code == engine.LFG_ERR_NOT_SPD
