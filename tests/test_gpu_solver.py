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


@pytest.mark.parametrize("refine_tol,bound", [(1e-12, 1e-10), (None, 1e-8)], ids=["tight", "default"])
@pytest.mark.parametrize("n,vf,seed", [(500, 0.5, 13)])
def test_fp32_refine_matches_oracle(oracle, engine, n, vf, seed, refine_tol, bound):
    """FP32 factor + FP64 refinement against the oracle's FP64 solve: with a
    tight tolerance to the FP64 form's accuracy, with the default one (2e-10
    relative residual) within the 1e-8 target."""
    p, o, d15, r, c, o18 = _assembled(oracle, n, vf, seed)
    rng = np.random.default_rng(seed)
    b = rng.standard_normal((4, 6 * n))
    x_ref = o.solve_assembled(b)
    opts = {} if refine_tol is None else {"refine_tol": refine_tol}
    s = engine.Solver(n, engine.PREC_FP32_REFINE, **opts)
    s.set_blocks(d15, r, c, o18, True, positions=p.position)
    s.factorize()
    x = s.solve(b)
    rel = np.abs(x - x_ref).max() / np.abs(x_ref).max()
    assert rel < bound, rel
    assert s.last.refine_iters >= 1
    assert s.last.refine_residual <= (refine_tol or 2e-10)


def test_not_spd_reported(oracle, engine):
    p, o, d15, r, c, o18 = _assembled(oracle, 200, 0.45, 14)
    bad = d15.copy()
    bad[37, 0] = -1e6  # a strongly negative translational diagonal entry
    s = engine.Solver(200, engine.PREC_FP64)
    s.set_blocks(bad, r, c, o18, True, positions=p.position)
    with pytest.raises(engine.LFGError) as ei:
        s.factorize()
    assert ei.value.code == engine.LFG_ERR_NOT_SPD


@pytest.mark.parametrize("precision,tol", [(0, 1e-11), (1, 2e-6)], ids=["fp64", "fp32"])
def test_multiply_L_is_a_square_root(oracle, engine, precision, tol):
    """lfg_solver_multiply_factor (StokesSolver::compute_LTRHS): x = L b with
    L L^T = R.  The engine's L is its own (nested-dissection) square root, so
    the checks are the identities every square root satisfies: L L^T = R
    column by column, and (L a)^T R^-1 (L b) = a^T b."""
    import _golden as G
    n = 60
    p, o, d15, r, c, o18 = _assembled(oracle, n, 0.45, 21)
    R = G.dense_from_blocks(oracle, d15, r, c, o18, n)
    s = engine.Solver(n, precision)
    s.set_blocks(d15, r, c, o18, True, positions=p.position)
    s.factorize()
    m = 6 * n
    Lm = np.zeros((m, m))
    for j0 in range(0, m, 4):
        E = np.zeros((4, m))
        for q in range(4):
            if j0 + q < m:
                E[q, j0 + q] = 1.0
        Y = s.multiply_L(E)
        for q in range(4):
            if j0 + q < m:
                Lm[:, j0 + q] = Y[q]
    rel = np.abs(Lm @ Lm.T - R).max() / np.abs(R).max()
    assert rel < tol, rel
    rng = np.random.default_rng(5)
    a = rng.standard_normal((2, m))
    y = s.multiply_L(a)
    x = np.linalg.solve(R, y.T).T
    lhs = y[0] @ x[1]
    assert abs(lhs - a[0] @ a[1]) < 50 * tol * np.abs(a[0]) @ np.abs(a[1])
