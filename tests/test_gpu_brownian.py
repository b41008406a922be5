"""The Brownian force the engine draws itself (no injected force).

System::setBrownianForceToParticle (System.cpp:1665-1710, with
StokesSolver::compute_LTRHS of StokesSolver.cpp:627) sets
F_B = L (sqrt(2 kT/dt) psi), psi a vector of 6n independent standard normals
and L L^T = R the resistance matrix of the predictor's configuration.  Whatever square root L is, chol(R)^-1 F_B /
sqrt(2 kT/dt) is an orthogonal transform of psi, so its 6n components are
again independent standard normals; that is what is checked here, with R
assembled by the engine before the step and factorised by numpy.  The
reference seeds its generator from the clock, so there are no reference
draws to compare with: the tests check the distribution, that a seed repeats
its trajectory and that another seed does not.
"""
import math

import numpy as np
import pytest

import _golden as G

pytestmark = pytest.mark.gpu

FC_BROWNIAN = 4


def _make(engine, F, seed, precision):
    lx, ly, lz = G.box(F)
    p = G.params(F)
    p["seed"] = seed
    g = engine.Sim(p, F["s0_pre_position"].reshape(-1, 3), F["param_radius"], lx, ly, lz,
                   F["s0_pre_shear_disp"], precision=precision)
    G.restore(g, F, 0)
    return g, p


def _normal_cdf(x):
    return 0.5 * (1.0 + np.vectorize(math.erf)(x / math.sqrt(2.0)))


@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "fp32refine"])
def test_brownian_draws_are_standard_normal_through_R(engine, oracle, precision):
    F = G.load(G.BROWNIAN_CASES[0])
    n = len(F["param_radius"])
    g, p = _make(engine, F, 12345, precision)
    scale = math.sqrt(2.0 * p["brownian"] / p["dt"])
    ws = []
    for _ in range(3):
        d15, r, c, o18 = g.assemble()
        R = G.dense_from_blocks(oracle, d15, r, c, o18, n)
        g.step(calc_stress=False)
        fb = g.force_component(FC_BROWNIAN).reshape(-1)
        assert np.isfinite(fb).all()
        ws.append(np.linalg.solve(np.linalg.cholesky(R), fb) / scale)
    g.close()
    w = np.concatenate(ws)
    m = len(w)
    # 6 sigma bounds on the sample mean and variance of m standard normals
    assert abs(w.mean()) < 6.0 / math.sqrt(m), w.mean()
    assert abs(w.var() - 1.0) < 6.0 * math.sqrt(2.0 / m), w.var()
    assert np.abs(w).max() < 6.5
    # Kolmogorov-Smirnov distance to the normal CDF (2.0/sqrt(m): p < 1e-3)
    ws_ = np.sort(w)
    cdf = _normal_cdf(ws_)
    k = np.arange(1, m + 1)
    D = max((k / m - cdf).max(), (cdf - (k - 1) / m).max())
    assert D < 2.0 / math.sqrt(m), D
    # successive draws are independent: no correlation between the steps' psi
    for a in range(3):
        for b in range(a + 1, 3):
            rho = float(np.dot(ws[a], ws[b]) / math.sqrt(np.dot(ws[a], ws[a]) * np.dot(ws[b], ws[b])))
            assert abs(rho) < 6.0 / math.sqrt(6 * n), (a, b, rho)


def test_brownian_seed_repeats_and_differs(engine):
    F = G.load(G.BROWNIAN_CASES[0])
    runs = {}
    for key, seed in (("a", 7), ("b", 7), ("c", 8)):
        g, _ = _make(engine, F, seed, 0)
        fbs = []
        for _ in range(3):
            g.step(calc_stress=True)
            fbs.append(g.force_component(FC_BROWNIAN).reshape(-1))
        runs[key] = (np.stack(fbs), g.particles()["pos"], g.scalars()["total_stress"])
        g.close()
    fa, pa, sa = runs["a"]
    fb_, pb, sb = runs["b"]
    fc, pc, _ = runs["c"]
    assert np.array_equal(fa[0], fb_[0])          # the same draw and the same product
    assert np.abs(fa - fb_).max() <= 1e-12 * np.abs(fa).max()
    assert np.abs(pa - pb).max() <= 1e-12 * np.abs(pa).max()
    assert np.abs(sa - sb).max() <= 1e-10 * np.abs(sa).max()
    # another seed: other forces (the largest difference of two independent
    # draws of 6n components is of the order of the largest component),
    # different trajectory
    assert np.abs(fa[0] - fc[0]).max() > 0.1 * np.abs(fa[0]).max()
    assert np.abs(pa - pc).max() > 0
    # successive steps of one run draw fresh forces
    assert not np.allclose(fa[0], fa[1])
