"""The GPU engine against LF_DEM's own C++ directly (fixtures in
tests/golden/): every time step replayed from the reference's state on the
device, compared with the reference's next state."""
import numpy as np
import pytest

import _golden as G

pytestmark = pytest.mark.gpu


def _make(engine, F, k, precision=0):
    lx, ly, lz = G.box(F)
    g = engine.Sim(G.params(F), F[f"s{k}_pre_position"].reshape(-1, 3), F["param_radius"], lx, ly, lz,
                   F[f"s{k}_pre_shear_disp"], precision=precision)
    G.restore(g, F, k)
    return g


@pytest.mark.parametrize("name", G.CASES)
def test_matrix_matches_reference(engine, oracle, name):
    F = G.load(name)
    n = len(F["param_radius"])
    g = _make(engine, F, 0)
    d15, r, c, o18 = g.assemble()
    A = G.dense_from_blocks(oracle, d15, r, c, o18, n)
    Aref = G.csc_to_blocks(F, n)
    assert np.abs(A - Aref).max() <= 1e-13 * np.abs(Aref).max()


@pytest.mark.parametrize("precision,tol", [(0, 1e-10), (1, 1e-8)], ids=["fp64", "fp32refine"])
@pytest.mark.parametrize("name", G.CASES)
def test_steps_match_reference(engine, name, precision, tol):
    F = G.load(name)
    nsteps = int(F["nsteps"][0])
    skip = G.removal_steps(F)
    for k in range(nsteps):
        g = _make(engine, F, k, precision)
        g.step(calc_stress=True)
        pi, pd = G.pairs(F, k, "post")
        pg = g.pairs()
        assert np.array_equal(np.stack([pg["p0"], pg["p1"]], 1), pi[:, :2]), k
        if k in skip:
            continue
        assert np.array_equal(pg["contact_active"], pi[:, 2]), k
        assert np.array_equal(pg["state"], pi[:, 3]), k
        s = g.scalars()
        for key in ("shear_rate", "dt", "strain"):
            ref = float(F[f"s{k}_post_{key}"][0])
            assert abs(s[key] - ref) <= tol * abs(ref), (k, key)
        p = g.particles()
        for ours, theirs in (("pos", "position"), ("vel", "velocity"), ("ang", "ang_velocity"),
                             ("na_vel", "na_velocity")):
            ref = F[f"s{k}_post_{theirs}"].reshape(-1, 3)
            err = np.abs(p[ours] - ref).max() / np.abs(ref).max()
            assert err <= tol, (k, ours, err)
        ts = F[f"s{k}_post_total_stress"]
        assert np.abs(s["total_stress"] - ts).max() <= tol * np.abs(ts).max(), k
        g.close()


@pytest.mark.parametrize("name", G.BROWNIAN_CASES)
@pytest.mark.parametrize("precision,tol", [(0, 1e-9), (1, 1e-8)], ids=["fp64", "fp32refine"])
def test_brownian_steps_match_reference(engine, name, precision, tol):
    """Mid-point (predictor-corrector) steps with the Brownian force the
    reference drew for that step (System::timeEvolutionPredictorCorrectorMethod,
    System.cpp:888-983; the force is reused in the corrector; fixed dt; the
    Banchio-Brady stress of Stress.cpp:270-286)."""
    F = G.load(name)
    skip = G.removal_steps(F)
    assert len(skip) < int(F["nsteps"][0]) - 2, "too few steps without an interaction removal"
    for k in range(int(F["nsteps"][0])):
        g = _make(engine, F, k, precision)
        g.set_brownian_force(F[f"s{k}_post_brownian_force"])
        g.step(calc_stress=True)
        pi, _ = G.pairs(F, k, "post")
        pg = g.pairs()
        assert np.array_equal(np.stack([pg["p0"], pg["p1"]], 1), pi[:, :2]), k
        if k in skip:
            continue   # the reference's swap-removal side effect (see _golden.removal_steps)
        assert np.array_equal(pg["contact_active"], pi[:, 2]), k
        s = g.scalars()
        for key in ("dt", "strain"):
            ref = float(F[f"s{k}_post_{key}"][0])
            assert abs(s[key] - ref) <= tol * abs(ref), (k, key)
        p = g.particles()
        for ours, theirs in (("pos", "position"), ("vel", "velocity"), ("ang", "ang_velocity"),
                             ("na_vel", "na_velocity")):
            ref = F[f"s{k}_post_{theirs}"].reshape(-1, 3)
            err = np.abs(p[ours] - ref).max() / np.abs(ref).max()
            assert err <= tol, (k, ours, err)
        ts = F[f"s{k}_post_total_stress"]
        assert np.abs(s["total_stress"] - ts).max() <= tol * np.abs(ts).max(), k
        g.close()
