"""GPU engine against the CPU oracle at the sizes of the configured workloads.

- The benchmarked workload itself: N = 4096 bidisperse spheres, phi = 0.56,
  stress control 10 cl with the critical-load friction model, the same seeded
  packing and parameters bench.py times.  One predictor-corrector step from
  the packing, in the plain FP64 form (velocities, angular velocities,
  stresses, contact forces within 1e-10; pair list and contact states
  bit-exact) and in the FP32 + FP64-refinement form (1e-8).
- The 2D monolayer: N = 8192 discs, areal fraction 0.78, rate control, one
  step, same bars.
- The 3D plain-method run (N = 500, phi = 0.50, rate control): the engine
  runs the suspension forward; at ten points spread over the run its state
  (positions, Lees-Edwards offset, contact springs, clock) is handed to a
  fresh engine and to the oracle, both advance one step with stresses, and
  the results agree within 1e-10.

Tolerances are relative to the largest magnitude of each compared quantity.
"""
import numpy as np
import pytest

import bench
from _systems import RATE_PARAMS
from lf_dem_gb300 import packing as PK

pytestmark = pytest.mark.gpu

TOL64 = 1e-10
TOL32 = 1e-8


def _rel(a, b):
    a, b = np.asarray(a, dtype=float), np.asarray(b, dtype=float)
    scale = max(np.abs(b).max(), 1e-300)
    return float(np.abs(a - b).max() / scale)


def _rel_scalar(a, b):
    return abs(a - b) / max(abs(b), 1e-300)


def _oracle_step(oracle, params, p):
    o = oracle.OracleSim(params, p.position, p.radius, p.lx, p.ly, p.lz)
    o.first_time()
    o.step(calc_stress=True)
    return {"part": o.particles(), "pairs": o.pairs(), "sc": o.scalars()}


def _compare(ref, g, tol, exact_lists):
    """Engine state after its step against the oracle's result `ref`."""
    pg, sg, qg = g.particles(), g.scalars(), g.pairs()
    po, so, qo = ref["part"], ref["sc"], ref["pairs"]
    errs = {k: _rel(pg[k], po[k]) for k in ("pos", "vel", "ang", "na_vel")}
    errs["total_stress"] = _rel(sg["total_stress"], so["total_stress"])
    for k in ("viscosity", "N1", "N2", "shear_rate", "dt"):
        errs[k] = _rel_scalar(sg[k], so[k])
    keys_o = np.stack([qo["p0"], qo["p1"]], 1)
    keys_g = np.stack([qg["p0"], qg["p1"]], 1)
    if exact_lists:
        assert np.array_equal(keys_o, keys_g), "pair lists differ"
        assert np.array_equal(qo["contact_active"], qg["contact_active"]), "contact states differ"
        assert np.array_equal(qo["state"], qg["state"]), "friction states differ"
    assert len(keys_o) == len(keys_g)
    errs["contact_force"] = _rel(np.asarray(qg["f_spring_total"]), np.asarray(qo["f_spring_total"]))
    bad = {k: v for k, v in errs.items() if not v <= tol}
    assert not bad, (bad, errs)
    return errs


@pytest.fixture(scope="module")
def cfg2(oracle):
    p = PK.generate(bench.N_PART, bench.VF, seed=2000)
    prm = bench.workload_params()
    return p, prm, _oracle_step(oracle, prm, p)


@pytest.mark.parametrize("precision,tol", [(0, TOL64), (1, TOL32)], ids=["fp64", "fp32_refine"])
def test_benchmarked_workload_step_matches_oracle(engine, cfg2, precision, tol):
    p, prm, ref = cfg2
    g = engine.Sim(prm, p.position, p.radius, p.lx, p.ly, p.lz, precision=precision)
    g.step(calc_stress=True)
    errs = _compare(ref, g, tol, exact_lists=True)
    print(f"N=4096 phi=0.56 stress 10cl, precision {precision}: " +
          ", ".join(f"{k} {v:.1e}" for k, v in errs.items()))
    g.close()


@pytest.fixture(scope="module")
def cfg3(oracle):
    p = PK.generate(8192, 0.78, seed=3000, twodim=True)
    prm = dict(RATE_PARAMS)
    return p, prm, _oracle_step(oracle, prm, p)


@pytest.mark.parametrize("precision,tol", [(0, TOL64), (1, TOL32)], ids=["fp64", "fp32_refine"])
def test_monolayer_8192_step_matches_oracle(engine, cfg3, precision, tol):
    p, prm, ref = cfg3
    g = engine.Sim(prm, p.position, p.radius, p.lx, p.ly, p.lz, precision=precision)
    g.step(calc_stress=True)
    errs = _compare(ref, g, tol, exact_lists=True)
    # a monolayer stays in the plane: no y displacement, rotation only about y
    part = g.particles()
    vmax, wmax = np.abs(part["vel"]).max(), np.abs(part["ang"]).max()
    assert np.abs(part["vel"][:, 1]).max() <= 1e-14 * vmax
    assert max(np.abs(part["ang"][:, 0]).max(), np.abs(part["ang"][:, 2]).max()) <= 1e-14 * wmax
    print(f"2D N=8192 phi=0.78 rate 1r, precision {precision}: " +
          ", ".join(f"{k} {v:.1e}" for k, v in errs.items()))
    g.close()


REPLAY_POINTS = 10
REPLAY_STEPS_BETWEEN = 150


def test_plain_run_replayed_at_ten_points(engine, oracle):
    """N = 500, phi = 0.50, rate control 1r: one-step parity from ten states
    spread over the engine's own run (dense suspensions are chaotic, so a
    free-running comparison would only test round-off growth)."""
    p = PK.generate(500, 0.50, seed=1000)
    prm = dict(RATE_PARAMS)
    run = engine.Sim(prm, p.position, p.radius, p.lx, p.ly, p.lz)
    worst = {}
    strains = []
    for point in range(REPLAY_POINTS):
        run.run(REPLAY_STEPS_BETWEEN)
        sc = run.scalars()
        strains.append(sc["strain"])
        pos = run.particles()["pos"]
        c0, c1, dtan, _ = run.contact_states()
        contacts = [(int(a), int(b), d) for a, b, d in zip(c0, c1, dtan)]
        le = tuple(sc["shear_disp"])
        clock = (sc["time"], sc["strain"], sc["dt"], sc["shear_rate"], sc["max_velocity"],
                 sc["max_sliding_velocity"])
        g = engine.Sim(prm, pos, p.radius, p.lx, p.ly, p.lz, le_disp=le, contacts=contacts)
        o = oracle.OracleSim(prm, pos, p.radius, p.lx, p.ly, p.lz, le_disp=le, contacts=contacts)
        o.first_time()
        g.set_clock(*clock)
        o.set_clock(*clock)
        o.step(calc_stress=True)
        g.step(calc_stress=True)
        ref = {"part": o.particles(), "pairs": o.pairs(), "sc": o.scalars()}
        errs = _compare(ref, g, TOL64, exact_lists=True)
        for comp in range(8):
            so_ = o.particle_stress(comp)
            if so_ is None:
                continue
            e = _rel(g.particle_stress(comp), so_)
            assert e <= TOL64, (point, comp, e)
        for k, v in errs.items():
            worst[k] = max(worst.get(k, 0.0), v)
        g.close()
        del o
    run.close()
    assert strains[-1] > strains[0] > 0
    print(f"N=500 replay at strains {strains[0]:.3g}..{strains[-1]:.3g}: " +
          ", ".join(f"{k} {v:.1e}" for k, v in worst.items()))
