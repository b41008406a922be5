"""GPU engine (lfg_sim_*) against the CPU oracle: stage-level parity (R_FU
blocks, force components) and whole predictor-corrector steps (positions,
velocities, pair list and contact states, stresslets) on seeded packings."""
import numpy as np
import pytest

from _systems import RATE_PARAMS, ROLLING_PARAMS, STRESS_PARAMS, make_packing

pytestmark = pytest.mark.gpu

TOL = 1e-10   # relative, FP64 plain form


def _pair_keys(p):
    return np.stack([p["p0"], p["p1"]], 1)


def _make(oracle, engine, params, n, vf, seed, precision=0):
    p = make_packing(n, vf, seed)
    o = oracle.OracleSim(params, p.position, p.radius, p.lx, p.ly, p.lz)
    o.first_time()
    g = engine.Sim(params, p.position, p.radius, p.lx, p.ly, p.lz, precision=precision)
    return p, o, g


@pytest.mark.parametrize("params", [RATE_PARAMS, STRESS_PARAMS], ids=["rate", "stress"])
def test_initial_pairs_and_blocks(oracle, engine, params):
    p, o, g = _make(oracle, engine, params, 200, 0.45, 31)
    po, pg = o.pairs(), g.pairs()
    assert np.array_equal(_pair_keys(po), _pair_keys(pg))
    assert np.array_equal(po["contact_active"], pg["contact_active"])
    assert np.array_equal(po["lub_active"], pg["lub_active"])
    d_o, r_o, c_o, od_o = o.assemble()
    d_g, r_g, c_g, od_g = g.assemble()
    assert np.array_equal(r_o, r_g) and np.array_equal(c_o, c_g)
    # same accumulation order; the log(1/(h+lambda)) terms use CUDA's log (<= 1 ulp from glibc)
    assert np.abs(d_o - d_g).max() <= 1e-13 * np.abs(d_o).max()
    assert np.abs(od_o - od_g).max() <= 1e-14 * np.abs(od_o).max()
    for comp in range(4):
        fo, fg = o.force_component(comp), g.force_component(comp)
        if fo is None:
            continue
        scale = max(np.abs(fo).max(), 1e-300)
        assert np.abs(fo - fg).max() <= 1e-12 * scale, comp


@pytest.mark.parametrize("params,n,vf,seed", [(RATE_PARAMS, 200, 0.45, 32), (STRESS_PARAMS, 200, 0.5, 33),
                                              (RATE_PARAMS, 500, 0.5, 34), (ROLLING_PARAMS, 300, 0.52, 35)],
                         ids=["rate200", "stress200", "rate500", "rolling300"])
def test_steps_match_oracle(oracle, engine, params, n, vf, seed):
    p, o, g = _make(oracle, engine, params, n, vf, seed)
    for k in range(4):
        calc = k == 3
        o.step(calc_stress=calc)
        g.step(calc_stress=calc)
        so, sg = o.scalars(), g.scalars()
        assert abs(so["dt"] - sg["dt"]) <= TOL * abs(so["dt"])
        assert abs(so["shear_rate"] - sg["shear_rate"]) <= TOL * abs(so["shear_rate"])
        po, pg = o.particles(), g.particles()
        for key in ("pos", "vel", "ang", "na_vel"):
            scale = max(np.abs(po[key]).max(), 1e-300)
            err = np.abs(po[key] - pg[key]).max() / scale
            assert err <= TOL, (k, key, err)
        qo, qg = o.pairs(), g.pairs()
        assert np.array_equal(_pair_keys(qo), _pair_keys(qg)), k
        assert np.array_equal(qo["contact_active"], qg["contact_active"])
        assert np.array_equal(qo["state"], qg["state"])
        assert np.abs(qo["disp_tan"] - qg["disp_tan"]).max() <= 1e-9 * max(np.abs(qo["disp_tan"]).max(), 1e-12)
    # stresses of the stress-computing step
    for comp in range(8):
        so_ = o.particle_stress(comp)
        if so_ is None:
            continue
        sg_ = g.particle_stress(comp)
        scale = max(np.abs(so_).max(), 1e-300)
        assert np.abs(so_ - sg_).max() <= TOL * scale, comp
    so, sg = o.scalars(), g.scalars()
    assert np.abs(so["total_stress"] - sg["total_stress"]).max() <= TOL * np.abs(so["total_stress"]).max()


def test_fp32_refine_step(oracle, engine):
    p, o, g = _make(oracle, engine, STRESS_PARAMS, 500, 0.5, 35, precision=1)
    for k in range(2):
        o.step()
        g.step()
    po, pg = o.particles(), g.particles()
    err = np.abs(po["vel"] - pg["vel"]).max() / np.abs(po["vel"]).max()
    assert err <= 1e-8, err


@pytest.mark.parametrize("params,n,vf,seed,twod", [(RATE_PARAMS, 400, 0.52, 36, False),
                                                  (RATE_PARAMS, 500, 0.75, 37, True)], ids=["3d", "2d"])
def test_thin_skin_rebuilds_keep_pair_lists(oracle, engine, params, n, vf, seed, twod):
    """A thin pair-superset skin makes the per-step superset check (one CTA
    per cell, neighbour cells staged in shared memory) trigger rebuilds
    often; every step's interactions must still be exactly the oracle's."""
    from lf_dem_gb300 import packing as PK
    p = PK.generate(n, vf, seed=seed, twodim=twod)
    o = oracle.OracleSim(params, p.position, p.radius, p.lx, p.ly, p.lz)
    o.first_time()
    g = engine.Sim(params, p.position, p.radius, p.lx, p.ly, p.lz, skin=0.001)
    for k in range(25):
        o.step()
        g.step()
        qo, qg = o.pairs(), g.pairs()
        assert np.array_equal(_pair_keys(qo), _pair_keys(qg)), k
        assert np.array_equal(qo["contact_active"], qg["contact_active"]), k
        err = np.abs(o.particles()["pos"] - g.particles()["pos"]).max()
        assert err <= 1e-10 * max(p.lx, p.lz), k
    assert g.scalars()["n_symbolic_runs"] >= 3
    g.close()


@pytest.mark.parametrize("params", [RATE_PARAMS, STRESS_PARAMS], ids=["rate", "stress"])
def test_scalar_interaction_counts(engine, params):
    """lfg_sim_scalars' interaction counts (a device reduction) against the interaction list."""
    p = make_packing(300, 0.52, 41)
    g = engine.Sim(params, p.position, p.radius, p.lx, p.ly, p.lz)
    for _ in range(3):
        g.run(2)
        s = g.scalars()
        pg = g.pairs()
        assert s["n_pairs"] == len(pg)
        assert s["n_contacts"] == int(np.count_nonzero(pg["contact_active"]))
        assert s["n_lub"] == int(np.count_nonzero(pg["lub_active"]))
        assert 0 < s["n_resistance_pairs"] <= s["n_pairs"]
    g.close()


def test_run_timing_covers_every_step(engine):
    """lfg_sim_timing.run_ms: one event pair around a whole lfg_sim_run, so it
    counts every step and the gaps between them (at least the sum of the
    per-step event times, and not far above it)."""
    p = make_packing(400, 0.52, 42)
    g = engine.Sim(STRESS_PARAMS, p.position, p.radius, p.lx, p.ly, p.lz, precision=1)
    g.run(2)
    g.clear_step_times()
    g.run(5)
    t = g.timing()
    ms, _ = g.step_times()
    assert t["run_steps"] == 5 and len(ms) == 5
    assert t["run_ms"] >= 0.999 * float(np.sum(ms))
    assert t["run_ms"] <= 2.0 * float(np.sum(ms)) + 5.0
    g.close()
