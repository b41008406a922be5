"""The CPU oracle against LF_DEM's own C++ (fixtures in tests/golden/): the
resolved parameters, R_FU entry by entry, force components, and every time
step replayed from the reference's state (positions, velocities, pair list,
contact and friction states, tangential springs, shear rate, stresslets)."""
import numpy as np
import pytest

import _golden as G

NAMES = {"contact": 0, "dashpot": 1, "hydro": 2, "repulsion": 3}
STRESS = {"contact": 0, "dashpot": 1, "hydro": 2, "repulsion": 3, "M_E_hydro": 4}


def _make(oracle, F, k):
    lx, ly, lz = G.box(F)
    o = oracle.OracleSim(G.params(F), F[f"s{k}_pre_position"].reshape(-1, 3), F["param_radius"], lx, ly, lz,
                         F[f"s{k}_pre_shear_disp"])
    o.first_time()
    G.restore(o, F, k)
    return o


@pytest.mark.parametrize("name", G.CASES)
def test_initial_matrix_and_forces(oracle, name):
    F = G.load(name)
    n = len(F["param_radius"])
    o = _make(oracle, F, 0)
    pi, _ = G.pairs(F, 0, "pre")
    po = o.pairs()
    assert np.array_equal(np.stack([po["p0"], po["p1"]], 1), pi[:, :2])
    assert np.array_equal(po["contact_active"], pi[:, 2])
    d15, r, c, o18 = o.assemble()
    A = G.dense_from_blocks(oracle, d15, r, c, o18, n)
    Aref = G.csc_to_blocks(F, n)
    assert np.abs(A - Aref).max() <= 1e-13 * np.abs(Aref).max()
    # force components at the rate the reference used for them (1 under stress control)
    if F["param_control"][0] == 1:
        o.set_clock(float(F["s0_pre_time"][0]), float(F["s0_pre_strain"][0]), float(F["s0_pre_dt"][0]), 1.0,
                    0.0, float(F["s0_pre_max_sliding_velocity"][0]))
    for nm, comp in NAMES.items():
        key = "s0_stage_force_" + nm
        if key not in F:
            continue
        ref = F[key].reshape(-1, 6)
        got = o.force_component(comp)
        assert np.abs(got - ref).max() <= 1e-12 * max(np.abs(ref).max(), 1e-300), nm


@pytest.mark.parametrize("name", G.CASES)
def test_steps_replayed_from_reference_state(oracle, name):
    F = G.load(name)
    nsteps = int(F["nsteps"][0])
    skip = G.removal_steps(F)
    checked = 0
    for k in range(nsteps):
        o = _make(oracle, F, k)
        last = k == nsteps - 1
        o.step(calc_stress=True)
        pi, pd = G.pairs(F, k, "post")
        po = o.pairs()
        assert np.array_equal(np.stack([po["p0"], po["p1"]], 1), pi[:, :2]), k
        if k in skip:
            continue
        checked += 1
        assert np.array_equal(po["contact_active"], pi[:, 2]), k
        assert np.array_equal(po["state"], pi[:, 3]), k
        assert np.abs(po["disp_tan"] - pd[:, 5:8]).max() <= 1e-9 * max(np.abs(pd[:, 5:8]).max(), 1e-12)
        s = o.scalars()
        for key in ("shear_rate", "dt", "strain"):
            ref = float(F[f"s{k}_post_{key}"][0])
            assert abs(s[key] - ref) <= 1e-10 * abs(ref), (k, key)
        p = o.particles()
        for ours, theirs in (("pos", "position"), ("vel", "velocity"), ("ang", "ang_velocity"),
                             ("na_vel", "na_velocity")):
            ref = F[f"s{k}_post_{theirs}"].reshape(-1, 3)
            err = np.abs(p[ours] - ref).max() / np.abs(ref).max()
            assert err <= 1e-10, (k, ours, err)
        ts = F[f"s{k}_post_total_stress"]
        assert np.abs(s["total_stress"] - ts).max() <= 1e-10 * np.abs(ts).max(), k
        if last:
            for nm, comp in STRESS.items():
                key = f"s{k}_post_stress_{nm}"
                if key not in F:
                    continue
                ref = F[key].reshape(-1, 6)
                got = o.particle_stress(comp)
                assert np.abs(got - ref).max() <= 1e-10 * np.abs(ref).max(), nm
    assert checked >= 1
