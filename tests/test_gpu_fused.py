"""The fused batch (lfg_batch_create_fused): suspensions of uneven N advanced
in lockstep through one joint factorisation and solve of the block-diagonal
system of all of them.  Every suspension's result must be what it gets alone
(lfg_sim): within 1e-12 relative in FP64 (the joint factor's fronts are the
suspensions' own, computed by the same kernels) and within the refinement's
1e-8 in FP32 + refinement (the joint refinement may take more iterations than
one suspension alone); pair lists and contact states identical.  A fused step
launches far fewer kernels than the suspensions stepping one by one."""
import numpy as np
import pytest

from _systems import RATE_PARAMS, STRESS_PARAMS, make_packing

pytestmark = pytest.mark.gpu

CASES = [(RATE_PARAMS, 150, 0.45, 81), (STRESS_PARAMS, 260, 0.5, 82), (RATE_PARAMS, 340, 0.52, 83),
         (dict(RATE_PARAMS, shear_rate=0.1), 420, 0.5, 84)]
TOL = {0: 1e-12, 1: 1e-8}


def _rel(a, b):
    return float(np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(np.asarray(b)).max(), 1e-300))


def _packs():
    return [make_packing(n, vf, seed) for _, n, vf, seed in CASES]


def _compare(g, h, tol, what):
    pa, pb = g.particles(), h.particles()
    for key in ("pos", "vel", "ang", "na_vel"):
        assert _rel(pb[key], pa[key]) <= tol, (what, key, _rel(pb[key], pa[key]))
    qa, qb = g.pairs(), h.pairs()
    assert np.array_equal(np.stack([qa["p0"], qa["p1"]], 1), np.stack([qb["p0"], qb["p1"]], 1)), what
    assert np.array_equal(qa["contact_active"], qb["contact_active"]), what
    sa, sb = g.scalars(), h.scalars()
    assert _rel(sb["total_stress"], sa["total_stress"]) <= tol, what
    assert abs(sb["strain"] - sa["strain"]) <= tol * max(abs(sa["strain"]), 1e-300), what
    assert sa["total_num_timesteps"] == sb["total_num_timesteps"], what


@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "fp32refine"])
def test_fused_run_matches_alone(engine, precision):
    packs = _packs()
    b = engine.Batch(fused=True, precision=precision)
    for (params, *_), p in zip(CASES, packs):
        b.add(params, p.position, p.radius, p.lx, p.ly, p.lz)
    nsteps = 6
    b.run(nsteps)
    fused_kernels = b.stats()["kernels"]
    alone_kernels = 0
    for slot, ((params, *_), p) in enumerate(zip(CASES, packs)):
        g = engine.Sim(params, p.position, p.radius, p.lx, p.ly, p.lz, precision=precision)
        g.run(nsteps)
        _, k = g.step_times()
        alone_kernels += k
        _compare(g, b.sim(slot), TOL[precision], slot)
        g.close()
    st = b.stats()
    assert st["fused"] == 1 and st["joint_analyses"] >= 1
    # one launch per level and stage serves every suspension
    assert fused_kernels < 0.6 * alone_kernels, (fused_kernels, alone_kernels)
    b.close()


def test_fused_advance_matches_alone(engine):
    packs = _packs()
    targets = [0.004, 0.002, 0.003, 0.0015]
    b = engine.Batch(fused=True, precision=1)
    for (params, *_), p in zip(CASES, packs):
        b.add(params, p.position, p.radius, p.lx, p.ly, p.lz)
    b.advance(targets)
    for slot, ((params, *_), p) in enumerate(zip(CASES, packs)):
        g = engine.Sim(params, p.position, p.radius, p.lx, p.ly, p.lz, precision=1)
        g.advance(strain_end=targets[slot])
        assert g.scalars()["strain"] >= targets[slot] - 1e-8
        _compare(g, b.sim(slot), TOL[1], slot)
        # the stress-computing last step ran for this suspension too
        sa, sb = g.particle_stress(0), b.sim(slot).particle_stress(0)
        assert _rel(sb, sa) <= TOL[1]
        g.close()
    b.close()


def test_fused_superset_rebuild_keeps_parity(engine):
    """A thin pair-superset skin, so that supersets run out of it within the
    run: a suspension's pattern change redoes the joint analysis mid-run."""
    params, n, vf, seed = CASES[2]
    p = make_packing(n, vf, seed)
    q = make_packing(200, 0.5, 85)
    skin = 0.002
    b = engine.Batch(fused=True, precision=0)
    b.add(params, p.position, p.radius, p.lx, p.ly, p.lz, skin=skin)
    b.add(RATE_PARAMS, q.position, q.radius, q.lx, q.ly, q.lz, skin=skin)
    nsteps = 40
    b.run(nsteps)
    assert b.stats()["joint_analyses"] >= 3
    for slot, (prm, pk) in enumerate(((params, p), (RATE_PARAMS, q))):
        g = engine.Sim(prm, pk.position, pk.radius, pk.lx, pk.ly, pk.lz, precision=0, skin=skin)
        g.run(nsteps)
        _compare(g, b.sim(slot), 1e-10, slot)
        g.close()
    b.close()


def test_fused_autotune_and_refusals(engine):
    packs = _packs()
    b = engine.Batch(fused=True, precision=1)
    for (params, *_), p in zip(CASES[:2], packs[:2]):
        b.add(params, p.position, p.radius, p.lx, p.ly, p.lz)
    b.autotune((8, 32), steps=1)
    assert b.tuned_leaf(CASES[0][1], 1) in (8, 32)
    b.run(1)
    # a Brownian suspension is refused, and a member cannot step on its own
    brown = dict(RATE_PARAMS, brownian=1.0)
    pk = packs[0]
    with pytest.raises(engine.LFGError):
        b.add(brown, pk.position, pk.radius, pk.lx, pk.ly, pk.lz)
    with pytest.raises(engine.LFGError):
        b.sim(0).step()
    b.close()
