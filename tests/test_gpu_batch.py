"""Many suspensions on one GPU: the batch (lfg_batch_*) and the request server
(lfg_server_*).  Every suspension's result must be the same alone and among
others -- bit for bit, since the kernels are deterministic and suspensions
share nothing -- the autotuner must pick one of its candidate leaf sizes, and
admission must respect the slot count and the HBM budget."""
import numpy as np
import pytest

from _systems import RATE_PARAMS, STRESS_PARAMS, make_packing

pytestmark = pytest.mark.gpu

CASES = [(RATE_PARAMS, 150, 0.45, 71), (STRESS_PARAMS, 260, 0.5, 72), (RATE_PARAMS, 340, 0.52, 73)]


def _packs():
    return [make_packing(n, vf, seed) for _, n, vf, seed in CASES]


def _alone_steps(engine, params, p, nsteps, precision):
    g = engine.Sim(params, p.position, p.radius, p.lx, p.ly, p.lz, precision=precision)
    g.run(nsteps)
    pos = g.particles()["pos"].copy()
    g.close()
    return pos


@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "fp32refine"])
def test_batch_run_matches_alone(engine, precision):
    packs = _packs()
    b = engine.Batch(nthreads=3)
    for (params, *_), p in zip(CASES, packs):
        b.add(params, p.position, p.radius, p.lx, p.ly, p.lz, precision=precision)
    b.run(4)
    for slot, ((params, *_), p) in enumerate(zip(CASES, packs)):
        ref = _alone_steps(engine, params, p, 4, precision)
        got = b.sim(slot).particles()["pos"]
        assert np.array_equal(ref, got), slot
    b.close()


def test_batch_advance_matches_alone(engine):
    packs = _packs()
    targets = [0.004, 0.002, 0.003]
    b = engine.Batch(nthreads=2)
    for (params, *_), p in zip(CASES, packs):
        b.add(params, p.position, p.radius, p.lx, p.ly, p.lz, precision=1)
    b.advance(targets)
    for slot, ((params, *_), p) in enumerate(zip(CASES, packs)):
        g = engine.Sim(params, p.position, p.radius, p.lx, p.ly, p.lz, precision=1)
        g.advance(strain_end=targets[slot])
        sa, sb = g.scalars(), b.sim(slot).scalars()
        assert sa["strain"] >= targets[slot] - 1e-8
        assert sa["total_num_timesteps"] == sb["total_num_timesteps"]
        assert np.array_equal(g.particles()["pos"], b.sim(slot).particles()["pos"]), slot
        g.close()
    b.close()


def test_autotune_picks_a_candidate(engine):
    packs = _packs()
    b = engine.Batch(nthreads=2)
    for (params, *_), p in zip(CASES, packs):
        b.add(params, p.position, p.radius, p.lx, p.ly, p.lz, precision=1)
    b.autotune((8, 32), steps=1)
    for _, n, _, _ in CASES:
        assert b.tuned_leaf(n, 1) in (8, 32)
    b.run(2)   # the re-analysed suspensions keep stepping
    for slot in range(len(CASES)):
        assert np.isfinite(b.sim(slot).particles()["pos"]).all()
    b.close()


def _serve(engine, max_active, budget, packs, strains):
    s = engine.Server(max_active=max_active, hbm_budget_bytes=budget)
    for i, ((params, *_), p) in enumerate(zip(CASES, packs)):
        s.submit(i, params, p.position, p.radius, p.lx, p.ly, p.lz, strain_end=strains[i])
    s.wait(timeout_s=600)
    res = {r.id: r for r in s.poll()}
    pos = {i: s.final_positions(i) for i in res}
    st = s.stats()
    s.close()
    return res, pos, st


def test_server_results_same_alone_and_in_the_mix(engine):
    packs = _packs()
    strains = [0.003, 0.002, 0.002]
    big = 1 << 40
    res1, pos1, st1 = _serve(engine, 1, big, packs, strains)
    res3, pos3, st3 = _serve(engine, 3, big, packs, strains)
    assert st1["peak_active"] == 1
    assert st3["peak_active"] >= 2
    for i in range(len(CASES)):
        assert res1[i].status == 0 and res3[i].status == 0, (res1[i].msg, res3[i].msg)
        assert res1[i].t_submit <= res1[i].t_admit <= res1[i].t_done
        assert res3[i].steps == res1[i].steps
        assert res3[i].strain >= strains[i] - 1e-8
        assert np.array_equal(pos1[i], pos3[i]), i


def test_server_admission_respects_budget(engine):
    packs = _packs()
    strains = [0.002, 0.002, 0.002]
    est = max(engine.footprint_estimate(n, 1) for _, n, _, _ in CASES)
    budget = int(1.5 * est)   # one suspension at a time fits, two do not
    res, _, st = _serve(engine, 3, budget, packs, strains)
    assert all(r.status == 0 for r in res.values())
    assert st["peak_reserved_bytes"] <= budget
    assert st["admitted"] == len(CASES)
