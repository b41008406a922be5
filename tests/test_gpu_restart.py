"""Checkpoint and restart through LF_DEM's own file formats: the engine runs a
few steps, saves its state as conf_*.dat (positions, box, contact springs)
and chk_*.dat (strain, time), a new engine and the CPU oracle both restart
from those files, and the restarted runs agree (FP64, 1e-10 relative)."""
import numpy as np
import pytest

from _systems import ROLLING_PARAMS, make_packing

pytestmark = pytest.mark.gpu


def test_restart_from_checkpoint_matches_oracle(engine, oracle, tmp_path):
    p = make_packing(300, 0.52, 91)
    g = engine.Sim(ROLLING_PARAMS, p.position, p.radius, p.lx, p.ly, p.lz)
    g.run(3)
    sc = g.scalars()
    c0, c1, dt, dr = g.contact_states()
    assert len(c0) > 0 and np.abs(dr).max() > 0
    conf, chk = tmp_path / "conf.dat", tmp_path / "chk.dat"
    pos = g.particles()["pos"]
    engine.write_conf_binary(conf, pos, p.radius, p.lx, p.ly, p.lz, p.vf, tuple(sc["shear_disp"]), (c0, c1, dt, dr))
    engine.write_checkpoint(chk, sc["strain"], sc["time"], sc["time"])
    g.close()

    c = engine.read_conf_binary(conf)
    strain, time, _ = engine.read_checkpoint(chk)
    contacts = [(int(a), int(b), t) for a, b, t in zip(c["p0"], c["p1"], c["disp_tan"])]
    r = engine.Sim(ROLLING_PARAMS, c["position"], c["radius"], c["lx"], c["ly"], c["lz"], le_disp=c["le_disp"],
                   contacts=contacts)
    o = oracle.OracleSim(ROLLING_PARAMS, c["position"], c["radius"], c["lx"], c["ly"], c["lz"], le_disp=c["le_disp"],
                         contacts=contacts)
    for a, b, d in zip(c["p0"], c["p1"], c["disp_rolling"]):
        r.set_contact_rolling(int(a), int(b), d)
        o.set_contact_rolling(int(a), int(b), d)
    r.refresh()   # creation already ran the first-time force update; redo it with the rolling springs
    o.first_time()
    for sim in (r, o):
        sim.set_clock(time, strain, sc["dt"], sc["shear_rate"], sc["max_velocity"], sc["max_sliding_velocity"])
    for _ in range(3):
        r.step()
        o.step()
    pr, po = r.particles(), o.particles()
    for key in ("pos", "vel", "ang"):
        scale = max(np.abs(po[key]).max(), 1e-300)
        assert np.abs(pr[key] - po[key]).max() <= 1e-10 * scale, key
    assert abs(r.scalars()["strain"] - o.scalars()["strain"]) <= 1e-12
