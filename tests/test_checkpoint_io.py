"""LF_DEM checkpoint files (conf_*.dat binary configuration, chk_*.dat state)
read and written by the engine library, against files the reference itself
wrote at the end of each golden run (Simulation::checkpoint): the parsed
positions, radii, box and contact springs equal the reference's final state,
writing them back reproduces the reference's bytes, the old unlabelled format
with unsigned-short particle numbers is recognised, and the state file round
trips.  Host I/O only (runs on the CPU)."""
import os
import struct

import numpy as np
import pytest

import _golden as G


@pytest.fixture(scope="module")
def E():
    import lf_dem_gb300 as E
    from lf_dem_gb300 import build as B
    B.build()
    E._lib = None
    E.load()
    return E


@pytest.mark.parametrize("name", G.CASES)
def test_reference_checkpoint_roundtrip(E, name, tmp_path):
    F = G.load(name)
    last = int(F["nsteps"][0]) - 1
    conf = tmp_path / "conf_ref.dat"
    conf.write_bytes(bytes(F["conf_bin"]))
    c = E.read_conf_binary(conf)
    assert c["format"] == 2
    n = len(F["param_radius"])
    pos = F[f"s{last}_post_position"].reshape(-1, 3)
    assert np.array_equal(c["position"], pos) and np.array_equal(c["radius"], F["param_radius"])
    assert (c["lx"], c["ly"], c["lz"]) == G.box(F)
    assert c["le_disp"] == tuple(F[f"s{last}_post_shear_disp"])
    # contacts: the active ones of the final pair dump, with their springs
    pi, pd = G.pairs(F, last, "post")
    act = pi[:, 2] == 1
    ref = {(int(a), int(b)): (d[5:8], d[16:19]) for (a, b), d in zip(pi[act, :2], pd[act])}
    got = {(int(a), int(b)): (t, r) for a, b, t, r in zip(c["p0"], c["p1"], c["disp_tan"], c["disp_rolling"])}
    assert set(got) == set(ref)
    for k, (t, r) in got.items():
        assert np.array_equal(t, ref[k][0]) and np.array_equal(r, ref[k][1]), k
    out = tmp_path / "conf_out.dat"
    E.write_conf_binary(out, c["position"], c["radius"], c["lx"], c["ly"], c["lz"], c["vf"], c["le_disp"],
                        (c["p0"], c["p1"], c["disp_tan"], c["disp_rolling"]))
    assert out.read_bytes() == bytes(F["conf_bin"])
    chk = tmp_path / "chk_ref.dat"
    chk.write_bytes(bytes(F["chk_bin"]))
    strain, time, tsim = E.read_checkpoint(chk)
    assert strain == float(F[f"s{last}_post_strain"][0]) and time == float(F[f"s{last}_post_time"][0])
    chk2 = tmp_path / "chk_out.dat"
    E.write_checkpoint(chk2, strain, time, tsim)
    assert chk2.read_bytes() == bytes(F["chk_bin"])
    assert n == len(c["radius"])


def test_old_unsigned_short_contact_format(E, tmp_path):
    # unlabelled header (np first), contacts with unsigned short particle numbers
    np_, vf, lx, ly, lz = 3, 0.3, 10.0, 0.0, 10.0
    pos = [(1.0, 0.0, 1.0, 1.0), (3.0, 0.0, 1.0, 1.0), (5.0, 0.0, 1.0, 1.4)]
    raw = struct.pack("<i6d", np_, vf, lx, ly, lz, 0.25, 0.0)
    for p in pos:
        raw += struct.pack("<4d", *p)
    raw += struct.pack("<I", 2)
    raw += struct.pack("<HH6d", 0, 1, 0.1, 0.2, 0.3, 0.0, 0.0, 0.0)
    raw += struct.pack("<HH6d", 1, 2, -0.1, 0.0, 0.5, 0.01, 0.02, 0.03)
    f = tmp_path / "old.dat"
    f.write_bytes(raw)
    c = E.read_conf_binary(f)
    assert c["format"] == 1 and c["le_disp"] == (0.25, 0.0)
    assert list(c["p0"]) == [0, 1] and list(c["p1"]) == [1, 2]
    assert np.array_equal(c["disp_tan"][1], [-0.1, 0.0, 0.5]) and np.array_equal(c["disp_rolling"][1], [0.01, 0.02, 0.03])
    assert np.array_equal(c["position"][2], [5.0, 0.0, 1.0]) and c["radius"][2] == 1.4
    with pytest.raises(E.LFGError):
        E.read_conf_binary(tmp_path / "missing.dat")
