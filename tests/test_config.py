"""LF_DEM's Parameter_File and unit system (lfg_config_resolve) against the
parameters the reference itself resolved for the golden fixtures (the
harness dumps ParameterSet after Simulation::setupSimulation and
System::setupParameters): every used value bit for bit, and time_end /
strain_end.  Forces that the input never sets are left uninitialised by the
reference and are not compared.  Runs on the CPU (no device call)."""
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


@pytest.mark.parametrize("name", G.CASES+G.BROWNIAN_CASES)
def test_resolved_parameters_match_reference(E, name):
    F = G.load(name)
    text = bytes(F["param_file"]).decode()
    ctl = bytes(F["control_arg"]).decode().split()
    d, time_end, strain_end = E.resolve_config(text, ctl[0][1], ctl[1])
    for k in G.PARAM_KEYS:
        if "param_" + k not in F:
            continue
        if k == "critical_load" and d["friction_model"] not in (2, 3):
            continue
        if k == "repulsion" and not d["repulsion_on"]:
            continue
        got = d[k]
        if k == "interaction_range" and got == -1:
            got = 2 + d["lub_max_gap"]   # the reference stores the lubrication range it then uses
        got = np.atleast_1d(np.asarray(got, dtype=float))
        ref = np.atleast_1d(F["param_" + k].astype(float))
        assert np.array_equal(got, ref), (k, got, ref)
    assert time_end == float(F["param_time_end"][0])
    assert strain_end == float(F["param_strain_end"][0])


def test_units_and_errors(E):
    # kt given as a fraction of kn, contact relaxation in repulsive units, rate 2r
    d, te, se = E.resolve_config("kn = 1e4r; kt = 0.5kn; contact_relaxation_time = 2e-3r; time_end = 3h;", "r", "2r")
    assert d["repulsion"] == 0.5 and d["kn"] == 5e3 and d["kt"] == 2.5e3
    assert d["contact_relaxation_time"] == 2e-3 / 0.5 and d["shear_rate"] == 1.0
    assert (te, se) == (-1.0, 3.0)
    # stress control in critical-load units forces the critical-load friction model
    d, te, se = E.resolve_config("kn = 1e4cl;", "s", "10cl")
    assert d["friction_model"] == 2 and d["critical_load"] == 1.0 and d["control"] == 1
    assert d["target_stress"] == 10 / 6 / np.pi
    for bad in ("kn = 1e4r // comment;", "unknown_key = 1;", "kn = 1e4;", "kn = 1e4q;", "brownian = 1r;"):
        with pytest.raises(E.LFGError):
            E.resolve_config(bad, "r", "1r")
    # a comment drops the text before it in the statement, as the reference's reader does
    d, _, _ = E.resolve_config("/* stiff */ kn = 3e4r; mu_static = 0.5;", "r", "1r")
    assert d["kn"] == 3e4 and d["mu_static"] == 0.5
