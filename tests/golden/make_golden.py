#!/usr/bin/env python3
"""Generate the golden fixtures in tests/golden/ by running LF_DEM's own C++
(compiled from the reference sources into oracle/_ref by `make -C oracle ref`)
on seeded packings, one time step at a time.

Each fixture holds the resolved (non-dimensionalised) parameters, the
configuration, and for every step: the state before the step, the reference's
R_FU (lower CSC) and force / velocity / stress components at that state, and
the state after the step.  The tests replay each step from the stored state
with the CPU oracle and with the GPU engine and compare.

usage: LFDEM_REF=<LF_DEM source dir> make -C oracle ref && python tests/golden/make_golden.py [case | writers_case | writers_pst_case ...]
"""
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)

from lf_dem_gb300 import packing  # noqa: E402
from refdump import read_records  # noqa: E402

HARNESS = os.path.join(ROOT, "oracle", "_ref", "lfdem_ref_harness")

# Parameter files in LF_DEM's Parameter_File syntax (key = value; with unit
# suffixes), resolved by the reference's own unit system inside the harness.
CASES = {
    "rate_n200": dict(n=200, vf=0.45, seed=101, control="r", value="1", suffix="r", steps=4, calc_stress=1,
                      params="""
lub_reduce_parameter = 1e-3;
lub_max_gap = 0.5;
kn = 1e4r;
kt = 0.5kn;
mu_static = 1;
time_end = 2h;
"""),
    "stress_n200": dict(n=200, vf=0.5, seed=102, control="s", value="10", suffix="cl", steps=4, calc_stress=1,
                        params="""
lub_reduce_parameter = 1e-3;
mu_static = 1;
kn = 1e4cl;
kt = 0.5kn;
time_end = 5h;
"""),
    "rate_normal_n200": dict(n=200, vf=0.5, seed=103, control="r", value="2", suffix="r", steps=4,
                             calc_stress=1, params="""
lubrication_model = normal;
friction_model = 0;
lub_reduce_parameter = 1e-2;
kn = 5e3r;
repulsive_length = 0.02;
contact_relaxation_time = 2e-3r;
sd_coeff = 0.5;
time_end = 1h;
"""),
    # rolling friction (mu_rolling > 0, Contact.cpp:162-180, 283-305, 431-435)
    "rolling_n200": dict(n=200, vf=0.5, seed=105, control="r", value="1", suffix="r", steps=4, calc_stress=1,
                         params="""
lub_reduce_parameter = 1e-3;
lub_max_gap = 0.5;
kn = 1e4r;
kt = 0.5kn;
kr = 0.5kn;
mu_static = 1;
mu_rolling = 0.2;
time_end = 2h;
"""),
    # Brownian force at Pe = 1000 (hydro internal units, fixed dt, mid-point
    # predictor-corrector; System.cpp:888-983, 1665-1710, Stress.cpp:270-286);
    # the harness records each step's Brownian force
    "brownian_n200": dict(n=200, vf=0.45, seed=106, control="r", value="1000", suffix="b", steps=6, calc_stress=1,
                          params="""
lub_reduce_parameter = 1e-3;
lub_max_gap = 0.5;
kn = 1e4h;
kt = 0.5kn;
mu_static = 1;
time_end = 1h;
"""),
    # 2D monolayer (ly = 0 in the configuration): the reference's twodimension path
    "rate_2d_n200": dict(n=200, vf=0.7, seed=104, control="r", value="1", suffix="r", steps=4, calc_stress=1,
                         twodim=True, params="""
lub_reduce_parameter = 1e-3;
lub_max_gap = 0.5;
kn = 1e4r;
kt = 0.5kn;
mu_static = 1;
time_end = 2h;
"""),
}


def run_case(name, c, workdir):
    p = packing.generate(c["n"], c["vf"], seed=c["seed"], twodim=c.get("twodim", False))
    conf = os.path.join(workdir, f"{name}.dat")
    packing.write_conf(p, conf)
    par = os.path.join(workdir, f"{name}_params.txt")
    with open(par, "w") as f:
        f.write(c["params"])
    out = os.path.join(workdir, name)
    os.makedirs(out, exist_ok=True)
    r = subprocess.run([HARNESS, conf, par, c["control"], c["value"], c["suffix"], str(c["steps"]), out,
                        str(c["calc_stress"]), "1"], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"harness failed for {name}: {r.stderr[-2000:]}")
    P = read_records(os.path.join(out, "params.bin"))
    data = {"param_" + k: v for k, v in P.items()}
    data["param_file"] = np.frombuffer(c["params"].encode(), dtype=np.uint8)
    data["control_arg"] = np.frombuffer(f"-{c['control']} {c['value']}{c['suffix']}".encode(), dtype=np.uint8)
    with open(conf) as f:
        data["conf_file"] = np.frombuffer(f.read().encode(), dtype=np.uint8)
    keep_pre = {"pre_position", "pre_shear_disp", "pre_time", "pre_strain", "pre_dt", "pre_shear_rate",
                "pre_max_velocity", "pre_max_sliding_velocity", "pre_pairs_i", "pre_pairs_d"}
    keep_post = {"post_position", "post_velocity", "post_ang_velocity", "post_na_velocity", "post_shear_rate",
                 "post_dt", "post_strain", "post_time", "post_shear_disp", "post_pairs_i", "post_pairs_d",
                 "post_total_stress", "post_max_velocity", "post_max_sliding_velocity", "post_brownian_force"}
    for k in range(c["steps"]):
        R = read_records(os.path.join(out, f"step_{k:04d}.bin"))
        last = k == c["steps"]-1
        for key, v in R.items():
            if key.endswith("pairs_d"):
                # keep r, gap, n, disp_tan, f_spring_total, lub coefficients, repulsion and
                # disp_rolling; drop rvec and the sliding velocity
                v = v.reshape(-1, 23)
                v = np.concatenate([v[:, :16], v[:, 20:23]], axis=1).reshape(-1)
            if key in keep_pre or key in keep_post or (k == 0 and key.startswith("stage_")) or \
                    (last and key.startswith("post_stress_")):
                data[f"s{k}_{key}"] = v
    data["nsteps"] = np.array([c["steps"]])
    # the reference's checkpoint of the final state (Simulation::checkpoint)
    for fn, key in (("conf.bin", "conf_bin"), ("chk.bin", "chk_bin")):
        with open(os.path.join(out, fn), "rb") as f:
            data[key] = np.frombuffer(f.read(), dtype=np.uint8)
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **data)
    return os.path.getsize(os.path.join(HERE, f"{name}.npz"))


# Output files: the reference advances to strains k * WRITER_DSTRAIN (k = 1,
# 2) with its own System::timeEvolution and writes data_/st_/par_/int_
# through Simulation::generateOutput (harness output mode).
WRITER_CASES = ["rate_n200", "stress_n200", "rate_normal_n200", "rate_2d_n200"]
WRITER_DSTRAIN = 1e-4
WRITER_OUTPUTS = 2
# The per-particle stress file pst_ (Simulation::outputPstFileTxt): the same
# runs with out_particle_stress letters appended to the Parameter_File; every
# group letter, and one letter outside the reference's table (its group has
# the empty name and no components)
PST_CASES = {"stress_n200": "tcldrb", "rate_normal_n200": "rcxt"}


def run_writers(name, c, workdir, pst=None):
    p = packing.generate(c["n"], c["vf"], seed=c["seed"], twodim=c.get("twodim", False))
    conf = os.path.join(workdir, f"w_{name}.dat")
    packing.write_conf(p, conf)
    par = os.path.join(workdir, f"w_{name}_params.txt")
    params = c["params"] + (f'out_particle_stress = "{pst}";\n' if pst else "")
    with open(par, "w") as f:
        f.write(params)
    out = os.path.join(workdir, ("p_" if pst else "w_") + name)
    os.makedirs(out, exist_ok=True)
    env = dict(os.environ, HARNESS_OUTPUT_DSTRAIN=repr(WRITER_DSTRAIN))
    r = subprocess.run([HARNESS, conf, par, c["control"], c["value"], c["suffix"], str(WRITER_OUTPUTS), out],
                       capture_output=True, text=True, env=env)
    if r.returncode != 0:
        raise RuntimeError(f"harness (output mode) failed for {name}: {r.stderr[-2000:]}")
    data = {"param_file": np.frombuffer(params.encode(), dtype=np.uint8),
            "control": np.frombuffer(c["control"].encode(), dtype=np.uint8),
            "control_value": np.frombuffer((c["value"]+c["suffix"]).encode(), dtype=np.uint8),
            "dstrain": np.array([WRITER_DSTRAIN]), "outputs": np.array([WRITER_OUTPUTS])}
    with open(conf) as f:
        data["conf_file"] = np.frombuffer(f.read().encode(), dtype=np.uint8)
    for kind in (("pst",) if pst else ("data", "st", "par", "int")):
        files = [f for f in os.listdir(out) if f.startswith(kind + "_") and f.endswith(".dat")]
        assert len(files) == 1, (kind, files)
        with open(os.path.join(out, files[0]), "rb") as f:
            data[kind] = np.frombuffer(f.read(), dtype=np.uint8)
    path = os.path.join(HERE, f"writers_pst_{name}.npz" if pst else f"writers_{name}.npz")
    np.savez_compressed(path, **data)
    return os.path.getsize(path)


def main(only=None):
    if not os.path.exists(HARNESS):
        subprocess.run(["make", "-C", os.path.join(ROOT, "oracle"), "ref"], check=True)
    with tempfile.TemporaryDirectory() as wd:
        for name, c in CASES.items():
            if only and name not in only and "writers_" + name not in only:
                continue
            if not only or name in only:
                size = run_case(name, c, wd)
                print(f"{name}: {size/1e3:.0f} kB")
            if name in WRITER_CASES and (not only or name in only or "writers_" + name in only):
                size = run_writers(name, c, wd)
                print(f"writers_{name}: {size/1e3:.0f} kB")
            if name in PST_CASES and (not only or name in only or "writers_pst_" + name in only):
                size = run_writers(name, c, wd, pst=PST_CASES[name])
                print(f"writers_pst_{name}: {size/1e3:.0f} kB")


if __name__ == "__main__":
    main(sys.argv[1:] or None)
