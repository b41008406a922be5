"""Access to the reference fixtures in tests/golden/ (written by
tests/golden/make_golden.py from LF_DEM's own C++ run step by step)."""
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CASES = ["rate_n200", "stress_n200", "rate_normal_n200", "rate_2d_n200", "rolling_n200"]
# Brownian runs: the reference draws its Brownian force from a clock-seeded
# generator; each step's force is recorded and replayed (the CPU oracle has
# no Brownian path, so these are engine-only)
BROWNIAN_CASES = ["brownian_n200"]
PARAM_KEYS = ["kn", "kt", "mu_static", "mu_dynamic", "critical_load", "ft_max", "friction_model", "repulsion_on",
              "repulsion", "repulsive_length", "repulsive_max_length", "lubrication_model", "lub_reduce_parameter",
              "lub_max_gap", "interaction_range", "sd_coeff", "contact_relaxation_time",
              "contact_relaxation_time_tan", "disp_max", "dt", "dt_max", "dt_min", "fixed_dt",
              "integration_method", "control", "shear_rate", "target_stress", "Ehat", "Ohat",
              "init_strain_shear_rate_limit", "init_shear_rate_limit", "mu_rolling", "kr", "brownian"]


def load(name):
    return dict(np.load(os.path.join(GOLDEN, name + ".npz")))


def params(F):
    d = {}
    for k in PARAM_KEYS:
        if "param_" + k not in F:
            continue
        v = F["param_" + k]
        d[k] = tuple(v) if k in ("Ehat", "Ohat") else float(v[0])
    # the reference resolved interaction_range = -1 to 2 + lub_max_gap and
    # kept the lubrication-range function (System.cpp:405-410)
    d["interaction_range"] = -1.0
    return d


def box(F):
    return float(F["param_lx"][0]), float(F["param_ly"][0]), float(F["param_lz"][0])


def pairs(F, k, when):
    pi = F[f"s{k}_{when}_pairs_i"].reshape(-1, 6)
    raw = F[f"s{k}_{when}_pairs_d"]
    pd = raw.reshape(len(pi), -1) if len(pi) else raw.reshape(0, 19)
    o = np.lexsort((pi[:, 1], pi[:, 0]))
    return pi[o], pd[o]


def removal_steps(F):
    """Steps whose result depends on LF_DEM's swap-removal side effect: when an
    interaction leaves the range, System::updateInteractions moves the last
    vector element into its slot through the copy-swap assignment, which
    re-runs Interaction::activateForceMembers on it (Interaction.cpp:57-66,
    System.cpp:1395-1400) and so resets that pair's tangential spring and
    zeroes its spring and repulsive forces until its next update.  Which pair
    is moved depends on the heap-address-ordered cell lists, so these steps
    are compared on the pair set only."""
    n = int(F["nsteps"][0])
    bad = set()
    for k in range(n):
        a = {tuple(x) for x in pairs(F, k, "pre")[0][:, :2]}
        b = {tuple(x) for x in pairs(F, k, "post")[0][:, :2]}
        if a - b:
            bad.add(k)
            bad.add(k + 1)
    return bad


def restore(sim, F, k):
    """Put a simulation (oracle or engine, same method names) into the
    reference's state before step k."""
    pi, pd = pairs(F, k, "pre")
    for a, d in zip(pi, pd):
        if a[2]:  # contact active
            sim.set_contact(int(a[0]), int(a[1]), int(a[3]), d[5:8].copy())
            if len(d) >= 19:
                sim.set_contact_rolling(int(a[0]), int(a[1]), d[16:19].copy())
    sim.refresh()
    sim.set_clock(float(F[f"s{k}_pre_time"][0]), float(F[f"s{k}_pre_strain"][0]), float(F[f"s{k}_pre_dt"][0]),
                  float(F[f"s{k}_pre_shear_rate"][0]), float(F[f"s{k}_pre_max_velocity"][0]),
                  float(F[f"s{k}_pre_max_sliding_velocity"][0]))


def csc_to_blocks(F, n):
    """Reference CSC (lower, 6n x 6n) -> dense symmetric matrix."""
    cp, ci, cx = F["s0_stage_csc_p"], F["s0_stage_csc_i"], F["s0_stage_csc_x"]
    A = np.zeros((6 * n, 6 * n))
    for j in range(6 * n):
        sl = slice(cp[j], cp[j + 1])
        A[ci[sl], j] += cx[sl]
    return A + np.tril(A, -1).T


def dense_from_blocks(mod, d15, r, c, o18, n):
    A = np.zeros((6 * n, 6 * n))
    for i in range(n):
        A[6 * i:6 * i + 6, 6 * i:6 * i + 6] = mod.dblock_dense(d15[i])
    for e in range(len(r)):
        M = mod.odblock_dense(o18[e])
        A[6 * r[e]:6 * r[e] + 6, 6 * c[e]:6 * c[e] + 6] = M
        A[6 * c[e]:6 * c[e] + 6, 6 * r[e]:6 * r[e] + 6] = M.T
    return A
