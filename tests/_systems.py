"""Shared test inputs: seeded packings and flat parameter sets for the oracle
and the GPU engine (same values, two structs)."""
import numpy as np

from lf_dem_gb300 import packing

# cfg1-like: rate control "-r 1r" (hydro units: shear rate 1, repulsion 1),
# kn = 1e4, kt = 0.5 kn, mu = 1, lambda = 1e-3, lub_max_gap = 0.5
RATE_PARAMS = dict(kn=1e4, kt=5e3, mu_static=1.0, mu_dynamic=1.0, friction_model=1, repulsion_on=1,
                   repulsion=1.0, repulsive_length=0.05, repulsive_max_length=-1.0, lubrication_model=2,
                   lub_reduce_parameter=1e-3, lub_max_gap=0.5, interaction_range=-1.0, sd_coeff=1.0,
                   contact_relaxation_time=1e-3, contact_relaxation_time_tan=-1.0, disp_max=1e-3, dt=1e-4,
                   dt_max=-1.0, dt_min=-1.0, fixed_dt=0, integration_method=1, control=0, shear_rate=1.0,
                   target_stress=0.0, Ehat=(0, 0, 0.5, 0, 0, 0), Ohat=(0, 0.5, 0),
                   init_strain_shear_rate_limit=0.0, init_shear_rate_limit=999.0, critical_load=0.0,
                   ft_max=0.0)

# cfg2-like: stress control "-s 10cl" (critical-load units, friction_model 2)
STRESS_PARAMS = dict(RATE_PARAMS)
STRESS_PARAMS.update(friction_model=2, critical_load=1.0, repulsion_on=0, repulsion=0.0, control=1,
                     shear_rate=0.0, target_stress=10.0 / 6 / np.pi)


# rolling friction on top of the rate-controlled set (Contact.cpp:162-180, 283-305)
ROLLING_PARAMS = dict(RATE_PARAMS)
ROLLING_PARAMS.update(mu_rolling=0.2, kr=5e3)


def make_packing(n, vf, seed):
    return packing.generate(n, vf, seed=seed)
