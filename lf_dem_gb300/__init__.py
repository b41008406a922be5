"""lf_dem_gb300 -- GB300 (sm_103a) engine for LF_DEM's per-timestep hydrodynamic core.

The product is the C-ABI shared library lf_dem_gb300/_lib/liblfdem_gb300.so
(declared in include/lfdem_gb300.h).  This module is a thin ctypes front-end
used by the tests and the benchmark; it loads the library and fails loudly if
it is missing or if no GB300 is present.  There is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "liblfdem_gb300.so")

LFG_OK = 0
LFG_ERR_BAD_ARG = 1
LFG_ERR_OOM = 2
LFG_ERR_NOT_SPD = 3
LFG_ERR_TIMEOUT = 4
LFG_ERR_CUDA = 5
LFG_ERR_NO_DEVICE = 6
LFG_ERR_NOT_CONVERGED = 7
PREC_FP64 = 0
PREC_FP32_REFINE = 1


class Status(C.Structure):
    _fields_ = [("code", C.c_int), ("info", C.c_int), ("refine_iters", C.c_int), ("pad_", C.c_int),
                ("refine_residual", C.c_double), ("msg", C.c_char * 200)]


class OutputUnits(C.Structure):
    _fields_ = [("unit", C.c_char * 32), ("internal_to_output", C.c_double), ("input_value", C.c_double),
                ("out_data_particle", C.c_int), ("out_data_interaction", C.c_int), ("origin_zero_flow", C.c_int),
                ("pad_", C.c_int), ("out_particle_stress", C.c_char * 32)]


class OutputConfig(C.Structure):
    _fields_ = [("directory", C.c_char_p), ("simu_name", C.c_char_p), ("version", C.c_char_p),
                ("unit", C.c_char_p), ("internal_to_output", C.c_double), ("input_value", C.c_double),
                ("volume_fraction", C.c_double), ("out_data_particle", C.c_int),
                ("out_data_interaction", C.c_int), ("origin_zero_flow", C.c_int), ("diminish_output", C.c_int),
                ("force_overwrite", C.c_int), ("out_particle_stress", C.c_char_p)]


class Params(C.Structure):
    _fields_ = [
        ("kn", C.c_double), ("kt", C.c_double),
        ("mu_static", C.c_double), ("mu_dynamic", C.c_double),
        ("critical_load", C.c_double), ("ft_max", C.c_double),
        ("friction_model", C.c_int), ("repulsion_on", C.c_int),
        ("repulsion", C.c_double), ("repulsive_length", C.c_double),
        ("repulsive_max_length", C.c_double),
        ("lubrication_model", C.c_int),
        ("lub_reduce_parameter", C.c_double), ("lub_max_gap", C.c_double),
        ("interaction_range", C.c_double), ("sd_coeff", C.c_double),
        ("contact_relaxation_time", C.c_double), ("contact_relaxation_time_tan", C.c_double),
        ("disp_max", C.c_double), ("dt", C.c_double), ("dt_max", C.c_double), ("dt_min", C.c_double),
        ("fixed_dt", C.c_int), ("integration_method", C.c_int), ("control", C.c_int),
        ("shear_rate", C.c_double), ("target_stress", C.c_double),
        ("Ehat", C.c_double * 6), ("Ohat", C.c_double * 3),
        ("init_strain_shear_rate_limit", C.c_double), ("init_shear_rate_limit", C.c_double),
        ("mu_rolling", C.c_double), ("kr", C.c_double), ("brownian", C.c_double), ("seed", C.c_uint64),
    ]


class Options(C.Structure):
    _fields_ = [("precision", C.c_int), ("device", C.c_int), ("refine_tol", C.c_double),
                ("refine_max_iter", C.c_int), ("pad0_", C.c_int), ("skin", C.c_double),
                ("use_graphs", C.c_int), ("leaf_size", C.c_int), ("dof_2d", C.c_int), ("pad2_", C.c_int)]


class SolverStats(C.Structure):
    _fields_ = [("n_blocks", C.c_int), ("n_supernodes", C.c_int), ("n_levels", C.c_int),
                ("max_front", C.c_int), ("nnz_L", C.c_int64), ("flops_factor", C.c_double),
                ("front_bytes", C.c_int64), ("n_factor_launches", C.c_int), ("n_solve_launches", C.c_int)]


class SimScalars(C.Structure):
    _fields_ = [
        ("time", C.c_double), ("strain", C.c_double), ("shear_rate", C.c_double), ("dt", C.c_double),
        ("shear_disp", C.c_double * 2), ("max_velocity", C.c_double), ("max_sliding_velocity", C.c_double),
        ("total_stress", C.c_double * 6), ("viscosity", C.c_double), ("N1", C.c_double), ("N2", C.c_double),
        ("rate_prop_shearstress", C.c_double), ("rate_indep_shearstress", C.c_double),
        ("total_num_timesteps", C.c_int64), ("n_pairs", C.c_int), ("n_contacts", C.c_int),
        ("n_lub", C.c_int), ("n_resistance_pairs", C.c_int), ("n_superset_pairs", C.c_int),
        ("n_symbolic_runs", C.c_int), ("last_refine_iters", C.c_int), ("pad_", C.c_int),
        ("last_refine_residual", C.c_double),
    ]


class Pair(C.Structure):
    _fields_ = [
        ("p0", C.c_int32), ("p1", C.c_int32), ("z_offset", C.c_int32), ("contact_active", C.c_int32),
        ("state", C.c_int32), ("lub_active", C.c_int32), ("pad0_", C.c_int32), ("pad1_", C.c_int32),
        ("r", C.c_double), ("reduced_gap", C.c_double),
        ("nvec", C.c_double * 3), ("rvec", C.c_double * 3), ("disp_tan", C.c_double * 3),
        ("f_spring_total", C.c_double * 3), ("lub_coeff", C.c_double), ("log_lub_coeff", C.c_double),
        ("rep_force", C.c_double * 3),
    ]


class Request(C.Structure):
    _fields_ = [("id", C.c_int64), ("params", C.c_void_p), ("options", C.c_void_p), ("n", C.c_int),
                ("pos", C.c_void_p), ("radius", C.c_void_p), ("lx", C.c_double), ("ly", C.c_double),
                ("lz", C.c_double), ("strain_end", C.c_double)]


class Result(C.Structure):
    _fields_ = [("id", C.c_int64), ("status", C.c_int), ("n", C.c_int), ("steps", C.c_int64),
                ("t_submit", C.c_double), ("t_admit", C.c_double), ("t_done", C.c_double),
                ("strain", C.c_double), ("shear_rate", C.c_double), ("viscosity", C.c_double),
                ("N1", C.c_double), ("N2", C.c_double), ("footprint_est", C.c_int64),
                ("footprint_bytes", C.c_int64), ("msg", C.c_char * 120)]


class ServerStats(C.Structure):
    _fields_ = [("submitted", C.c_int64), ("admitted", C.c_int64), ("active", C.c_int), ("queued", C.c_int),
                ("peak_active", C.c_int), ("pad_", C.c_int), ("reserved_bytes", C.c_int64),
                ("peak_reserved_bytes", C.c_int64), ("budget_bytes", C.c_int64)]


class BatchStats(C.Structure):
    _fields_ = [("kernels", C.c_int64), ("joint_analyses", C.c_int), ("last_refine_iters", C.c_int),
                ("factor_flops", C.c_double), ("fused", C.c_int), ("pad_", C.c_int)]


class SimTiming(C.Structure):
    _fields_ = [("ms", C.c_double * 8), ("launches", C.c_int64), ("factor_flops", C.c_double),
                ("solve_bytes", C.c_double), ("rebuild_ms", C.c_double), ("rebuilds", C.c_int), ("run_steps", C.c_int),
                ("run_ms", C.c_double)]


# Every extern "C" symbol declared in include/lfdem_gb300.h.
EXPORTS = [
    "lfg_default_options", "lfg_device_info",
    "lfg_solver_create", "lfg_solver_set_blocks", "lfg_solver_factorize", "lfg_solver_solve",
    "lfg_solver_solve_device", "lfg_solver_get_stats", "lfg_solver_destroy",
    "lfg_sim_create", "lfg_sim_advance", "lfg_sim_step", "lfg_sim_run", "lfg_sim_get_scalars",
    "lfg_sim_get_particles", "lfg_sim_get_num_pairs", "lfg_sim_get_pairs", "lfg_sim_get_particle_stress",
    "lfg_sim_get_velocity_component", "lfg_sim_set_contact", "lfg_sim_set_clock", "lfg_sim_refresh",
    "lfg_sim_assemble", "lfg_sim_force_component", "lfg_sim_get_timing", "lfg_sim_get_step_times",
    "lfg_sim_clear_step_times", "lfg_sim_destroy", "lfg_sim_force_component_noalloc",
    "lfg_sim_advance_partial", "lfg_sim_set_contact_rolling", "lfg_config_resolve",
    "lfg_sim_get_contact_states", "lfg_conf_write_binary", "lfg_conf_read_binary", "lfg_checkpoint_write",
    "lfg_checkpoint_read", "lfg_sim_set_leaf_size", "lfg_sim_device_bytes", "lfg_footprint_estimate",
    "lfg_batch_create", "lfg_batch_add", "lfg_batch_size", "lfg_batch_sim", "lfg_batch_run", "lfg_batch_advance",
    "lfg_batch_autotune", "lfg_batch_tuned_leaf", "lfg_batch_destroy", "lfg_batch_create_fused",
    "lfg_batch_get_stats",
    "lfg_server_create", "lfg_server_submit", "lfg_server_poll", "lfg_server_wait", "lfg_server_final_positions",
    "lfg_server_get_stats", "lfg_server_destroy",
    "lfg_config_output", "lfg_output_open", "lfg_output_write", "lfg_output_close", "lfg_solver_multiply_factor",
    "lfg_sim_set_brownian_force",
]

_lib = None


class LFGError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"lfg error {code}: {msg}")
        self.code = code


def load(path: str | None = None):
    """Load the engine library (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise RuntimeError(f"{p} not found: build it with `python -m lf_dem_gb300.build` "
                           "(or __graft_entry__.build()); there is no CPU fallback")
    L = C.CDLL(p)
    vp = C.c_void_p
    pst = C.POINTER(Status)
    L.lfg_default_options.argtypes = [C.POINTER(Options)]
    L.lfg_default_options.restype = None
    L.lfg_device_info.argtypes = [C.c_int, C.c_char_p, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int),
                                  C.POINTER(C.c_int)]
    L.lfg_solver_create.argtypes = [C.c_int, C.c_int, C.POINTER(Options), C.POINTER(vp), pst]
    L.lfg_solver_set_blocks.argtypes = [vp, vp, C.c_int, vp, vp, vp, C.c_int, vp, pst]
    L.lfg_solver_factorize.argtypes = [vp, pst]
    L.lfg_solver_solve.argtypes = [vp, C.c_int, vp, vp, pst]
    L.lfg_solver_multiply_factor.argtypes = [vp, C.c_int, vp, vp, pst]
    L.lfg_solver_solve_device.argtypes = [vp, C.c_int, vp, vp, pst]
    L.lfg_solver_get_stats.argtypes = [vp, C.POINTER(SolverStats)]
    L.lfg_solver_destroy.argtypes = [vp]
    L.lfg_solver_destroy.restype = None
    L.lfg_conf_write_binary.argtypes = [C.c_char_p, C.c_int, C.c_double, C.c_double, C.c_double, C.c_double,
                                        vp, vp, vp, C.c_int, vp, vp, vp, vp, pst]
    L.lfg_conf_read_binary.argtypes = [C.c_char_p, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int),
                                       vp, vp, vp, vp, vp, vp, vp, pst]
    L.lfg_checkpoint_write.argtypes = [C.c_char_p, C.c_double, C.c_double, C.c_double, pst]
    L.lfg_checkpoint_read.argtypes = [C.c_char_p, C.POINTER(C.c_double), C.POINTER(C.c_double),
                                      C.POINTER(C.c_double), pst]
    L.lfg_config_resolve.argtypes = [C.c_char_p, C.c_char, C.c_char_p, C.POINTER(Params), C.POINTER(C.c_double),
                                     C.POINTER(C.c_double), pst]
    L.lfg_config_output.argtypes = [C.c_char_p, C.c_char, C.c_char_p, C.POINTER(OutputUnits), pst]
    if hasattr(L, "lfg_sim_create"):
        L.lfg_sim_create.argtypes = [C.POINTER(Params), C.POINTER(Options), C.c_int, vp, vp, C.c_double,
                                     C.c_double, C.c_double, vp, C.c_int, vp, vp, vp, C.POINTER(vp), pst]
        L.lfg_sim_advance.argtypes = [vp, C.c_double, C.c_double, pst]
        L.lfg_sim_set_brownian_force.argtypes = [vp, vp, pst]
        L.lfg_output_open.argtypes = [vp, C.POINTER(OutputConfig), C.POINTER(vp), pst]
        L.lfg_output_write.argtypes = [vp, pst]
        L.lfg_output_close.argtypes = [vp]
        L.lfg_output_close.restype = None
        L.lfg_sim_step.argtypes = [vp, C.c_int, C.c_double, C.c_double, pst]
        L.lfg_sim_run.argtypes = [vp, C.c_int, C.c_double, C.c_double, pst]
        L.lfg_sim_get_scalars.argtypes = [vp, C.POINTER(SimScalars)]
        L.lfg_sim_get_particles.argtypes = [vp, vp, vp, vp, vp, vp]
        L.lfg_sim_get_num_pairs.argtypes = [vp]
        L.lfg_sim_get_pairs.argtypes = [vp, vp, C.c_int]
        L.lfg_sim_get_particle_stress.argtypes = [vp, C.c_int, vp]
        L.lfg_sim_get_velocity_component.argtypes = [vp, C.c_int, vp]
        L.lfg_sim_set_contact.argtypes = [vp, C.c_int, C.c_int, C.c_int, vp]
        L.lfg_sim_set_contact_rolling.argtypes = [vp, C.c_int, C.c_int, vp]
        L.lfg_sim_get_contact_states.argtypes = [vp, vp, vp, vp, vp, C.c_int]
        L.lfg_sim_set_clock.argtypes = [vp, C.c_double, C.c_double, C.c_double, C.c_double, C.c_double,
                                        C.c_double]
        L.lfg_sim_refresh.argtypes = [vp]
        L.lfg_sim_assemble.argtypes = [vp, vp, vp, vp, vp, C.c_int, C.POINTER(C.c_int)]
        L.lfg_sim_force_component.argtypes = [vp, C.c_int, vp]
        L.lfg_sim_force_component_noalloc.argtypes = [vp, C.c_int, vp, pst]
        L.lfg_sim_get_timing.argtypes = [vp, C.POINTER(SimTiming)]
        L.lfg_sim_get_step_times.argtypes = [vp, vp, C.c_int, C.POINTER(C.c_int64)]
        L.lfg_sim_clear_step_times.argtypes = [vp]
        L.lfg_sim_clear_step_times.restype = None
        L.lfg_sim_destroy.argtypes = [vp]
        L.lfg_sim_destroy.restype = None
        L.lfg_sim_advance_partial.argtypes = [vp, C.c_double, C.c_double, C.c_int, C.POINTER(C.c_int), pst]
        L.lfg_sim_set_leaf_size.argtypes = [vp, C.c_int, pst]
        L.lfg_sim_device_bytes.argtypes = [vp]
        L.lfg_sim_device_bytes.restype = C.c_int64
        L.lfg_footprint_estimate.argtypes = [C.c_int, C.c_int]
        L.lfg_footprint_estimate.restype = C.c_int64
        L.lfg_batch_create.argtypes = [C.c_int, C.c_int, C.POINTER(vp), pst]
        L.lfg_batch_add.argtypes = [vp, C.POINTER(Params), C.POINTER(Options), C.c_int, vp, vp, C.c_double,
                                    C.c_double, C.c_double, vp, C.POINTER(C.c_int), pst]
        L.lfg_batch_size.argtypes = [vp]
        L.lfg_batch_sim.argtypes = [vp, C.c_int]
        L.lfg_batch_sim.restype = vp
        L.lfg_batch_run.argtypes = [vp, C.c_int, pst]
        L.lfg_batch_advance.argtypes = [vp, vp, pst]
        L.lfg_batch_autotune.argtypes = [vp, vp, C.c_int, C.c_int, pst]
        L.lfg_batch_tuned_leaf.argtypes = [vp, C.c_int, C.c_int]
        L.lfg_batch_destroy.argtypes = [vp]
        L.lfg_batch_destroy.restype = None
        L.lfg_batch_create_fused.argtypes = [C.c_int, C.c_int, C.POINTER(vp), pst]
        L.lfg_batch_get_stats.argtypes = [vp, C.POINTER(BatchStats)]
        L.lfg_server_create.argtypes = [C.c_int, C.c_int, C.c_int64, C.POINTER(vp), pst]
        L.lfg_server_submit.argtypes = [vp, C.POINTER(Request), pst]
        L.lfg_server_poll.argtypes = [vp, C.POINTER(Result), C.c_int]
        L.lfg_server_wait.argtypes = [vp, C.c_double, pst]
        L.lfg_server_final_positions.argtypes = [vp, C.c_int64, vp, C.c_int]
        L.lfg_server_get_stats.argtypes = [vp, C.POINTER(ServerStats)]
        L.lfg_server_destroy.argtypes = [vp]
        L.lfg_server_destroy.restype = None
    _lib = L
    return L


def _check(rc, st: Status):
    if rc != LFG_OK:
        raise LFGError(rc, st.msg.decode(errors="replace"))


def default_options(**kw) -> Options:
    o = Options()
    load().lfg_default_options(C.byref(o))
    for k, v in kw.items():
        setattr(o, k, v)
    return o


def device_info(device: int = 0):
    name = C.create_string_buffer(128)
    a, b, c = C.c_int(), C.c_int(), C.c_int()
    rc = load().lfg_device_info(device, name, 128, C.byref(a), C.byref(b), C.byref(c))
    return rc, name.value.decode(), (a.value, b.value), c.value


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


class Solver:
    """Device resistance solver (lfg_solver_*): the StokesSolver linear algebra."""

    def __init__(self, n: int, precision: int = PREC_FP64, dof: int = 6, **opts):
        L = load()
        self.n = n
        self.dof = dof
        self.opt = default_options(precision=precision, **opts)
        h = C.c_void_p()
        st = Status()
        _check(L.lfg_solver_create(n, dof, C.byref(self.opt), C.byref(h), C.byref(st)), st)
        self.h = h
        self.last = st

    def set_blocks(self, dblocks, od_row, od_col, odblocks, pattern_changed=True, positions=None):
        d = np.ascontiguousarray(dblocks, dtype=np.float64)
        r = np.ascontiguousarray(od_row, dtype=np.int32)
        c = np.ascontiguousarray(od_col, dtype=np.int32)
        o = np.ascontiguousarray(odblocks, dtype=np.float64)
        pos = None if positions is None else np.ascontiguousarray(positions, dtype=np.float64)
        st = Status()
        _check(load().lfg_solver_set_blocks(self.h, _ptr(d), len(r), _ptr(r), _ptr(c), _ptr(o),
                                            int(pattern_changed), None if pos is None else _ptr(pos),
                                            C.byref(st)), st)

    def factorize(self):
        st = Status()
        rc = load().lfg_solver_factorize(self.h, C.byref(st))
        self.last = st
        _check(rc, st)

    def multiply_L(self, b):
        """x = L b with the current factor (R = L L^T; lfg_solver_multiply_factor)."""
        b = np.ascontiguousarray(b, dtype=np.float64)
        k = b.size // (6 * self.n)
        x = np.zeros_like(b)
        st = Status()
        _check(load().lfg_solver_multiply_factor(self.h, k, _ptr(b), _ptr(x), C.byref(st)), st)
        return x

    def solve(self, b):
        b = np.ascontiguousarray(b, dtype=np.float64)
        k = b.size // (6 * self.n)
        x = np.zeros_like(b)
        st = Status()
        rc = load().lfg_solver_solve(self.h, k, _ptr(b), _ptr(x), C.byref(st))
        self.last = st
        _check(rc, st)
        return x

    def stats(self) -> dict:
        s = SolverStats()
        load().lfg_solver_get_stats(self.h, C.byref(s))
        return {k: getattr(s, k) for k, _ in SolverStats._fields_}

    def close(self):
        if getattr(self, "h", None):
            load().lfg_solver_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def resolve_config(parameter_text: str, control: str, control_value: str):
    """LF_DEM's Parameter_File + `-r value` / `-s value` resolved by the
    reference's unit system (lfg_config_resolve): (parameter dict, time_end,
    strain_end)."""
    p = Params()
    te, se = C.c_double(), C.c_double()
    st = Status()
    rc = load().lfg_config_resolve(parameter_text.encode(), control.encode(), control_value.encode(), C.byref(p),
                                   C.byref(te), C.byref(se), C.byref(st))
    _check(rc, st)
    d = {}
    for k, _ in Params._fields_:
        v = getattr(p, k)
        d[k] = tuple(v) if k in ("Ehat", "Ohat") else v
    return d, te.value, se.value


def output_units(parameter_text: str, control: str, control_value: str) -> dict:
    """Output unit, internal-to-output factor, control number and output
    switches of a Parameter_File + control value (lfg_config_output)."""
    u = OutputUnits()
    st = Status()
    _check(load().lfg_config_output(parameter_text.encode(), control.encode(), control_value.encode(), C.byref(u),
                                    C.byref(st)), st)
    return {"unit": u.unit.decode(), "internal_to_output": u.internal_to_output, "input_value": u.input_value,
            "out_data_particle": u.out_data_particle, "out_data_interaction": u.out_data_interaction,
            "origin_zero_flow": u.origin_zero_flow, "out_particle_stress": u.out_particle_stress.decode()}


class Output:
    """LF_DEM's data_/st_/par_/int_ files (and pst_ when units name
    out_particle_stress groups) for a Sim (lfg_output_*)."""

    def __init__(self, sim, simu_name: str, units: dict, volume_fraction: float, directory: str = "",
                 version: str = "lf_dem_gb300", diminish_output: bool = False, force_overwrite: bool = False):
        L = load()
        self._keep = [directory.encode(), simu_name.encode(), version.encode(), units["unit"].encode(),
                      units.get("out_particle_stress", "").encode()]
        cfg = OutputConfig(self._keep[0], self._keep[1], self._keep[2], self._keep[3],
                           units["internal_to_output"], units["input_value"], volume_fraction,
                           int(units.get("out_data_particle", 1)), int(units.get("out_data_interaction", 1)),
                           int(units.get("origin_zero_flow", 1)), int(diminish_output), int(force_overwrite),
                           self._keep[4])
        h = C.c_void_p()
        st = Status()
        _check(L.lfg_output_open(sim.h, C.byref(cfg), C.byref(h), C.byref(st)), st)
        self.h = h

    def write(self):
        st = Status()
        _check(load().lfg_output_write(self.h, C.byref(st)), st)

    def close(self):
        if self.h:
            load().lfg_output_close(self.h)
            self.h = None


def write_conf_binary(path, position, radius, lx, ly, lz, vf, le_disp=(0.0, 0.0), contacts=None):
    """LF_DEM binary configuration (format 2).  contacts: (p0, p1, disp_tan,
    disp_rolling) arrays or None."""
    pos = np.ascontiguousarray(position, dtype=np.float64).reshape(-1)
    rad = np.ascontiguousarray(radius, dtype=np.float64)
    led = np.ascontiguousarray(le_disp, dtype=np.float64)
    st = Status()
    if contacts is not None and len(contacts[0]):
        p0 = np.ascontiguousarray(contacts[0], dtype=np.int32)
        p1 = np.ascontiguousarray(contacts[1], dtype=np.int32)
        dt = np.ascontiguousarray(contacts[2], dtype=np.float64).reshape(-1)
        dr = np.ascontiguousarray(contacts[3], dtype=np.float64).reshape(-1)
        args = (len(p0), _ptr(p0), _ptr(p1), _ptr(dt), _ptr(dr))
    else:
        args = (0, None, None, None, None)
    _check(load().lfg_conf_write_binary(str(path).encode(), len(rad), vf, lx, ly, lz, _ptr(led), _ptr(pos), _ptr(rad),
                                        *args, C.byref(st)), st)


def read_conf_binary(path):
    """LF_DEM binary configuration -> dict(format, vf, lx, ly, lz, le_disp,
    position, radius, p0, p1, disp_tan, disp_rolling)."""
    L = load()
    np_, nc, fmt = C.c_int(), C.c_int(), C.c_int()
    st = Status()
    _check(L.lfg_conf_read_binary(str(path).encode(), C.byref(np_), C.byref(nc), C.byref(fmt), None, None, None, None,
                                  None, None, None, C.byref(st)), st)
    n, k = np_.value, nc.value
    meta, pos, rad = np.zeros(6), np.zeros(3 * n), np.zeros(n)
    p0, p1 = np.zeros(max(k, 1), dtype=np.int32), np.zeros(max(k, 1), dtype=np.int32)
    dt, dr = np.zeros(3 * max(k, 1)), np.zeros(3 * max(k, 1))
    _check(L.lfg_conf_read_binary(str(path).encode(), C.byref(np_), C.byref(nc), C.byref(fmt), _ptr(meta), _ptr(pos),
                                  _ptr(rad), _ptr(p0), _ptr(p1), _ptr(dt), _ptr(dr), C.byref(st)), st)
    return dict(format=fmt.value, vf=meta[0], lx=meta[1], ly=meta[2], lz=meta[3], le_disp=tuple(meta[4:6]),
                position=pos.reshape(-1, 3), radius=rad, p0=p0[:k], p1=p1[:k], disp_tan=dt[:3 * k].reshape(-1, 3),
                disp_rolling=dr[:3 * k].reshape(-1, 3))


def write_checkpoint(path, strain, time, time_in_simulation_units):
    st = Status()
    _check(load().lfg_checkpoint_write(str(path).encode(), strain, time, time_in_simulation_units, C.byref(st)), st)


def read_checkpoint(path):
    a, b, c = C.c_double(), C.c_double(), C.c_double()
    st = Status()
    _check(load().lfg_checkpoint_read(str(path).encode(), C.byref(a), C.byref(b), C.byref(c), C.byref(st)), st)
    return a.value, b.value, c.value


def make_params(d: dict) -> Params:
    """lfg_params from a dict of already non-dimensionalised values."""
    p = Params()
    defaults = dict(mu_dynamic=-1.0, repulsive_max_length=-1.0, interaction_range=-1.0, sd_coeff=1.0,
                    contact_relaxation_time=1e-3, contact_relaxation_time_tan=-1.0, disp_max=1e-3,
                    dt=1e-4, dt_max=-1.0, dt_min=-1.0, integration_method=1, lubrication_model=2,
                    lub_reduce_parameter=1e-3, lub_max_gap=0.5, friction_model=1, mu_static=1.0,
                    repulsive_length=0.05, init_strain_shear_rate_limit=0.0, init_shear_rate_limit=999.0,
                    Ehat=(0, 0, 0.5, 0, 0, 0), Ohat=(0, 0.5, 0))
    full = dict(defaults)
    full.update(d)
    for k, _ in Params._fields_:
        if k not in full:
            continue
        v = full[k]
        if k in ("Ehat", "Ohat"):
            arr = getattr(p, k)
            for i, x in enumerate(v):
                arr[i] = float(x)
        elif isinstance(getattr(p, k), int):
            setattr(p, k, int(v))
        else:
            setattr(p, k, float(v))
    return p


class Sim:
    """One suspension advanced on the device (lfg_sim_*): System::timeEvolution."""

    def __init__(self, params: dict, position, radius, lx, ly, lz, le_disp=(0.0, 0.0), contacts=None,
                 precision: int = PREC_FP64, **opts):
        L = load()
        self.n = len(radius)
        self.p = make_params(params)
        self.opt = default_options(precision=precision, **opts)
        pos = np.ascontiguousarray(position, dtype=np.float64).reshape(-1)
        rad = np.ascontiguousarray(radius, dtype=np.float64)
        led = np.ascontiguousarray(le_disp, dtype=np.float64)
        h = C.c_void_p()
        st = Status()
        if contacts:
            c0 = np.ascontiguousarray([c[0] for c in contacts], dtype=np.int32)
            c1 = np.ascontiguousarray([c[1] for c in contacts], dtype=np.int32)
            cd = np.ascontiguousarray([c[2] for c in contacts], dtype=np.float64).reshape(-1)
            rc = L.lfg_sim_create(C.byref(self.p), C.byref(self.opt), self.n, _ptr(pos), _ptr(rad), lx, ly, lz,
                                  _ptr(led), len(contacts), _ptr(c0), _ptr(c1), _ptr(cd), C.byref(h), C.byref(st))
        else:
            rc = L.lfg_sim_create(C.byref(self.p), C.byref(self.opt), self.n, _ptr(pos), _ptr(rad), lx, ly, lz,
                                  _ptr(led), 0, None, None, None, C.byref(h), C.byref(st))
        _check(rc, st)
        self.h = h

    @classmethod
    def _borrowed(cls, handle, n):
        """A view of a simulation owned by a Batch (not destroyed by close)."""
        self = cls.__new__(cls)
        self.h = C.c_void_p(handle)
        self.n = n
        self._owned = False
        return self

    def close(self):
        if getattr(self, "h", None):
            if getattr(self, "_owned", True):
                load().lfg_sim_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def step(self, calc_stress=False, time_end=-1.0, strain_end=1e9):
        st = Status()
        _check(load().lfg_sim_step(self.h, int(calc_stress), time_end, strain_end, C.byref(st)), st)

    def run(self, nsteps, time_end=-1.0, strain_end=1e9):
        st = Status()
        _check(load().lfg_sim_run(self.h, int(nsteps), time_end, strain_end, C.byref(st)), st)

    def set_leaf_size(self, leaf):
        st = Status()
        _check(load().lfg_sim_set_leaf_size(self.h, int(leaf), C.byref(st)), st)

    def device_bytes(self) -> int:
        return int(load().lfg_sim_device_bytes(self.h))

    def advance(self, time_end=-1.0, strain_end=-1.0):
        st = Status()
        _check(load().lfg_sim_advance(self.h, time_end, strain_end, C.byref(st)), st)

    def scalars(self) -> dict:
        s = SimScalars()
        load().lfg_sim_get_scalars(self.h, C.byref(s))
        out = {}
        for k, _ in SimScalars._fields_:
            v = getattr(s, k)
            out[k] = np.array(v[:]) if hasattr(v, "__len__") else v
        return out

    def particles(self) -> dict:
        arrs = {k: np.zeros(3 * self.n) for k in ("pos", "vel", "ang", "na_vel", "na_ang")}
        load().lfg_sim_get_particles(self.h, *[_ptr(a) for a in arrs.values()])
        return {k: v.reshape(-1, 3) for k, v in arrs.items()}

    def pairs(self) -> np.ndarray:
        L = load()
        n = L.lfg_sim_get_num_pairs(self.h)
        buf = (Pair * max(n, 1))()
        L.lfg_sim_get_pairs(self.h, buf, n)
        return np.ctypeslib.as_array(buf)[:n].copy()

    def particle_stress(self, comp: int):
        out = np.zeros(6 * self.n)
        rc = load().lfg_sim_get_particle_stress(self.h, comp, _ptr(out))
        return None if rc else out.reshape(-1, 6)

    def velocity_component(self, comp: int):
        out = np.zeros(6 * self.n)
        rc = load().lfg_sim_get_velocity_component(self.h, comp, _ptr(out))
        return None if rc else out.reshape(-1, 6)

    def set_contact(self, p0, p1, state, disp_tan):
        d = np.ascontiguousarray(disp_tan, dtype=np.float64)
        rc = load().lfg_sim_set_contact(self.h, int(p0), int(p1), int(state), _ptr(d))
        if rc:
            raise LFGError(rc, f"no pair ({p0},{p1})")

    def contact_states(self):
        """Active contacts (p0, p1, disp_tan, disp_rolling), sorted by (p0, p1)."""
        L = load()
        k = L.lfg_sim_get_contact_states(self.h, None, None, None, None, 0)
        if k < 0:
            raise LFGError(-k, "contact states")
        p0, p1 = np.zeros(max(k, 1), dtype=np.int32), np.zeros(max(k, 1), dtype=np.int32)
        dt, dr = np.zeros(3 * max(k, 1)), np.zeros(3 * max(k, 1))
        L.lfg_sim_get_contact_states(self.h, _ptr(p0), _ptr(p1), _ptr(dt), _ptr(dr), k)
        return p0[:k], p1[:k], dt[:3 * k].reshape(-1, 3), dr[:3 * k].reshape(-1, 3)

    def set_contact_rolling(self, p0, p1, disp_rolling):
        d = np.ascontiguousarray(disp_rolling, dtype=np.float64)
        rc = load().lfg_sim_set_contact_rolling(self.h, int(p0), int(p1), _ptr(d))
        if rc:
            raise LFGError(rc, f"no pair ({p0}, {p1})")
    def set_brownian_force(self, fb):
        """The Brownian force (6n) the next predictor uses instead of a draw."""
        f = np.ascontiguousarray(fb, dtype=np.float64)
        st = Status()
        _check(load().lfg_sim_set_brownian_force(self.h, _ptr(f), C.byref(st)), st)

    def set_clock(self, time, strain, dt, shear_rate, max_velocity, max_sliding_velocity):
        load().lfg_sim_set_clock(self.h, time, strain, dt, shear_rate, max_velocity, max_sliding_velocity)

    def refresh(self):
        load().lfg_sim_refresh(self.h)

    def assemble(self):
        L = load()
        nb = C.c_int()
        L.lfg_sim_assemble(self.h, None, None, None, None, 0, C.byref(nb))
        k = nb.value
        d = np.zeros(15 * self.n)
        r = np.zeros(max(k, 1), dtype=np.int32)
        c = np.zeros(max(k, 1), dtype=np.int32)
        o = np.zeros(18 * max(k, 1))
        L.lfg_sim_assemble(self.h, _ptr(d), _ptr(r), _ptr(c), _ptr(o), k, C.byref(nb))
        return d.reshape(-1, 15), r[:k], c[:k], o[:18 * k].reshape(-1, 18)

    def force_component(self, comp: int):
        out = np.zeros(6 * self.n)
        rc = load().lfg_sim_force_component(self.h, comp, _ptr(out))
        return None if rc else out.reshape(-1, 6)

    def force_component_noalloc(self, comp: int, d_out: int):
        """Force component comp into the device buffer at address d_out (6n
        doubles) through the entry point that allocates nothing."""
        st = Status()
        rc = load().lfg_sim_force_component_noalloc(self.h, comp, C.c_void_p(d_out), C.byref(st))
        _check(rc, st)

    def step_times(self):
        L = load()
        kern = C.c_int64()
        n = L.lfg_sim_get_step_times(self.h, None, 0, C.byref(kern))
        buf = np.zeros(max(n, 1))
        L.lfg_sim_get_step_times(self.h, _ptr(buf), n, C.byref(kern))
        return buf[:n].copy(), kern.value

    def clear_step_times(self):
        load().lfg_sim_clear_step_times(self.h)

    def timing(self) -> dict:
        t = SimTiming()
        load().lfg_sim_get_timing(self.h, C.byref(t))
        return {"ms": list(t.ms), "launches": t.launches, "factor_flops": t.factor_flops,
                "solve_bytes": t.solve_bytes, "rebuild_ms": t.rebuild_ms, "rebuilds": t.rebuilds,
                "run_steps": t.run_steps, "run_ms": t.run_ms}


def footprint_estimate(n: int, precision: int = PREC_FP32_REFINE) -> int:
    return int(load().lfg_footprint_estimate(int(n), int(precision)))


class Batch:
    """Many suspensions on one GPU (lfg_batch_*), stepped together."""

    def __init__(self, device: int = 0, nthreads: int = 0, fused: bool = False, precision: int = PREC_FP32_REFINE):
        """fused: lockstep through one joint factorisation and solve
        (lfg_batch_create_fused, all suspensions in `precision`); otherwise
        each suspension on its own stream, driven by nthreads host workers."""
        L = load()
        h = C.c_void_p()
        st = Status()
        if fused:
            _check(L.lfg_batch_create_fused(device, precision, C.byref(h), C.byref(st)), st)
        else:
            _check(L.lfg_batch_create(device, nthreads, C.byref(h), C.byref(st)), st)
        self.h = h
        self.n = []
        self._keep = []

    def add(self, params: dict, position, radius, lx, ly, lz, precision: int = PREC_FP64, **opts) -> int:
        L = load()
        p = make_params(params)
        o = default_options(precision=precision, **opts)
        pos = np.ascontiguousarray(position, dtype=np.float64).reshape(-1)
        rad = np.ascontiguousarray(radius, dtype=np.float64)
        slot = C.c_int()
        st = Status()
        _check(L.lfg_batch_add(self.h, C.byref(p), C.byref(o), len(rad), _ptr(pos), _ptr(rad), lx, ly, lz, None,
                               C.byref(slot), C.byref(st)), st)
        self.n.append(len(rad))
        return slot.value

    def sim(self, slot: int) -> "Sim":
        return Sim._borrowed(load().lfg_batch_sim(self.h, slot), self.n[slot])

    def run(self, nsteps: int):
        st = Status()
        _check(load().lfg_batch_run(self.h, int(nsteps), C.byref(st)), st)

    def advance(self, strain_end):
        se = np.ascontiguousarray(strain_end, dtype=np.float64)
        st = Status()
        _check(load().lfg_batch_advance(self.h, _ptr(se), C.byref(st)), st)

    def autotune(self, leaf_sizes=(8, 16, 32, 64), steps: int = 2):
        ls = np.ascontiguousarray(leaf_sizes, dtype=np.int32)
        st = Status()
        _check(load().lfg_batch_autotune(self.h, _ptr(ls), len(ls), int(steps), C.byref(st)), st)

    def tuned_leaf(self, n: int, precision: int) -> int:
        return int(load().lfg_batch_tuned_leaf(self.h, int(n), int(precision)))

    def stats(self) -> dict:
        s = BatchStats()
        load().lfg_batch_get_stats(self.h, C.byref(s))
        return {k: getattr(s, k) for k, _ in BatchStats._fields_ if k != "pad_"}

    def close(self):
        if getattr(self, "h", None):
            load().lfg_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Server:
    """Request loop (lfg_server_*): admission by estimated factor footprint,
    continuous batching, per-request timing."""

    def __init__(self, max_active: int, hbm_budget_bytes: int, device: int = 0):
        L = load()
        h = C.c_void_p()
        st = Status()
        _check(L.lfg_server_create(device, int(max_active), int(hbm_budget_bytes), C.byref(h), C.byref(st)), st)
        self.h = h
        self._n = {}

    def submit(self, rid: int, params: dict, position, radius, lx, ly, lz, strain_end: float,
               precision: int = PREC_FP32_REFINE, **opts):
        p = make_params(params)
        o = default_options(precision=precision, **opts)
        pos = np.ascontiguousarray(position, dtype=np.float64).reshape(-1)
        rad = np.ascontiguousarray(radius, dtype=np.float64)
        r = Request(id=rid, params=C.cast(C.pointer(p), C.c_void_p), options=C.cast(C.pointer(o), C.c_void_p),
                    n=len(rad), pos=pos.ctypes.data, radius=rad.ctypes.data, lx=lx, ly=ly, lz=lz,
                    strain_end=strain_end)
        st = Status()
        _check(load().lfg_server_submit(self.h, C.byref(r), C.byref(st)), st)   # copies the inputs
        self._n[rid] = len(rad)

    def poll(self, cap: int = 256):
        buf = (Result * cap)()
        k = load().lfg_server_poll(self.h, buf, cap)
        return [buf[i] for i in range(k)]

    def wait(self, timeout_s: float = 0.0):
        st = Status()
        _check(load().lfg_server_wait(self.h, float(timeout_s), C.byref(st)), st)

    def final_positions(self, rid: int):
        n = self._n[rid]
        out = np.zeros(3 * n)
        rc = load().lfg_server_final_positions(self.h, int(rid), _ptr(out), n)
        if rc:
            raise LFGError(rc, f"no final positions for request {rid}")
        return out.reshape(-1, 3)

    def stats(self) -> dict:
        s = ServerStats()
        load().lfg_server_get_stats(self.h, C.byref(s))
        return {k: getattr(s, k) for k, _ in ServerStats._fields_ if k != "pad_"}

    def close(self):
        if getattr(self, "h", None):
            load().lfg_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
