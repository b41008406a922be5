"""ctypes front-end of the CPU oracle (oracle/lfdem_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
cpu_baseline / reference legs of bench.py, never by the lf_dem_gb300 package.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "liblfdem_oracle.so")


def build(quiet: bool = True) -> str:
    """Compile the C restatement (make -C oracle)."""
    out = subprocess.run(["make", "-C", HERE, "all"], capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + out.stdout + out.stderr)
    return LIB_PATH


class Params(C.Structure):
    """Mirror of lfo_params (lfdem_oracle.h)."""
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
        ("mu_rolling", C.c_double), ("kr", C.c_double),
    ]


class PairOut(C.Structure):
    _fields_ = [
        ("p0", C.c_int), ("p1", C.c_int), ("z_offset", C.c_int), ("contact_active", C.c_int),
        ("state", C.c_int), ("lub_active", C.c_int), ("dashpot_active", C.c_int), ("pad_", C.c_int),
        ("r", C.c_double), ("reduced_gap", C.c_double),
        ("nvec", C.c_double * 3), ("rvec", C.c_double * 3), ("disp_tan", C.c_double * 3),
        ("f_spring_total", C.c_double * 3), ("lub_coeff", C.c_double), ("log_lub_coeff", C.c_double),
        ("rep_force", C.c_double * 3),
    ]


class Scalars(C.Structure):
    _fields_ = [
        ("time", C.c_double), ("strain", C.c_double), ("shear_rate", C.c_double), ("dt", C.c_double),
        ("shear_disp", C.c_double * 2), ("max_velocity", C.c_double), ("max_sliding_velocity", C.c_double),
        ("total_stress", C.c_double * 6), ("viscosity", C.c_double), ("N1", C.c_double), ("N2", C.c_double),
        ("rate_prop_shearstress", C.c_double), ("rate_indep_shearstress", C.c_double),
        ("total_num_timesteps", C.c_longlong), ("n_pairs", C.c_int), ("n_contacts", C.c_int),
        ("n_lub", C.c_int), ("n_resistance_pairs", C.c_int), ("pad_", C.c_int),
    ]


PARAM_KEYS = [f[0] for f in Params._fields_]

_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = C.CDLL(LIB_PATH)
        dp = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
        ip = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
        L.lfo_create.restype = C.c_void_p
        L.lfo_create.argtypes = [C.POINTER(Params), C.c_int, dp, dp, C.c_double, C.c_double, C.c_double,
                                 dp, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]
        L.lfo_destroy.argtypes = [C.c_void_p]
        L.lfo_time_evolution.argtypes = [C.c_void_p, C.c_double, C.c_double]
        L.lfo_step.argtypes = [C.c_void_p, C.c_int, C.c_double, C.c_double]
        L.lfo_first_time.argtypes = [C.c_void_p]
        L.lfo_get_scalars.argtypes = [C.c_void_p, C.POINTER(Scalars)]
        L.lfo_get_particles.argtypes = [C.c_void_p] + [C.c_void_p] * 5
        L.lfo_get_num_pairs.argtypes = [C.c_void_p]
        L.lfo_get_pairs.argtypes = [C.c_void_p, C.c_void_p]
        L.lfo_get_particle_stress.argtypes = [C.c_void_p, C.c_int, dp]
        L.lfo_get_velocity_component.argtypes = [C.c_void_p, C.c_int, dp]
        L.lfo_assemble.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
        L.lfo_solve_assembled.argtypes = [C.c_void_p, C.c_int, dp, dp]
        L.lfo_force_component.argtypes = [C.c_void_p, C.c_int, dp]
        L.lfo_bsr_solve.argtypes = [C.c_int, dp, C.c_int, ip, ip, dp, C.c_int, dp, dp]
        L.lfo_set_contact.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, dp]
        L.lfo_set_contact.restype = C.c_int
        L.lfo_set_contact_rolling.argtypes = [C.c_void_p, C.c_int, C.c_int, dp]
        L.lfo_set_contact_rolling.restype = C.c_int
        L.lfo_set_clock.argtypes = [C.c_void_p, C.c_double, C.c_double, C.c_double, C.c_double,
                                    C.c_double, C.c_double, C.c_int]
        L.lfo_refresh.argtypes = [C.c_void_p]
        L.lfo_num_threads.restype = C.c_int
        L.lfo_set_num_threads.argtypes = [C.c_int]
        L.lfo_set_blas.argtypes = [C.c_void_p] * 5 + [C.c_int]
        L.lfo_blas_ready.restype = C.c_int
        L.lfo_factor_stats.argtypes = [C.c_void_p, C.c_void_p]
        L.lfo_dblock_to_dense.argtypes = [dp, dp]
        L.lfo_odblock_to_dense.argtypes = [dp, dp]
        _lib = L
    return _lib


def make_params(d: dict) -> Params:
    p = Params()
    defaults = dict(mu_dynamic=-1.0, repulsive_max_length=-1.0, interaction_range=-1.0, sd_coeff=1.0,
                    contact_relaxation_time=1e-3, contact_relaxation_time_tan=-1.0, disp_max=1e-3,
                    dt=1e-4, dt_max=-1.0, dt_min=-1.0, integration_method=1, lubrication_model=2,
                    lub_reduce_parameter=1e-3, lub_max_gap=0.5, friction_model=1, mu_static=1.0,
                    repulsive_length=0.05, init_strain_shear_rate_limit=0.0, init_shear_rate_limit=999.0,
                    Ehat=(0, 0, 0.5, 0, 0, 0), Ohat=(0, 0.5, 0))
    full = dict(defaults)
    full.update(d)
    for k in PARAM_KEYS:
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


class OracleSim:
    """One oracle System (CPU, FP64)."""

    def __init__(self, params: dict, position, radius, lx, ly, lz, le_disp=(0.0, 0.0),
                 contacts=None):
        L = lib()
        self.n = len(radius)
        self.p = make_params(params)
        pos = np.ascontiguousarray(position, dtype=np.float64).reshape(-1)
        rad = np.ascontiguousarray(radius, dtype=np.float64)
        led = np.ascontiguousarray(le_disp, dtype=np.float64)
        if contacts:
            c0 = np.ascontiguousarray([c[0] for c in contacts], dtype=np.int32)
            c1 = np.ascontiguousarray([c[1] for c in contacts], dtype=np.int32)
            cd = np.ascontiguousarray([c[2] for c in contacts], dtype=np.float64).reshape(-1)
            self._keep = (c0, c1, cd)
            h = L.lfo_create(C.byref(self.p), self.n, pos, rad, lx, ly, lz, led, len(contacts),
                             c0.ctypes.data, c1.ctypes.data, cd.ctypes.data)
        else:
            h = L.lfo_create(C.byref(self.p), self.n, pos, rad, lx, ly, lz, led, 0, None, None, None)
        if not h:
            raise RuntimeError("lfo_create failed")
        self.h = h

    def __del__(self):
        if getattr(self, "h", None):
            lib().lfo_destroy(self.h)
            self.h = None

    def first_time(self):
        lib().lfo_first_time(self.h)

    def step(self, calc_stress=False, time_end=-1.0, strain_end=1e9):
        st = lib().lfo_step(self.h, int(calc_stress), time_end, strain_end)
        if st:
            raise RuntimeError(f"lfo_step failed: {st}")

    def time_evolution(self, time_end=-1.0, strain_end=-1.0):
        st = lib().lfo_time_evolution(self.h, time_end, strain_end)
        if st:
            raise RuntimeError(f"lfo_time_evolution failed: {st}")

    def scalars(self) -> dict:
        s = Scalars()
        lib().lfo_get_scalars(self.h, C.byref(s))
        out = {}
        for k, _ in Scalars._fields_:
            v = getattr(s, k)
            out[k] = np.array(v[:]) if hasattr(v, "__len__") else v
        return out

    def particles(self) -> dict:
        arrs = {k: np.zeros(3 * self.n) for k in ("pos", "vel", "ang", "na_vel", "na_ang")}
        lib().lfo_get_particles(self.h, *[a.ctypes.data for a in arrs.values()])
        return {k: v.reshape(-1, 3) for k, v in arrs.items()}

    def pairs(self) -> np.ndarray:
        n = lib().lfo_get_num_pairs(self.h)
        buf = (PairOut * n)()
        lib().lfo_get_pairs(self.h, buf)
        return np.ctypeslib.as_array(buf).copy() if n else np.zeros(0, dtype=np.dtype(PairOut))

    def particle_stress(self, comp: int):
        out = np.zeros(6 * self.n)
        st = lib().lfo_get_particle_stress(self.h, comp, out)
        return None if st else out.reshape(-1, 6)

    def velocity_component(self, comp: int):
        out = np.zeros(6 * self.n)
        st = lib().lfo_get_velocity_component(self.h, comp, out)
        return None if st else out.reshape(-1, 6)

    def force_component(self, comp: int):
        out = np.zeros(6 * self.n)
        st = lib().lfo_force_component(self.h, comp, out)
        return None if st else out.reshape(-1, 6)

    def assemble(self):
        L = lib()
        nb = L.lfo_assemble(self.h, None, None, None, None)
        d = np.zeros(15 * self.n)
        r = np.zeros(nb, dtype=np.int32)
        c = np.zeros(nb, dtype=np.int32)
        o = np.zeros(18 * max(nb, 1))
        L.lfo_assemble(self.h, d.ctypes.data, r.ctypes.data, c.ctypes.data, o.ctypes.data)
        return d.reshape(-1, 15), r, c, o[:18 * nb].reshape(-1, 18)

    def solve_assembled(self, b):
        b = np.ascontiguousarray(b, dtype=np.float64)
        k = b.size // (6 * self.n)
        x = np.zeros_like(b)
        st = lib().lfo_solve_assembled(self.h, k, b.reshape(-1), x.reshape(-1))
        if st:
            raise RuntimeError(f"oracle factorisation failed: {st}")
        return x

    def set_contact(self, p0, p1, state, disp_tan):
        st = lib().lfo_set_contact(self.h, int(p0), int(p1), int(state),
                                   np.ascontiguousarray(disp_tan, dtype=np.float64))
        if st:
            raise RuntimeError(f"no pair ({p0},{p1}) in the oracle")

    def set_contact_rolling(self, p0, p1, disp_rolling):
        d = np.ascontiguousarray(disp_rolling, dtype=np.float64)
        if lib().lfo_set_contact_rolling(self.h, int(p0), int(p1), d) != 0:
            raise ValueError(f"no pair ({p0}, {p1})")
    def set_clock(self, time, strain, dt, shear_rate, max_velocity, max_sliding_velocity, firsttime_done=1):
        lib().lfo_set_clock(self.h, time, strain, dt, shear_rate, max_velocity, max_sliding_velocity,
                            int(firsttime_done))

    def refresh(self):
        lib().lfo_refresh(self.h)


def factor_stats(sim) -> dict:
    """Factorisations so far, the last one's ordering flops, seconds in the
    ordering + symbolic analysis and in the numeric factorisation."""
    out = np.zeros(4)
    lib().lfo_factor_stats(sim.h, out.ctypes.data)
    return {"factorisations": int(out[0]), "factor_flops": float(out[1]), "analyze_s": float(out[2]),
            "factor_s": float(out[3])}


def _capsule_ptr(capsule) -> int:
    get_name = C.pythonapi.PyCapsule_GetName
    get_name.restype = C.c_char_p
    get_name.argtypes = [C.py_object]
    get_ptr = C.pythonapi.PyCapsule_GetPointer
    get_ptr.restype = C.c_void_p
    get_ptr.argtypes = [C.py_object, C.c_char_p]
    return get_ptr(capsule, get_name(capsule))


def use_blas(threads: int = 0) -> bool:
    """Switch the oracle's factorisation to the supernodal one with dense
    BLAS-3 kernels (the method of CHOLMOD's supernodal factorisation), taking
    dpotrf, dtrsm, dsyrk and dgemm from scipy's BLAS/LAPACK (Fortran
    interface, through scipy.linalg.cython_blas / cython_lapack) and the
    OpenBLAS thread setter of scipy's bundled OpenBLAS when there is one.
    threads: BLAS threads for the large fronts (0: the OpenMP thread count).
    Returns False when scipy is not available (the block factorisation stays)."""
    try:
        import scipy.linalg.cython_blas as cb
        import scipy.linalg.cython_lapack as cl
    except ImportError:
        return False
    potrf = _capsule_ptr(cl.__pyx_capi__["dpotrf"])
    trsm = _capsule_ptr(cb.__pyx_capi__["dtrsm"])
    syrk = _capsule_ptr(cb.__pyx_capi__["dsyrk"])
    gemm = _capsule_ptr(cb.__pyx_capi__["dgemm"])
    setter = None
    import glob
    import scipy
    libdir = os.path.join(os.path.dirname(os.path.dirname(scipy.__file__)), "scipy.libs")
    for path in sorted(glob.glob(os.path.join(libdir, "*openblas*.so*"))):
        try:
            blas = C.CDLL(path)
        except OSError:
            continue
        for name in ("scipy_openblas_set_num_threads", "openblas_set_num_threads"):
            fn = getattr(blas, name, None)
            if fn is not None:
                setter = C.cast(fn, C.c_void_p).value
                break
        if setter:
            break
    lib().lfo_set_blas(potrf, trsm, syrk, gemm, setter, int(threads) if threads > 0 else num_threads())
    return bool(lib().lfo_blas_ready())


def set_num_threads(n: int) -> None:
    """OpenMP threads of the oracle's later parallel regions."""
    lib().lfo_set_num_threads(int(n))


def num_threads() -> int:
    return lib().lfo_num_threads()


def dblock_dense(d15):
    out = np.zeros(36)
    lib().lfo_dblock_to_dense(np.ascontiguousarray(d15, dtype=np.float64), out)
    return out.reshape(6, 6)


def odblock_dense(o18):
    out = np.zeros(36)
    lib().lfo_odblock_to_dense(np.ascontiguousarray(o18, dtype=np.float64), out)
    return out.reshape(6, 6)
