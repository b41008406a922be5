"""lfg_sim_force_component_noalloc (static device scratch, nothing allocated)
against lfg_sim_force_component on the same simulation state, called twice in
a row for every component.  Both run the same kernels in the same summation
order; the tolerance below is the one the test holds them to."""
import ctypes as C

import numpy as np
import pytest

from _systems import RATE_PARAMS, STRESS_PARAMS, make_packing

pytestmark = pytest.mark.gpu

RTOL = 1e-12


def _cudart():
    # the runtime the engine library is linked against (already loaded with it)
    rt = C.CDLL("libcudart.so.13")
    rt.cudaMalloc.argtypes = [C.POINTER(C.c_void_p), C.c_size_t]
    rt.cudaFree.argtypes = [C.c_void_p]
    rt.cudaMemset.argtypes = [C.c_void_p, C.c_int, C.c_size_t]
    rt.cudaMemcpy.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t, C.c_int]
    rt.cudaDeviceSynchronize.argtypes = []
    return rt


@pytest.mark.parametrize("params,vf,seed", [(RATE_PARAMS, 0.5, 61), (STRESS_PARAMS, 0.52, 62)],
                         ids=["rate", "stress"])
def test_noalloc_force_components_match(engine, params, vf, seed):
    p = make_packing(300, vf, seed)
    g = engine.Sim(params, p.position, p.radius, p.lx, p.ly, p.lz)
    g.run(3)
    n = g.n
    rt = _cudart()
    nbytes = 8 * 6 * n
    dptr = C.c_void_p()
    assert rt.cudaMalloc(C.byref(dptr), nbytes) == 0
    try:
        for call in range(2):
            for comp in range(4):
                ref = g.force_component(comp)
                assert ref is not None
                # fill with NaN bytes so that an unwritten output cannot pass
                assert rt.cudaMemset(dptr, 0xFF, nbytes) == 0
                assert rt.cudaDeviceSynchronize() == 0
                g.force_component_noalloc(comp, dptr.value)
                got = np.empty(6 * n)
                assert rt.cudaMemcpy(got.ctypes.data, dptr, nbytes, 2) == 0   # device to host
                got = got.reshape(-1, 6)
                assert np.isfinite(got).all(), (call, comp)
                scale = max(np.abs(ref).max(), 1e-300)
                assert np.abs(got - ref).max() <= RTOL * scale, (call, comp)
        # a host buffer is refused with a status, not written through
        host = np.zeros(6 * n)
        with pytest.raises(engine.LFGError):
            g.force_component_noalloc(0, host.ctypes.data)
        # only the pair-force components 0..3 have a scratch slot: the Brownian
        # component (4) and out-of-range values are refused, the output untouched
        assert rt.cudaMemset(dptr, 0, nbytes) == 0
        for bad in (4, 5, -1):
            with pytest.raises(engine.LFGError):
                g.force_component_noalloc(bad, dptr.value)
        got = np.empty(6 * n)
        assert rt.cudaMemcpy(got.ctypes.data, dptr, nbytes, 2) == 0
        assert not got.any()
    finally:
        rt.cudaFree(dptr)
        g.close()
