"""The allocation-free energy entry point, kvft_ft_cc_energy_noalloc.

Some callers cannot let a library allocate device memory: a host process
whose own pool owns the device, a serving loop that cannot absorb the
synchronisation cudaMalloc may imply, a plugin host that forbids foreign
allocations.  For them the energy reduction keeps its scratch in a fixed
static device array.  This file checks, through the C ABI, that two calls in a
row give the value of the allocating entry point kvft_ft_cc_energy, and that
a problem beyond the static scratch is refused.  It is named so that pytest
collects it last.
"""
import ctypes

import numpy
import pytest

from kelvin_gb300 import _lib

pytestmark = pytest.mark.gpu

TOL = 1e-12
PER_THREAD_STREAM = ctypes.c_void_p(2)     # cudaStreamPerThread


def _inputs(rng, ng, nv, no):
    T1 = rng.standard_normal((ng, nv, no)) * 0.1
    T2 = rng.standard_normal((ng, nv, nv, no, no)) * 0.1
    f = rng.standard_normal((no, nv))
    eri = rng.standard_normal((no, no, nv, nv))
    g = numpy.abs(rng.standard_normal(ng))
    return T1, T2, f, eri, g


def test_noalloc_energy_matches_allocating_entry_point():
    # the context and the allocation-free call share the per-thread default
    # stream, so their work is ordered without extra synchronisation
    ctx = _lib.Context(0, stream=PER_THREAD_STREAM)
    rng = numpy.random.default_rng(99)
    out = _lib.DeviceArray(ctx, (1,))
    try:
        for call, (ng, nv, no, beta, qterm) in enumerate([(5, 8, 6, 2.5, 1), (7, 9, 9, 0.7, 0)]):
            arrs = _inputs(rng, ng, nv, no)
            dev = [_lib.DeviceArray.from_host(ctx, a) for a in arrs]
            ref = ctypes.c_double()
            ctx.check(ctx.L.kvft_ft_cc_energy(ctx.h, ng, nv, no, *[d.ptr for d in dev], beta,
                                              qterm, ctypes.byref(ref)), "kvft_ft_cc_energy")
            st = ctx.L.kvft_ft_cc_energy_noalloc(PER_THREAD_STREAM, ng, nv, no,
                                                 *[d.ptr for d in dev], beta, qterm, out.ptr)
            assert st == 0, "call %d: status %d" % (call, st)
            got = float(out.to_host()[0])
            assert abs(got - ref.value) <= TOL * max(1.0, abs(ref.value)), (call, got, ref.value)
    finally:
        ctx.close()


def test_noalloc_energy_rejects_problems_beyond_its_scratch():
    L = _lib.lib()
    ctx = _lib.Context(0, stream=PER_THREAD_STREAM)
    try:
        tiny = _lib.DeviceArray(ctx, (1,))
        # 100 x 100 pairs -> 313 * 313 tiles > 32767: refused before any launch
        st = L.kvft_ft_cc_energy_noalloc(PER_THREAD_STREAM, 2, 100, 100, tiny.ptr, tiny.ptr,
                                         tiny.ptr, tiny.ptr, tiny.ptr, 1.0, 1, tiny.ptr)
        assert st == 1                       # KVFT_EINVAL
    finally:
        ctx.close()
