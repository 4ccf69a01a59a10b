"""ctypes binding of libkvft.so (the C ABI declared in include/kvft.h).

The library is required: importing an entry point without it raises, there is
no CPU fallback.  Build it with ``kelvin_gb300.build.build()``.
"""
import ctypes
import os
import threading

import numpy

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libkvft.so")

c_double_p = ctypes.POINTER(ctypes.c_double)
vp = ctypes.c_void_p

PREC_FP64 = 0
PREC_FP64_TC = 1
PREC_MIXED = 2

STATUS = {0: "ok", 1: "invalid argument", 2: "device memory exhausted",
          3: "iteration diverged", 4: "device wait timed out", 5: "CUDA error",
          6: "not converged"}


class KvftError(Exception):
    """A libkvft call failed; ``status`` holds the kvft_status code."""

    def __init__(self, msg, status):
        super().__init__(msg)
        self.status = status


class SolveOpts(ctypes.Structure):
    _fields_ = [("econv", ctypes.c_double), ("tconv", ctypes.c_double),
                ("damp", ctypes.c_double), ("max_iter", ctypes.c_int),
                ("full", ctypes.c_int), ("guess", ctypes.c_int),
                ("verbose", ctypes.c_int)]


class Result(ctypes.Structure):
    _fields_ = [("omega_cc", ctypes.c_double), ("e_guess", ctypes.c_double),
                ("res", ctypes.c_double), ("iterations", ctypes.c_int),
                ("converged", ctypes.c_int)]


class ProfileStats(ctypes.Structure):
    _fields_ = [("launches", ctypes.c_uint64 * 6), ("ms", ctypes.c_double * 6),
                ("work", ctypes.c_double * 6)]


PROFILE_CATEGORIES = ("gemm6", "gemm", "quad", "energy", "elem", "pack")

# name -> (restype, argtypes)
_SIGS = {
    "kvft_profile_begin": (ctypes.c_int, [vp]),
    "kvft_profile_end": (ctypes.c_int, [vp, ctypes.POINTER(ProfileStats)]),
    "kvft_profile_records": (ctypes.c_int, [vp, ctypes.c_int, ctypes.POINTER(ctypes.c_int),
                                            vp, vp, vp]),
    "kvft_profile_shapes": (ctypes.c_int, [vp, ctypes.c_int, ctypes.POINTER(ctypes.c_int), vp]),
    "kvft_ctx_create": (ctypes.c_int, [ctypes.c_int, vp, ctypes.POINTER(vp)]),
    "kvft_ctx_destroy": (ctypes.c_int, [vp]),
    "kvft_last_error": (ctypes.c_char_p, [vp]),
    "kvft_status_string": (ctypes.c_char_p, [ctypes.c_int]),
    "kvft_set_precision": (ctypes.c_int, [vp, ctypes.c_int, ctypes.c_int]),
    "kvft_alloc": (ctypes.c_int, [vp, ctypes.c_size_t, ctypes.POINTER(vp)]),
    "kvft_free": (ctypes.c_int, [vp, vp]),
    "kvft_h2d": (ctypes.c_int, [vp, vp, vp, ctypes.c_size_t]),
    "kvft_d2h": (ctypes.c_int, [vp, vp, vp, ctypes.c_size_t]),
    "kvft_memset": (ctypes.c_int, [vp, vp, ctypes.c_int, ctypes.c_size_t]),
    "kvft_sync": (ctypes.c_int, [vp]),
    "kvft_event_record": (ctypes.c_int, [vp, ctypes.c_int]),
    "kvft_event_elapsed_ms": (ctypes.c_int, [vp, ctypes.c_int, ctypes.c_int,
                                             ctypes.POINTER(ctypes.c_float)]),
    "kvft_launch_count": (ctypes.c_int, [vp, ctypes.POINTER(ctypes.c_uint64)]),
    "kvft_flush_l2": (ctypes.c_int, [vp]),
    "kvft_int_tbar1": (ctypes.c_int, [vp, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                      vp, vp, vp, vp, ctypes.c_int, vp]),
    "kvft_int_tbar2": (ctypes.c_int, [vp, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                      vp, vp, vp, vp, ctypes.c_int, vp]),
    "kvft_int_tbar1_single": (ctypes.c_int, [vp, ctypes.c_int, ctypes.c_int,
                                             ctypes.c_int, ctypes.c_int, vp, vp, vp,
                                             vp, vp]),
    "kvft_int_tbar2_single": (ctypes.c_int, [vp, ctypes.c_int, ctypes.c_int,
                                             ctypes.c_int, ctypes.c_int, vp, vp, vp,
                                             vp, vp]),
    "kvft_ft_cc_energy": (ctypes.c_int, [vp, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                         vp, vp, vp, vp, vp, ctypes.c_double,
                                         ctypes.c_int, c_double_p]),
    "kvft_ccsd_stanton": (ctypes.c_int, [vp, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                         ctypes.POINTER(vp), ctypes.POINTER(vp), vp, vp,
                                         vp, vp, vp, vp, ctypes.c_int, vp, vp]),
    "kvft_stanton_residual": (ctypes.c_int, [vp, ctypes.c_int, ctypes.c_int,
                                             ctypes.c_int, ctypes.POINTER(vp),
                                             ctypes.POINTER(vp), vp, vp,
                                             ctypes.c_double, vp, vp]),
    "kvft_lambda_residual": (ctypes.c_int, [vp, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                            ctypes.POINTER(vp), ctypes.POINTER(vp), vp, vp,
                                            vp, vp, vp, vp]),
    "kvft_ccsd_lambda": (ctypes.c_int, [vp, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                        ctypes.POINTER(vp), ctypes.POINTER(vp), vp, vp, vp,
                                        vp, vp, vp, vp, vp, vp, vp, vp]),
    "kvft_lambda_densities": (ctypes.c_int, [vp, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                             ctypes.POINTER(vp), ctypes.POINTER(vp), vp, vp,
                                             vp, vp, vp, vp, vp, vp, vp, ctypes.POINTER(vp),
                                             ctypes.POINTER(vp)]),
    "kvft_lambda_solve": (ctypes.c_int, [vp, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                         ctypes.POINTER(vp), ctypes.POINTER(vp), vp, vp, vp,
                                         vp, vp, vp, vp, ctypes.c_double, ctypes.c_double,
                                         ctypes.c_int, ctypes.c_int, vp, vp, vp,
                                         ctypes.POINTER(ctypes.c_int)]),
    "kvft_set_lambda_spin_blocks": (ctypes.c_int, [vp, ctypes.c_int]),
    "kvft_set_residual_spin_blocks": (ctypes.c_int, [vp, ctypes.c_int]),
    "kvft_set_workspace_limit": (ctypes.c_int, [vp, ctypes.c_size_t]),
    "kvft_solver_step_begin": (ctypes.c_int, [vp, ctypes.c_double]),
    "kvft_solver_set_acceleration": (ctypes.c_int, [vp, ctypes.c_int]),
    "kvft_solver_set_graph": (ctypes.c_int, [vp, ctypes.c_int, ctypes.POINTER(ctypes.c_int)]),
    "kvft_solver_step_end": (ctypes.c_int, [vp, c_double_p, c_double_p]),
    "kvft_mem_info": (ctypes.c_int, [vp, ctypes.POINTER(ctypes.c_size_t),
                                     ctypes.POINTER(ctypes.c_size_t)]),
    "kvft_lambda_guess": (ctypes.c_int, [vp, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                         ctypes.POINTER(vp), ctypes.POINTER(vp), vp,
                                         ctypes.c_double, ctypes.c_int, vp, vp]),
    "kvft_einsum_plan": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_char_p,
                                        ctypes.c_char_p, ctypes.c_char_p,
                                        ctypes.POINTER(ctypes.c_int),
                                        ctypes.POINTER(ctypes.c_int),
                                        ctypes.POINTER(ctypes.c_longlong)]),
    "kvft_dryrun_create": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.POINTER(vp)]),
    "kvft_dryrun_count": (ctypes.c_int, [vp, ctypes.POINTER(ctypes.c_int)]),
    "kvft_dryrun_op": (ctypes.c_int, [vp, ctypes.c_int, ctypes.POINTER(ctypes.c_int),
                                      ctypes.POINTER(ctypes.c_longlong),
                                      ctypes.POINTER(ctypes.c_double), ctypes.POINTER(vp)]),
    "kvft_dryrun_scratch": (ctypes.c_int, [vp, ctypes.c_int, ctypes.POINTER(vp),
                                           ctypes.POINTER(ctypes.c_size_t)]),
    "kvft_ft_cc_energy_noalloc": (ctypes.c_int, [vp, ctypes.c_int, ctypes.c_int,
                                                 ctypes.c_int, vp, vp, vp, vp, vp,
                                                 ctypes.c_double, ctypes.c_int, vp]),
    "kvft_gemm": (ctypes.c_int, [vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                 ctypes.c_int, ctypes.c_int, vp, vp, vp]),
    "kvft_ueg_eri": (ctypes.c_int, [vp, ctypes.c_int, vp, ctypes.c_double, vp]),
    "kvft_hubbard_eri": (ctypes.c_int, [vp, ctypes.c_int, ctypes.c_double, vp]),
    "kvft_ft_integrals": (ctypes.c_int, [vp, ctypes.c_int, vp, vp, vp, ctypes.c_double,
                                         ctypes.c_double, ctypes.POINTER(vp),
                                         ctypes.POINTER(vp)]),
    "kvft_solver_create": (ctypes.c_int, [vp, ctypes.c_int, ctypes.c_int, vp, vp, vp,
                                          ctypes.c_double, ctypes.c_double, vp, vp, vp,
                                          ctypes.POINTER(vp)]),
    "kvft_solver_create_blocks": (ctypes.c_int, [vp, ctypes.c_int, ctypes.c_int,
                                                 ctypes.c_int, ctypes.POINTER(vp),
                                                 ctypes.POINTER(vp), vp, vp,
                                                 ctypes.c_double, vp, vp, vp,
                                                 ctypes.POINTER(vp)]),
    "kvft_solver_destroy": (ctypes.c_int, [vp]),
    "kvft_solver_run": (ctypes.c_int, [vp, ctypes.POINTER(SolveOpts),
                                       ctypes.POINTER(Result)]),
    "kvft_solver_step": (ctypes.c_int, [vp, ctypes.c_double, c_double_p, c_double_p]),
    "kvft_solver_run_point": (ctypes.c_int, [vp, ctypes.POINTER(SolveOpts),
                                             ctypes.POINTER(Result)]),
    "kvft_solver_get_amplitudes": (ctypes.c_int, [vp, vp, vp]),
    "kvft_solver_read_amplitudes": (ctypes.c_int, [vp, vp, vp, ctypes.c_int]),
    "kvft_solver_set_amplitudes": (ctypes.c_int, [vp, vp, vp]),
    "kvft_solver_device_amplitudes": (ctypes.c_int, [vp, ctypes.POINTER(vp),
                                                     ctypes.POINTER(vp)]),
    "kvft_solver_set_spin_blocks": (ctypes.c_int, [vp, ctypes.c_int,
                                                   ctypes.POINTER(ctypes.c_int)]),
    "kvft_solver_lambda": (ctypes.c_int, [vp, ctypes.c_int, ctypes.c_double, ctypes.c_double,
                                          ctypes.c_int, ctypes.c_int, vp, vp, vp,
                                          ctypes.POINTER(ctypes.c_int)]),
    "kvft_solver_lambda_densities": (ctypes.c_int, [vp, vp, vp, ctypes.POINTER(vp),
                                                    ctypes.POINTER(vp)]),
    "kvft_solver_footprint": (ctypes.c_size_t, [ctypes.c_int, ctypes.c_int,
                                                ctypes.c_int]),
}

_lib = None
_lock = threading.Lock()


def lib():
    """Load libkvft.so (raises if it is missing: no fallback exists)."""
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(LIB_PATH):
                raise RuntimeError("libkvft.so is not built (%s); run "
                                   "kelvin_gb300.build.build()" % LIB_PATH)
            L = ctypes.CDLL(LIB_PATH)
            for name, (res, args) in _SIGS.items():
                fn = getattr(L, name)
                fn.restype = res
                fn.argtypes = args
            _lib = L
    return _lib


def exported_symbols():
    """Names of the C entry points the binding declares."""
    return sorted(_SIGS)


class Context(object):
    """One CUDA device + stream (kvft_ctx)."""

    def __init__(self, device=0, stream=None):
        L = lib()
        h = vp()
        st = L.kvft_ctx_create(int(device), stream, ctypes.byref(h))
        if st != 0:
            raise KvftError("kvft_ctx_create(device=%d): %s" % (device, STATUS.get(st, st)), st)
        self.h = h
        self.device = device
        self.L = L

    def check(self, st, what):
        if st != 0:
            msg = self.L.kvft_last_error(self.h).decode(errors="replace")
            raise KvftError("%s: %s (%s)" % (what, STATUS.get(st, st), msg), st)

    def set_precision(self, precision, digits=7):
        self.check(self.L.kvft_set_precision(self.h, int(precision), int(digits)),
                   "kvft_set_precision")
        self._precision = (int(precision), int(digits))

    def sync(self):
        self.check(self.L.kvft_sync(self.h), "kvft_sync")

    def record(self, slot):
        self.check(self.L.kvft_event_record(self.h, slot), "kvft_event_record")

    def elapsed_ms(self, s0, s1):
        ms = ctypes.c_float()
        self.check(self.L.kvft_event_elapsed_ms(self.h, s0, s1, ctypes.byref(ms)),
                   "kvft_event_elapsed_ms")
        return float(ms.value)

    def launches(self):
        c = ctypes.c_uint64()
        self.check(self.L.kvft_launch_count(self.h, ctypes.byref(c)), "kvft_launch_count")
        return int(c.value)

    def flush_l2(self):
        self.check(self.L.kvft_flush_l2(self.h), "kvft_flush_l2")

    def mem_info(self):
        """(free, total) bytes of the context's device."""
        f, t = ctypes.c_size_t(), ctypes.c_size_t()
        self.check(self.L.kvft_mem_info(self.h, ctypes.byref(f), ctypes.byref(t)),
                   "kvft_mem_info")
        return int(f.value), int(t.value)

    def set_workspace_limit(self, nbytes):
        """Cap the tau-chunk workspace of this context's solvers (0: default)."""
        self.check(self.L.kvft_set_workspace_limit(self.h, int(nbytes)),
                   "kvft_set_workspace_limit")

    def set_residual_spin_blocks(self, half):
        """Assert spin blocks (alpha half h) for kvft_stanton_residual /
        kvft_ccsd_stanton on this context; 0 turns them off."""
        self.check(self.L.kvft_set_residual_spin_blocks(self.h, int(half)),
                   "kvft_set_residual_spin_blocks")

    def profile_begin(self):
        self.check(self.L.kvft_profile_begin(self.h), "kvft_profile_begin")

    def profile_records(self):
        """[(category, device ms, algorithmic work)] of every timed scope so
        far, in completion order (call before profile_end)."""
        n = ctypes.c_int()
        self.check(self.L.kvft_profile_records(self.h, 0, ctypes.byref(n), None, None, None),
                   "kvft_profile_records")
        cat = (ctypes.c_int * max(n.value, 1))()
        ms = (ctypes.c_float * max(n.value, 1))()
        work = (ctypes.c_double * max(n.value, 1))()
        self.check(self.L.kvft_profile_records(self.h, n.value, ctypes.byref(n), cat, ms, work),
                   "kvft_profile_records")
        return [(PROFILE_CATEGORIES[cat[i]], float(ms[i]), float(work[i]))
                for i in range(n.value)]

    def profile_shapes(self):
        """[(M, N, K, batch)] of the contraction behind each record (zeros for
        scopes that are not a contraction or its packing)."""
        n = ctypes.c_int()
        self.check(self.L.kvft_profile_shapes(self.h, 0, ctypes.byref(n), None),
                   "kvft_profile_shapes")
        sh = (ctypes.c_int * max(4 * n.value, 4))()
        self.check(self.L.kvft_profile_shapes(self.h, n.value, ctypes.byref(n), sh),
                   "kvft_profile_shapes")
        return [tuple(sh[4 * i:4 * i + 4]) for i in range(n.value)]

    def profile_end(self):
        """{category: (launches, total ms, algorithmic work)}."""
        st = ProfileStats()
        self.check(self.L.kvft_profile_end(self.h, ctypes.byref(st)), "kvft_profile_end")
        return {c: (int(st.launches[i]), float(st.ms[i]), float(st.work[i]))
                for i, c in enumerate(PROFILE_CATEGORIES)}

    def close(self):
        if self.h:
            self.L.kvft_ctx_destroy(self.h)
            self.h = None


_contexts = {}


def context(device=0):
    """Process-wide default context of a device."""
    with _lock:
        ctx = _contexts.get(device)
    if ctx is None:
        ctx = Context(device)
        with _lock:
            _contexts[device] = ctx
    return ctx


class DeviceArray(object):
    """A float64 device buffer with a shape (owned unless ``owner`` is set)."""

    def __init__(self, ctx, shape, ptr=None, owner=None):
        self.ctx = ctx
        self.shape = tuple(int(s) for s in shape)
        self.size = int(numpy.prod(self.shape)) if self.shape else 1
        self.nbytes = 8 * self.size
        self.owner = owner
        if ptr is None:
            p = vp()
            ctx.check(ctx.L.kvft_alloc(ctx.h, max(self.nbytes, 16), ctypes.byref(p)),
                      "kvft_alloc(%d bytes)" % self.nbytes)
            self.ptr = p
            self._own = True
        else:
            self.ptr = ptr if isinstance(ptr, vp) else vp(ptr)
            self._own = False

    @classmethod
    def from_host(cls, ctx, a):
        a = numpy.ascontiguousarray(a, dtype=numpy.float64)
        d = cls(ctx, a.shape)
        if a.size:
            ctx.check(ctx.L.kvft_h2d(ctx.h, d.ptr, a.ctypes.data_as(vp), a.nbytes), "kvft_h2d")
        return d

    def to_host(self, out=None):
        out = numpy.empty(self.shape) if out is None else out
        if self.size:
            self.ctx.check(self.ctx.L.kvft_d2h(self.ctx.h, out.ctypes.data_as(vp), self.ptr,
                                               self.nbytes), "kvft_d2h")
        return out

    def zero(self):
        self.ctx.check(self.ctx.L.kvft_memset(self.ctx.h, self.ptr, 0, self.nbytes),
                       "kvft_memset")

    def free(self):
        """Release the buffer now (it is released on collection otherwise)."""
        if self._own and self.ctx.h and self.ptr:
            self.ctx.L.kvft_free(self.ctx.h, self.ptr)
        self.ptr = vp()
        self._own = False

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


def as_device(ctx, a):
    """DeviceArray for ``a`` (copied in when it is a host array)."""
    if isinstance(a, DeviceArray):
        return a
    return DeviceArray.from_host(ctx, a)


def ptr_array(arrs):
    """ctypes array of device pointers."""
    return (vp * len(arrs))(*[a.ptr for a in arrs])
