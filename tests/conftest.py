import os
import sys

import numpy
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU and libkvft.so")


def golden(name):
    return numpy.load(os.path.join(GOLDEN, name))


@pytest.fixture(scope="session")
def ctx():
    from kelvin_gb300 import _lib
    return _lib.context(0)


class Blocks(object):
    pass


def unpack_blocks(d, prefix):
    """(F, I) containers from a fixture written by make_golden.pack_blocks."""
    F, I = Blocks(), Blocks()
    for b in ("oo", "ov", "vo", "vv"):
        setattr(F, b, d[prefix + "F_" + b])
    for b in ("vvvv", "vvvo", "vovv", "vvoo", "vovo", "oovv", "vooo", "ooov", "oooo"):
        setattr(I, b, d[prefix + "I_" + b])
    return F, I


def random_system(rng, no, nv, scale_f=0.2, scale_g=0.1):
    """Consistent random F/I blocks sliced from a full antisymmetric tensor."""
    n = no + nv
    f = rng.standard_normal((n, n)) * scale_f
    g = rng.standard_normal((n, n, n, n)) * scale_g
    g = g - g.transpose(1, 0, 2, 3)
    g = g - g.transpose(0, 1, 3, 2)
    o, v = slice(0, no), slice(no, n)
    sl = {'o': o, 'v': v}
    F, I = Blocks(), Blocks()
    for b in ("oo", "ov", "vo", "vv"):
        setattr(F, b, numpy.ascontiguousarray(f[sl[b[0]], sl[b[1]]]))
    for b in ("vvvv", "vvvo", "vovv", "vvoo", "vovo", "oovv", "vooo", "ooov", "oooo"):
        setattr(I, b, numpy.ascontiguousarray(g[tuple(sl[c] for c in b)]))
    return F, I


def random_T(rng, ng, nv, no, scale=0.05):
    T1 = rng.standard_normal((ng, nv, no)) * scale
    T2 = rng.standard_normal((ng, nv, nv, no, no)) * scale
    T2 = T2 - T2.transpose(0, 2, 1, 3, 4)
    T2 = T2 - T2.transpose(0, 1, 2, 4, 3)
    return T1, T2
