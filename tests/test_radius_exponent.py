"""The stencils' power-of-two scale comes from frexp(sqrt(r2max)); the kernels take its
exponent from r2max's bit pattern instead (sqrt_frexp_exponent in stencil_common.cuh:
(E + 1) >> 1 for r2max = m 2^E, m in [0.5, 1)).  That rule is checked here against IEEE
square roots over the normal range, every power of two and its neighbours included (the
device's sqrt is correctly rounded, as numpy's)."""
import struct

import numpy as np


def exponent_rule(x):
    b = struct.unpack("<q", struct.pack("<d", x))[0]
    return ((((b >> 52) & 0x7FF) - 1022) + 1) >> 1


def test_rule_equals_frexp_of_sqrt():
    rng = np.random.default_rng(0)
    xs = list(np.exp(rng.uniform(-700, 700, 50000)))
    for a in range(-1021, 1023):
        p = 2.0 ** a
        xs += [p, np.nextafter(p, 0.0), np.nextafter(p, np.inf), np.nextafter(np.nextafter(p, 0.0), 0.0)]
    xs = [x for x in xs if np.isfinite(x) and x >= np.finfo(np.float64).tiny]
    bad = [x for x in xs if exponent_rule(x) != int(np.frexp(np.sqrt(x))[1])]
    assert not bad, bad[:5]
