"""The roofline's measuring probes on the GPU: the DFMA peak and the cost of
CUDA's FP64 functions in units of it (the measured transcendental weights of
the scan's roofline numerator)."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

import cortrace as ct

pytestmark = pytest.mark.gpu

NAMES = ["loop", "exp", "log", "sin", "cos", "atan", "asin", "atan2", "pow", "div", "sqrt"]


def test_fp64_probes(ctx):
    peak = C.c_double(0.0)
    ctx._check(ctx.lib.cor_probe_fp64_peak(ctx.h, C.byref(peak)), "peak")
    w = np.zeros(11)
    ctx._check(ctx.lib.cor_probe_fp64_functions(ctx.h, w.ctypes.data), "functions")
    print(f"FP64 peak {peak.value / 1e12:.3f} TFLOP/s; flops per call:",
          {n: round(float(v), 1) for n, v in zip(NAMES, w)})
    assert peak.value > 1e11
    assert w[0] == 0.0
    # every function costs more than one FMA and less than a few hundred
    assert np.all(w[1:] > 2.0) and np.all(w[1:] < 1000.0)
    # a division or square root is cheaper than a transcendental
    assert w[9] < w[8] and w[10] < w[8]
