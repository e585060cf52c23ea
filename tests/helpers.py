"""Shared helpers for the test-suite (geometry records for the oracle probes)."""
import ctypes as C

import numpy as np

from gartus_gb300 import abi


def geometry(kind, *vals):
    g = abi.gt_geometry()
    g.kind = kind
    flat = [float(x) for v in vals for x in (v if isinstance(v, (tuple, list)) else (v,))]
    for i, x in enumerate(flat):
        g.p[i] = x
    return g


def dptr(values):
    arr = (C.c_double * len(values))(*[float(v) for v in values])
    return arr


def material(kind, color=(0.0, 0.0, 0.0), param=0.0):
    m = abi.gt_material()
    m.kind = kind
    for i in range(3):
        m.color[i] = color[i]
    m.param = param
    return m


def rel_err(a, b, floor=1e-6):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return np.abs(a - b) / np.maximum(np.maximum(np.abs(a), np.abs(b)), floor)
