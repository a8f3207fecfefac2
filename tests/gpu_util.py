"""Shared helpers for the GPU tests."""
import os

import numpy as np

from opendeformer_gb300 import api

_ctx = None


def ctx():
    global _ctx
    if _ctx is None:
        if not os.path.exists(api.LIB_PATH):
            from opendeformer_gb300 import build
            build.build()
        _ctx = api.Context(0)
    return _ctx


def material(name, rho, E, nu, thr):
    return api.Material(name, float(rho), float(E), float(nu), float(thr))


def rel_err(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))
