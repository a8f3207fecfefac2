"""The mixed-precision path's double-float stiffness contraction (FP32
pairs, operands split and results rebuilt with integer bit operations)
against the exact FP64 one, on displaced meshes: every assembled stiffness
value within 1e-12 of the largest (the FP32 rounding of a plain FP32
contraction was 5.7e-8).  The invertible elements' internal forces stay FP64
and equal bit for bit; the corotational element's are the reference's sum
regrouped in FP64 (R sum_b K0_ab (R^T x_b - X_b)), within 1e-12 of the
largest."""
import os

import numpy as np
import pytest

from opendeformer_gb300 import api, meshgen
from tests.gpu_util import ctx

pytestmark = pytest.mark.gpu


def evaluate(s, df):
    old = os.environ.get("OD_GB300_ELEMENT_DF")
    os.environ["OD_GB300_ELEMENT_DF"] = "1" if df else "0"
    try:
        return s.evaluate()
    finally:
        if old is None:
            os.environ.pop("OD_GB300_ELEMENT_DF", None)
        else:
            os.environ["OD_GB300_ELEMENT_DF"] = old


@pytest.mark.parametrize("kind", ["neohookean", "stvk", "corotational"])
@pytest.mark.parametrize("scale", [0.002, 0.02])
def test_double_float_contraction_matches_fp64(kind, scale):
    g = meshgen.tet_grid(10, 4, 4, h=0.05, jitter=0.15, seed=21)
    cd = meshgen.constrained_dofs_for_nodes(g.face_nodes(0, 0))
    mat = api.Material(kind, 1000.0, 1e5, 0.45, 0.1)
    s = api.Scene(ctx(), g.X, g.tets, g.facets, cd, mat)
    rng = np.random.default_rng(5)
    u = rng.normal(scale=scale, size=(g.n_nodes, 3))
    u[g.face_nodes(0, 0)] = 0.0
    s.set_displacements(u)
    k64, f64 = evaluate(s, False)
    kdf, fdf = evaluate(s, True)
    s.close()
    assert np.abs(k64).max() > 0
    assert np.abs(kdf - k64).max() <= 1e-12 * np.abs(k64).max()
    if kind == "corotational":
        assert np.abs(f64).max() > 0
        assert np.abs(fdf - f64).max() <= 1e-12 * np.abs(f64).max()
    else:
        assert np.array_equal(fdf, f64)
