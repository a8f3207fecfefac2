"""The mixed-precision path's element evaluation against the FP64 one, on
displaced meshes up to inverted elements.  Stiffness: the double-float
contraction (FP32 pairs, operands split and results rebuilt with integer
bit operations; a plain FP32 contraction was 5.7e-8 of the largest value
off).  Forces: the
invertible elements' stay FP64, their SVD's first eigenvalue taken from
FP32 trigonometry and refined by Newton steps; the corotational element's
are the reference's sum regrouped in FP64 (R sum_b K0_ab (R^T x_b - X_b)).
The corotational values within 1e-12 of the largest.  The invertible
elements' values within 1e-10: the refined eigenvalue can differ from the
FP64 trigonometric one by an ulp, and where two singular values nearly
coincide the eigenvectors turn by about ulp / gap (up to 1.4e-11 of the
largest stiffness value on these meshes; typical entries 1e-15).  At the
largest displacement (four element sizes: most elements inverted and
clamped, singular values near the clamp) the ulp-level differences of the
mixed path's reciprocal roots and products grow to about 1e-9 of the
largest force; that case is held to 1e-8."""
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
@pytest.mark.parametrize("scale", [0.002, 0.02, 0.2])
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
    bound = 1e-12 if kind == "corotational" else (1e-10 if scale < 0.1 else 1e-8)
    assert np.abs(k64).max() > 0
    assert np.abs(kdf - k64).max() <= bound * np.abs(k64).max()
    assert np.abs(f64).max() > 0
    assert np.abs(fdf - f64).max() <= bound * np.abs(f64).max()
