"""GPU path against the golden fixtures made by the reference's own CPU code."""
import numpy as np
import pytest

import golden_cases

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", ["double", "single"])
def test_gpu_matches_reference_golden(precision):
    import galario_gb300 as g
    impl = getattr(g, precision)
    d = golden_cases.load(precision)
    # double: the reference's own results to 1e-12; single: the single-precision
    # tolerance 1e-5.  The reference's single build runs every stage in float
    # (FP32 index and phase) and differs from its double build by up to 2.1e-6
    # on these cases; the GPU path keeps the index and phase in double-float.
    tol = 1e-12 if precision == "double" else 1e-5
    for name, got, exp in golden_cases.run_all(impl, d):
        assert np.shape(got) == np.shape(exp), name
        assert golden_cases.rel(got, exp) <= tol, (name, golden_cases.rel(got, exp))
