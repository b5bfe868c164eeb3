"""Elastostatic Kelvin matrices (sod_elastostatic_assemble), collocation and Galerkin, against the
FP64 oracle restatement of src/elastics_bem_matrix_collection.cpp:43-385.  Tolerance: <= 1e-5 relative Frobenius
norm (FP32 regular faces; FP64 singular faces and diagonal correction).  The corrected H annihilates
rigid translations to FP64 rounding."""
import numpy as np
import pytest

from surfaceonlydeformables_gb300.meshes import Material, make_icosphere_mesh

from .conftest import rel_fro

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", params=[(2, 0.3), (3, 0.45)])
def case(request, gpu_ctx):
    from surfaceonlydeformables_gb300 import api

    level, nu = request.param
    m = make_icosphere_mesh(level, 0.1, axes=(1.3, 0.8, 1.0), jitter=0.1, seed=level)
    return m, api.Mesh(gpu_ctx, m), Material(1e5, nu, 1000.0)


@pytest.mark.parametrize("kind", ["G", "H"])
def test_elastostatic_vs_oracle(gpu_ctx, oracle, case, kind):
    from surfaceonlydeformables_gb300 import _lib as L
    from surfaceonlydeformables_gb300 import api

    m, dm, mat = case
    got = api.elastostatic(gpu_ctx, dm, kind, mat)
    ref = oracle.elastostatic(kind, m, mat)
    assert rel_fro(got, ref) <= 1e-5
    got32 = api.elastostatic(gpu_ctx, dm, kind, mat, dtype=L.F32)
    assert rel_fro(got32, ref) <= 1e-5


def test_elastostatic_H_rigid_translations(gpu_ctx, case):
    from surfaceonlydeformables_gb300 import api

    m, dm, mat = case
    H = api.elastostatic(gpu_ctx, dm, "H", mat)
    for d in range(3):
        t = np.zeros(3 * m.nV)
        t[d::3] = 1.0
        assert np.abs(H @ t).max() <= 1e-12 * np.abs(H).max() * m.nV


def test_elastostatic_deterministic(gpu_ctx, case):
    from surfaceonlydeformables_gb300 import api

    m, dm, mat = case
    a = api.elastostatic(gpu_ctx, dm, "H", mat)
    b = api.elastostatic(gpu_ctx, dm, "H", mat)
    assert np.array_equal(a, b)


@pytest.fixture(scope="module", params=[(1, 0.3), (2, 0.45)])
def gcase(request, gpu_ctx):
    from surfaceonlydeformables_gb300 import api

    level, nu = request.param
    m = make_icosphere_mesh(level, 0.1, axes=(1.2, 0.9, 1.0), jitter=0.1, seed=10 + level)
    return m, api.Mesh(gpu_ctx, m), Material(1e5, nu, 1000.0)


@pytest.mark.parametrize("kind", ["G", "H"])
def test_elastostatic_galerkin_vs_oracle(gpu_ctx, oracle, gcase, kind):
    """Galerkin G and H (H with the mass matrix and the rigid-mode diagonal correction,
    src/elastics_bem_matrix_collection.cpp:246-385) against the FP64 oracle: <= 1e-5."""
    from surfaceonlydeformables_gb300 import _lib as L
    from surfaceonlydeformables_gb300 import api

    m, dm, mat = gcase
    got = api.elastostatic(gpu_ctx, dm, kind, mat, order=3, sorder=3, method=L.GALERKIN)
    ref = oracle.elastostatic(kind, m, mat, galerkin=True, order=3, sorder=3)
    assert rel_fro(got, ref) <= 1e-5, rel_fro(got, ref)
    if kind == "G":
        # the Galerkin single layer is symmetric up to the quadrature: the Sauter-Schwab maps of the
        # singular pairs do not treat x and y alike (same bound as the Laplace-domain Galerkin G)
        assert rel_fro(got, got.T) <= 1e-4
    else:
        for d in range(3):
            t = np.zeros(3 * m.nV)
            t[d::3] = 1.0
            assert np.abs(got @ t).max() <= 1e-12 * np.abs(got).max() * m.nV
    again = api.elastostatic(gpu_ctx, dm, kind, mat, order=3, sorder=3, method=L.GALERKIN)
    assert np.array_equal(got, again)
