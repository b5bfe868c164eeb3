"""Dense LU solves on the device (sod_solver: the H_0 factorisation, u_p = H_0^-1 G_0', the inverse,
and the fused per-step u = H_0^-1 b) against numpy.linalg in FP64.

Tolerance: relative Frobenius norm <= 1e-11 for the random well-conditioned systems and <= 1e-10
against H_0 of a real precompute (FP64 LU with partial pivoting in both)."""
import numpy as np
import pytest

from surfaceonlydeformables_gb300.meshes import Material, make_icosphere_mesh

from .conftest import rel_fro

pytestmark = pytest.mark.gpu


def make_solver(api, L, ctx, A):
    try:
        return api.Solver(ctx, A)
    except L.SodError as e:
        if e.code == L.SOD_ERR_UNSUPPORTED:
            pytest.skip(str(e))
        raise


def test_solver_random_systems(gpu_ctx):
    from surfaceonlydeformables_gb300 import _lib as L
    from surfaceonlydeformables_gb300 import api

    rng = np.random.default_rng(0)
    n = 301
    A = rng.normal(size=(n, n)) + n ** 0.5 * np.eye(n)
    S = make_solver(api, L, gpu_ctx, A)
    b = rng.normal(size=n)
    assert rel_fro(S.solve(b), np.linalg.solve(A, b)) <= 1e-11
    B = rng.normal(size=(n, 7))
    assert rel_fro(S.solve(B), np.linalg.solve(A, B)) <= 1e-11
    assert rel_fro(S.inverse(), np.linalg.inv(A)) <= 1e-11


def test_solver_singular_matrix(gpu_ctx):
    from surfaceonlydeformables_gb300 import _lib as L
    from surfaceonlydeformables_gb300 import api

    A = np.ones((4, 4))
    with pytest.raises(L.SodError) as e:
        make_solver(api, L, gpu_ctx, A)
    assert e.value.code == L.SOD_ERR_INVALID_ARG


def test_solver_u_p_from_precompute(gpu_ctx):
    """u_p = H_0^-1 G_0 and H_0^-1 B_trans_0 (src/elastodynamics_cqbem_matrix_collection.cpp:204-214)."""
    import torch

    from surfaceonlydeformables_gb300 import _lib as L
    from surfaceonlydeformables_gb300 import api

    m = make_icosphere_mesh(2, 0.1)
    dm = api.Mesh(gpu_ctx, m)
    w = api.precompute(gpu_ctx, dm, Material(1e5, 0.3, 1000.0), 2, 0.01, 8, kinds=("G", "H", "B_trans"))
    H0, G0, Bt0 = (w[k][0].contiguous() for k in ("H", "G", "B_trans"))
    S = make_solver(api, L, gpu_ctx, H0)  # device input
    up = torch.empty_like(G0)
    S.solve(G0, out=up)  # device in, device out
    torch.cuda.synchronize()
    ref = np.linalg.solve(H0.cpu().numpy(), G0.cpu().numpy())
    assert rel_fro(up.cpu().numpy(), ref) <= 1e-10
    assert rel_fro(S.solve(Bt0.cpu().numpy()), np.linalg.solve(H0.cpu().numpy(), Bt0.cpu().numpy())) <= 1e-10


@pytest.mark.parametrize("R", [1, 16])
def test_history_convolve_solve(gpu_ctx, R):
    """One served step on the device: u = A^-1 b with b the bank's convolution."""
    from surfaceonlydeformables_gb300 import _lib as L
    from surfaceonlydeformables_gb300 import api

    rng = np.random.default_rng(R)
    n, K = 120, 4
    bank = api.HistoryBank(gpu_ctx, n, n, K, R, L.F32)
    for k in range(1, K + 1):
        bank.set_weights(k, rng.normal(size=(n, n)), rng.normal(size=(n, n)))
    shape = (n, R) if R > 1 else (n,)
    for _ in range(K + 1):
        bank.push(rng.normal(size=shape), rng.normal(size=shape))
    A = rng.normal(size=(n, n)) + n ** 0.5 * np.eye(n)
    S = make_solver(api, L, gpu_ctx, A)
    b = bank.convolve()
    u = bank.convolve_solve(S)
    assert rel_fro(u, np.linalg.solve(A, b)) <= 1e-11
    S.keep_inverse()  # the per-step form: GEMV with the resident inverse
    u2 = bank.convolve_solve(S)
    assert rel_fro(u2, np.linalg.solve(A, b)) <= 1e-11
    assert np.array_equal(u2, bank.convolve_solve(S))  # deterministic
