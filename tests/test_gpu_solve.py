"""Dense solves on the device in FP64:
- sod_solver (the H_0 factorisation, u_p = H_0^-1 G_0', the inverse, the fused per-step
  u = H_0^-1 b) against numpy.linalg;
- sod_lstsq (the complete orthogonal decompositions B_trans_inv / B_euler_inv) against the oracle's
  restatement of the same algorithm;
- sod_elastostatic_u_p (the regularised elastostatic solve) against the oracle's restatement.

Tolerances (relative Frobenius): <= 1e-11 for random well-conditioned systems, <= 1e-10 against
H_0 of a real precompute, <= 1e-12 for least squares with well-conditioned B.  The regularised
elastostatic system has condition numbers of 1e6-1e7, where FP64 solvers of different kinds differ
by up to 2.5e-10: u_p is held to 1e-8 against the oracle, and its backward error
||H' u_p - G'|| / ||G'|| to 1e-12."""
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


def make_lstsq(api, L, ctx, B):
    try:
        return api.LeastSquares(ctx, B)
    except L.SodError as e:
        if e.code == L.SOD_ERR_UNSUPPORTED:
            pytest.skip(str(e))
        raise


def test_lstsq_full_rank(gpu_ctx):
    from oracle import oracle

    from surfaceonlydeformables_gb300 import _lib as L
    from surfaceonlydeformables_gb300 import api

    rng = np.random.default_rng(3)
    m, k = 1000, 3
    B = rng.normal(size=(m, k))
    Y = rng.normal(size=(m, 37))
    S = make_lstsq(api, L, gpu_ctx, B)
    assert S.rank == 3
    assert rel_fro(S.solve(Y), oracle.cod_solve(B, Y)) <= 1e-12
    assert rel_fro(S.solve(Y[:, 0]), oracle.cod_solve(B, Y[:, 0])) <= 1e-12
    assert rel_fro(S.pinv(), oracle.cod_solve(B, np.eye(m))) <= 1e-12
    assert np.array_equal(S.solve(Y), S.solve(Y))  # deterministic


@pytest.mark.parametrize("k,rank", [(3, 2), (6, 4), (8, 8), (1, 1)])
def test_lstsq_rank_deficient(gpu_ctx, k, rank):
    """Planted linear dependencies: the minimum-norm solution of the complete orthogonal decomposition."""
    from oracle import oracle

    from surfaceonlydeformables_gb300 import _lib as L
    from surfaceonlydeformables_gb300 import api

    rng = np.random.default_rng(k)
    m = 257
    B = rng.normal(size=(m, k))
    for c in range(rank, k):  # columns beyond `rank` are combinations of earlier ones
        B[:, c] = B[:, c - rank] - 0.5 * B[:, (c + 1) % rank]
    Y = rng.normal(size=(m, 11))
    S = make_lstsq(api, L, gpu_ctx, B)
    assert S.rank == rank
    ref = oracle.cod_solve(B, Y)
    assert rel_fro(ref, np.linalg.pinv(B, rcond=1e-10) @ Y) <= 1e-12  # oracle = pseudo-inverse
    assert rel_fro(S.solve(Y), ref) <= 1e-10


def test_lstsq_zero_and_bad_shapes(gpu_ctx):
    from surfaceonlydeformables_gb300 import _lib as L
    from surfaceonlydeformables_gb300 import api

    S = make_lstsq(api, L, gpu_ctx, np.zeros((20, 3)))
    assert S.rank == 0
    assert np.array_equal(S.solve(np.ones((20, 4))), np.zeros((3, 4)))
    for shape in [(2, 3), (40, 9)]:
        with pytest.raises(L.SodError) as e:
            api.LeastSquares(gpu_ctx, np.ones(shape))
        assert e.value.code == L.SOD_ERR_INVALID_ARG


def test_lstsq_b_trans_from_precompute(gpu_ctx):
    """B_trans_inv.solve(H_0), .solve(G_0), B_euler_inv.solve(B_trans)
    (src/elastodynamics_cqbem_matrix_collection.cpp:184-191) on a real precompute, device buffers."""
    import torch
    from oracle import oracle

    from surfaceonlydeformables_gb300 import _lib as L
    from surfaceonlydeformables_gb300 import api

    m = make_icosphere_mesh(2, 0.1)
    dm = api.Mesh(gpu_ctx, m)
    w = api.precompute(gpu_ctx, dm, Material(1e5, 0.3, 1000.0), 2, 0.01, 8,
                       kinds=("G", "H", "B_trans", "B_euler"))
    H0, G0, Bt0, Be0 = (w[k][0].contiguous() for k in ("H", "G", "B_trans", "B_euler"))
    St = make_lstsq(api, L, gpu_ctx, Bt0)
    Se = make_lstsq(api, L, gpu_ctx, Be0)
    assert St.rank == 3 and Se.rank == 3
    X = torch.empty((3, H0.shape[1]), dtype=torch.float64, device=H0.device)
    St.solve(H0, out=X)
    torch.cuda.synchronize()
    h, g, bt, be = (t.cpu().numpy() for t in (H0, G0, Bt0, Be0))
    assert rel_fro(X.cpu().numpy(), oracle.cod_solve(bt, h)) <= 1e-10
    assert rel_fro(St.solve(g), oracle.cod_solve(bt, g)) <= 1e-10
    # on a centred sphere B_trans is nearly orthogonal to the range of B_euler, so B_euler^+ B_trans is
    # small (~1e-8 relative) and all cancellation: compare on the scale ||B_euler^+|| ||B_trans||
    d = Se.solve(bt) - oracle.cod_solve(be, bt)
    assert np.linalg.norm(d) <= 1e-12 * np.linalg.norm(np.linalg.pinv(be)) * np.linalg.norm(bt)


def test_rigid_modes_match_oracle(gpu_ctx):
    from oracle import oracle

    from surfaceonlydeformables_gb300 import api

    m = make_icosphere_mesh(2, 0.1)
    dm = api.Mesh(gpu_ctx, m)
    assert rel_fro(api.rigid_modes(gpu_ctx, dm), oracle.rigid_modes(m)) <= 1e-14


@pytest.mark.parametrize("galerkin", [False, True])
def test_elastostatic_u_p(gpu_ctx, galerkin):
    """u_p = (H^T H + c^2 T^T T)^-1 H^T G (I - T^T (T T^T)^-1 T)
    (src/elastostatics_bem_matrix_collection.cpp:58-89) from the library's own H and G."""
    import torch
    from oracle import oracle

    from surfaceonlydeformables_gb300 import _lib as L
    from surfaceonlydeformables_gb300 import api

    m = make_icosphere_mesh(2, 0.1)
    dm = api.Mesh(gpu_ctx, m)
    mat = Material(1e5, 0.3, 1000.0)
    method = L.GALERKIN if galerkin else L.COLLOCATION
    kw = dict(order=5, subdiv=1, sorder=5, ssub=1, method=method)
    H = api.elastostatic(gpu_ctx, dm, "H", mat, **kw)
    G = api.elastostatic(gpu_ctx, dm, "G", mat, **kw)
    try:
        up = api.elastostatic_u_p(gpu_ctx, dm, H, G)
    except L.SodError as e:
        if e.code == L.SOD_ERR_UNSUPPORTED:
            pytest.skip(str(e))
        raise
    T = oracle.rigid_modes(m)
    ref = oracle.elastostatic_u_p(H, G, T)
    assert rel_fro(up, ref) <= 1e-8
    n = H.shape[0]
    Hr = H.T @ H + (np.trace(H) / n) ** 2 * (T.T @ T)
    Gp = H.T @ G @ (np.eye(n) - T.T @ np.linalg.solve(T @ T.T, T))
    assert rel_fro(Hr @ up, Gp) <= 1e-12
    # rigid tractions are projected out: u_p T^T = 0
    assert np.linalg.norm(up @ T.T) <= 1e-9 * np.linalg.norm(up) * np.linalg.norm(T)
    # device buffers in and out give the same bits
    dH, dG = torch.from_numpy(H).cuda(), torch.from_numpy(G).cuda()
    dup = torch.empty_like(dH)
    api.elastostatic_u_p(gpu_ctx, dm, dH, dG, out=dup)
    torch.cuda.synchronize()
    assert np.array_equal(dup.cpu().numpy(), up)
