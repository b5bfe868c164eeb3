"""Galerkin assembly of G and H (method SOD_GALERKIN) against the FP64 oracle restatement of
src/elastodynamics_cqbem_{G,H}_galerkin_non_singular.cu and src/elastodynamics_cqbem_galerkin_singular.cpp.
Tolerances: whole rows <= 1e-5 relative Frobenius (FP32 regular pairs); the singular face pairs alone
(double-float Sauter-Schwab quadrature) <= 1e-10."""
import numpy as np
import pytest

from surfaceonlydeformables_gb300.meshes import Material, make_icosphere_mesh

from .conftest import rel_fro

pytestmark = pytest.mark.gpu
MAT = Material(1e5, 0.45, 1000.0)


@pytest.fixture(scope="module")
def small(gpu_ctx):
    from surfaceonlydeformables_gb300 import api

    m = make_icosphere_mesh(1, 0.1, jitter=0.2, seed=3)
    return m, api.Mesh(gpu_ctx, m)


def freq(sodlib, l=3):
    s, R, L = sodlib.cq_frequencies(2, 1 / 200, 64)
    return s[l]


@pytest.mark.parametrize("kind", ["G", "H", "B_trans", "B_angular"])
@pytest.mark.parametrize("order", [5, 7])
def test_galerkin_parts_vs_oracle(gpu_ctx, oracle, sodlib, small, kind, order):
    from surfaceonlydeformables_gb300 import _lib as L
    from surfaceonlydeformables_gb300 import api

    m, dm = small
    s = freq(sodlib)
    for parts, tol in ((L.PART_REGULAR, 1e-5), (L.PART_SINGULAR, 1e-10), (L.PART_ALL, 1e-5)):
        got = api.assemble(gpu_ctx, dm, kind, MAT, s, order=order, sorder=5, ssub=1, method=L.GALERKIN,
                           parts=parts)
        ref = oracle.galerkin(kind, m, MAT, s, order=order, sorder=5, ssub=1, parts=parts)
        assert rel_fro(got, ref) <= tol, (parts, rel_fro(got, ref))


def test_galerkin_rows_sampled_642(gpu_ctx, oracle, sodlib):
    """Row-sampled oracle on 642 vertices (the rows of the sampled vertices are exact)."""
    from surfaceonlydeformables_gb300 import _lib as L
    from surfaceonlydeformables_gb300 import api

    m = make_icosphere_mesh(3, 0.1, jitter=0.2, seed=5)
    dm = api.Mesh(gpu_ctx, m)
    s = freq(sodlib, 7)
    rows = np.array([0, 17, 100, 333, 641], dtype=np.int32)
    for kind in ("G", "H"):
        got = api.assemble(gpu_ctx, dm, kind, MAT, s, order=7, sorder=5, ssub=1, method=L.GALERKIN)
        ref = oracle.galerkin(kind, m, MAT, s, order=7, sorder=5, ssub=1, rows=rows)
        sel = np.concatenate([np.arange(3 * r, 3 * r + 3) for r in rows])
        assert rel_fro(got[sel], ref) <= 1e-5, kind


def test_galerkin_G_symmetric(gpu_ctx, sodlib, small):
    """The Galerkin single layer is symmetric (U_ab = U_ba^T): to FP32 rounding over the regular
    pairs; to the quadrature error of the Sauter-Schwab maps (which treat the two triangles
    differently) with the singular pairs, the oracle's own bound."""
    from surfaceonlydeformables_gb300 import _lib as L
    from surfaceonlydeformables_gb300 import api

    m, dm = small
    Ur = api.assemble(gpu_ctx, dm, "G", MAT, freq(sodlib), order=7, method=L.GALERKIN, parts=L.PART_REGULAR)
    assert np.linalg.norm(Ur - Ur.T) / np.linalg.norm(Ur) <= 1e-6
    U = api.assemble(gpu_ctx, dm, "G", MAT, freq(sodlib), order=7, method=L.GALERKIN)
    assert np.linalg.norm(U - U.T) / np.linalg.norm(U) <= 1e-4


def test_galerkin_all_kinds_in_one_call(gpu_ctx, oracle, sodlib, small):
    """G, H, B_trans and B_angular together (B fused into the G pass) match the single-kind calls."""
    from surfaceonlydeformables_gb300 import _lib as L
    from surfaceonlydeformables_gb300 import api

    m, dm = small
    s, R, Lq = sodlib.cq_frequencies(2, 1 / 200, 16)
    allk = api.assemble_all(gpu_ctx, dm, MAT, s[:3], order=5, method=L.GALERKIN)
    for kind in ("G", "H", "B_trans", "B_angular"):
        one = api.assemble_frequencies(gpu_ctx, dm, kind, MAT, s[:3], order=5, method=L.GALERKIN)
        assert rel_fro(allk[kind], one) <= 1e-6, kind
        ref = oracle.galerkin(kind, m, MAT, s[2], order=5, sorder=5, ssub=1)
        assert rel_fro(allk[kind][2], ref) <= 1e-5, kind


def test_galerkin_row_block_beyond_shared_memory(gpu_ctx, oracle, sodlib):
    """The reference's 3485-vertex bunny: the test-point rows of H (9 x 3485 complex FP32) exceed
    shared memory, so each CTA accumulates directly in its global-memory output row.  Sampled rows
    of G (with the B kinds) and H against the row-sampled FP64 oracle, <= 1e-5."""
    import os

    import torch

    from surfaceonlydeformables_gb300 import _lib as L
    from surfaceonlydeformables_gb300 import api
    from surfaceonlydeformables_gb300.meshes import SurfaceMesh

    b = np.load(os.path.join(os.path.dirname(__file__), "golden", "bunny_mesh.npz"))
    m = SurfaceMesh.from_arrays(b["V"], b["F"])
    dm = api.Mesh(gpu_ctx, m)
    s, R, Lq = sodlib.cq_frequencies(1, 0.003, 5)
    rows = np.array([11, 1800], dtype=np.int32)
    n3 = 3 * m.nV
    for kind in ("H", "G"):
        out = torch.empty((1, n3, n3), dtype=torch.complex128, device="cuda")
        api.assemble_frequencies(gpu_ctx, dm, kind, MAT, s[1:2], order=5, sorder=5, ssub=1, method=L.GALERKIN,
                                 out=out)
        torch.cuda.synchronize()
        got = np.concatenate([out[0, 3 * v:3 * v + 3].cpu().numpy() for v in rows])
        ref = oracle.galerkin(kind, m, MAT, s[1], order=5, sorder=5, ssub=1, rows=rows)
        assert rel_fro(got, ref) <= 1e-5, (kind, rel_fro(got, ref))
        del out
