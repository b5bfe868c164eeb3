"""GPU test of the allocation-free assembly entry point (sod_cqbem_assemble_noalloc).

Some callers cannot allocate device memory while they run (a host program that owns the whole
device memory budget, a real-time step loop where cudaMalloc would stall the device).  For them the
library offers one entry point whose only scratch is a fixed device array inside the library.
This file is named so that pytest collects it last; it creates its own context and meshes, so it
also passes when run alone in a fresh process.

Checks, through the C ABI: two calls in a row match the regular entry point within the Laplace-
domain tolerance of the other tests (1e-5 relative Frobenius) for every kind, with complex128 and
complex64 outputs; frequencies are chunked to fit the scratch; a warm call leaves the device's free
memory (cudaMemGetInfo) unchanged; and meshes beyond the scratch or beyond the shared-memory row
block are rejected with SOD_ERR_CAPACITY.
"""
import ctypes

import numpy as np
import pytest

from surfaceonlydeformables_gb300.meshes import Material, make_icosphere_mesh

pytestmark = pytest.mark.gpu

MAT = Material(1e5, 0.3, 1000.0)
TOL = 1e-5


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def _noalloc(L, ctx, mesh, kind, s, out, dtype):
    sv = np.ascontiguousarray(np.asarray(s, dtype=np.complex128)).view(np.float64)
    return L.load().sod_cqbem_assemble_noalloc(ctx.handle, mesh.handle, L.KINDS[kind], MAT.c1, MAT.c2, MAT.rho,
                                               L.ptr(sv), len(s), 5, 1, 5, 1, ctypes.c_void_p(out.data_ptr()), dtype)


@pytest.mark.parametrize("kind,c64", [("G", False), ("H", False), ("B_trans", False), ("B_angular", False),
                                      ("G", True), ("B_trans", True)])
def test_noalloc_matches_regular_entry_point(sodlib, kind, c64):
    import torch

    from surfaceonlydeformables_gb300 import _lib as L
    from surfaceonlydeformables_gb300 import api

    dt_lib = L.C64 if c64 else L.C128
    dt_torch = torch.complex64 if c64 else torch.complex128
    ctx = api.Context(0)
    mesh = api.Mesh(ctx, make_icosphere_mesh(3, 0.1))  # 642 vertices: G/H need several chunks
    s, R, Lq = L.cq_frequencies(2, 0.01, 32)
    ref = api.assemble_frequencies(ctx, mesh, kind, MAT, s, dtype=dt_lib)  # also builds the schedule
    out = torch.empty(ref.shape, dtype=dt_torch, device="cuda")
    free_after_first = None
    for call in range(2):
        out.zero_()
        torch.cuda.synchronize()
        rc = _noalloc(L, ctx, mesh, kind, s, out, dt_lib)
        assert rc == L.SOD_OK, L.load().sod_last_error()
        ctx.synchronize()
        free_now = torch.cuda.mem_get_info()[0]
        if call == 0:
            free_after_first = free_now  # the first call may load kernels (lazy module loading)
        else:
            assert free_now == free_after_first, "a warm call changed the device's free memory"
        got = out.cpu().numpy().reshape(ref.shape)
        assert _rel(got, ref) <= TOL, (kind, c64, call, _rel(got, ref))


def test_noalloc_rejects_meshes_beyond_the_scratch(sodlib):
    import torch

    from surfaceonlydeformables_gb300 import _lib as L
    from surfaceonlydeformables_gb300 import api

    ctx = api.Context(0)
    big = api.Mesh(ctx, make_icosphere_mesh(5, 0.1))  # 10242 vertices
    s, R, Lq = L.cq_frequencies(2, 0.01, 4)
    out = torch.empty(1, dtype=torch.complex128, device="cuda")
    rc = _noalloc(L, ctx, big, "G", s, out, L.C128)
    assert rc == L.SOD_ERR_CAPACITY
    assert b"scratch" in L.load().sod_last_error()


def test_noalloc_rejects_row_blocks_beyond_shared_memory(sodlib):
    """H needs 72 bytes of shared memory per vertex for its row block; a 3300-vertex mesh fits the
    scratch but not shared memory, and the entry point says so (it has no global-memory variant)."""
    import torch

    from surfaceonlydeformables_gb300 import _lib as L
    from surfaceonlydeformables_gb300 import api
    from surfaceonlydeformables_gb300.meshes import SurfaceMesh

    g = np.load(__import__("os").path.join(__import__("os").path.dirname(__file__), "golden", "bunny_mesh.npz"))
    ctx = api.Context(0)
    bunny = api.Mesh(ctx, SurfaceMesh.from_arrays(g["V"], g["F"]))  # 3485 vertices
    s, R, Lq = L.cq_frequencies(1, 0.003, 1)
    out = torch.empty(1, dtype=torch.complex128, device="cuda")
    rc = _noalloc(L, ctx, bunny, "H", s[:1], out, L.C128)
    assert rc == L.SOD_ERR_CAPACITY
    assert b"shared memory" in L.load().sod_last_error()
