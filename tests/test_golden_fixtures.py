"""The real-mesh fixtures of tests/golden (the reference's cube scene meshes and FP64 oracle rows on
them, written by tests/golden/make_fixtures.py): the meshes are closed 2-manifolds, the split
vertices of the discontinuous cube sit on their canonical vertices, and the oracle still reproduces
the stored rows (relative Frobenius <= 1e-12 for the FP64 singular rows, <= 1e-6 for the full rows
stored as complex64)."""
import os

import numpy as np
import pytest

from surfaceonlydeformables_gb300.meshes import SurfaceMesh

from .conftest import rel_fro

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.fixture(scope="module")
def fixtures():
    return np.load(os.path.join(GOLDEN, "cube_meshes.npz")), np.load(os.path.join(GOLDEN, "cube_oracle_rows.npz"))


def test_cube_meshes_are_closed(fixtures):
    m, _ = fixtures
    for tag in ("cont", "disc"):
        F = m[f"F_{tag}"]
        canon = m["vmap_disc"][F] if tag == "disc" else F
        e = np.sort(np.concatenate([canon[:, [0, 1]], canon[:, [1, 2]], canon[:, [2, 0]]]), axis=1)
        _, counts = np.unique(e, axis=0, return_counts=True)
        assert np.all(counts == 2), tag  # every edge between exactly two faces (over canonical vertices)
    V, F = m["V_cont"], m["F_cont"]
    assert len(V) - len(np.unique(np.sort(np.concatenate([F[:, [0, 1]], F[:, [1, 2]], F[:, [2, 0]]]), axis=1),
                                  axis=0)) + len(F) == 2  # Euler characteristic of a sphere
    vm = m["vmap_disc"]
    assert np.array_equal(m["V_disc"][vm], m["V_disc"]) and len(np.unique(vm)) == len(V)


def test_oracle_reproduces_cube_rows(fixtures, oracle):
    import importlib.util

    spec = importlib.util.spec_from_file_location("make_fixtures", os.path.join(GOLDEN, "make_fixtures.py"))
    mf = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mf)
    m, r = fixtures
    mat = mf.material()
    for tag in ("cont", "disc"):
        mesh = SurfaceMesh.from_arrays(m[f"V_{tag}"], m[f"F_{tag}"])
        vmap = m["vmap_disc"] if tag == "disc" else None
        verts = r[f"verts_{tag}"]
        for kind in ("G", "H"):
            got = oracle.collocation(kind, mesh, mat, r["s"][0], order=mf.ORDER, subdiv=mf.SUBDIV, rows=verts,
                                     parts=2, vmap=vmap)
            assert rel_fro(got, r[f"{tag}_{kind}_sing"][0]) <= 1e-12, (tag, kind)
        got = oracle.collocation("B_trans", mesh, mat, r["s"][-1], order=mf.ORDER, subdiv=mf.SUBDIV, rows=verts,
                                 vmap=vmap)
        assert rel_fro(got, r[f"{tag}_B_trans_all"]) <= 1e-12, tag
