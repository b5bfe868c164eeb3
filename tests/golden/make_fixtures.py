"""Builds the real-mesh fixtures of tests/golden from the reference's scene meshes.

Reads data/cube_reordered.obj and data/cube_reordered_discontinuous.obj of a reference checkout
(its directory is the required first argument) and writes:
  cube_meshes.npz      V, F of both meshes, centred at the volume centroid as the reference's
                       PhysicsBaseMatrixCollection::init does (src/physics_base_matrix_collection.cpp:
                       41-45); vmap of the discontinuous mesh: each split vertex maps to the first
                       vertex with the same coordinates (the reference's vertex_map_inverse)
  bunny_mesh.npz       V, F of data/bunny_reordered.obj (3485 vertices, the bunny scene of
                       data/bunny_friction.json), centred; its H row block (9 x 3485 complex FP32)
                       is larger than shared memory, so it exercises the global-memory accumulator
  cube_oracle_rows.npz FP64 oracle rows (G, H, B_trans, B_angular) of a few vertices, with the scene's
                       material and quadrature: the singular part at two CQ frequencies (FP64,
                       for the 1e-10 check) and the full rows at the second one (G and H stored
                       as complex64, enough for the 1e-5 check)
                       (data/cube_drop.json: mu 1e5, nu 0.45, rho 1000, BDF1, dt 0.005, order 5,
                       subdivision 2)
Run from the repository root: python tests/golden/make_fixtures.py <reference_checkout_dir>
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", ".."))

from oracle import oracle  # noqa: E402
from surfaceonlydeformables_gb300 import meshes  # noqa: E402

MU, NU, RHO = 100000.0, 0.44999998807907104, 1000.0
BDF, DT, NSTEPS = 1, 0.004999999888241291, 16
ORDER, SUBDIV = 5, 2
FREQ_INDEX = [0, 4]
KINDS = ["G", "H", "B_trans", "B_angular"]


def read_obj(path):
    V, F = [], []
    with open(path) as f:
        for line in f:
            t = line.split()
            if not t:
                continue
            if t[0] == "v":
                V.append([float(x) for x in t[1:4]])
            elif t[0] == "f":
                F.append([int(x.split("/")[0]) - 1 for x in t[1:4]])
    return np.array(V, dtype=np.float64), np.array(F, dtype=np.int32)


def material():
    return meshes.Material(2.0 * MU * (1.0 + NU), NU, RHO)


def sample_vertices(V, vmap=None):
    """A corner, an edge and a face-interior vertex of the cube (and, with vmap, a split vertex)."""
    a = np.abs(V)
    m = a.max()
    on = (np.abs(a - m) < 1e-9 * m).sum(axis=1)  # coordinates on the cube's boundary planes
    picks = [int(np.flatnonzero(on == 3)[0]), int(np.flatnonzero(on == 2)[0]), int(np.flatnonzero(on == 1)[0])]
    if vmap is not None:
        split = np.flatnonzero(vmap != np.arange(len(vmap)))
        picks += [int(split[0]), int(vmap[split[0]])]
    return np.array(sorted(set(picks)), dtype=np.int32)


def main():
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_fixtures.py <reference_checkout_dir>")
    ref = sys.argv[1]
    out = {}
    for tag, name in (("cont", "cube_reordered.obj"), ("disc", "cube_reordered_discontinuous.obj")):
        V, F = read_obj(os.path.join(ref, "data", name))
        V = meshes.center_mesh(V, F)
        out[f"V_{tag}"], out[f"F_{tag}"] = V, F
    V = out["V_disc"]
    _, first = np.unique(V, axis=0, return_index=True)
    key = {tuple(V[i]): i for i in sorted(first)}
    out["vmap_disc"] = np.array([key[tuple(v)] for v in V], dtype=np.int32)
    np.savez_compressed(os.path.join(HERE, "cube_meshes.npz"), **out)
    V, F = read_obj(os.path.join(ref, "data", "bunny_reordered.obj"))
    np.savez_compressed(os.path.join(HERE, "bunny_mesh.npz"), V=meshes.center_mesh(V, F), F=F)

    s, R, L = oracle.cq_frequencies(BDF, DT, NSTEPS)
    s = np.asarray(s)[FREQ_INDEX]
    mat = material()
    rows = {"s": s}
    for tag in ("cont", "disc"):
        m = meshes.SurfaceMesh.from_arrays(out[f"V_{tag}"], out[f"F_{tag}"])
        vmap = out["vmap_disc"] if tag == "disc" else None
        verts = sample_vertices(m.V, vmap)
        rows[f"verts_{tag}"] = verts
        for kind in KINDS:
            rows[f"{tag}_{kind}_sing"] = np.stack([
                oracle.collocation(kind, m, mat, sl, order=ORDER, subdiv=SUBDIV, rows=verts, parts=2, vmap=vmap)
                for sl in s])
            full = oracle.collocation(kind, m, mat, s[-1], order=ORDER, subdiv=SUBDIV, rows=verts, vmap=vmap)
            rows[f"{tag}_{kind}_all"] = full.astype(np.complex64) if kind in ("G", "H") else full
    np.savez_compressed(os.path.join(HERE, "cube_oracle_rows.npz"), **rows)


if __name__ == "__main__":
    main()
