"""Surface-mesh input preparation for the CQBEM precomputation.

Restates the subset of the reference's mesh set-up that the assembly depends on
(src/physics_base_matrix_collection.cpp:32-57): vertices are centred at the volume centroid of
the closed surface (igl::centroid at :41-45) and per-face unit normals are taken as
normalize((v1 - v0) x (v2 - v0)) (igl::per_face_normals, src/elastodynamics_cqbem_matrix_collection.cpp:73-74).

It also synthesises the seeded test meshes used by the benchmarks: subdivided icosahedra
("icospheres": 162 / 642 / 2562 vertices at levels 2 / 3 / 4), optionally jittered tangentially
and scaled to ellipsoids.  The reference reads OBJ files instead; mesh tooling (subdivision schemes,
decimation, OpenCCL reordering) is outside the accelerated path.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np


@dataclass
class Material:
    """Isotropic elastic material given by Young's modulus E, Poisson ratio nu and density rho.

    The reference configures materials by (mu, nu, rho) (src/elastics_bem_matrix_collection.cpp:19-20);
    mu = E / (2 (1 + nu)).  Wave speeds follow src/elastodynamics_cqbem_matrix_collection.cpp:59-61.
    """

    E: float
    nu: float
    rho: float

    @property
    def mu(self) -> float:
        return self.E / (2.0 * (1.0 + self.nu))

    @property
    def lam(self) -> float:
        return 2.0 * self.nu * self.mu / (1.0 - 2.0 * self.nu)

    @property
    def c1(self) -> float:
        return float(np.sqrt((self.lam + 2.0 * self.mu) / self.rho))

    @property
    def c2(self) -> float:
        return float(np.sqrt(self.mu / self.rho))


def icosphere(level: int, radius: float = 1.0) -> tuple[np.ndarray, np.ndarray]:
    """Subdivided icosahedron projected on a sphere; outward-oriented (counter-clockwise) faces.

    Returns V (nV x 3 float64) and F (nF x 3 int32) with nV = 10 * 4**level + 2.
    """
    t = (1.0 + 5.0 ** 0.5) / 2.0
    V = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t), (0, -1, -t), (0, 1, -t),
         (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    V = [np.array(v, dtype=np.float64) / np.linalg.norm(v) for v in V]
    F = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4), (11, 10, 2),
         (10, 7, 6), (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9), (4, 9, 5),
         (2, 4, 11), (6, 2, 10), (8, 6, 7), (9, 8, 1)]
    for _ in range(level):
        mid: dict[tuple[int, int], int] = {}

        def midpoint(a: int, b: int) -> int:
            key = (a, b) if a < b else (b, a)
            if key not in mid:
                m = V[a] + V[b]
                V.append(m / np.linalg.norm(m))
                mid[key] = len(V) - 1
            return mid[key]

        nf = []
        for a, b, c in F:
            ab, bc, ca = midpoint(a, b), midpoint(b, c), midpoint(c, a)
            nf += [(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)]
        F = nf
    return np.asarray(V) * radius, np.asarray(F, dtype=np.int32)


def face_normals(V: np.ndarray, F: np.ndarray) -> np.ndarray:
    """Unit face normals normalize((v1-v0) x (v2-v0)); zero for degenerate faces."""
    n = np.cross(V[F[:, 1]] - V[F[:, 0]], V[F[:, 2]] - V[F[:, 0]])
    ln = np.linalg.norm(n, axis=1, keepdims=True)
    return np.where(ln > 0, n / np.where(ln > 0, ln, 1.0), 0.0)


def double_areas(V: np.ndarray, F: np.ndarray) -> np.ndarray:
    return np.linalg.norm(np.cross(V[F[:, 1]] - V[F[:, 0]], V[F[:, 2]] - V[F[:, 0]]), axis=1)


def volume_centroid(V: np.ndarray, F: np.ndarray) -> tuple[np.ndarray, float]:
    """Centroid and volume of the solid bounded by a closed oriented surface.

    Sum over the tetrahedra (origin, a, b, c): volume a.(b x c)/6 with centroid (a+b+c)/4.
    """
    a, b, c = V[F[:, 0]], V[F[:, 1]], V[F[:, 2]]
    vol = np.einsum("ij,ij->i", a, np.cross(b, c)) / 6.0
    tot = vol.sum()
    cm = (vol[:, None] * (a + b + c)).sum(axis=0) / (4.0 * tot)
    return cm, float(tot)


def center_mesh(V: np.ndarray, F: np.ndarray) -> np.ndarray:
    """Translate V so that the volume centroid sits at the origin (physics_base_matrix_collection.cpp:41-45)."""
    cm, _ = volume_centroid(V, F)
    return V - cm


def mean_edge_length(V: np.ndarray, F: np.ndarray) -> float:
    e = np.concatenate([V[F[:, 1]] - V[F[:, 0]], V[F[:, 2]] - V[F[:, 1]], V[F[:, 0]] - V[F[:, 2]]])
    return float(np.linalg.norm(e, axis=1).mean())


def jitter_tangential(V: np.ndarray, F: np.ndarray, sigma_rel: float, seed: int) -> np.ndarray:
    """Seeded Gaussian jitter in each vertex's tangent plane (sphere about the origin), sigma =
    sigma_rel x mean edge length, then projected back to the vertex's original radius."""
    rng = np.random.default_rng(seed)
    sigma = sigma_rel * mean_edge_length(V, F)
    d = rng.normal(0.0, sigma, size=V.shape)
    rad = np.linalg.norm(V, axis=1, keepdims=True)
    nrm = V / rad
    d -= np.einsum("ij,ij->i", d, nrm)[:, None] * nrm
    W = V + d
    return W / np.linalg.norm(W, axis=1, keepdims=True) * rad


@dataclass
class SurfaceMesh:
    """A centred closed triangle mesh with its face normals, ready for assembly."""

    V: np.ndarray  # nV x 3 float64, centred at the volume centroid
    F: np.ndarray  # nF x 3 int32
    N: np.ndarray  # nF x 3 float64 unit normals

    @property
    def nV(self) -> int:
        return int(self.V.shape[0])

    @property
    def nF(self) -> int:
        return int(self.F.shape[0])

    @classmethod
    def from_arrays(cls, V, F) -> "SurfaceMesh":
        V = np.ascontiguousarray(V, dtype=np.float64)
        F = np.ascontiguousarray(F, dtype=np.int32)
        V = np.ascontiguousarray(center_mesh(V, F))
        return cls(V, F, np.ascontiguousarray(face_normals(V, F)))


def make_icosphere_mesh(level: int, radius: float = 0.1, jitter: float = 0.0, axes=(1.0, 1.0, 1.0),
                        seed: int = 0) -> SurfaceMesh:
    """Seeded synthetic mesh: icosphere of `level`, optional tangential jitter, ellipsoid axes scaling."""
    V, F = icosphere(level, 1.0)
    if jitter > 0:
        V = jitter_tangential(V, F, jitter, seed)
    V = V * np.asarray(axes, dtype=np.float64)[None, :] * radius
    return SurfaceMesh.from_arrays(V, F)
