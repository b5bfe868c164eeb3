"""GPU time-domain precomputation (sod_cqbem_precompute) against the FP64 oracle pipeline:
inverse transform, free term on H_0, B_trans shift of B_angular, B_euler.

  * pipeline exactness: the oracle pipeline applied to the GPU's own Laplace-domain matrices
    agrees with the GPU to <= 1e-10 (relative Frobenius, stacked over n)
  * accuracy vs FP64: the inverse transform multiplies the late weights by up to R^-N = 1e5, so
    FP32 noise of the Laplace-domain entries (~1e-7) would become ~1e-3 of the stacked weights;
    the precompute's regular pass is compensated (double-float) by default, and every kind --
    G, H, B_trans, B_angular, B_euler -- must be within 1e-5 of the FP64 pipeline, stacked over n.
    With the regular pass forced to FP32 the same weights are no better than the reference's own
    mixed-precision pipeline (that test records the level the compensated pass removes).
"""
import numpy as np
import pytest

from surfaceonlydeformables_gb300.meshes import Material, make_icosphere_mesh

from .conftest import rel_fro

pytestmark = pytest.mark.gpu
MAT = Material(1e5, 0.3, 1000.0)
KINDS = ("G", "H", "B_trans", "B_angular")


def oracle_pipeline(oracle, mesh, X, L, R, cm, mat=MAT):
    nV = mesh.nV
    out = {k: oracle.inverse_transform(X[k], L, R) for k in KINDS}
    C = oracle.c_matrix_collocation(mesh, mat.nu).reshape(nV, 3, 3)
    for v in range(nV):
        out["H"][0, 3 * v:3 * v + 3, 3 * v:3 * v + 3] += C[v]
    Ba = out["B_angular"].reshape(L, 3 * nV, 3, 3)
    Ba = np.stack([oracle.b_angular_shift(Ba[n], out["B_trans"][n], mesh.V, np.asarray(cm)) for n in range(L)])
    out["B_angular"] = Ba
    out["B_euler"] = np.stack([oracle.b_euler(Ba[n]) for n in range(L)])
    return out


@pytest.fixture(scope="module")
def setup(gpu_ctx, sodlib):
    from surfaceonlydeformables_gb300 import api

    m = make_icosphere_mesh(2, 0.1)
    dm = api.Mesh(gpu_ctx, m)
    N, dt = 16, 0.01
    s, R, L = sodlib.cq_frequencies(2, dt, N)
    cm = (0.0, 0.0, 0.0)  # the mesh is centred at its volume centroid
    pre = api.precompute(gpu_ctx, dm, MAT, 2, dt, N, cm=cm)
    gpu_ctx.synchronize()
    got = {k: v.cpu().numpy() for k, v in pre.items()}
    return m, dm, s, R, L, cm, got


def test_precompute_pipeline_exact(gpu_ctx, oracle, sodlib, setup):
    from surfaceonlydeformables_gb300 import api

    from surfaceonlydeformables_gb300 import _lib as L_

    m, dm, s, R, L, cm, got = setup
    gpu_ctx.set_precision(L_.PRECISION_COMPENSATED)  # the precompute's own Laplace-domain pass
    try:
        X = api.assemble_all(gpu_ctx, dm, MAT, s)
    finally:
        gpu_ctx.set_precision(L_.PRECISION_AUTO)
    X = {k: (v.reshape(len(s), 3 * m.nV, 3, 3) if k == "B_angular" else v) for k, v in X.items()}
    ref = oracle_pipeline(oracle, m, X, L, R, cm)
    for k in ("G", "H", "B_trans", "B_angular", "B_euler"):
        assert rel_fro(got[k], ref[k]) <= 1e-10, (k, rel_fro(got[k], ref[k]))


@pytest.fixture(scope="module")
def fp64_and_mixed(oracle, setup):
    m, dm, s, R, L, cm, got = setup
    X64 = {k: np.stack([oracle.collocation(k, m, MAT, sl, mode=oracle.FP64) for sl in s]) for k in KINDS}
    Xmx = {k: np.stack([oracle.collocation(k, m, MAT, sl, mode=oracle.MIXED) for sl in s]) for k in KINDS}
    for X in (X64, Xmx):
        X["B_angular"] = X["B_angular"].reshape(len(s), 3 * m.nV, 3, 3)
    return oracle_pipeline(oracle, m, X64, L, R, cm), oracle_pipeline(oracle, m, Xmx, L, R, cm)


def test_precompute_accuracy_vs_fp64(setup, fp64_and_mixed):
    m, dm, s, R, L, cm, got = setup
    ref, mix = fp64_and_mixed
    for k in ("G", "H", "B_trans", "B_angular", "B_euler"):
        e = rel_fro(got[k], ref[k])
        print(f"{k}: GPU stacked err {e:.2e}, reference-mixed {rel_fro(mix[k], ref[k]):.2e}")
        assert e <= 1e-5, (k, e)
        assert rel_fro(got[k][0], ref[k][0]) <= 1e-5, k


def test_precompute_fp32_regular_pass_level(gpu_ctx, setup, fp64_and_mixed):
    """The same precompute with the regular pass forced to FP32: the late weights carry the amplified
    FP32 noise, at the level of the reference's own mixed-precision pipeline (G, B kinds)."""
    from surfaceonlydeformables_gb300 import _lib as L_
    from surfaceonlydeformables_gb300 import api

    m, dm, s, R, L, cm, got = setup
    ref, mix = fp64_and_mixed
    gpu_ctx.set_precision(L_.PRECISION_FP32)
    try:
        pre = api.precompute(gpu_ctx, dm, MAT, 2, 0.01, 16, cm=cm)
        gpu_ctx.synchronize()
        f32 = {k: v.cpu().numpy() for k, v in pre.items()}
    finally:
        gpu_ctx.set_precision(L_.PRECISION_AUTO)
    fp32_level = max(rel_fro(mix[k], ref[k]) for k in ("G", "B_trans", "B_angular"))
    for k in ("G", "B_trans", "B_angular"):
        e = rel_fro(f32[k], ref[k])
        print(f"{k}: FP32 regular pass stacked err {e:.2e}, compensated {rel_fro(got[k], ref[k]):.2e}")
        assert 1e-5 < e <= 3 * fp32_level, (k, e, fp32_level)


def test_precompute_galerkin_pipeline_exact(gpu_ctx, oracle, sodlib):
    """Galerkin path: H_0 gets the Galerkin mass matrix (src/elastodynamics_cqbem_H.cu:184-186,
    src/elastics_bem_matrix_collection.cpp:447-467); the pipeline on the GPU's own Galerkin
    Laplace-domain matrices agrees to <= 1e-10."""
    from surfaceonlydeformables_gb300 import _lib as L
    from surfaceonlydeformables_gb300 import api

    m = make_icosphere_mesh(1, 0.1)
    dm = api.Mesh(gpu_ctx, m)
    N, dt = 8, 0.01
    s, R, Lq = sodlib.cq_frequencies(2, dt, N)
    cm = (0.0, 0.0, 0.0)
    got = {k: v.cpu().numpy() for k, v in api.precompute(gpu_ctx, dm, MAT, 2, dt, N, order=4, sorder=4,
                                                         method=L.GALERKIN, cm=cm).items()}
    # the same all-kinds call the precompute makes (same fused passes, so the same FP32 sums)
    X = api.assemble_all(gpu_ctx, dm, MAT, s, order=4, sorder=4, method=L.GALERKIN)
    X["B_angular"] = X["B_angular"].reshape(len(s), 3 * m.nV, 3, 3)
    nV = m.nV
    ref = {k: oracle.inverse_transform(X[k], Lq, R) for k in KINDS}
    ref["H"][0] += oracle.c_matrix_galerkin(m)
    Ba = ref["B_angular"].reshape(Lq, 3 * nV, 3, 3)
    Ba = np.stack([oracle.b_angular_shift(Ba[n], ref["B_trans"][n], m.V, np.asarray(cm)) for n in range(Lq)])
    ref["B_angular"] = Ba
    ref["B_euler"] = np.stack([oracle.b_euler(Ba[n]) for n in range(Lq)])
    for k in ("G", "H", "B_trans", "B_angular", "B_euler"):
        assert rel_fro(got[k], ref[k]) <= 1e-10, (k, rel_fro(got[k], ref[k]))


def test_write_cache_matches_precompute(gpu_ctx, setup, tmp_path):
    """sod_cqbem_write_cache writes the reference's cache files (G_k, H_k, B_k = [B_trans | B_euler],
    src/elastodynamics_cqbem_matrix_collection.cpp:76-176) from device-resident precompute outputs."""
    from surfaceonlydeformables_gb300 import api

    m, dm, s, R, L, cm, got = setup
    import torch

    w = {k: torch.from_numpy(got[k]).cuda() for k in ("G", "H", "B_trans", "B_euler")}
    api.write_cache(gpu_ctx, str(tmp_path), m.nV, w)
    n3 = 3 * m.nV
    for k in (0, L // 2, L - 1):
        for name in ("G", "H"):
            raw = open(tmp_path / f"{name}_{k}.mat", "rb").read()
            assert np.frombuffer(raw[:16], dtype=np.int64).tolist() == [n3, n3]
            assert np.array_equal(np.frombuffer(raw[16:], dtype=np.float64).reshape(n3, n3), got[name][k])
        B = api.mat_read(gpu_ctx, str(tmp_path / f"B_{k}.mat"), n3, 6)
        assert np.array_equal(B[:, :3], got["B_trans"][k]) and np.array_equal(B[:, 3:], got["B_euler"][k])
