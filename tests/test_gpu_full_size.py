"""GPU parity at the benchmarked sizes, against the FP64 oracle.

The row-sampled oracle integrates every face for the listed field vertices only, so the sampled
rows are the exact FP64 rows (not an approximation); a relative Frobenius error over those rows is
reported per kind.

  * the 2562-vertex shared-memory scatter (G with B_trans / B_angular fused, and H) at three Laplace
    frequencies of the N = 32, dt = 1/200 BDF2 set of the mixed-size workload: <= 1e-5 on sampled rows;
  * a batch that holds a 2562-vertex object next to 642- and 162-vertex objects (ellipsoids, mixed
    materials, N 32 / 16): <= 1e-5 on sampled rows of every object and kind;
  * the 642-vertex single-object case (E 1e5, nu 0.3, dt 0.01, BDF2, N = 32, all 17 frequencies,
    7-point rule): every Laplace-domain matrix of every kind <= 1e-5 against the full FP64 oracle;
  * the Galerkin case (2562 vertices jittered by 0.2 x the mean edge, nu 0.45, dt 1/200, N = 64,
    13-point regular rule, Sauter-Schwab order 5): three of the 33 frequencies, G and H <= 1e-5 on
    sampled rows.
"""
import numpy as np
import pytest

from surfaceonlydeformables_gb300.meshes import Material, make_icosphere_mesh

from .conftest import rel_fro

pytestmark = pytest.mark.gpu
KINDS = ("G", "H", "B_trans", "B_angular")
TOL = 1e-5


def sample_rows(nV, k, seed):
    rng = np.random.default_rng(seed)
    return np.sort(rng.choice(nV, size=k, replace=False)).astype(np.int32)


def row_index(kind, rows):
    return np.concatenate([np.arange(3 * v, 3 * v + 3) for v in rows])


def test_scatter_2562_vertices_rows_vs_oracle(gpu_ctx, oracle):
    from surfaceonlydeformables_gb300 import _lib as L
    from surfaceonlydeformables_gb300 import api

    m = make_icosphere_mesh(4, 0.1)
    mat = Material(1e5, 0.3, 1000.0)
    dm = api.Mesh(gpu_ctx, m)
    s, R, Lq = L.cq_frequencies(2, 1 / 200, 32)
    sel = s[[1, 8, 16]]
    got = api.assemble_all(gpu_ctx, dm, mat, sel, dtype=L.C64,
                           outs=api.alloc_outputs(dm, len(sel), KINDS, L.C64))
    gpu_ctx.synchronize()  # device outputs: the call returns before its kernels finish
    rows = sample_rows(m.nV, 6, 11)
    idx = row_index("G", rows)
    for kind in KINDS:
        g = got[kind].cpu().numpy()
        for l, sl in enumerate(sel):
            ref = oracle.collocation(kind, m, mat, sl, rows=rows)
            e = rel_fro(g[l][idx], ref)
            assert e <= TOL, (kind, l, e)


def test_batch_with_a_2562_vertex_object_vs_oracle(gpu_ctx, oracle):
    from surfaceonlydeformables_gb300 import _lib as L
    from surfaceonlydeformables_gb300 import api

    specs = [(4, (1.4, 0.8, 1.1), Material(2.2e5, 0.31, 1000.0), 32),
             (3, (0.7, 1.5, 1.0), Material(3e4, 0.42, 1000.0), 16),
             (2, (1.2, 1.0, 0.6), Material(6e5, 0.24, 1000.0), 32)]
    b = api.Batch(gpu_ctx, KINDS, L.C64)
    objs = []
    for k, (lev, axes, mat, N) in enumerate(specs):
        m = make_icosphere_mesh(lev, 0.1, axes=axes, seed=40 + k)
        dm = api.Mesh(gpu_ctx, m)
        s, R, Lq = L.cq_frequencies(2, 1 / 200, N)
        out = api.alloc_outputs(dm, len(s), KINDS, L.C64)
        b.add(dm, mat, s, out)
        objs.append((m, dm, mat, s, out))
    b.finalize()
    b.run()
    gpu_ctx.synchronize()
    for j, (m, dm, mat, s, out) in enumerate(objs):
        rows = sample_rows(m.nV, 4, 50 + j)
        idx = row_index("G", rows)
        for kind in KINDS:
            g = out[kind].cpu().numpy()
            for l in (0, len(s) // 2, len(s) - 1):
                ref = oracle.collocation(kind, m, mat, s[l], rows=rows)
                e = rel_fro(g[l][idx], ref)
                assert e <= TOL, (j, kind, l, e)


@pytest.fixture(scope="module")
def case642(gpu_ctx, oracle):
    """642 vertices, N = 32 (17 Laplace frequencies), the full FP64 oracle of every kind."""
    from surfaceonlydeformables_gb300 import _lib as L
    from surfaceonlydeformables_gb300 import api

    m = make_icosphere_mesh(3, 0.1)
    mat = Material(1e5, 0.3, 1000.0)
    dm = api.Mesh(gpu_ctx, m)
    s, R, Lq = L.cq_frequencies(2, 0.01, 32)
    ref = {k: np.stack([oracle.collocation(k, m, mat, sl) for sl in s]) for k in KINDS}
    return m, dm, mat, s, R, Lq, ref


def test_single_object_642_all_frequencies(gpu_ctx, case642):
    from surfaceonlydeformables_gb300 import _lib as L
    from surfaceonlydeformables_gb300 import api

    m, dm, mat, s, R, Lq, ref = case642
    assert len(s) == 17
    got = api.assemble_all(gpu_ctx, dm, mat, s, dtype=L.C128)
    for kind in KINDS:
        for l in range(len(s)):
            e = rel_fro(got[kind][l], ref[kind][l])
            assert e <= TOL, (kind, l, e)
        print(f"{kind}: worst frequency {max(rel_fro(got[kind][l], ref[kind][l]) for l in range(len(s))):.2e}")


@pytest.mark.parametrize("kind", ["G", "H"])
def test_galerkin_2562_jittered_rows_vs_oracle(gpu_ctx, oracle, kind):
    from surfaceonlydeformables_gb300 import _lib as L
    from surfaceonlydeformables_gb300 import api

    m = make_icosphere_mesh(4, 0.1, jitter=0.2, seed=2)
    mat = Material(1e5, 0.45, 1000.0)
    dm = api.Mesh(gpu_ctx, m)
    s, R, Lq = L.cq_frequencies(2, 1 / 200, 64)
    assert len(s) == 33
    sel = s[[1, 16, 32]]
    n = 3 * m.nV
    import torch

    out = torch.empty((len(sel), n, n), dtype=torch.complex64, device="cuda")
    api.assemble_frequencies(gpu_ctx, dm, kind, mat, sel, order=7, sorder=5, ssub=1, method=L.GALERKIN, out=out,
                             dtype=L.C64)
    gpu_ctx.synchronize()
    rows = sample_rows(m.nV, 3, 7)
    idx = row_index(kind, rows)
    g = out.cpu().numpy()
    for l, sl in enumerate(sel):
        ref = oracle.galerkin(kind, m, mat, sl, order=7, sorder=5, ssub=1, rows=rows)
        e = rel_fro(g[l][idx], ref)
        assert e <= TOL, (kind, l, e)


def test_single_object_642_time_domain(gpu_ctx, oracle, case642):
    """The 642-vertex case's time-domain weights (L = 33 of each kind, H_0 with the free term, B_angular
    with the B_trans shift, B_euler) through sod_cqbem_precompute (compensated regular pass) against the
    oracle pipeline on the FP64 Laplace-domain matrices: <= 1e-5 stacked over n for every kind."""
    from surfaceonlydeformables_gb300 import api

    from .test_gpu_precompute import oracle_pipeline

    m, dm, mat, s, R, Lq, ref = case642
    X = dict(ref)
    X["B_angular"] = X["B_angular"].reshape(len(s), 3 * m.nV, 3, 3)
    want = oracle_pipeline(oracle, m, X, Lq, R, (0.0, 0.0, 0.0), mat=mat)
    pre = api.precompute(gpu_ctx, dm, mat, 2, 0.01, 32)
    gpu_ctx.synchronize()
    got = {k: v.cpu().numpy() for k, v in pre.items()}
    for k in ("G", "H", "B_trans", "B_angular", "B_euler"):
        e = rel_fro(got[k], want[k])
        per_n = [rel_fro(got[k][n], want[k][n]) for n in (0, Lq // 2, Lq - 1)]
        print(f"{k}: stacked {e:.2e}, n = 0 / {Lq // 2} / {Lq - 1}: " + " / ".join(f"{v:.1e}" for v in per_n))
        assert e <= TOL, (k, e)
