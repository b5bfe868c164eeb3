"""Request loop (sod_server): assembly and step requests of several objects in flight at once.
Each step result equals, bit for bit, the same object's requests served alone, and matches the plain
drop-in (CQ precompute + history sum in FP64 on the host) to <= 1e-5 relative."""
import numpy as np
import pytest

from surfaceonlydeformables_gb300.meshes import Material, make_icosphere_mesh

from .conftest import rel_fro

pytestmark = pytest.mark.gpu

OBJS = [(2, Material(1e5, 0.3, 1000.0), 16, (1.0, 1.0, 1.0)),
        (1, Material(3e4, 0.42, 1000.0), 8, (1.6, 0.7, 1.1)),
        (2, Material(5e5, 0.25, 1000.0), 8, (0.6, 1.3, 0.9))]


def serve(objs, steps_per_obj, seed=0, cap=8 << 30, slots=2):
    from surfaceonlydeformables_gb300 import api

    srv = api.Server(0, cap, slots, 700)
    rng = np.random.default_rng(seed)
    ids, step_ids = [], {}
    meshes = [make_icosphere_mesh(lev, 0.1, axes=ax, seed=k) for k, (lev, _, _, ax) in enumerate(objs)]
    for m, (lev, mat, N, ax) in zip(meshes, objs):
        ids.append(srv.submit_assembly(m, mat, 2, 1 / 200, N))
    hist = {k: [] for k in range(len(objs))}
    for t in range(steps_per_obj):
        for k, m in enumerate(meshes):
            p = rng.normal(size=3 * m.nV) * 10.0
            u = rng.normal(size=3 * m.nV) * 1e-4
            hist[k].append((p, u))
            step_ids.setdefault(k, []).append(srv.submit_step(ids[k], p, u))
    srv.drain(300)
    done = {i: (st, lat) for i, st, lat in srv.poll(100000)}
    results = {k: [srv.result(r) for r in step_ids[k]] for k in step_ids}
    return srv, meshes, ids, hist, results, done


def test_served_results_alone_vs_mix(gpu_ctx):
    from surfaceonlydeformables_gb300 import api

    srv, meshes, ids, hist, mix, done = serve(OBJS, 5)
    assert all(st == 0 for st, _ in done.values())
    assert all(lat > 0 for _, lat in done.values())
    srv.close()
    for k, (lev, mat, N, ax) in enumerate(OBJS):
        alone = api.Server(0, 8 << 30, 1, 700)
        oid = alone.submit_assembly(meshes[k], mat, 2, 1 / 200, N)
        rids = [alone.submit_step(oid, p, u) for p, u in hist[k]]
        alone.drain(300)
        got = [alone.result(r) for r in rids]
        alone.close()
        for a, b in zip(mix[k], got):
            assert np.array_equal(a.view(np.uint8), b.view(np.uint8))


def test_served_matches_plain_path(gpu_ctx, sodlib):
    from surfaceonlydeformables_gb300 import _lib as L
    from surfaceonlydeformables_gb300 import api

    srv, meshes, ids, hist, res, done = serve(OBJS[:2], 4, seed=3)
    srv.close()
    for k, m in enumerate(meshes):
        lev, mat, N, ax = OBJS[k]
        pre = api.precompute(gpu_ctx, api.Mesh(gpu_ctx, m), mat, 2, 1 / 200, N, kinds=("G", "H"))
        G = pre["G"].cpu().numpy()
        H = pre["H"].cpu().numpy()
        for t in range(len(hist[k])):
            b = np.zeros(3 * m.nV)
            for i in range(min(t + 1, N)):
                p, u = hist[k][t - i]
                b += G[i + 1] @ p - H[i + 1] @ u
            assert rel_fro(res[k][t], b) <= 1e-5


def test_server_capacity_and_eviction(gpu_ctx):
    from surfaceonlydeformables_gb300 import _lib as L
    from surfaceonlydeformables_gb300 import api

    m = make_icosphere_mesh(2, 0.1, seed=1)
    mat = Material(1e5, 0.3, 1000.0)
    tiny = api.Server(0, 1 << 20, 1, 700)
    rid = tiny.submit_assembly(m, mat, 2, 1 / 200, 8)
    tiny.drain(60)
    (i, st, _), = tiny.poll()
    assert i == rid and st == L.SOD_ERR_CAPACITY
    tiny.close()
    # room for one 162-vertex object with N = 8 (bank + assembly buffers) but not two
    n = 3 * m.nV
    bank = 4 * 8 * 2 * n * ((n + 7) // 8 * 8) + 4 * 8 * 2 * ((n + 7) // 8 * 8)
    one = bank + 4 * 2 * 9 * n * n  # bank + the assembly's time-domain buffers
    srv = api.Server(0, int(one + 0.5 * bank), 1, 700)
    a = srv.submit_assembly(m, mat, 2, 1 / 200, 8)
    srv.drain(60)
    b = srv.submit_assembly(m, mat, 2, 1 / 200, 8)
    srv.drain(60)
    s = srv.submit_step(a, np.ones(n), np.zeros(n))  # a was evicted to admit b
    srv.drain(60)
    st = {i: code for i, code, _ in srv.poll()}
    assert st[a] == 0 and st[b] == 0 and st[s] == L.SOD_ERR_INVALID_ARG
    # a step whose vectors are not the object's 3V long is rejected on the host; the object still steps
    bad = srv.submit_step(b, np.ones(n - 3), np.zeros(n - 3))
    good = srv.submit_step(b, np.ones(n), np.zeros(n))
    srv.drain(60)
    st = {i: code for i, code, _ in srv.poll()}
    assert st[bad] == L.SOD_ERR_INVALID_ARG and st[good] == 0
    assert srv.result(good).shape == (n,)
    srv.close()
