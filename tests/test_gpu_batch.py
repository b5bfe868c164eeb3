"""Batched persistent assembly under a CUDA graph (sod_batch): every object matches its per-object
assembly and the FP64 oracle, an object's result is bitwise the same alone and in the mix, and
replays are bitwise reproducible."""
import numpy as np
import pytest

from surfaceonlydeformables_gb300.meshes import Material, make_icosphere_mesh

from .conftest import rel_fro

pytestmark = pytest.mark.gpu
KINDS = ("G", "H", "B_trans", "B_angular")


@pytest.fixture(scope="module")
def objects(gpu_ctx, sodlib):
    from surfaceonlydeformables_gb300 import api

    specs = [(3, (1.0, 1.0, 1.0), Material(1e5, 0.3, 1000.0), 16),
             (2, (1.6, 0.7, 1.1), Material(3e4, 0.42, 1000.0), 8),
             (2, (0.6, 1.3, 0.9), Material(5e5, 0.25, 1000.0), 16)]
    objs = []
    for k, (lev, axes, mat, N) in enumerate(specs):
        m = make_icosphere_mesh(lev, 0.1, axes=axes, seed=k)
        s, R, L = sodlib.cq_frequencies(2, 1 / 200, N)
        objs.append(dict(host=m, dev=api.Mesh(gpu_ctx, m), mat=mat, s=s))
    return objs


def run_batch(ctx, objs):
    from surfaceonlydeformables_gb300 import _lib as L
    from surfaceonlydeformables_gb300 import api

    b = api.Batch(ctx, KINDS, L.C64)
    outs = []
    for o in objs:
        out = api.alloc_outputs(o["dev"], len(o["s"]), KINDS, L.C64)
        b.add(o["dev"], o["mat"], o["s"], out)
        outs.append(out)
    b.finalize()
    b.run()
    ctx.synchronize()
    return b, [{k: v.cpu().numpy() for k, v in out.items()} for out in outs]


def test_batch_matches_per_object_and_oracle(gpu_ctx, objects, oracle):
    from surfaceonlydeformables_gb300 import _lib as L
    from surfaceonlydeformables_gb300 import api

    b, res = run_batch(gpu_ctx, objects)
    assert b.launches_per_step >= 5
    for o, r in zip(objects, res):
        single = api.assemble_all(gpu_ctx, o["dev"], o["mat"], o["s"], dtype=L.C64)
        for k in KINDS:
            assert rel_fro(r[k], single[k]) <= 1e-6, k
        l = len(o["s"]) // 2
        for k in KINDS:
            ref = oracle.collocation(k, o["host"], o["mat"], o["s"][l])
            assert rel_fro(r[k][l], ref) <= 1e-5, k


def test_same_result_alone_and_in_the_mix(gpu_ctx, objects):
    _, mix = run_batch(gpu_ctx, objects)
    for j in range(len(objects)):
        _, alone = run_batch(gpu_ctx, [objects[j]])
        for k in KINDS:
            assert np.array_equal(alone[0][k].view(np.uint8), mix[j][k].view(np.uint8)), (j, k)


def test_batch_replay_reproducible(gpu_ctx, objects):
    from surfaceonlydeformables_gb300 import _lib as L
    from surfaceonlydeformables_gb300 import api

    b = api.Batch(gpu_ctx, KINDS, L.C64)
    outs = []
    for o in objects:
        out = api.alloc_outputs(o["dev"], len(o["s"]), KINDS, L.C64)
        b.add(o["dev"], o["mat"], o["s"], out)
        outs.append(out)
    b.finalize()
    b.run()
    gpu_ctx.synchronize()
    first = [{k: v.clone() for k, v in out.items()} for out in outs]
    for out in outs:
        for v in out.values():
            v.zero_()
    b.run()
    gpu_ctx.synchronize()
    for a, c in zip(first, outs):
        for k in KINDS:
            assert bool((a[k] == c[k]).all()), k


def test_batch_profile_reports_every_launch(gpu_ctx, objects):
    from surfaceonlydeformables_gb300 import _lib as L
    from surfaceonlydeformables_gb300 import api

    b = api.Batch(gpu_ctx, KINDS, L.C64)
    for o in objects:
        b.add(o["dev"], o["mat"], o["s"], api.alloc_outputs(o["dev"], len(o["s"]), KINDS, L.C64))
    b.finalize()
    prof = b.profile()
    assert len(prof) == b.launches_per_step
    passes = {p["pass"] for p in prof}
    # with G in the batch the B kinds ride along in the G scatter: no separate reduction launch
    assert {"singular_polar", "singular_guiggiani", "combine_GB", "combine_H", "scatter_G", "scatter_H"} == passes
    assert all(p["ms"] > 0 and p["evals"] > 0 for p in prof)
    # regular evaluations of the G scatter: nfreq * (nV nF - 3 nF) * 7 points, summed over objects
    want = sum(len(o["s"]) * (o["host"].nV * o["host"].nF - 3 * o["host"].nF) * 7 for o in objects)
    assert sum(p["evals"] for p in prof if p["pass"] == "scatter_G") == want


@pytest.mark.parametrize("kinds", [("B_trans", "B_angular"), ("H", "B_angular"), ("G", "B_trans")])
def test_batch_kind_subsets(gpu_ctx, objects, oracle, kinds):
    """Batches of a subset of the kinds (B without G runs the separate reduction pass)."""
    from surfaceonlydeformables_gb300 import _lib as L
    from surfaceonlydeformables_gb300 import api

    b = api.Batch(gpu_ctx, kinds, L.C64)
    outs = []
    for o in objects[1:]:
        out = api.alloc_outputs(o["dev"], len(o["s"]), kinds, L.C64)
        b.add(o["dev"], o["mat"], o["s"], out)
        outs.append(out)
    b.run()
    gpu_ctx.synchronize()
    if "G" not in kinds:
        assert "reduce_B" in {p["pass"] for p in b.profile()} or not set(kinds) & {"B_trans", "B_angular"}
    for o, out in zip(objects[1:], outs):
        single = api.assemble_all(gpu_ctx, o["dev"], o["mat"], o["s"], dtype=L.C64)
        l = len(o["s"]) - 1
        for k in kinds:
            r = out[k].cpu().numpy()
            assert rel_fro(r, single[k]) <= 1e-6, k
            assert rel_fro(r[l], oracle.collocation(k, o["host"], o["mat"], o["s"][l])) <= 1e-5, k


def test_batch_with_row_block_beyond_shared_memory(gpu_ctx, sodlib, oracle):
    """The reference's 3485-vertex bunny in a batch with a small sphere: its H row block exceeds
    shared memory, so the batch gives it a launch with the accumulators in global memory.  Results
    match the per-object path and sampled FP64 oracle rows."""
    import os

    from surfaceonlydeformables_gb300 import _lib as L
    from surfaceonlydeformables_gb300 import api
    from surfaceonlydeformables_gb300.meshes import SurfaceMesh

    b = np.load(os.path.join(os.path.dirname(__file__), "golden", "bunny_mesh.npz"))
    bunny = SurfaceMesh.from_arrays(b["V"], b["F"])
    s, R, Lq = sodlib.cq_frequencies(1, 0.003, 5)
    mat = Material(2.0 * 1e6 * 1.3, 0.3, 3000.0)
    small = make_icosphere_mesh(2, 0.1)
    objs = [dict(host=bunny, dev=api.Mesh(gpu_ctx, bunny), mat=mat, s=s[:2]),
            dict(host=small, dev=api.Mesh(gpu_ctx, small), mat=mat, s=s[:2])]
    bt, res = run_batch(gpu_ctx, objs)
    for o, r in zip(objs, res):
        single = api.assemble_all(gpu_ctx, o["dev"], o["mat"], o["s"], dtype=L.C64)
        for k in KINDS:
            assert rel_fro(r[k], single[k]) <= 1e-6, k
    verts = np.array([7, 2000], dtype=np.int32)
    for k in ("G", "H"):
        got = np.concatenate([res[0][k][1][3 * v:3 * v + 3] for v in verts])
        ref = oracle.collocation(k, bunny, mat, s[1], rows=verts)
        assert rel_fro(got, ref) <= 1e-5, k
