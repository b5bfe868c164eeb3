"""GPU parity of the collocation assembly and the inverse transform against the FP64 oracle.

Tolerances (relative Frobenius norm):
  * whole Laplace-domain matrix (FP32 regular + FP64 singular)     <= 1e-5
  * FP64 singular pass alone vs the oracle's singular pass          <= 1e-10
  * inverse transform of identical frequency data                   <= 1e-10
Everything goes through the C ABI (host numpy buffers or device torch tensors).
"""
import numpy as np
import pytest

from surfaceonlydeformables_gb300.meshes import Material, make_icosphere_mesh

from .conftest import rel_fro

pytestmark = pytest.mark.gpu

KINDS = ["G", "H", "B_trans", "B_angular"]
MAT = Material(1e5, 0.3, 1000.0)


@pytest.fixture(scope="module")
def meshes():
    return {lev: make_icosphere_mesh(lev, 0.1) for lev in (1, 2)}


@pytest.fixture(scope="module")
def dev_meshes(gpu_ctx, meshes):
    from surfaceonlydeformables_gb300.api import Mesh

    return {lev: Mesh(gpu_ctx, m) for lev, m in meshes.items()}


@pytest.fixture(scope="module")
def freqs(sodlib):
    s, R, L = sodlib.cq_frequencies(2, 0.01, 32)
    return s[[0, 5, 16]]


@pytest.mark.parametrize("kind", KINDS)
@pytest.mark.parametrize("lev", [1, 2])
def test_collocation_matches_fp64_oracle(gpu_ctx, dev_meshes, meshes, oracle, freqs, kind, lev):
    from surfaceonlydeformables_gb300 import api

    for s in freqs:
        got = api.assemble(gpu_ctx, dev_meshes[lev], kind, MAT, s, order=5, subdiv=1)
        ref = oracle.collocation(kind, meshes[lev], MAT, s, order=5, subdiv=1)
        assert rel_fro(got, ref) <= 1e-5, (kind, lev, s, rel_fro(got, ref))


@pytest.mark.parametrize("kind", KINDS)
def test_singular_pass_small_s(gpu_ctx, dev_meshes, meshes, oracle, kind):
    """|s| r -> 0: the reference's literal kernel formulas cancel (up to ~9 digits in FP64 for the
    strongly singular H); the device and the accuracy oracle both evaluate the cancellation-free
    form, so the singular pass still agrees to 1e-10."""
    from surfaceonlydeformables_gb300 import _lib as L
    from surfaceonlydeformables_gb300 import api

    for s in (5.0 + 0.0j, 0.5 + 2.0j):
        got = api.assemble(gpu_ctx, dev_meshes[2], kind, MAT, s, parts=L.PART_SINGULAR)
        ref = oracle.collocation(kind, meshes[2], MAT, s, parts=2)
        assert rel_fro(got, ref) <= 1e-10, (kind, s, rel_fro(got, ref))


@pytest.mark.parametrize("kind", KINDS)
def test_singular_pass_is_fp64(gpu_ctx, dev_meshes, meshes, oracle, freqs, kind):
    from surfaceonlydeformables_gb300 import _lib as L
    from surfaceonlydeformables_gb300 import api

    for s in freqs:
        got = api.assemble(gpu_ctx, dev_meshes[2], kind, MAT, s, parts=L.PART_SINGULAR)
        ref = oracle.collocation(kind, meshes[2], MAT, s, parts=2)
        assert rel_fro(got, ref) <= 1e-10, (kind, s, rel_fro(got, ref))


@pytest.mark.parametrize("kind", KINDS)
def test_regular_pass(gpu_ctx, dev_meshes, meshes, oracle, freqs, kind):
    from surfaceonlydeformables_gb300 import _lib as L
    from surfaceonlydeformables_gb300 import api

    s = freqs[1]
    got = api.assemble(gpu_ctx, dev_meshes[2], kind, MAT, s, parts=L.PART_REGULAR)
    ref = oracle.collocation(kind, meshes[2], MAT, s, parts=1)
    assert rel_fro(got, ref) <= 1e-5


@pytest.mark.parametrize("order,subdiv", [(1, 1), (3, 2), (7, 1), (5, 2)])
def test_quadrature_variants(gpu_ctx, dev_meshes, meshes, oracle, freqs, order, subdiv):
    from surfaceonlydeformables_gb300 import api

    s = freqs[2]
    for kind in ("G", "H"):
        got = api.assemble(gpu_ctx, dev_meshes[1], kind, MAT, s, order=order, subdiv=subdiv,
                           sorder=min(order, 5), ssub=subdiv)
        ref = oracle.collocation(kind, meshes[1], MAT, s, order=order, subdiv=subdiv, sorder=min(order, 5),
                                 ssub=subdiv)
        assert rel_fro(got, ref) <= 1e-5, (kind, order, subdiv)


def test_bitwise_reproducible(gpu_ctx, dev_meshes, freqs):
    from surfaceonlydeformables_gb300 import api

    for kind in KINDS:
        a = api.assemble(gpu_ctx, dev_meshes[2], kind, MAT, freqs[1])
        b = api.assemble(gpu_ctx, dev_meshes[2], kind, MAT, freqs[1])
        assert np.array_equal(a.view(np.uint8), b.view(np.uint8)), kind


def test_thread_count_does_not_change_results(gpu_ctx, dev_meshes, freqs):
    from surfaceonlydeformables_gb300 import api

    base = api.assemble(gpu_ctx, dev_meshes[2], "H", MAT, freqs[0])
    for t in (64, 256, 512):
        gpu_ctx.set_tuning(t, 0)
        other = api.assemble(gpu_ctx, dev_meshes[2], "H", MAT, freqs[0])
        assert rel_fro(other, base) < 1e-6
    gpu_ctx.set_tuning(0, 0)


def test_device_pointer_path_and_c64(gpu_ctx, dev_meshes, freqs):
    import torch

    from surfaceonlydeformables_gb300 import _lib as L
    from surfaceonlydeformables_gb300 import api

    m = dev_meshes[2]
    host = api.assemble(gpu_ctx, m, "G", MAT, freqs[1])
    dev = torch.empty((3 * m.nV, 3 * m.nV), dtype=torch.complex128, device="cuda")
    api.assemble(gpu_ctx, m, "G", MAT, freqs[1], out=dev)
    gpu_ctx.synchronize()
    assert np.array_equal(dev.cpu().numpy(), host)
    c64 = api.assemble(gpu_ctx, m, "G", MAT, freqs[1], dtype=L.C64)
    assert c64.dtype == np.complex64 and rel_fro(c64, host) < 1e-6


def test_inverse_transform_matches_fp64(gpu_ctx, oracle, sodlib):
    from surfaceonlydeformables_gb300 import _lib as L
    from surfaceonlydeformables_gb300 import api

    rng = np.random.default_rng(3)
    for N in (32, 64, 5):
        s, R, Lq = sodlib.cq_frequencies(2, 0.005, N)
        X = (rng.normal(size=(len(s), 777)) + 1j * rng.normal(size=(len(s), 777))) / (1 + np.abs(s))[:, None]
        ref = oracle.inverse_transform(X, Lq, R)
        got = api.inverse_transform(gpu_ctx, X, Lq, R)
        assert rel_fro(got, ref) <= 1e-10, (N, rel_fro(got, ref))
        # complex64 input: compare with the FP64 transform of the same (rounded) data
        X32 = X.astype(np.complex64)
        ref32 = oracle.inverse_transform(X32.astype(np.complex128), Lq, R)
        got32 = api.inverse_transform(gpu_ctx, X32, Lq, R)
        assert rel_fro(got32, ref32) <= 1e-10
        got32f = api.inverse_transform(gpu_ctx, X32, Lq, R, out_dtype=L.F32)
        assert rel_fro(got32f, ref32) <= 2e-7  # the FP32 rounding of the outputs
        # complex128 input, FP32 output (the request loop's banks): double-float accumulation
        got64f = api.inverse_transform(gpu_ctx, X, Lq, R, out_dtype=L.F32)
        assert rel_fro(got64f, ref) <= 2e-7, (N, rel_fro(got64f, ref))


def test_inverse_transform_closed_form_weights(gpu_ctx, sodlib):
    """K(s) = 1/s under BDF1: the weights are dt / (1 - R^L) for every n (aliased sum)."""
    from surfaceonlydeformables_gb300 import api

    dt, N = 0.01, 24
    s, R, L = sodlib.cq_frequencies(1, dt, N)
    w = api.inverse_transform(gpu_ctx, (1.0 / s)[:, None].copy(), L, R)[:, 0]
    amp = R ** -np.arange(L)
    assert np.all(np.abs(w - dt / (1 - R ** L)) / dt < 1e-13 * amp)


def test_inverse_transform_real_data_fp64(gpu_ctx, dev_meshes, meshes, oracle, sodlib):
    """Real G data cancels heavily in the late weights; the FP64 kernel must still match to 1e-10."""
    from surfaceonlydeformables_gb300 import api

    s, R, Lq = sodlib.cq_frequencies(2, 0.01, 8)
    X = api.assemble_frequencies(gpu_ctx, dev_meshes[1], "G", MAT, s)
    got = api.inverse_transform(gpu_ctx, X, Lq, R)
    ref = oracle.inverse_transform(X, Lq, R)
    assert rel_fro(got, ref) <= 1e-10


def test_multi_frequency_launch_matches_single(gpu_ctx, dev_meshes, sodlib):
    """One launch over all frequencies (split into chunks above 40) equals per-frequency calls."""
    from surfaceonlydeformables_gb300 import api

    s, R, Lq = sodlib.cq_frequencies(2, 1 / 200, 96)  # 49 frequencies -> two chunks
    for kind in KINDS:
        allf = api.assemble_frequencies(gpu_ctx, dev_meshes[1], kind, MAT, s)
        for l in (0, 39, 40, 48):
            one = api.assemble(gpu_ctx, dev_meshes[1], kind, MAT, s[l])
            assert np.array_equal(allf[l], one), (kind, l)


def test_torch_stream_ordering(dev_meshes, sodlib, freqs):
    """Work issued on a torch stream is visible to torch events and later torch work on that stream."""
    import torch

    from surfaceonlydeformables_gb300 import _lib as L
    from surfaceonlydeformables_gb300 import api

    st = torch.cuda.Stream()
    ctx = api.Context(0, stream=st)
    m = api.Mesh(ctx, dev_meshes[2].host)
    with torch.cuda.stream(st):
        out = torch.zeros((3 * m.nV, 3 * m.nV), dtype=torch.complex64, device="cuda")
        api.assemble(ctx, m, "H", MAT, freqs[0], out=out, dtype=L.C64)
        total = out.abs().sum()
    st.synchronize()
    ref = api.assemble(ctx, m, "H", MAT, freqs[0], dtype=L.C64)
    assert abs(float(total) - np.abs(ref).sum()) < 1e-3 * np.abs(ref).sum()


def test_assemble_all_matches_per_kind(gpu_ctx, dev_meshes, meshes, oracle, sodlib):
    """The fused all-kinds call (shared FP64 radial terms) equals the per-kind calls to FP32 rounding
    (different kernel instantiations may contract FP32 operations differently) and matches the oracle."""
    from surfaceonlydeformables_gb300 import api

    s, R, Lq = sodlib.cq_frequencies(2, 0.01, 8)
    allk = api.assemble_all(gpu_ctx, dev_meshes[2], MAT, s)
    for kind in KINDS:
        one = api.assemble_frequencies(gpu_ctx, dev_meshes[2], kind, MAT, s)
        assert rel_fro(allk[kind], one) < 1e-6, kind
        ref = oracle.collocation(kind, meshes[2], MAT, s[2])
        assert rel_fro(allk[kind][2], ref) <= 1e-5, kind
    part = api.assemble_all(gpu_ctx, dev_meshes[2], MAT, s, kinds=("G", "B_angular"))
    assert set(part) == {"G", "B_angular"} and rel_fro(part["G"], allk["G"]) < 1e-6


@pytest.mark.parametrize("dtype_name", ["C128", "C64"])
def test_pinned_host_output_written_in_place(gpu_ctx, dev_meshes, freqs, dtype_name):
    """Page-locked host outputs are written by the kernels directly (no staging copy); the result
    must be bit-identical to a pageable host buffer and to a device buffer, for every kind and for
    the multi-frequency call."""
    import torch

    from surfaceonlydeformables_gb300 import _lib as L
    from surfaceonlydeformables_gb300 import api

    dt = getattr(L, dtype_name)
    tdt = torch.complex128 if dt == L.C128 else torch.complex64
    m = dev_meshes[2]
    for kind in KINDS:
        shape = api.out_shape(L.KINDS[kind], m.nV)
        pageable = api.assemble(gpu_ctx, m, kind, MAT, freqs[1], dtype=dt)
        pinned = torch.full(shape, complex(np.nan, np.nan), dtype=tdt).pin_memory()
        api.assemble(gpu_ctx, m, kind, MAT, freqs[1], out=pinned.numpy(), dtype=dt)
        dev = torch.empty(shape, dtype=tdt, device="cuda")
        api.assemble(gpu_ctx, m, kind, MAT, freqs[1], out=dev, dtype=dt)
        torch.cuda.synchronize()
        assert np.array_equal(pinned.numpy().view(np.uint8), pageable.view(np.uint8)), kind
        assert np.array_equal(dev.cpu().numpy().view(np.uint8), pageable.view(np.uint8)), kind
        many = torch.full((len(freqs),) + shape, complex(np.nan, np.nan), dtype=tdt).pin_memory()
        api.assemble_frequencies(gpu_ctx, m, kind, MAT, freqs, out=many.numpy(), dtype=dt)
        ref = api.assemble_frequencies(gpu_ctx, m, kind, MAT, freqs, dtype=dt)
        assert np.array_equal(many.numpy().view(np.uint8), ref.view(np.uint8)), kind


def test_large_host_output_pipelined(gpu_ctx, freqs):
    """Host outputs of 16 MB and more are staged and copied in row chunks while later rows compute;
    the result is bit-identical to a device buffer (642 vertices: 59 MB complex128 G/H, two chunks),
    for pageable and page-locked buffers and for the all-kinds call."""
    import torch

    from surfaceonlydeformables_gb300 import _lib as L
    from surfaceonlydeformables_gb300 import api
    from surfaceonlydeformables_gb300.api import Mesh

    m = make_icosphere_mesh(3, 0.1)
    dm = Mesh(gpu_ctx, m)
    for kind in ("G", "H"):
        shape = api.out_shape(L.KINDS[kind], m.nV)
        dev = torch.empty(shape, dtype=torch.complex128, device="cuda")
        api.assemble(gpu_ctx, dm, kind, MAT, freqs[1], out=dev)
        torch.cuda.synchronize()
        ref = dev.cpu().numpy()
        pageable = api.assemble(gpu_ctx, dm, kind, MAT, freqs[1])
        pinned = torch.full(shape, complex(np.nan, np.nan), dtype=torch.complex128).pin_memory()
        api.assemble(gpu_ctx, dm, kind, MAT, freqs[1], out=pinned.numpy())
        assert np.array_equal(pageable.view(np.uint8), ref.view(np.uint8)), kind
        assert np.array_equal(pinned.numpy().view(np.uint8), ref.view(np.uint8)), kind
    host = api.assemble_all(gpu_ctx, dm, MAT, freqs[:2])
    devs = {k: torch.empty((2,) + api.out_shape(L.KINDS[k], m.nV), dtype=torch.complex128, device="cuda")
            for k in KINDS}
    api.assemble_all(gpu_ctx, dm, MAT, freqs[:2], outs=devs)
    torch.cuda.synchronize()
    for k in KINDS:
        assert np.array_equal(host[k].view(np.uint8), devs[k].cpu().numpy().view(np.uint8)), k


def test_colour_phase_wait_timeout_is_reported(gpu_ctx, sodlib):
    """The scatter kernels' colour-phase waits are bounded.  With the context's test hook the barrier
    expects one arrival more than ever comes, so every wait runs out (about a second): the call returns
    SOD_ERR_TIMEOUT instead of hanging, and the context stays usable -- the next call reproduces the
    result bit for bit."""
    from surfaceonlydeformables_gb300 import _lib as L
    from surfaceonlydeformables_gb300 import api

    dm = api.Mesh(gpu_ctx, make_icosphere_mesh(1, 0.1))
    mat = Material(1e5, 0.3, 1000.0)
    s = complex(sodlib.cq_frequencies(2, 0.01, 4)[0][1])
    want = api.assemble(gpu_ctx, dm, "G", mat, s)
    gpu_ctx.set_wait_test(True)
    try:
        with pytest.raises(L.SodError) as e:
            api.assemble(gpu_ctx, dm, "G", mat, s)
        assert e.value.code == L.SOD_ERR_TIMEOUT
    finally:
        gpu_ctx.set_wait_test(False)
    got = api.assemble(gpu_ctx, dm, "G", mat, s)
    assert np.array_equal(got, want)
    gpu_ctx.synchronize()  # no error left behind


@pytest.mark.parametrize("kind", KINDS)
def test_compensated_regular_pass(gpu_ctx, dev_meshes, meshes, oracle, freqs, kind):
    """SOD_PRECISION_COMPENSATED: the frequency-dependent terms and the sums in double-float, the
    geometry in FP32.  The whole matrix is then limited by the FP32 geometry (~3e-8 for G and B,
    ~1.5e-7 for H, whose 1/r^2 kernel is more sensitive to it), below the FP32 pass."""
    from surfaceonlydeformables_gb300 import _lib as L
    from surfaceonlydeformables_gb300 import api

    gpu_ctx.set_precision(L.PRECISION_COMPENSATED)
    try:
        for s in freqs:
            got = api.assemble(gpu_ctx, dev_meshes[2], kind, MAT, s)
            ref = oracle.collocation(kind, meshes[2], MAT, s)
            print(kind, s, f"{rel_fro(got, ref):.2e}")
            assert rel_fro(got, ref) <= 3e-7, (kind, s, rel_fro(got, ref))
    finally:
        gpu_ctx.set_precision(L.PRECISION_AUTO)
