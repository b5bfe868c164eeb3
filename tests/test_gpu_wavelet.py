"""Wavelet-compressed history bank (sod_history_create_compressed) against the oracle's restatement of
the reference's CompressedMatrix<1> / CompressedVector<1> path.

Tolerances: the kept coefficients (row pointers, columns, values) are bit-identical to the oracle
(both evaluate the decomposition in FP64 in the reference's order without contraction, and both keep
ties at the threshold in (row, column) order); the per-step convolution <= 1e-12 relative (FP64 sums
in a different order); keeping every coefficient it matches the dense convolution to <= 1e-12."""
import struct

import numpy as np
import pytest

from surfaceonlydeformables_gb300.meshes import Material, make_icosphere_mesh

from .conftest import rel_fro

pytestmark = pytest.mark.gpu


def _weights(gpu_ctx, level, N):
    """Time-domain G_k, H_k (k = 0..N) of an icosphere from the library's precompute."""
    from surfaceonlydeformables_gb300 import api

    m = make_icosphere_mesh(level, 0.1)
    dm = api.Mesh(gpu_ctx, m)
    w = api.precompute(gpu_ctx, dm, Material(1e5, 0.3, 1000.0), 2, 0.01, N, kinds=("G", "H"))
    return m.nV, w["G"].cpu().numpy(), w["H"].cpu().numpy()


@pytest.mark.parametrize("level,ratio", [(1, 0.1), (2, 0.1), (2, 0.02), (1, 1e-9)])
def test_compressed_matrices_bit_exact(gpu_ctx, level, ratio):
    from oracle import oracle

    from surfaceonlydeformables_gb300 import api

    K = 3
    nV, G, H = _weights(gpu_ctx, level, K)
    bank = api.HistoryBank.compressed(gpu_ctx, nV, K, ratio)
    for k in range(1, K + 1):
        bank.set_weights(k, G[k], H[k])
    total = 0
    for k in range(1, K + 1):
        for which, (W, sign) in enumerate(((G[k], 1.0), (H[k], -1.0))):
            rp, col, val = bank.compressed_matrix(k, which)
            ref = oracle.wavelet_compress(W, nV, ratio, sign)
            assert np.array_equal(rp, ref[0]) and np.array_equal(col, ref[1]), (k, which)
            assert np.array_equal(val, ref[2]), (k, which)
            total += len(val)
    assert bank.weight_bytes == 12 * total


def test_compressed_ties_at_threshold(gpu_ctx):
    """A matrix of ones has many coefficients of equal magnitude: the ratio cuts through a tie."""
    from oracle import oracle

    from surfaceonlydeformables_gb300 import api

    nV = 10
    N = 3 * nV
    W = np.ones((N, N))
    W[::2, 1::3] = 2.0
    bank = api.HistoryBank.compressed(gpu_ctx, nV, 1, 0.05)
    bank.set_weights(1, W, -W)
    for which, sign in ((0, 1.0), (1, -1.0)):
        rp, col, val = bank.compressed_matrix(1, which)
        ref = oracle.wavelet_compress(W if which == 0 else -W, nV, 0.05, sign)
        assert len(val) == int(N * N * 0.05)
        assert np.array_equal(rp, ref[0]) and np.array_equal(col, ref[1]) and np.array_equal(val, ref[2])


@pytest.mark.parametrize("ratio", [0.1, 1e-9])
def test_compressed_convolution(gpu_ctx, ratio):
    """b over a partly and a fully filled ring, with B terms, against the oracle's compressed history;
    keeping every coefficient, against the dense convolution."""
    import torch
    from oracle import oracle

    from surfaceonlydeformables_gb300 import api

    K = 4
    nV, G, H = _weights(gpu_ctx, 2, K)
    N = 3 * nV
    rng = np.random.default_rng(3)
    B = [np.zeros((N, 6))] + [rng.normal(size=(N, 6)) * 1e-3 for _ in range(K)]
    bank = api.HistoryBank.compressed(gpu_ctx, nV, K, ratio)
    for k in range(1, K + 1):
        bank.set_weights(k, torch.from_numpy(G[k]).cuda(), torch.from_numpy(H[k]).cuda())  # device inputs
        bank.set_b(k, B[k])
    Gc = {k: oracle.wavelet_compress(G[k], nV, ratio) for k in range(1, K + 1)}
    Hc = {k: oracle.wavelet_compress(H[k], nV, ratio, -1.0) for k in range(1, K + 1)}
    ps, us, As = [], [], []
    for step in range(6):
        p, u, a = rng.normal(size=N) * 10.0, rng.normal(size=N) * 1e-4, rng.normal(size=6)
        bank.push(p, u, a)
        ps.insert(0, p), us.insert(0, u), As.insert(0, a)
        if step in (1, 5):
            n = min(len(ps), K)
            got = bank.convolve()
            ph, uh, ah = np.array(ps[:n]), np.array(us[:n]), np.array(As[:n])
            ref = oracle.wavelet_history_convolution(Gc, Hc, ph, uh, nV, np.stack(B), ah)
            assert rel_fro(got, ref) <= 1e-12, step
            if ratio < 1e-6:
                dense = oracle.history_convolution(G[:n + 1], H[:n + 1], ph, uh, np.stack(B[:n + 1]), ah)
                assert rel_fro(got, dense) <= 1e-12, step
    assert np.array_equal(bank.convolve(), bank.convolve())  # deterministic
    bank.reset()
    assert np.array_equal(bank.convolve(), np.zeros(N))


def test_cpmat_file(gpu_ctx, tmp_path):
    """save_compressed_matrix layout: int N; int64 rows, cols, nonZeros, outerSize, innerSize; values;
    outerSize row starts; column indices."""
    from surfaceonlydeformables_gb300 import api

    nV, G, H = _weights(gpu_ctx, 1, 1)
    bank = api.HistoryBank.compressed(gpu_ctx, nV, 1, 0.1)
    bank.set_weights(1, G[1], H[1])
    path = str(tmp_path / "H_1_0.100000.cpmat")
    bank.write_cpmat(1, 1, path)
    rp, col, val = bank.compressed_matrix(1, 1)
    raw = open(path, "rb").read()
    N, rows, cols, nnz, outer, inner = struct.unpack_from("<iqqqqq", raw, 0)
    assert N == 3 * nV and rows == cols == outer == inner == len(rp) - 1 and nnz == len(val)
    o = 4 + 5 * 8
    assert np.array_equal(np.frombuffer(raw, np.float64, nnz, o), val)
    o += 8 * nnz
    assert np.array_equal(np.frombuffer(raw, np.int32, outer, o), rp[:-1])
    o += 4 * outer
    assert np.array_equal(np.frombuffer(raw, np.int32, nnz, o), col)
    assert o + 4 * nnz == len(raw)


def test_compressed_bank_arguments(gpu_ctx):
    from surfaceonlydeformables_gb300 import _lib as L
    from surfaceonlydeformables_gb300 import api

    for nV, K, ratio in ((10, 2, 0.0), (10, 2, 1.5), (5462, 2, 0.1), (10, 0, 0.1)):
        with pytest.raises(L.SodError) as e:
            api.HistoryBank.compressed(gpu_ctx, nV, K, ratio)
        assert e.value.code == L.SOD_ERR_INVALID_ARG
    bank = api.HistoryBank.compressed(gpu_ctx, 10, 2, 0.1)
    with pytest.raises(L.SodError):
        bank.set_engine(L.HISTORY_ENGINE_TENSOR_CORES)
    with pytest.raises(L.SodError):
        bank.compressed_matrix(1, 0)  # weights not set yet
