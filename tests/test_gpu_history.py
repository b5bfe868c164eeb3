"""History convolution (sod_history) against the FP64 oracle restatement of
src/elastodynamics_cqbem_object.cpp:44-48.

Tolerances (relative Frobenius norm of b):
  FP32 weights : <= 2e-6 (FP32 rounding of weights and history vectors);
  BF16 weights : <= 4e-3 (8-bit significand of the weights; per-row power-of-two scales);
  BF16, tensor cores against CUDA cores on the same bank: <= 3e-5 (the tensor-core path carries the
  history as two BF16 terms, a 16-bit significand, and accumulates in FP32 in another order);
  FP32 on the tensor cores (3xTF32: w_hi x_hi + w_hi x_lo + w_lo x_hi, 22-bit split operands):
  the FP32 tolerance, <= 2e-6."""
import numpy as np
import pytest

from .conftest import rel_fro

pytestmark = pytest.mark.gpu


def decaying_bank(rng, K, n, m):
    """G_k, H_k with the magnitude decay of CQ weights (index 0 unused, as in the oracle)."""
    G = np.zeros((K + 1, n, m))
    H = np.zeros((K + 1, n, m))
    for k in range(1, K + 1):
        G[k] = rng.normal(size=(n, m)) * 1e-6 * 0.8 ** k
        H[k] = rng.normal(size=(n, m)) * 0.8 ** k
    return G, H


def run(gpu_ctx, oracle, n, m, K, R, wdt, nsteps, with_b, seed=0, engine=0):
    from surfaceonlydeformables_gb300 import _lib as L
    from surfaceonlydeformables_gb300 import api

    rng = np.random.default_rng(seed)
    G, H = decaying_bank(rng, K, n, m)
    B = rng.normal(size=(K + 1, n, 6)) * 1e-3 if with_b else None
    bank = api.HistoryBank(gpu_ctx, n, m, K, R, wdt)
    bank.set_engine(engine)
    for k in range(1, K + 1):
        bank.set_weights(k, G[k], H[k])
        if with_b:
            bank.set_b(k, B[k])
    shape = (m, R) if R > 1 else (m,)
    ps, us, as_ = [], [], []
    for step in range(nsteps):
        p = rng.normal(size=shape) * 10.0
        u = rng.normal(size=shape) * 1e-4
        a = rng.normal(size=(6, R) if R > 1 else (6,))
        bank.push(p, u, a if with_b else None)
        ps.append(p), us.append(u), as_.append(a)
    got = bank.convolve()
    used = min(nsteps, K)
    ph = np.stack(ps[::-1][:used])
    uh = np.stack(us[::-1][:used])
    ref = oracle.history_convolution(G, H, ph, uh, B if with_b else None, np.stack(as_[::-1][:used]) if with_b else None)
    return got, ref, bank


@pytest.mark.parametrize("R", [1, 16])
@pytest.mark.parametrize("nsteps", [3, 11])  # fewer steps than K, and a wrapped ring
def test_history_fp32(gpu_ctx, oracle, R, nsteps):
    from surfaceonlydeformables_gb300 import _lib as L

    got, ref, bank = run(gpu_ctx, oracle, 126, 126, 8, R, L.F32, nsteps, with_b=True)
    assert got.shape == ref.shape
    assert rel_fro(got, ref) <= 2e-6
    again = bank.convolve()
    assert np.array_equal(got.view(np.uint8), again.view(np.uint8))  # bitwise reproducible


@pytest.mark.parametrize("R", [1, 16])
def test_history_bf16(gpu_ctx, oracle, R):
    from surfaceonlydeformables_gb300 import _lib as L

    got, ref, bank = run(gpu_ctx, oracle, 126, 130, 8, R, L.BF16, 9, with_b=False, seed=3)
    assert rel_fro(got, ref) <= 4e-3
    assert bank.weight_bytes == 8 * 2 * 126 * 136 * 2 + 8 * 2 * 126 * 4


@pytest.mark.parametrize("R", [1, 16])
@pytest.mark.parametrize("n,m,K,nsteps", [(126, 130, 8, 9), (300, 200, 4, 2), (1926, 1926, 24, 30)])
def test_history_bf16_tensor_cores(gpu_ctx, oracle, n, m, K, nsteps, R):
    """tcgen05 path: row counts that are not a multiple of the 128-row tile, column counts that are
    not a multiple of the 64-column K tile, a partly filled and a wrapped ring, the B term."""
    from surfaceonlydeformables_gb300 import _lib as L

    tc, ref, bank = run(gpu_ctx, oracle, n, m, K, R, L.BF16, nsteps, with_b=True, seed=7,
                        engine=L.HISTORY_ENGINE_TENSOR_CORES)
    cc, _, _ = run(gpu_ctx, oracle, n, m, K, R, L.BF16, nsteps, with_b=True, seed=7,
                   engine=L.HISTORY_ENGINE_CUDA_CORES)
    assert rel_fro(tc, ref) <= 4e-3
    assert rel_fro(tc, cc) <= 3e-5
    again = bank.convolve()
    assert np.array_equal(tc.view(np.uint8), again.view(np.uint8))  # bitwise reproducible


@pytest.mark.parametrize("R", [1, 16])
@pytest.mark.parametrize("n,m,K,nsteps", [(126, 130, 8, 9), (300, 200, 4, 2), (1926, 1926, 24, 30)])
def test_history_fp32_tensor_cores(gpu_ctx, oracle, n, m, K, nsteps, R):
    """3xTF32 path for FP32 banks: same shapes as the BF16 case, FP32 tolerance against the oracle."""
    from surfaceonlydeformables_gb300 import _lib as L

    tc, ref, bank = run(gpu_ctx, oracle, n, m, K, R, L.F32, nsteps, with_b=True, seed=9,
                        engine=L.HISTORY_ENGINE_TENSOR_CORES)
    cc, _, _ = run(gpu_ctx, oracle, n, m, K, R, L.F32, nsteps, with_b=True, seed=9,
                   engine=L.HISTORY_ENGINE_CUDA_CORES)
    assert rel_fro(tc, ref) <= 2e-6, rel_fro(tc, ref)
    assert rel_fro(cc, ref) <= 2e-6
    again = bank.convolve()
    assert np.array_equal(tc.view(np.uint8), again.view(np.uint8))  # bitwise reproducible


@pytest.mark.parametrize("R", [1, 16])
def test_history_fp32_tensor_cores_truncated_operands(gpu_ctx, R):
    """The FP32 tensor-core path takes w_hi as the top 19 bits the TF32 MMA reads.  Weights in [1, 2)
    whose low 13 bits are at least half a TF32 unit would be off by about 2^-11 if the tensor core
    rounded its operands.  With x = 1 (x_lo = 0) the result is w_hi + TF32(w_lo), which misses w only by
    the bits of w_lo below TF32's 11: less than 2^-21 relative."""
    from surfaceonlydeformables_gb300 import _lib as L
    from surfaceonlydeformables_gb300 import api

    n = 200
    rng = np.random.default_rng(11)
    bits = rng.integers(0x3F800000, 0x40000000, n).astype(np.uint32)
    bits = (bits & np.uint32(0xFFFFE000)) | np.uint32(0x1000) | (rng.integers(0, 0x1000, n).astype(np.uint32))
    w = bits.view(np.float32).astype(np.float64) * np.where(rng.random(n) < 0.5, -1.0, 1.0)
    bank = api.HistoryBank(gpu_ctx, n, n, 1, R, L.F32)
    bank.set_engine(L.HISTORY_ENGINE_TENSOR_CORES)
    bank.set_weights(1, np.diag(w), np.zeros((n, n)))
    bank.push(np.ones((n, R)) if R > 1 else np.ones(n), np.zeros((n, R)) if R > 1 else np.zeros(n))
    got = bank.convolve()
    want = np.repeat(w[:, None], R, axis=1) if R > 1 else w
    err = np.max(np.abs(got - want) / np.abs(want))
    assert err < 2.0**-21, err


def test_history_engine_selection(gpu_ctx):
    from surfaceonlydeformables_gb300 import _lib as L
    from surfaceonlydeformables_gb300 import api

    f32 = api.HistoryBank(gpu_ctx, 10, 10, 2, 16, L.F32)  # AUTO: tensor cores (3xTF32)
    f32.set_weights(1, 2.0 * np.eye(10), np.zeros((10, 10)))
    f32.push(np.ones((10, 16)), np.zeros((10, 16)))
    assert np.allclose(f32.convolve(), 2.0)
    f32.set_engine(L.HISTORY_ENGINE_TENSOR_CORES)  # same engine as AUTO here: the ring is kept
    assert np.allclose(f32.convolve(), 2.0)
    bf = api.HistoryBank(gpu_ctx, 10, 10, 2, 16, L.BF16)
    bf.set_weights(1, np.eye(10), np.zeros((10, 10)))
    bf.push(np.ones((10, 16)), np.zeros((10, 16)))
    assert np.allclose(bf.convolve(), 1.0)
    bf.set_engine(L.HISTORY_ENGINE_CUDA_CORES)  # the ring is emptied
    assert np.all(bf.convolve() == 0.0)
    with pytest.raises(L.SodError):
        bf.set_engine(7)


def test_history_larger_object(gpu_ctx, oracle):
    """3V = 1926 (642 vertices), K = 24, 16 right-hand sides, ring wrapped, with the B term."""
    from surfaceonlydeformables_gb300 import _lib as L

    got, ref, _ = run(gpu_ctx, oracle, 1926, 1926, 24, 16, L.F32, 30, with_b=True, seed=5)
    assert rel_fro(got, ref) <= 2e-6


def test_history_empty_and_reset(gpu_ctx):
    from surfaceonlydeformables_gb300 import _lib as L
    from surfaceonlydeformables_gb300 import api

    bank = api.HistoryBank(gpu_ctx, 10, 10, 4, 1, L.F32)
    assert np.all(bank.convolve() == 0.0)
    bank.set_weights(1, np.eye(10), np.zeros((10, 10)))
    bank.push(np.arange(10.0), np.zeros(10))
    assert np.allclose(bank.convolve(), np.arange(10.0))
    bank.reset()
    assert np.all(bank.convolve() == 0.0)


@pytest.mark.parametrize("wdt_name,R,tol", [("F32", 1, 2e-6), ("F32", 16, 2e-6), ("BF16", 1, 4e-3), ("BF16", 16, 4e-3)])
def test_history_full_size_against_fp64(gpu_ctx, wdt_name, R, tol):
    """The benchmarked bank: one 2562-vertex object (3V = 7686) with K = 64 steps of FP64 weights
    (G_k ~ 1e-6 x 0.8^k, H_k ~ 0.8^k), the ring wrapped, default engine.  The FP64 reference
    b = sum_k G_k p_{n-k} - H_k u_{n-k} is formed on the device in FP64 from the same FP64 weights
    (regenerated from per-k seeds), so the bank's FP32 / BF16 storage is what is measured."""
    import torch

    from surfaceonlydeformables_gb300 import _lib as L
    from surfaceonlydeformables_gb300 import api

    n, K, nsteps = 7686, 64, 67
    ctx = api.Context(0, stream=torch.cuda.current_stream())  # torch's and the bank's work in one stream order
    bank = api.HistoryBank(ctx, n, n, K, R, getattr(L, wdt_name))
    gen = torch.Generator(device="cuda")

    def weights(k):
        gen.manual_seed(1000 + k)
        G = torch.randn((n, n), dtype=torch.float64, device="cuda", generator=gen) * (1e-6 * 0.8 ** k)
        H = torch.randn((n, n), dtype=torch.float64, device="cuda", generator=gen) * (0.8 ** k)
        return G, H

    for k in range(1, K + 1):
        G, H = weights(k)
        bank.set_weights(k, G, H)
        del G, H
    gen.manual_seed(7)
    shape = (n, R) if R > 1 else (n,)
    ps, us = [], []
    for _ in range(nsteps):
        p = torch.randn(shape, dtype=torch.float64, device="cuda", generator=gen) * 10.0
        u = torch.randn(shape, dtype=torch.float64, device="cuda", generator=gen) * 1e-4
        bank.push(p, u)
        ps.append(p), us.append(u)
    got = torch.empty(shape, dtype=torch.float64, device="cuda")
    bank.convolve(got)
    torch.cuda.synchronize()
    ref = torch.zeros(shape, dtype=torch.float64, device="cuda")
    for i in range(K):  # G_{i+1} p_{n-1-i} - H_{i+1} u_{n-1-i}
        G, H = weights(i + 1)
        ref += G @ ps[nsteps - 1 - i] - H @ us[nsteps - 1 - i]
        del G, H
    err = float(torch.linalg.norm(got - ref) / torch.linalg.norm(ref))
    bank.close()
    ctx.close()
    torch.cuda.empty_cache()
    assert err <= tol, (wdt_name, R, err)
