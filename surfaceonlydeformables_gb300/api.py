"""Thin object layer over the C ABI: Context (device + stream + scratch) and Mesh (device-resident
geometry), plus the per-frequency assembly and inverse-transform calls."""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib as L
from .meshes import Material, SurfaceMesh


def _torch():
    import torch  # deferred: the package itself needs only numpy

    return torch


class Context:
    """A device, a CUDA stream and the library's scratch buffers (sod_context)."""

    def __init__(self, device: int = 0, stream=None):
        self._h = ctypes.c_void_p()
        L.check(L.load().sod_context_create(device, ctypes.byref(self._h)))
        self.device = device
        if stream is not None:
            self.set_stream(stream)

    def set_stream(self, stream) -> None:
        """stream: a torch.cuda.Stream or a raw cudaStream_t integer (0 = CUDA's default stream)."""
        raw = int(getattr(stream, "cuda_stream", stream) or 0)
        L.check(L.load().sod_context_set_stream(self._h, ctypes.c_void_p(raw) if raw else None))

    def synchronize(self) -> None:
        L.check(L.load().sod_context_synchronize(self._h))

    def set_tuning(self, coll_threads: int = 0, galerkin_threads: int = 0) -> None:
        L.check(L.load().sod_context_set_tuning(self._h, coll_threads, galerkin_threads))

    def set_precision(self, precision: int) -> None:
        """Regular-pass precision: L.PRECISION_AUTO (FP32 for Laplace-domain outputs, compensated for
        time-domain outputs), L.PRECISION_FP32 or L.PRECISION_COMPENSATED."""
        L.check(L.load().sod_context_set_precision(self._h, precision))

    def set_wait_test(self, stall: bool) -> None:
        """Test hook: make the collocation scatter kernels' bounded colour-phase waits run out."""
        L.check(L.load().sod_context_set_wait_test(self._h, 1 if stall else 0))

    @property
    def launches(self) -> int:
        return int(L.load().sod_context_launch_count(self._h))

    @property
    def handle(self):
        return self._h

    def close(self) -> None:
        if self._h:
            L.load().sod_context_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Mesh:
    """Device-resident mesh with precomputed stars, neighbour slots and face colourings."""

    def __init__(self, ctx: Context, mesh: SurfaceMesh, vmap=None):
        self.ctx = ctx
        self.host = mesh
        self.nV, self.nF = mesh.nV, mesh.nF
        self._vmap = None if vmap is None else np.ascontiguousarray(vmap, dtype=np.int32)
        self._h = ctypes.c_void_p()
        L.check(L.load().sod_mesh_create(ctx.handle, L.ptr(mesh.V), mesh.nV, L.ptr(mesh.F), mesh.nF, L.ptr(mesh.N),
                                         L.ptr(self._vmap), ctypes.byref(self._h)))

    @property
    def handle(self):
        return self._h

    def close(self) -> None:
        if self._h:
            L.load().sod_mesh_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def out_shape(kind: int, nV: int) -> tuple[int, int]:
    return (3 * nV, 3 * nV) if kind in (L.G, L.H) else ((3 * nV, 3) if kind == L.B_TRANS else (3 * nV, 9))


def assemble(ctx: Context, mesh: Mesh, kind, mat: Material, s: complex, order: int = 5, subdiv: int = 1,
             sorder: int | None = None, ssub: int | None = None, method: int = L.COLLOCATION,
             parts: int = L.PART_ALL, out=None, dtype: int = L.C128):
    """Laplace-domain matrix of `kind` at frequency s (drop-in for the reference's per-row kernels).

    out: numpy (host) or torch CUDA tensor of the right shape/dtype; allocated as numpy if None.
    B_angular comes back as (3V, 9) = [row][j*3+k]."""
    kind = L.KINDS.get(kind, kind)
    if out is None:
        out = np.empty(out_shape(kind, mesh.nV), dtype=np.complex128 if dtype == L.C128 else np.complex64)
    sorder = sorder or min(order, 5)
    ssub = ssub or subdiv
    L.check(L.load().sod_cqbem_assemble(ctx.handle, mesh.handle, kind, method, mat.c1, mat.c2, mat.rho,
                                        float(np.real(s)), float(np.imag(s)), order, subdiv, sorder, ssub, parts,
                                        L.ptr(out), dtype))
    return out


def assemble_frequencies(ctx: Context, mesh: Mesh, kind, mat: Material, s, order: int = 5, subdiv: int = 1,
                         sorder: int | None = None, ssub: int | None = None, method: int = L.COLLOCATION,
                         parts: int = L.PART_ALL, out=None, dtype: int = L.C128):
    """All listed Laplace frequencies in one launch: out has shape (len(s),) + out_shape(kind)."""
    kind = L.KINDS.get(kind, kind)
    s = np.ascontiguousarray(np.asarray(s, dtype=np.complex128).ravel())
    if out is None:
        out = np.empty((len(s),) + out_shape(kind, mesh.nV), dtype=np.complex128 if dtype == L.C128 else np.complex64)
    sorder = sorder or min(order, 5)
    ssub = ssub or subdiv
    L.check(L.load().sod_cqbem_assemble_frequencies(ctx.handle, mesh.handle, kind, method, mat.c1, mat.c2, mat.rho,
                                                    L.ptr(s.view(np.float64)), len(s), order, subdiv, sorder, ssub,
                                                    parts, L.ptr(out), dtype))
    return out


def assemble_all(ctx: Context, mesh: Mesh, mat: Material, s, order: int = 5, subdiv: int = 1,
                 sorder: int | None = None, ssub: int | None = None, method: int = L.COLLOCATION,
                 parts: int = L.PART_ALL, outs: dict | None = None, dtype: int = L.C128, kinds=("G", "H", "B_trans", "B_angular")):
    """Several kinds for all listed frequencies in one call (shared FP64 radial terms).  Returns a dict
    kind -> array of shape (len(s),) + out_shape(kind)."""
    s = np.ascontiguousarray(np.asarray(s, dtype=np.complex128).ravel())
    outs = dict(outs or {})
    cd = np.complex128 if dtype == L.C128 else np.complex64
    for k in kinds:
        if k not in outs:
            outs[k] = np.empty((len(s),) + out_shape(L.KINDS[k], mesh.nV), dtype=cd)
    sorder = sorder or min(order, 5)
    ssub = ssub or subdiv
    ptrs = [L.ptr(outs[k]) if k in outs else None for k in ("G", "H", "B_trans", "B_angular")]
    L.check(L.load().sod_cqbem_assemble_all(ctx.handle, mesh.handle, method, mat.c1, mat.c2, mat.rho,
                                            L.ptr(s.view(np.float64)), len(s), order, subdiv, sorder, ssub, parts,
                                            *ptrs, dtype))
    return outs


class Batch:
    """Many objects assembled by persistent kernels under one CUDA graph (sod_batch).

    add() takes device output tensors (torch CUDA) per kind; run() replays the captured step."""

    def __init__(self, ctx: Context, kinds=("G", "H", "B_trans", "B_angular"), dtype: int = L.C64):
        self.ctx = ctx
        self.kinds = tuple(kinds)
        self.dtype = dtype
        mask = 0
        for k in self.kinds:
            mask |= 1 << L.KINDS[k]
        self._h = ctypes.c_void_p()
        L.check(L.load().sod_batch_create(ctx.handle, mask, dtype, ctypes.byref(self._h)))
        self._keep = []

    def add(self, mesh: Mesh, mat: Material, s, outs: dict, order: int = 5, subdiv: int = 1,
            sorder: int | None = None, ssub: int | None = None) -> None:
        sv = np.ascontiguousarray(np.asarray(s, dtype=np.complex128).ravel())
        self._keep.append((mesh, outs))
        ptrs = [L.ptr(outs[k]) if k in self.kinds else None for k in ("G", "H", "B_trans", "B_angular")]
        L.check(L.load().sod_batch_add(self._h, mesh.handle, mat.c1, mat.c2, mat.rho, L.ptr(sv.view(np.float64)),
                                       len(sv), order, subdiv, sorder or min(order, 5), ssub or subdiv, *ptrs))

    def finalize(self) -> None:
        L.check(L.load().sod_batch_finalize(self._h))

    def run(self) -> None:
        L.check(L.load().sod_batch_run(self._h))

    @property
    def launches_per_step(self) -> int:
        return int(L.load().sod_batch_launch_count(self._h))

    PASS_NAMES = ("singular_polar", "singular_guiggiani", "scatter_G", "scatter_H", "reduce_B", "combine_GB",
                  "combine_H")

    def profile(self) -> list[dict]:
        """Per-launch device times of one eager (non-graph) step: [{pass, evals, ms}]."""
        n = self.launches_per_step
        which = np.zeros(n, dtype=np.int32)
        evals = np.zeros(n, dtype=np.float64)
        ms = np.zeros(n, dtype=np.float32)
        L.check(L.load().sod_batch_profile(self._h, n, L.ptr(which), L.ptr(evals), L.ptr(ms)))
        return [{"pass": self.PASS_NAMES[w], "evals": float(e), "ms": float(t)} for w, e, t in zip(which, evals, ms)]

    def close(self) -> None:
        if self._h:
            L.load().sod_batch_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def alloc_outputs(mesh: Mesh, nfreq: int, kinds=("G", "H", "B_trans", "B_angular"), dtype: int = L.C64, device=0):
    """torch CUDA output buffers for one object: kind -> (nfreq,) + out_shape(kind)."""
    torch = _torch()
    td = torch.complex64 if dtype == L.C64 else torch.complex128
    return {k: torch.empty((nfreq,) + out_shape(L.KINDS[k], mesh.nV), dtype=td, device=f"cuda:{device}") for k in kinds}


def precompute(ctx: Context, mesh: Mesh, mat: Material, bdf: int, dt: float, N: int, order: int = 5,
               subdiv: int = 1, sorder: int | None = None, ssub: int | None = None, method: int = L.COLLOCATION,
               cm=(0.0, 0.0, 0.0), out_dtype: int = L.F64, kinds=("G", "H", "B_trans", "B_angular", "B_euler")):
    """Time-domain CQ weights of one object (torch CUDA tensors): dict kind -> (L, ...) array."""
    torch = _torch()
    nV = mesh.nV
    Lq = N + 1
    shapes = {"G": (Lq, 3 * nV, 3 * nV), "H": (Lq, 3 * nV, 3 * nV), "B_trans": (Lq, 3 * nV, 3),
              "B_angular": (Lq, 3 * nV, 3, 3), "B_euler": (Lq, 3 * nV, 3)}
    dt_ = torch.float64 if out_dtype == L.F64 else torch.float32
    outs = {k: torch.empty(shapes[k], dtype=dt_, device=f"cuda:{ctx.device}") for k in kinds}
    cmv = np.ascontiguousarray(np.asarray(cm, dtype=np.float64))
    ptrs = [L.ptr(outs[k]) if k in outs else None for k in ("G", "H", "B_trans", "B_angular", "B_euler")]
    L.check(L.load().sod_cqbem_precompute(ctx.handle, mesh.handle, method, mat.c1, mat.c2, mat.rho, mat.nu, bdf, dt,
                                          N, order, subdiv, sorder or min(order, 5), ssub or subdiv, L.ptr(cmv),
                                          *ptrs, out_dtype))
    return outs


def inverse_transform(ctx: Context, Xhat, L_: int, R: float, out=None, out_dtype: int = L.F64):
    """Time-domain CQ weights from Laplace-domain blocks: Xhat (L/2+1, ...) complex -> (L, ...) real."""
    in_dtype = L.C128 if str(Xhat.dtype).endswith("complex128") else L.C64
    nfreq = Xhat.shape[0]
    M = int(np.prod(Xhat.shape[1:]))
    if out is None:
        out = np.empty((L_,) + tuple(Xhat.shape[1:]), dtype=np.float64 if out_dtype == L.F64 else np.float32)
    L.check(L.load().sod_cq_inverse_transform(ctx.handle, L.ptr(Xhat), in_dtype, M, nfreq, L_, R, L.ptr(out),
                                              out_dtype))
    return out


def elastostatic(ctx: Context, mesh: Mesh, kind: str, mat: Material, order: int = 5, subdiv: int = 1,
                 sorder: int | None = None, ssub: int | None = None, method: int = L.COLLOCATION, out=None,
                 dtype: int = L.F64):
    """Elastostatic Kelvin G or H (3nV x 3nV; H with the rigid-mode diagonal correction)."""
    if out is None:
        out = np.empty((3 * mesh.nV, 3 * mesh.nV), dtype=np.float64 if dtype == L.F64 else np.float32)
    L.check(L.load().sod_elastostatic_assemble(ctx.handle, mesh.handle, L.KINDS[kind], method, mat.nu, mat.mu, order,
                                               subdiv, sorder or min(order, 5), ssub or subdiv, L.ptr(out), dtype))
    return out


class Solver:
    """Dense LU (partial pivoting, FP64) of a row-major n x n matrix on the device (sod_solver): the
    H_0 factorisation of the reference's matrix collection and its solves."""

    def __init__(self, ctx: Context, A):
        A = A if hasattr(A, "data_ptr") else np.ascontiguousarray(np.asarray(A, dtype=np.float64))
        self.ctx, self.n = ctx, A.shape[0]
        self._h = ctypes.c_void_p()
        L.check(L.load().sod_solver_create(ctx.handle, self.n, L.ptr(A), ctypes.byref(self._h)))

    def solve(self, B, out=None):
        B = B if hasattr(B, "data_ptr") else np.ascontiguousarray(np.asarray(B, dtype=np.float64))
        nrhs = 1 if B.ndim == 1 else B.shape[1]
        if out is None:
            out = np.empty(B.shape, dtype=np.float64)
        L.check(L.load().sod_solver_solve(self._h, nrhs, L.ptr(B), L.ptr(out)))
        return out

    def inverse(self, out=None):
        if out is None:
            out = np.empty((self.n, self.n), dtype=np.float64)
        L.check(L.load().sod_solver_inverse(self._h, L.ptr(out)))
        return out

    def keep_inverse(self) -> None:
        """Keep A^-1 resident: the per-step HistoryBank.convolve_solve becomes one FP64 GEMV."""
        L.check(L.load().sod_solver_keep_inverse(self._h))

    def close(self) -> None:
        if self._h:
            L.load().sod_solver_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class LeastSquares:
    """Minimum-norm least squares with a tall m x k matrix B (sod_lstsq): the reference's
    CompleteOrthogonalDecomposition B_trans_inv / B_euler_inv.  solve(Y) = B^+ Y."""

    def __init__(self, ctx: Context, B):
        B = B if hasattr(B, "data_ptr") else np.ascontiguousarray(np.asarray(B, dtype=np.float64))
        self.ctx, self.m, self.k = ctx, B.shape[0], B.shape[1]
        self._h = ctypes.c_void_p()
        L.check(L.load().sod_lstsq_create(ctx.handle, self.m, self.k, L.ptr(B), ctypes.byref(self._h)))

    @property
    def rank(self) -> int:
        r = ctypes.c_int()
        L.check(L.load().sod_lstsq_rank(self._h, ctypes.byref(r)))
        return r.value

    def solve(self, Y, out=None):
        Y = Y if hasattr(Y, "data_ptr") else np.ascontiguousarray(np.asarray(Y, dtype=np.float64))
        ncols = 1 if Y.ndim == 1 else Y.shape[1]
        if out is None:
            out = np.empty((self.k,) if Y.ndim == 1 else (self.k, ncols), dtype=np.float64)
        L.check(L.load().sod_lstsq_solve(self._h, ncols, L.ptr(Y), L.ptr(out)))
        return out

    def pinv(self, out=None):
        if out is None:
            out = np.empty((self.k, self.m), dtype=np.float64)
        L.check(L.load().sod_lstsq_pinv(self._h, L.ptr(out)))
        return out

    def close(self) -> None:
        if self._h:
            L.load().sod_lstsq_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def elastostatic_u_p(ctx: Context, mesh: Mesh, H, G, out=None):
    """u_p of the elastostatic matrix collection: the regularised, force-free-projected solve of
    src/elastostatics_bem_matrix_collection.cpp:58-89 (FP64, 3nV x 3nV)."""
    H = H if hasattr(H, "data_ptr") else np.ascontiguousarray(np.asarray(H, dtype=np.float64))
    G = G if hasattr(G, "data_ptr") else np.ascontiguousarray(np.asarray(G, dtype=np.float64))
    if out is None:
        out = np.empty((3 * mesh.nV, 3 * mesh.nV), dtype=np.float64)
    L.check(L.load().sod_elastostatic_u_p(ctx.handle, mesh.handle, L.ptr(H), L.ptr(G), L.ptr(out)))
    return out


def rigid_modes(ctx: Context, mesh: Mesh, out=None):
    """Area-weighted rigid modes T (6 x 3nV) of the elastostatic regularisation."""
    if out is None:
        out = np.empty((6, 3 * mesh.nV), dtype=np.float64)
    L.check(L.load().sod_elastostatic_rigid_modes(ctx.handle, mesh.handle, L.ptr(out)))
    return out


def mat_write(ctx, path: str, M) -> None:
    """Matrix (2-D numpy array or CUDA tensor, float64/float32) to the reference's .mat file format.
    ctx may be None for host arrays."""
    M = M if hasattr(M, "data_ptr") else np.ascontiguousarray(M)
    dt = L.F32 if str(M.dtype) in ("float32", "torch.float32") else L.F64
    L.check(L.load().sod_mat_write(ctx.handle if ctx else None, path.encode(), L.ptr(M), M.shape[0], M.shape[1], dt))


def mat_read(ctx, path: str, rows: int, cols: int) -> np.ndarray:
    out = np.empty((rows, cols), dtype=np.float64)
    L.check(L.load().sod_mat_read(ctx.handle if ctx else None, path.encode(), L.ptr(out), rows, cols))
    return out


def write_cache(ctx: Context, folder: str, nV: int, weights: dict) -> None:
    """sod_cqbem_write_cache: `weights` as returned by precompute() (G, H, B_trans, B_euler; any
    subset, B_trans with B_euler)."""
    ref = next(iter(weights.values()))
    dt = L.F32 if str(ref.dtype) in ("float32", "torch.float32") else L.F64
    L_ = ref.shape[0]
    p = {k: (L.ptr(weights[k]) if k in weights else None) for k in ("G", "H", "B_trans", "B_euler")}
    L.check(L.load().sod_cqbem_write_cache(ctx.handle, folder.encode(), nV, L_, p["G"], p["H"], p["B_trans"],
                                           p["B_euler"], dt))


class HistoryBank:
    """Device-resident history convolution of one object (sod_history): G_k, -H_k (k = 1..K) as FP32
    or BF16 + per-row scales, a ring of the last K steps' vectors, b = sum G p - H u + B a."""

    def __init__(self, ctx: Context, nrow: int, ncol: int, K: int, R: int = 1, weight_dtype: int = L.F32):
        self.ctx, self.nrow, self.ncol, self.K, self.R = ctx, nrow, ncol, K, R
        self._h = ctypes.c_void_p()
        L.check(L.load().sod_history_create(ctx.handle, nrow, ncol, K, R, weight_dtype, ctypes.byref(self._h)))

    @staticmethod
    def _arr(x, dtype=np.float64):
        if hasattr(x, "data_ptr"):
            return x
        return np.ascontiguousarray(np.asarray(x, dtype=dtype))

    def set_weights(self, k: int, G, H) -> None:
        """G_k, H_k (nrow x ncol, float64 or float32; host arrays or CUDA tensors).  Device inputs are
        read in stream order on the context's stream, so they may be released right after the call
        when they were produced on that stream."""
        G, H = self._arr(G), self._arr(H)
        dt = L.F32 if (getattr(G, "dtype", None) in (np.float32,) or str(getattr(G, "dtype", "")) == "torch.float32") \
            else L.F64
        L.check(L.load().sod_history_set_weights(self._h, k, L.ptr(G), L.ptr(H), dt))

    def set_b(self, k: int, B) -> None:
        B = self._arr(B)
        L.check(L.load().sod_history_set_b(self._h, k, L.ptr(B)))

    def push(self, p, u, a=None) -> None:
        p, u = self._arr(p), self._arr(u)
        a = None if a is None else self._arr(a)
        L.check(L.load().sod_history_push(self._h, L.ptr(p), L.ptr(u), L.ptr(a) if a is not None else None))

    def convolve(self, out=None):
        if out is None:
            out = np.empty((self.nrow, self.R) if self.R > 1 else (self.nrow,), dtype=np.float64)
        L.check(L.load().sod_history_convolve(self._h, L.ptr(out)))
        return out

    def reset(self) -> None:
        L.check(L.load().sod_history_reset(self._h))

    def convolve_solve(self, solver: "Solver", out=None):
        """u = A^-1 b for the solver's A, with b this step's convolution (one device round trip)."""
        if out is None:
            out = np.empty((self.nrow, self.R) if self.R > 1 else (self.nrow,), dtype=np.float64)
        L.check(L.load().sod_history_convolve_solve(self._h, solver._h, L.ptr(out)))
        return out

    def set_engine(self, engine: int) -> None:
        """L.HISTORY_ENGINE_AUTO (tensor cores for BF16 banks and FP32 banks with R = 16), _CUDA_CORES or
        _TENSOR_CORES (FP32 banks there use a 3xTF32 split with FP32 accuracy).
        Switching engines empties the history ring."""
        L.check(L.load().sod_history_set_engine(self._h, engine))

    @property
    def weight_bytes(self) -> int:
        v = ctypes.c_int64()
        L.check(L.load().sod_history_bytes(self._h, ctypes.byref(v)))
        return int(v.value)

    @classmethod
    def compressed(cls, ctx: Context, nV: int, K: int, ratio: float) -> "HistoryBank":
        """Wavelet-compressed bank (sod_history_create_compressed): the reference's compressed
        history with CompressedMatrix<1> (Haar) at `ratio` (fraction of the 9 nV^2 entries kept)."""
        self = cls.__new__(cls)
        self.ctx, self.nrow, self.ncol, self.K, self.R = ctx, 3 * nV, 3 * nV, K, 1
        self._h = ctypes.c_void_p()
        L.check(L.load().sod_history_create_compressed(ctx.handle, nV, K, ratio, ctypes.byref(self._h)))
        return self

    def compressed_matrix(self, k: int, which: int):
        """(row_ptr, col, val) of the kept coefficients of G_k (which 0) or -H_k (which 1)."""
        nnz = ctypes.c_int64()
        L.check(L.load().sod_history_compressed_matrix(self._h, k, which, ctypes.byref(nnz), None, None, None))
        Np = 2
        while Np < self.nrow:
            Np *= 2
        rp = np.empty(2 * Np - 1, dtype=np.int32)
        col = np.empty(nnz.value, dtype=np.int32)
        val = np.empty(nnz.value, dtype=np.float64)
        L.check(L.load().sod_history_compressed_matrix(self._h, k, which, ctypes.byref(nnz), L.ptr(rp), L.ptr(col),
                                                       L.ptr(val)))
        return rp, col, val

    def write_cpmat(self, k: int, which: int, path: str) -> None:
        """The reference's .cpmat file of G_k (which 0) or -H_k (which 1)."""
        L.check(L.load().sod_history_write_cpmat(self._h, k, which, path.encode()))

    def close(self) -> None:
        if self._h:
            L.load().sod_history_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Server:
    """Request loop with continuous batching (sod_server): assembly requests create device-resident
    objects, step requests run their history convolution; completions carry per-request latency."""

    def __init__(self, device: int = 0, hbm_cap_bytes: int = 150 << 30, slots: int = 2, max_vertices: int = 2562):
        self._h = ctypes.c_void_p()
        L.check(L.load().sod_server_create(device, int(hbm_cap_bytes), slots, max_vertices, ctypes.byref(self._h)))
        self.n_of = {}

    def submit_assembly(self, mesh: SurfaceMesh, mat: Material, bdf: int, dt: float, N: int, order: int = 5,
                        subdiv: int = 1) -> int:
        V = np.ascontiguousarray(mesh.V, dtype=np.float64)
        F = np.ascontiguousarray(mesh.F, dtype=np.int32)
        rid = ctypes.c_int64()
        L.check(L.load().sod_server_submit_assembly(self._h, L.ptr(V), mesh.nV, L.ptr(F), mesh.nF, mat.E, mat.nu,
                                                    mat.rho, bdf, dt, N, order, subdiv, ctypes.byref(rid)))
        self.n_of[rid.value] = 3 * mesh.nV
        return rid.value

    def submit_step(self, obj: int, p, u) -> int:
        p = np.ascontiguousarray(p, dtype=np.float64)
        u = np.ascontiguousarray(u, dtype=np.float64)
        rid = ctypes.c_int64()
        L.check(L.load().sod_server_submit_step(self._h, obj, L.ptr(p), L.ptr(u), p.size, ctypes.byref(rid)))
        self.n_of[rid.value] = p.size
        return rid.value

    def poll(self, cap: int = 4096):
        ids = np.zeros(cap, dtype=np.int64)
        st = np.zeros(cap, dtype=np.int32)
        lat = np.zeros(cap, dtype=np.int64)
        n = ctypes.c_int()
        L.check(L.load().sod_server_poll(self._h, L.ptr(ids), L.ptr(st), L.ptr(lat), cap, ctypes.byref(n)))
        k = n.value
        return list(zip(ids[:k].tolist(), st[:k].tolist(), lat[:k].tolist()))

    def result(self, rid: int) -> np.ndarray:
        b = np.empty(self.n_of[rid], dtype=np.float64)
        L.check(L.load().sod_server_result(self._h, rid, L.ptr(b), b.size))
        return b

    def drain(self, timeout_s: float = 600.0) -> None:
        L.check(L.load().sod_server_drain(self._h, timeout_s))

    def close(self) -> None:
        if self._h:
            L.load().sod_server_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
