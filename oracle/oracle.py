"""ctypes front end of the CPU oracle (oracle/sod_oracle.cpp).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and bench.py's CPU
baseline / reference legs.  The product package never imports this module.
PARITY UNPINNED: see the header of sod_oracle.cpp.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libsod_oracle.so")
_lib = None

KIND = {"G": 0, "H": 1, "B_trans": 2, "B_angular": 3}
FP64, MIXED, LITERAL64 = 0, 1, 3  # accuracy oracle, reference-mixed baseline, FP64 with the literal formulas


def build(force: bool = False) -> str:
    """Compile the oracle with the committed Makefile (g++ -O3 -fopenmp)."""
    src = os.path.join(_HERE, "sod_oracle.cpp")
    if force or not os.path.exists(_LIB_PATH) or os.path.getmtime(_LIB_PATH) < os.path.getmtime(src):
        subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        _lib = ctypes.CDLL(_LIB_PATH)
        d, i, l, p = ctypes.c_double, ctypes.c_int, ctypes.c_long, ctypes.c_void_p
        _lib.oracle_collocation.argtypes = [i, i, p, i, p, i, p, p, d, d, d, d, d, i, i, i, i, p, i, i, p]
        _lib.oracle_galerkin.argtypes = [i, i, p, i, p, i, p, p, d, d, d, d, d, i, i, i, i, p, i, i, p]
        _lib.oracle_inverse_transform.argtypes = [i, i, d, p, l, p]
        _lib.oracle_cq_frequencies.argtypes = [i, d, i, p, p, p]
        _lib.oracle_c_matrix_collocation.argtypes = [p, i, p, i, p, d, p, p]
        _lib.oracle_c_matrix_galerkin.argtypes = [p, i, p, i, p]
        _lib.oracle_elastostatic.argtypes = [i, i, p, i, p, i, p, d, d, i, i, i, i, p]
        _lib.oracle_rigid_modes.argtypes = [p, i, p, i, p]
        _lib.oracle_tri_rule.argtypes = [i, p]
        _lib.oracle_set_threads.argtypes = [i]
    return _lib


def _ptr(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def set_threads(n: int) -> int:
    return lib().oracle_set_threads(int(n))


def tri_rule(order: int) -> np.ndarray:
    out = np.zeros((13, 4))
    n = lib().oracle_tri_rule(order, _ptr(out))
    return out[:n]


def cq_frequencies(bdf: int, dt: float, N: int):
    s = np.zeros(2 * (N + 1))
    R = ctypes.c_double()
    L = ctypes.c_int()
    lam = lib().oracle_cq_frequencies(bdf, dt, N, _ptr(s), ctypes.byref(R), ctypes.byref(L))
    return s[: 2 * lam].view(np.complex128).copy(), R.value, L.value


def _ncols(kind: int, nV: int) -> int:
    return 3 * nV if kind <= 1 else (3 if kind == 2 else 9)


def _assemble(fn, kind, mesh, mat, s, order, subdiv, sorder, ssub, rows, parts, mode, vmap):
    kind = KIND.get(kind, kind)
    rows_a = None if rows is None else np.ascontiguousarray(rows, dtype=np.int32)
    nr = mesh.nV if rows_a is None else len(rows_a)
    out = np.zeros((3 * nr, _ncols(kind, mesh.nV)), dtype=np.complex128)
    vm = None if vmap is None else np.ascontiguousarray(vmap, dtype=np.int32)
    rc = fn(kind, mode, _ptr(mesh.V), mesh.nV, _ptr(mesh.F), mesh.nF, _ptr(mesh.N), _ptr(vm),
            mat.c1, mat.c2, mat.rho, float(np.real(s)), float(np.imag(s)), order, subdiv, sorder, ssub,
            _ptr(rows_a), nr, parts, _ptr(out))
    if rc:
        raise ValueError(f"oracle rejected the arguments (code {rc})")
    return out


def collocation(kind, mesh, mat, s, order=5, subdiv=1, sorder=None, ssub=None, rows=None, parts=3,
                mode=FP64, vmap=None) -> np.ndarray:
    """Rows (3 per listed vertex) of U/P (3V cols), B_trans (3 cols) or B_angular (9 cols, [j][k])."""
    return _assemble(lib().oracle_collocation, kind, mesh, mat, s, order, subdiv,
                     sorder or order, ssub or subdiv, rows, parts, mode, vmap)


def galerkin(kind, mesh, mat, s, order=5, subdiv=1, sorder=5, ssub=1, rows=None, parts=3, mode=FP64,
             vmap=None) -> np.ndarray:
    return _assemble(lib().oracle_galerkin, kind, mesh, mat, s, order, subdiv, sorder, ssub, rows, parts,
                     mode, vmap)


def inverse_transform(Xhat: np.ndarray, L: int, R: float) -> np.ndarray:
    """Xhat: (Lambda, ...) complex -> (L, ...) real time-domain weights."""
    X = np.ascontiguousarray(Xhat, dtype=np.complex128)
    M = int(np.prod(X.shape[1:]))
    out = np.zeros((L,) + X.shape[1:], dtype=np.float64)
    rc = lib().oracle_inverse_transform(X.shape[0], L, R, _ptr(X), M, _ptr(out))
    if rc:
        raise ValueError("inverse transform: nfreq must equal L//2 + 1")
    return out


def c_matrix_collocation(mesh, nu: float, vmap=None) -> np.ndarray:
    out = np.zeros((3 * mesh.nV, 3))
    vm = None if vmap is None else np.ascontiguousarray(vmap, dtype=np.int32)
    lib().oracle_c_matrix_collocation(_ptr(mesh.V), mesh.nV, _ptr(mesh.F), mesh.nF, _ptr(mesh.N), nu, _ptr(vm),
                                      _ptr(out))
    return out


def c_matrix_galerkin(mesh) -> np.ndarray:
    out = np.zeros((3 * mesh.nV, 3 * mesh.nV))
    lib().oracle_c_matrix_galerkin(_ptr(mesh.V), mesh.nV, _ptr(mesh.F), mesh.nF, _ptr(out))
    return out


def elastostatic(kind, mesh, mat, galerkin=False, order=5, subdiv=1, sorder=None, ssub=None) -> np.ndarray:
    kind = KIND.get(kind, kind)
    out = np.zeros((3 * mesh.nV, 3 * mesh.nV))
    rc = lib().oracle_elastostatic(kind, int(galerkin), _ptr(mesh.V), mesh.nV, _ptr(mesh.F), mesh.nF,
                                   _ptr(mesh.N), mat.nu, mat.mu, order, subdiv, sorder or min(order, 5),
                                   ssub or subdiv, _ptr(out))
    if rc:
        raise ValueError("elastostatic: bad quadrature order")
    return out


def rigid_modes(mesh) -> np.ndarray:
    T = np.zeros((6, 3 * mesh.nV))
    lib().oracle_rigid_modes(_ptr(mesh.V), mesh.nV, _ptr(mesh.F), mesh.nF, _ptr(T))
    return T


def b_euler(B_angular_n: np.ndarray) -> np.ndarray:
    """B_euler(i,j) = B_ang(i,(j+2)%3,(j+1)%3) - B_ang(i,(j+1)%3,(j+2)%3)
    (src/elastodynamics_cqbem_matrix_collection.cpp:296-301).  B_angular_n: (3V, 3, 3)."""
    out = np.zeros(B_angular_n.shape[:2])
    for j in range(3):
        out[:, j] = B_angular_n[:, (j + 2) % 3, (j + 1) % 3] - B_angular_n[:, (j + 1) % 3, (j + 2) % 3]
    return out


def b_angular_shift(B_ang_n: np.ndarray, B_trans_n: np.ndarray, V: np.ndarray, cm: np.ndarray) -> np.ndarray:
    """B_ang(3v+i, j, k) += B_trans(3v+i, j) * (x_v - cm)_k  (src/elastodynamics_cqbem_B_angular.cu:167-175)."""
    d = np.repeat(V - cm[None, :], 3, axis=0)
    return B_ang_n + B_trans_n[:, :, None] * d[:, None, :]


def history_convolution(G, H, p_hist, u_hist, B=None, a_hist=None):
    """b = sum_{k=1..K} (G_k p_{n-k} - H_k u_{n-k} [+ B_k a_{n-k}])  (src/elastodynamics_cqbem_object.cpp:44-48;
    H is negated at load, src/elastodynamics_cqbem_matrix_collection.cpp:140).
    G, H: (N+1, 3V, 3V); p_hist/u_hist: (K, 3V[, R]) with index 0 the most recent step (n-1)."""
    K = p_hist.shape[0]
    b = np.zeros((G.shape[1],) + p_hist.shape[2:], dtype=np.float64)
    for k in range(1, K + 1):
        b += G[k].astype(np.float64) @ p_hist[k - 1] - H[k].astype(np.float64) @ u_hist[k - 1]
        if B is not None:
            b += B[k] @ a_hist[k - 1]
    return b


def cod_solve(B: np.ndarray, Y: np.ndarray) -> np.ndarray:
    """Minimum-norm least squares X = B^+ Y by the complete orthogonal decomposition, the algorithm
    of Eigen::CompleteOrthogonalDecomposition that the reference's B_trans_inv / B_euler_inv use
    (include/elastodynamics_cqbem_matrix_collection.hpp:43, src/elastodynamics_cqbem_matrix_collection.cpp:
    184-191): Householder QR with column pivoting (largest remaining column norm, first on ties),
    rank = leading |R_ii| > eps * min(m, k) * max |R_ii|, for rank r < k the R12 block removed by
    Householder reflections from the right, then x = P Z^T [T^-1 (Q^T y)_{1..r}; 0].  B: (m, k), m >= k."""
    A = np.array(B, dtype=np.float64)
    m, k = A.shape
    Y2 = np.asarray(Y, dtype=np.float64).reshape(m, -1).copy()
    perm = list(range(k))
    R = np.zeros((k, k))
    for j in range(k):
        norms = (A[j:, j:] ** 2).sum(axis=0)
        p = j + int(np.argmax(norms))
        A[:, [j, p]] = A[:, [p, j]]
        perm[j], perm[p] = perm[p], perm[j]
        x = A[j:, j].copy()
        sigma = float((x[1:] ** 2).sum())
        if sigma <= np.finfo(float).tiny:
            beta, tau, v = x[0], 0.0, np.zeros_like(x)
        else:
            beta = np.sqrt(x[0] ** 2 + sigma) * (-1.0 if x[0] >= 0 else 1.0)
            v = x / (x[0] - beta)
            tau = (beta - x[0]) / beta
        v[0] = 1.0
        A[j:, j] = 0.0
        A[j, j] = beta
        A[j:, j + 1:] -= tau * np.outer(v, v @ A[j:, j + 1:])
        Y2[j:] -= tau * np.outer(v, v @ Y2[j:])  # Q^T y, one reflector at a time
    R = np.triu(A[:k, :k])
    d = np.abs(np.diag(R))
    thr = d.max() * np.finfo(float).eps * k
    r = 0
    while r < k and d[r] > thr:
        r += 1
    X = np.zeros((k, Y2.shape[1]))
    if r == 0:
        return X.reshape((k,) + np.shape(Y)[1:])
    W = R[:r].copy()
    zs = []
    for i in range(r - 1, -1, -1):  # [R11 R12] = [T 0] Z
        idx = [i] + list(range(r, k))
        x = W[i, idx].copy()
        sigma = float((x[1:] ** 2).sum())
        if sigma <= np.finfo(float).tiny:
            zs.append((idx, 0.0, np.zeros_like(x)))
            continue
        beta = np.sqrt(x[0] ** 2 + sigma) * (-1.0 if x[0] >= 0 else 1.0)
        v = x / (x[0] - beta)
        v[0] = 1.0
        tau = (beta - x[0]) / beta
        W[:i + 1, idx] -= tau * np.outer(W[:i + 1, idx] @ v, v)
        zs.append((idx, tau, v))
    z = np.zeros((k, Y2.shape[1]))
    z[:r] = np.linalg.solve(np.triu(W[:r, :r]), Y2[:r])  # T^-1 c
    for idx, tau, v in reversed(zs):  # Z^T = H_{r-1} ... H_0: H_0 first
        z[idx] -= tau * np.outer(v, v @ z[idx])
    X[perm] = z
    return X.reshape((k,) + np.shape(Y)[1:])


def elastostatic_u_p(H: np.ndarray, G: np.ndarray, T: np.ndarray) -> np.ndarray:
    """u_p of ElastostaticsBEMMatrixCollection::init (src/elastostatics_bem_matrix_collection.cpp:58-89):
    H' = H^T H + (tr H / 3V)^2 T^T T, G' = H^T G (I - A^T (A A^T)^-1 A) with A = T, u_p = H'^-1 G'
    (the reference factors the symmetric H' by LDL^T; here LAPACK's symmetric-indefinite LDL^T solve)."""
    import scipy.linalg as sl

    n = H.shape[0]
    Hr = H.T @ H + (np.trace(H) / n) ** 2 * (T.T @ T)
    Gp = H.T @ G @ (np.eye(n) - T.T @ np.linalg.solve(T @ T.T, T))
    return sl.solve(Hr, Gp, assume_a="sym")


# ---- wavelet-compressed history (Haar, the reference's CompressedMatrix<1>) ----------------------
HAAR = 0.70710678118654752440  # M_SQRT1_2: h = (HAAR, HAAR), g = (HAAR, -HAAR) (include/wavelets.hpp:15-17)


def _haar_perm(nV: int) -> np.ndarray:
    """Permuted position of dof i: (i / 3) + (i % 3) nV (src/elastics_bem_matrix_collection.cpp:25-29)."""
    i = np.arange(3 * nV)
    return i // 3 + (i % 3) * nV


def _pow2(N: int) -> int:
    return 1 << max(1, int(np.ceil(np.log2(N))))


def wavelet_compress(M: np.ndarray, nV: int, ratio: float, sign: float = 1.0):
    """CompressedMatrix<1>(P (sign M) P^T, ratio) (include/wavelets.hpp:163-226, 402-420): the Haar
    non-standard form of the zero-padded permuted matrix (alpha = gg, beta = gh, gamma = hg blocks
    per level, the last scale coefficient at (2Np-3, 2Np-3)), keeping the (int)(N^2 ratio) entries of
    largest magnitude (all nonzero entries if that is <= 0).  Sums in the reference's order (k outer,
    m inner; (f_k f_m) s added to a running sum from 0).  Ties at the threshold are kept in (row,
    column) order (the reference's heap keeps an arbitrary subset of them).
    Returns (row_ptr, col, val) of the (2Np-2)^2 matrix, entries sorted by (row, column)."""
    N = 3 * nV
    Np = _pow2(N)
    sig = _haar_perm(nV)
    S = np.zeros((Np, Np))
    S[np.ix_(sig, sig)] = sign * np.asarray(M, dtype=np.float64)
    h, g = (HAAR, HAAR), (HAAR, -HAAR)

    def comb(fk, fm, s00, s01, s10, s11):
        a = 0.0 + (fk[0] * fm[0]) * s00
        a = a + (fk[0] * fm[1]) * s01
        a = a + (fk[1] * fm[0]) * s10
        return a + (fk[1] * fm[1]) * s11

    vals, cols, counts = [], [], []
    size, offset = Np // 2, 0
    while size >= 1:
        q = (S[0::2, 0::2], S[0::2, 1::2], S[1::2, 0::2], S[1::2, 1::2])
        alpha, beta, gamma, new_s = comb(g, g, *q), comb(g, h, *q), comb(h, g, *q), comb(h, h, *q)
        vals.append(np.hstack([alpha, beta]).ravel())
        cols.append(np.tile(offset + np.arange(2 * size), size))
        counts += [2 * size] * size
        vals.append(gamma.ravel())
        cols.append(np.tile(offset + np.arange(size), size))
        counts += [size] * size
        offset += 2 * size
        size //= 2
        S = new_s
    vals.append(np.array([S[0, 0]]))
    cols.append(np.array([offset - 1]))
    counts[-1] += 1  # the last gamma row also holds the final scale coefficient
    v = np.concatenate(vals)
    c = np.concatenate(cols)
    rows = np.repeat(np.arange(len(counts)), counts)
    a = np.abs(v)
    keep = int(N * N * ratio)
    if keep <= 0 or np.count_nonzero(a) <= keep:
        sel = a > 0
    else:
        t = np.partition(a, a.size - keep)[a.size - keep]  # keep-th largest magnitude
        sel = a > t
        eq = np.flatnonzero(a == t)
        sel[eq[:keep - int(sel.sum())]] = True
    L = 2 * Np - 2
    row_ptr = np.zeros(L + 1, dtype=np.int64)
    np.add.at(row_ptr, rows[sel] + 1, 1)
    return np.cumsum(row_ptr), c[sel].astype(np.int64), v[sel]


def wavelet_vector(x: np.ndarray, nV: int) -> np.ndarray:
    """CompressedVector<1>(P x) (include/wavelets.hpp:228-256, 383-399): per level the detail (g)
    then the scale (h) coefficients, 2Np-2 values."""
    N = 3 * nV
    Np = _pow2(N)
    s = np.zeros(Np)
    s[_haar_perm(nV)] = x
    out = np.zeros(2 * Np - 2)
    size, offset = Np // 2, 0
    while size >= 1:
        a, b = s[0::2], s[1::2]
        d = (0.0 + HAAR * a) + (-HAAR) * b
        ns = (0.0 + HAAR * a) + HAAR * b
        out[offset:offset + size] = d
        out[offset + size:offset + 2 * size] = ns
        s = ns
        offset += 2 * size
        size //= 2
    return out


def wavelet_reconstruct(y: np.ndarray, nV: int) -> np.ndarray:
    """CompressedMatrixVectorProduct<1> -> vector (include/wavelets.hpp:258-283, 372-376), then the
    inverse permutation: result[i] = reconstructed[(i / 3) + (i % 3) nV]."""
    Np = (len(y) + 2) // 2
    res = np.zeros(Np)
    size, offset = 1, -2
    while size <= Np // 2:
        base = 2 * Np - 2 + offset
        d = y[base:base + size]
        s = y[base + size:base + 2 * size] + res[:size]
        res[:2 * size] = 0.0
        res[0:2 * size:2] = 0.0 + (HAAR * s + HAAR * d)
        res[1:2 * size:2] = 0.0 + (HAAR * s + (-HAAR) * d)
        offset -= 4 * size
        size *= 2
    return res[_haar_perm(nV)]


def wavelet_history_convolution(Gc, Hc, p_hist, u_hist, nV, B=None, a_hist=None):
    """Compressed history of ElastodynamicsCQBEMObject::estimate_next_state
    (src/elastodynamics_cqbem_object.cpp:31-41): b = P^T reconstruct(sum_k D(-H_k) w(u_{n-k}) +
    D(G_k) w(p_{n-k})) + sum_k B_k a_{n-k}.  Gc[k], Hc[k] (k = 1..K): wavelet_compress of G_k and of
    H_k with sign -1; p_hist/u_hist: (K, 3V), index 0 the most recent step."""
    import scipy.sparse as sp

    N = 3 * nV
    Np = _pow2(N)
    L = 2 * Np - 2
    y = np.zeros(L)
    for k in range(1, p_hist.shape[0] + 1):
        for D, x in ((Hc[k], u_hist[k - 1]), (Gc[k], p_hist[k - 1])):
            y += sp.csr_matrix((D[2], D[1], D[0]), shape=(L, L)) @ wavelet_vector(x, nV)
    b = wavelet_reconstruct(y, nV)
    if B is not None:
        for k in range(1, p_hist.shape[0] + 1):
            b = b + B[k] @ a_hist[k - 1]
    return b
