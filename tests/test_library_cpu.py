"""The C-ABI library builds, loads and exports every symbol include/sod_gb300.h declares; its
host-only entry points agree with the oracle.  No compute call is made without a GPU."""
import ctypes
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_symbols():
    txt = open(os.path.join(ROOT, "include", "sod_gb300.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(sod_[a-z0-9_]+)\s*\(", txt)))


def test_header_symbols_all_exported(sodlib):
    lib = sodlib.load()
    names = header_symbols()
    assert len(names) >= 14
    for n in names:
        assert hasattr(lib, n), f"{n} declared in include/sod_gb300.h but not exported"
    assert sorted(sodlib.declared_symbols()) == names, "ctypes signatures out of sync with the header"


def test_triangle_rules_match_oracle(sodlib, oracle):
    for order in (1, 2, 3, 4, 5, 7):
        np.testing.assert_array_equal(sodlib.triangle_rule(order), oracle.tri_rule(order))
    with pytest.raises(sodlib.SodError) as e:
        sodlib.triangle_rule(6)
    assert e.value.code == sodlib.SOD_ERR_INVALID_ARG


@pytest.mark.parametrize("bdf,dt,N", [(2, 0.01, 32), (1, 0.005, 16), (2, 1 / 200, 64), (2, 0.01, 5)])
def test_cq_frequencies_match_oracle(sodlib, oracle, bdf, dt, N):
    s_lib, R_lib, L_lib = sodlib.cq_frequencies(bdf, dt, N)
    s_or, R_or, L_or = oracle.cq_frequencies(bdf, dt, N)
    assert L_lib == L_or and abs(R_lib - R_or) < 1e-15
    assert np.max(np.abs(s_lib - s_or) / np.abs(s_or)) < 1e-13


def test_bad_arguments_are_rejected(sodlib):
    lib = sodlib.load()
    R = ctypes.c_double()
    L = ctypes.c_int()
    s = np.zeros(8)
    assert lib.sod_cq_frequencies(3, 0.01, 4, sodlib.ptr(s), ctypes.byref(R), ctypes.byref(L)) == sodlib.SOD_ERR_INVALID_ARG
    assert b"BDF" in lib.sod_last_error()
    assert lib.sod_cq_frequencies(2, -1.0, 4, sodlib.ptr(s), ctypes.byref(R), ctypes.byref(L)) == sodlib.SOD_ERR_INVALID_ARG
    assert lib.sod_context_synchronize(None) == sodlib.SOD_ERR_INVALID_ARG


def test_no_device_fails_loudly(sodlib):
    """Without a GPU the compute path refuses to start (there is no CPU fallback)."""
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    h = ctypes.c_void_p()
    rc = sodlib.load().sod_context_create(0, ctypes.byref(h))
    assert rc == sodlib.SOD_ERR_NO_DEVICE
    from surfaceonlydeformables_gb300.api import Context

    with pytest.raises(sodlib.SodError):
        Context(0)


def test_mat_file_format_roundtrip(sodlib, tmp_path):
    """sod_mat_write / sod_mat_read use Eigen::save_matrix's layout (include/matrix_io.hpp:14-61):
    int64 rows, int64 cols, row-major doubles (the reference's matrices are row-major)."""
    import numpy as np

    from surfaceonlydeformables_gb300 import api

    rng = np.random.default_rng(1)
    M = rng.normal(size=(7, 5))
    p = str(tmp_path / "M.mat")
    api.mat_write(None, p, M)
    raw = open(p, "rb").read()
    assert np.frombuffer(raw[:16], dtype=np.int64).tolist() == [7, 5]
    assert np.array_equal(np.frombuffer(raw[16:], dtype=np.float64).reshape(7, 5), M)
    assert np.array_equal(api.mat_read(None, p, 7, 5), M)
    api.mat_write(None, p, M.astype(np.float32))  # FP32 input is written as doubles
    assert np.array_equal(api.mat_read(None, p, 7, 5), M.astype(np.float32).astype(np.float64))
    with pytest.raises(sodlib.SodError):
        api.mat_read(None, p, 5, 7)  # wrong dimensions are rejected
    # a file whose header claims negative sizes, and one cut short, are rejected as well
    lib = sodlib.load()
    out = np.empty(35)
    neg = str(tmp_path / "neg.mat")
    with open(neg, "wb") as fh:
        fh.write(np.array([-7, -5], dtype=np.int64).tobytes() + np.zeros(35).tobytes())
    assert lib.sod_mat_read(None, neg.encode(), sodlib.ptr(out), -7, -5) == sodlib.SOD_ERR_INVALID_ARG
    cut = str(tmp_path / "cut.mat")
    with open(cut, "wb") as fh:
        fh.write(raw[:16 + 8 * 20])
    assert lib.sod_mat_read(None, cut.encode(), sodlib.ptr(out), 7, 5) == sodlib.SOD_ERR_INVALID_ARG
    assert b"truncated" in lib.sod_last_error()


@pytest.mark.parametrize("level,axes", [(2, (1.0, 1.0, 1.0)), (3, (1.4, 0.8, 1.1)), (4, (1.0, 1.0, 1.0)),
                                        (4, (0.7, 1.5, 1.0))])
def test_face_colouring_is_a_proper_capacity_colouring(sodlib, level, axes):
    """The scatter schedule (sod_face_colouring): no two faces of a colour share a vertex (the
    colour-ordered adds need no atomics), no colour above the CTA size, every colour used, the same
    result on every call; on the 2562-vertex spheres the capacity search reaches ceil(nF / T)."""
    from surfaceonlydeformables_gb300.meshes import make_icosphere_mesh

    m = make_icosphere_mesh(level, 0.1, axes=axes, seed=5)
    F = np.ascontiguousarray(m.F, dtype=np.int32)
    lib = sodlib.load()
    for cap in (32, 128, 256, 480, 512):
        col = np.empty(m.nF, dtype=np.int32)
        n = ctypes.c_int()
        assert lib.sod_face_colouring(sodlib.ptr(F), m.nF, m.nV, cap, sodlib.ptr(col), ctypes.byref(n)) == 0
        k = n.value
        assert col.min() == 0 and col.max() == k - 1
        counts = np.bincount(col, minlength=k)
        assert counts.min() >= 1 and counts.max() <= cap
        # faces sharing a vertex: every pair of faces in one vertex star has distinct colours
        for v in range(m.nV):
            star = col[np.nonzero((F == v).any(axis=1))[0]]
            assert len(np.unique(star)) == len(star), (cap, v)
        col2 = np.empty_like(col)
        lib.sod_face_colouring(sodlib.ptr(F), m.nF, m.nV, cap, sodlib.ptr(col2), ctypes.byref(n))
        np.testing.assert_array_equal(col, col2)
        if level == 4 and cap >= 480:
            assert k == -(-m.nF // cap), (cap, k)
    bad = np.array([[0, 1, 99]], dtype=np.int32)
    col = np.empty(1, dtype=np.int32)
    assert lib.sod_face_colouring(sodlib.ptr(bad), 1, 3, 32, sodlib.ptr(col), ctypes.byref(n)) == sodlib.SOD_ERR_INVALID_ARG


@pytest.mark.parametrize("fixture,keys", [("bunny_mesh.npz", ("V", "F")), ("cube_meshes.npz", ("V_cont", "F_cont")),
                                          ("cube_meshes.npz", ("V_disc", "F_disc"))])
def test_face_colouring_on_scene_meshes(sodlib, fixture, keys):
    """The reference's own scene meshes (irregular valence; the split cube has duplicated vertices
    along its traction discontinuities): proper capacity colourings, never below the lower bound
    max(ceil(nF / T), largest vertex valence); the bunny reaches that bound."""
    d = np.load(os.path.join(ROOT, "tests", "golden", fixture))
    V, F = d[keys[0]], np.ascontiguousarray(d[keys[1]], dtype=np.int32)
    nV, nF = len(V), len(F)
    valence = int(np.bincount(F.ravel(), minlength=nV).max())
    lib = sodlib.load()
    for cap in (128, 256, 512):
        col = np.empty(nF, dtype=np.int32)
        n = ctypes.c_int()
        assert lib.sod_face_colouring(sodlib.ptr(F), nF, nV, cap, sodlib.ptr(col), ctypes.byref(n)) == 0
        k = n.value
        counts = np.bincount(col, minlength=k)
        assert col.min() == 0 and col.max() == k - 1 and counts.min() >= 1 and counts.max() <= cap
        star_of = [[] for _ in range(nV)]
        for f, tri in enumerate(F):
            for v in tri:
                star_of[v].append(f)
        for v in range(nV):
            star = col[star_of[v]]
            assert len(np.unique(star)) == len(star), (cap, v)
        bound = max(-(-nF // cap), valence)
        assert k >= bound
        if fixture == "bunny_mesh.npz":
            assert k == bound, (cap, k, bound)


_COLOUR_CASES = ((2, 96), (3, 160), (3, 224), (4, 448))  # (icosphere level, capacity): not used above

_COLOUR_CHILD = r"""
import ctypes, sys
import numpy as np
sys.path.insert(0, sys.argv[1])
from surfaceonlydeformables_gb300 import _lib
from surfaceonlydeformables_gb300.meshes import make_icosphere_mesh
lib = _lib.load()
out = []
for level, cap in %r:
    m = make_icosphere_mesh(level, 0.1, seed=5)
    F = np.ascontiguousarray(m.F, dtype=np.int32)
    col = np.empty(m.nF, dtype=np.int32)
    n = ctypes.c_int()
    assert lib.sod_face_colouring(_lib.ptr(F), m.nF, m.nV, cap, _lib.ptr(col), ctypes.byref(n)) == 0
    out.append(col)
np.savez(sys.argv[2], *out)
"""


def test_face_colouring_same_across_processes_and_threads(sodlib, tmp_path):
    """The scatter's summation order follows the colouring, so it must not depend on the process or
    on the cache: a fresh process (cold cache) and eight concurrent callers in this one (cache misses
    racing on the same connectivity, then hits) give the same colours."""
    import subprocess
    import sys
    import threading

    from surfaceonlydeformables_gb300.meshes import make_icosphere_mesh

    out = tmp_path / "colours.npz"
    subprocess.run([sys.executable, "-c", _COLOUR_CHILD % (_COLOUR_CASES,), ROOT, str(out)], check=True,
                   timeout=600)
    ref = np.load(out)
    ref = [ref[f"arr_{t}"] for t in range(len(_COLOUR_CASES))]
    lib = sodlib.load()
    meshes = []
    for level, cap in _COLOUR_CASES:
        m = make_icosphere_mesh(level, 0.1, seed=5)
        meshes.append((np.ascontiguousarray(m.F, dtype=np.int32), m.nF, m.nV, cap))
    got = [[None] * len(meshes) for _ in range(8)]
    errors = []

    def worker(w):
        try:
            for t in range(len(meshes)):
                i = (t + w) % len(meshes)  # callers start on different meshes
                F, nF, nV, cap = meshes[i]
                col = np.empty(nF, dtype=np.int32)
                n = ctypes.c_int()
                rc = lib.sod_face_colouring(sodlib.ptr(F), nF, nV, cap, sodlib.ptr(col), ctypes.byref(n))
                got[w][i] = (rc, col)
        except Exception as e:  # reported below, on the test's thread
            errors.append(e)

    threads = [threading.Thread(target=worker, args=(w,)) for w in range(8)]
    for th in threads:
        th.start()
    for th in threads:
        th.join()
    assert not errors, errors
    for w in range(8):
        for i in range(len(meshes)):
            rc, col = got[w][i]
            assert rc == 0
            np.testing.assert_array_equal(col, ref[i], err_msg=f"caller {w}, case {_COLOUR_CASES[i]}")
