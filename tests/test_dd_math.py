"""Accuracy of the double-float (float pair) math used by the singular quadrature kernels,
checked on the host build of the same header against mpmath at 40 digits.  The bound, 4e-14
relative (about 16 ulp of the 48-bit format), leaves room below the 1e-10 gate of the singular
passes."""
import ctypes
import os
import subprocess

import numpy as np
import pytest

mp = pytest.importorskip("mpmath")
mp.mp.dps = 40

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "..", "surfaceonlydeformables_gb300", "csrc")
TOL = 4e-14


@pytest.fixture(scope="module")
def lib(tmp_path_factory):
    out = tmp_path_factory.mktemp("dd") / "libdd_harness.so"
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fPIC", "-shared", "-I", CSRC,
                    os.path.join(HERE, "native", "dd_harness.cpp"), "-o", str(out)], check=True)
    return ctypes.CDLL(str(out))


def P(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def call(lib, name, *arrays, n):
    getattr(lib, name)(*[P(a) for a in arrays], ctypes.c_int(n))


def test_exp(lib):
    rng = np.random.default_rng(1)
    x = np.concatenate([rng.uniform(-69, 80, 4000), rng.uniform(-1e-3, 1e-3, 500), [0.0, -1e-30, 1.0, -1.0]])
    xin, out = np.empty_like(x), np.empty_like(x)
    call(lib, "dd_exp_eval", x, xin, out, n=len(x))
    err = max(abs(float((mp.mpf(o) - mp.exp(mp.mpf(v))) / mp.exp(mp.mpf(v)))) for v, o in zip(xin, out))
    assert err <= TOL, err


def test_sincos(lib):
    rng = np.random.default_rng(2)
    x = np.concatenate([rng.uniform(-390, 390, 3000), rng.uniform(-4, 4, 2000), [0.0, 1e-9, np.pi / 2]])
    xin, s, c = np.empty_like(x), np.empty_like(x), np.empty_like(x)
    call(lib, "dd_sincos_eval", x, xin, s, c, n=len(x))
    # absolute error (the functions are bounded by 1)
    es = max(abs(float(mp.mpf(o) - mp.sin(mp.mpf(v)))) for v, o in zip(xin, s))
    ec = max(abs(float(mp.mpf(o) - mp.cos(mp.mpf(v)))) for v, o in zip(xin, c))
    assert es <= TOL and ec <= TOL, (es, ec)


def test_sqrt(lib):
    rng = np.random.default_rng(4)
    x = rng.uniform(0.5, 2, 2000) * 10.0 ** rng.integers(-30, 30, 2000)
    xin, out = np.empty_like(x), np.empty_like(x)
    call(lib, "dd_sqrt_eval", x, xin, out, n=len(x))
    err = max(abs(float((mp.mpf(o) - mp.sqrt(mp.mpf(v))) / mp.sqrt(mp.mpf(v)))) for v, o in zip(xin, out))
    assert err <= TOL, err


def test_recip_and_fma(lib):
    rng = np.random.default_rng(3)
    x = rng.uniform(0.5, 2, 2000) * 10.0 ** rng.integers(-20, 20, 2000) * rng.choice([-1, 1], 2000)
    xin, out = np.empty_like(x), np.empty_like(x)
    call(lib, "dd_recip_eval", x, xin, out, n=len(x))
    err = max(abs(float((mp.mpf(o) - 1 / mp.mpf(v)) * mp.mpf(v))) for v, o in zip(xin, out))
    assert err <= TOL, err
    a, b, c = rng.normal(size=(3, 2000))
    abc, out = np.empty(3 * 2000), np.empty(2000)
    call(lib, "dd_fma_eval", a, b, c, abc, out, n=2000)
    abc = abc.reshape(-1, 3)
    err = max(abs(float(mp.mpf(o) - (mp.mpf(p[0]) * mp.mpf(p[1]) + mp.mpf(p[2]))))
              / max(1.0, abs(p[0] * p[1]) + abs(p[2])) for p, o in zip(abc, out))
    assert err <= TOL, err


def _psi_ref(z):
    z = mp.mpc(z)
    return ((1 + z) * mp.exp(-z) - 1) / z ** 2


@pytest.mark.parametrize("scale", [1e-4, 0.03, 0.06, 0.12, 1.0, 30.0])
def test_psi_and_cexp(lib, scale):
    rng = np.random.default_rng(int(scale * 1e4) + 7)
    n = 1500
    mag = scale * rng.uniform(0.5, 1.5, n)
    ang = rng.uniform(-np.pi / 2, np.pi / 2, n)  # Re z >= 0 as in e^{-s r / c}
    z = np.stack([mag * np.cos(ang), mag * np.sin(ang)], 1).ravel()
    zin, out = np.empty_like(z), np.empty_like(z)
    call(lib, "dd_cexp_neg_eval", z, zin, out, n=n)
    err = max(abs(complex(mp.mpc(o[0], o[1]) - mp.exp(-mp.mpc(v[0], v[1]))))
              / abs(complex(mp.exp(-mp.mpc(v[0], v[1])))) for v, o in zip(zin.reshape(-1, 2), out.reshape(-1, 2)))
    assert err <= TOL, ("cexp", err)
    call(lib, "dd_psi_eval", z, zin, out, n=n)
    err = max(abs(complex(mp.mpc(o[0], o[1]) - _psi_ref(mp.mpc(v[0], v[1])))) / abs(complex(_psi_ref(mp.mpc(v[0], v[1]))))
              for v, o in zip(zin.reshape(-1, 2), out.reshape(-1, 2)))
    # the closed form loses ~2 eps/|z|^2 just above the series threshold |z| = 0.1
    assert err <= (3e-12 if 0.06 <= scale < 0.2 else TOL * 10), ("psi", err)
