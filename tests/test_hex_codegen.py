"""The generated straight-line hex geometry (fierro_gb300/csrc/sgh_hex_geometry.cuh,
used by the element kernel) compiled as host C++ without contraction equals the
oracle's table-driven B matrix and volume bit for bit and its divergence sums
equal the reference's formulas evaluated term by term; the screened CFL minimum
(sgh_cfl.cuh) equals the exhaustive FP64 minimum of the reference's squared
distances (with the IEEE square d*d for the reference's pow(d, 2.0))."""
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT

SHIM = r'''
#include <cmath>
#include <cstdint>
#include <cstring>
#define __device__
#define __forceinline__ inline
static inline long long __double_as_longlong(double d) { long long b; std::memcpy(&b, &d, 8); return b; }
static inline double __longlong_as_double(long long b) { double d; std::memcpy(&d, &b, 8); return d; }
static inline float __uint_as_float(unsigned u) { float f; std::memcpy(&f, &u, 4); return f; }
static inline int __ffs(int v) { return __builtin_ffs(v); }
using std::fabs; using std::sqrt;
#include "sgh_hex_geometry.cuh"
#include "sgh_cfl.cuh"
extern "C" void geom(const double* x, const double* y, const double* z, const double* u, const double* v,
                     const double* w, double* bmat, double* out) {
  hex_geometry(x, y, z, u, v, w, bmat, 1, 0, out[0], out[1], out[2], out[3]);
}
extern "C" void bmat_adj(const double* x, const double* y, const double* z, const double* bbar, double* out) {
  for (int i = 0; i < 24; ++i) out[i] = 0.0;
  hex_bmatrix_adjoint(x, y, z, bbar, out, out + 8, out + 16);
}
extern "C" double vol_only(const double* x, const double* y, const double* z) { return hex_volume(x, y, z); }
extern "C" double cfl_min(const double* x, const double* y, const double* z) {
  double sx[8], sy[8], sz[8];
  for (int l = 0; l < 8; ++l) { sx[l] = x[l]; sy[l] = y[l]; sz[l] = z[l]; }
  return cfl::min_d2(x, y, z, sx, sy, sz, 1);
}
'''


@pytest.fixture(scope="module")
def geomlib(tmp_path_factory):
    d = tmp_path_factory.mktemp("hexgen")
    src = d / "shim.cpp"
    src.write_text(SHIM)
    so = d / "libgeom.so"
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fPIC", "-shared", "-I",
                    os.path.join(ROOT, "fierro_gb300", "csrc"), str(src), "-o", str(so)], check=True)
    lib = C.CDLL(str(so))
    lib.geom.argtypes = [C.c_void_p] * 8
    lib.bmat_adj.argtypes = [C.c_void_p] * 5
    lib.vol_only.argtypes = [C.c_void_p] * 3
    lib.vol_only.restype = C.c_double
    lib.cfl_min.argtypes = [C.c_void_p] * 3
    lib.cfl_min.restype = C.c_double
    return lib


def test_generated_geometry_is_current():
    """The committed .cuh is what the generator writes from sgh_hex.h."""
    import importlib.util
    path = os.path.join(ROOT, "fierro_gb300", "csrc", "gen_hex_geometry.py")
    target = os.path.join(ROOT, "fierro_gb300", "csrc", "sgh_hex_geometry.cuh")
    before = open(target).read()
    spec = importlib.util.spec_from_file_location("gen_hex_geometry", path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    mod.main()
    assert open(target).read() == before


def test_generated_geometry_bitwise(geomlib, oracle_built):
    from oracle import orc
    rng = np.random.default_rng(7)
    base = np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0], [0, 0, 1], [1, 0, 1], [1, 1, 1], [0, 1, 1]], float)
    pairs = [(a, b) for gap in range(1, 8) for a in range(0, 8 - gap) for b in [a + gap]]
    for trial in range(300):
        scale = 10 ** rng.uniform(-3, 1)
        h = (base + rng.uniform(-0.2, 0.2, base.shape)) * scale + rng.uniform(-5, 5, 3)
        vel = rng.normal(size=(8, 3))
        x, y, z = (np.ascontiguousarray(h[:, d]) for d in range(3))
        u, v, w = (np.ascontiguousarray(vel[:, d]) for d in range(3))
        bm = np.zeros(24)
        out = np.zeros(4)
        geomlib.geom(*(a.ctypes.data for a in (x, y, z, u, v, w, bm, out)))
        B = orc.bmatrix(x, y, z)
        assert np.array_equal(bm.reshape(8, 3), B)
        assert out[0] == orc.vol_hex(x, y, z)
        for c, vv in enumerate((u, v, w)):
            s = vv[0] * B[0, c]
            for p in range(1, 8):
                s = s + vv[p] * B[p, c]
            assert out[1 + c] == s


PAIRS = [(a, b) for gap in range(1, 8) for a in range(0, 8 - gap) for b in [a + gap]]


def exact_min_d2(h):
    best = None
    for a, b in PAIRS:
        dx, dy, dz = h[b, 0] - h[a, 0], h[b, 1] - h[a, 1], h[b, 2] - h[a, 2]
        d2 = (dx * dx + dy * dy) + dz * dz
        best = d2 if best is None else min(best, d2)
    return best


def _cfl(lib, h):
    x, y, z = (np.ascontiguousarray(h[:, d]) for d in range(3))
    return lib.cfl_min(x.ctypes.data, y.ctypes.data, z.ctypes.data)


def test_cfl_screening_is_exact(geomlib):
    """The FP32-screened CFL minimum equals the exhaustive FP64 minimum bit for bit:
    jittered hexes over many scales and offsets, exact cubes (12 tied edges) far
    from the origin, near-ties, coincident nodes, and coordinates outside the
    screening's range (full FP64 path)."""
    rng = np.random.default_rng(11)
    base = np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0], [0, 0, 1], [1, 0, 1], [1, 1, 1], [0, 1, 1]], float)
    cases = []
    for _ in range(3000):
        scale = 10 ** rng.uniform(-6, 3)
        off = rng.uniform(-1, 1, 3) * 10 ** rng.uniform(-3, 4)
        cases.append((base + rng.uniform(-0.2, 0.2, base.shape)) * scale + off)
    for _ in range(500):
        h = 10 ** rng.uniform(-4, 0)
        cases.append(base * h + rng.uniform(0, 1e3, 3))        # exact ties, large offset
        k = base.copy() * h + rng.uniform(0, 2, 3)
        k[1, 0] = np.nextafter(k[1, 0], np.inf)                 # 1-ulp near-tie
        cases.append(k)
        k = base.copy() * h
        k[6] = k[5]                                             # coincident nodes
        cases.append(k)
    cases.append(base * 2.0 ** 70)                              # outside [2^-60, 2^60]
    cases.append(base * 2.0 ** -70)
    cases.append(base * 1e-7)                                   # M < 2^-20
    for h in cases:
        got = _cfl(geomlib, h)
        assert got == exact_min_d2(h), h


def test_bmatrix_adjoint(geomlib, oracle_built):
    """hex_bmatrix_adjoint (the adjoint's corner-normal reverse) equals the
    gradient of sum(Bbar * B(x)): B is quadratic in the coordinates, so a central
    difference is exact up to rounding."""
    from oracle import orc
    rng = np.random.default_rng(11)
    base = np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0], [0, 0, 1], [1, 0, 1], [1, 1, 1], [0, 1, 1]], float)
    for trial in range(20):
        X = base + rng.uniform(-0.25, 0.25, base.shape)
        bbar = rng.normal(size=24)
        cols = [np.ascontiguousarray(X[:, d]) for d in range(3)]
        out = np.zeros(24)
        geomlib.bmat_adj(cols[0].ctypes.data, cols[1].ctypes.data, cols[2].ctypes.data, bbar.ctypes.data,
                         out.ctypes.data)
        h = 1e-3
        fd = np.zeros(24)
        for d in range(3):
            for p in range(8):
                Xp, Xm = X.copy(), X.copy()
                Xp[p, d] += h
                Xm[p, d] -= h
                Bp = orc.bmatrix(*[Xp[:, k] for k in range(3)]).ravel()
                Bm = orc.bmatrix(*[Xm[:, k] for k in range(3)]).ravel()
                fd[d * 8 + p] = (np.dot(bbar, Bp) - np.dot(bbar, Bm)) / (2 * h)
        assert np.max(np.abs(out - fd)) <= 1e-10 * max(1.0, np.max(np.abs(fd))), trial


def test_volume_gradient_is_bmatrix(oracle_built):
    """dV/dx_p = B_p for the exact hex volume (the adjoint's volume reverse)."""
    from oracle import orc
    rng = np.random.default_rng(12)
    base = np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0], [0, 0, 1], [1, 0, 1], [1, 1, 1], [0, 1, 1]], float)
    for trial in range(10):
        X = base + rng.uniform(-0.25, 0.25, base.shape)
        B = orc.bmatrix(*[X[:, k] for k in range(3)])
        h = 1e-5
        for p in range(8):
            for d in range(3):
                Xp, Xm = X.copy(), X.copy()
                Xp[p, d] += h
                Xm[p, d] -= h
                g = (orc.vol_hex(*[Xp[:, k] for k in range(3)]) - orc.vol_hex(*[Xm[:, k] for k in range(3)])) / (2 * h)
                assert abs(g - B[p, d]) <= 1e-8, (trial, p, d)


def test_generated_volume_alone_bitwise(geomlib, oracle_built):
    """hex_volume (the set-up kernel's volume) equals the oracle's get_vol_hex bit for bit."""
    from oracle import orc
    rng = np.random.default_rng(13)
    base = np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0], [0, 0, 1], [1, 0, 1], [1, 1, 1], [0, 1, 1]], float)
    for trial in range(300):
        X = (base + rng.uniform(-0.2, 0.2, base.shape)) * 10 ** rng.uniform(-3, 1) + rng.uniform(-5, 5, 3)
        cols = [np.ascontiguousarray(X[:, d]) for d in range(3)]
        a = geomlib.vol_only(*[c.ctypes.data for c in cols])
        b = orc.vol_hex(*cols)
        assert a == b, (trial, a, b)
