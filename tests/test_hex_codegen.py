"""The generated straight-line hex geometry (fierro_gb300/csrc/sgh_hex_geometry.cuh,
used by the element kernel) compiled as host C++ without contraction equals the
oracle's table-driven B matrix and volume bit for bit, and its divergence sums
and CFL minimum equal the reference's formulas evaluated term by term (with the
IEEE square d*d for the reference's pow(d, 2.0))."""
import ctypes as C
import math
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT

SHIM = r'''
#include <cstdint>
#include <cstring>
#define __device__
#define __forceinline__ inline
static inline long long okey(double d) { long long b; std::memcpy(&b, &d, 8); return b ^ ((b >> 63) & 0x7FFFFFFFFFFFFFFFLL); }
static inline double okey_decode(long long k) { long long b = k ^ ((k >> 63) & 0x7FFFFFFFFFFFFFFFLL); double d; std::memcpy(&d, &b, 8); return d; }
#include "sgh_hex_geometry.cuh"
extern "C" void geom(const double* x, const double* y, const double* z, const double* u, const double* v,
                     const double* w, double* bmat, double* out) {
  hex_geometry<true>(x, y, z, u, v, w, bmat, 1, 0, out[0], out[1], out[2], out[3], out[4]);
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
        out = np.zeros(5)
        geomlib.geom(*(a.ctypes.data for a in (x, y, z, u, v, w, bm, out)))
        B = orc.bmatrix(x, y, z)
        assert np.array_equal(bm.reshape(8, 3), B)
        assert out[0] == orc.vol_hex(x, y, z)
        for c, vv in enumerate((u, v, w)):
            s = vv[0] * B[0, c]
            for p in range(1, 8):
                s = s + vv[p] * B[p, c]
            assert out[1 + c] == s
        dist = []
        for a, b in pairs:
            dx, dy, dz = h[b, 0] - h[a, 0], h[b, 1] - h[a, 1], h[b, 2] - h[a, 2]
            dist.append(abs(math.sqrt((dx * dx + dy * dy) + dz * dz)))
        assert len(dist) == 28
        assert math.sqrt(out[4]) == min(dist)
