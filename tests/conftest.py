import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the libfierro_sgh kernels)")


def field_error(got: np.ndarray, ref: np.ndarray, floor: float = 1e-3) -> float:
    """Pointwise relative error with an absolute floor for near-zero values:
    max |got - ref| / max(|ref|, floor * max|ref|).  Values smaller than `floor`
    times the field's peak magnitude are compared at that scale."""
    got = np.asarray(got, dtype=np.float64)
    ref = np.asarray(ref, dtype=np.float64)
    scale = float(np.max(np.abs(ref))) if ref.size else 0.0
    if scale == 0.0:
        return float(np.max(np.abs(got))) if got.size else 0.0
    return float(np.max(np.abs(got - ref) / np.maximum(np.abs(ref), floor * scale)))


# Fields that are positive everywhere in every deck (density, pressure, energy,
# sound speed, volume, mass): the tight metric compares each value at its own
# scale.  The vector fields (positions on symmetry planes, velocities at rest)
# pass through zero and keep a floor.
POSITIVE_FIELDS = ("den", "pres", "sie", "sspd", "vol", "mass", "node_mass")
TIGHT_FLOOR = 1e-9


def field_error_tight(got: np.ndarray, ref: np.ndarray, key: str) -> float:
    """The tight parity metric: purely relative, max |got - ref| / |ref|, for the
    positive fields, so a quiescent cell (Sedov's 1e-10 background energy and
    pressure) is compared at its own scale; for positions and velocities the
    floor is 1e-9 of the field's peak instead of field_error's 1e-3."""
    got = np.asarray(got, dtype=np.float64)
    ref = np.asarray(ref, dtype=np.float64)
    if not ref.size:
        return 0.0
    if key in POSITIVE_FIELDS:
        return float(np.max(np.abs(got - ref) / np.maximum(np.abs(ref), 1e-300)))
    return field_error(got, ref, TIGHT_FLOOR)


def assert_fields_tight(got: dict, ref: dict, tol, keys=("coords", "vel", "den", "pres", "sie"), label: str = ""):
    """field_error_tight within `tol` (a number, or a dict field -> bound for
    the documented per-field bounds) for every key."""
    bad = {}
    for k in keys:
        t = tol[k] if isinstance(tol, dict) else tol
        e = field_error_tight(got[k], ref[k], k)
        if not e <= t:
            bad[k] = (e, t)
    assert not bad, "%s: fields over the tight bound (error, bound): %s" % (label, bad)


def assert_fields(got: dict, ref: dict, tol: float, keys=("coords", "vel", "den", "pres", "sie"),
                  floor: float = 1e-3, label: str = ""):
    bad = {}
    for k in keys:
        e = field_error(got[k], ref[k], floor)
        if not e <= tol:
            bad[k] = e
    assert not bad, "%s: fields over tolerance %g: %s" % (label, tol, bad)


def assert_bitwise(got: dict, ref: dict, keys, label: str = ""):
    bad = {k: int(np.sum(np.asarray(got[k]) != np.asarray(ref[k]))) for k in keys}
    bad = {k: v for k, v in bad.items() if v}
    assert not bad, "%s: values differing bit-for-bit: %s" % (label, bad)


def load_golden(name: str) -> dict:
    with np.load(os.path.join(GOLDEN, name + ".npz")) as z:
        return {k: z[k] for k in z.files}


@pytest.fixture(scope="session")
def oracle_built():
    from oracle import build_ref
    build_ref.build_oracle_lib()
    return True


@pytest.fixture(scope="session")
def lib_built():
    from fierro_gb300 import build
    build.build()
    return True
