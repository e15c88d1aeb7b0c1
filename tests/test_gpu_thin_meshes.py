"""Meshes one element thick, down to a single element (hex and 2D-RZ), on the
GPU against the restatement: the device set-up (Morton order, corner and neighbour lists,
boundary masks of a box whose every node is on the surface) and the cycle with a
lone element's limiter.  Exact mode bit for bit through both transfer paths; the
FMA mode within the one-cycle and full-run gates."""
import numpy as np
import pytest

from conftest import assert_bitwise, assert_fields, assert_fields_tight
from decks import THIN_SHAPES, THIN_SHAPES_RZ, thin_deck

pytestmark = pytest.mark.gpu

FIELDS = ("coords", "vel", "den", "pres", "sie", "sspd", "vol", "corner_force", "div", "node_mass")
GATED = ("coords", "vel", "den", "pres", "sie")


def _gpu(prob, cycles, fp_mode):
    from fierro_gb300 import sgh
    with sgh.SGHSolver(prob, fp_mode=fp_mode) as s:
        s.set_state(sgh.setup(prob))
        s.run(cycles)
        out = s.get_state()
        t = s.time()
    g = {"coords": out["node_coords"][1], "vel": out["node_vel"][1], "den": out["elem_den"],
         "pres": out["elem_pres"], "sie": out["elem_sie"][1], "sspd": out["elem_sspd"], "vol": out["elem_vol"],
         "corner_force": out["corner_force"], "div": out["elem_div"], "node_mass": out["node_mass"]}
    return g, t


@pytest.mark.parametrize("staged", ["0", "1"])
@pytest.mark.parametrize("shape", THIN_SHAPES + THIN_SHAPES_RZ)
def test_thin_mesh_exact_bitwise(oracle_built, lib_built, monkeypatch, shape, staged):
    from fierro_gb300 import sgh
    from oracle import orc
    monkeypatch.setenv("FIERRO_STAGED_TRANSFERS", staged)
    prob = thin_deck(shape)
    o = orc.Oracle(prob)
    o.run_cycles(30)
    r = o.state()
    g, t = _gpu(prob, 30, sgh.FP_EXACT)
    assert t[0] == r["time"]
    assert_bitwise(g, r, FIELDS, label="%s staged=%s" % (prob.name, staged))


@pytest.mark.parametrize("shape", THIN_SHAPES + THIN_SHAPES_RZ)
def test_thin_mesh_fma_within_gates(oracle_built, lib_built, shape):
    from fierro_gb300 import sgh
    from oracle import orc
    prob = thin_deck(shape)
    for cycles, tol in ((1, 1e-12), (30, 1e-9)):
        o = orc.Oracle(prob)
        o.run_cycles(cycles)
        r = o.state()
        g, _ = _gpu(prob, cycles, sgh.FP_FMA)
        assert_fields(g, r, tol, GATED, label="%s fma %d cycles" % (prob.name, cycles))
        assert_fields_tight(g, r, tol, GATED, label="%s fma %d cycles" % (prob.name, cycles))
