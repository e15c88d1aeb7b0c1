"""Seeded random decks against the restatement, bit for bit: hex and 2D-RZ box
meshes of uneven sizes and lengths, jittered or not, permuted or not; one to
three materials with random viscosity coefficients and gamma; global, box,
sphere and cylinder fills with cartesian, radial and spherical velocities;
reflecting and fixed planes at either end; one to three RK stages; 10 to 40
cycles.  Where the restatement's run goes non-finite (a random deck can invert
an element or cool one below zero energy), the GPU is compared bit for bit at
the last cycle whose state is finite, and the full run must return
FIERRO_ENUMERIC."""
import numpy as np
import pytest

from conftest import assert_bitwise
from decks import random_deck

pytestmark = pytest.mark.gpu

FIELDS = ("coords", "vel", "den", "pres", "sie", "sspd", "vol", "corner_force", "div", "node_mass")


@pytest.mark.parametrize("dims", [3, 2])
@pytest.mark.parametrize("seed", list(range(24)))
def test_random_deck_bitwise(oracle_built, lib_built, seed, dims):
    from fierro_gb300 import sgh
    from oracle import orc
    prob = random_deck(seed, dims)

    def finite(r):
        return all(np.isfinite(r[k]).all() for k in ("coords", "vel", "sie", "den", "pres", "sspd"))

    o = orc.Oracle(prob, variant="crpow")
    o.run_cycles(prob.params.cycle_stop)
    r = o.state()
    cycles = prob.params.cycle_stop
    if not finite(r):
        # the last cycle whose state is finite, and the failure reported by the GPU
        o = orc.Oracle(prob, variant="crpow")
        cycles = 0
        while True:
            o.run_cycles(1)
            if not finite(o.state()):
                break
            cycles += 1
        o = orc.Oracle(prob, variant="crpow")
        o.run_cycles(cycles)
        r = o.state()
        with sgh.SGHSolver(prob) as s:
            s.set_state(sgh.setup(prob))
            with pytest.raises(sgh.FierroError) as ei:
                s.run(prob.params.cycle_stop)
            assert ei.value.code == sgh.FIERRO_ENUMERIC
        if cycles == 0:
            return
    st = sgh.setup(prob)
    with sgh.SGHSolver(prob) as s:
        s.set_state(st)
        s.run(cycles)
        out = s.get_state()
        t = s.time()
    g = {"coords": out["node_coords"][1], "vel": out["node_vel"][1], "den": out["elem_den"],
         "pres": out["elem_pres"], "sie": out["elem_sie"][1], "sspd": out["elem_sspd"], "vol": out["elem_vol"],
         "corner_force": out["corner_force"], "div": out["elem_div"], "node_mass": out["node_mass"]}
    assert t[0] == r["time"] and t[3] == o.time()[3]
    assert_bitwise(g, r, FIELDS, label=prob.name)
