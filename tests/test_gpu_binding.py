"""The reference-side binding of the library as a reference maintainer would
add it: the reference's own driver sequence (input, EnSight/binary mesh read,
connectivity, get_vol, setup -- ref_harness.cpp, the call sequence of
driver.cpp:70-328 over the reference's node_t / elem_t / corner_t / mesh_t /
material_t / boundary_t) with its sgh_solve call (driver.cpp:280-313,
mesh.h:1175-1208) replaced by oracle/ref/fierro_sgh_call.inc -- the snippet the
integration notes show, verbatim -- compiled, linked against libfierro_sgh.so
and run.  Its final state must equal the C restatement with correctly rounded
pow bit for bit (the library's exact mode), and be within the parity gates
(1e-12 after one cycle, 1e-9 after the full run) of the reference's own
sgh_solve run on the same deck."""
import pytest

from conftest import assert_bitwise, assert_fields

pytestmark = pytest.mark.gpu

FIELDS = ("coords", "vel", "den", "pres", "sie", "sspd", "vol")


def _deck(case):
    from fierro_gb300 import problems
    if case == "sedov12":
        return problems.sedov(12, geo_digits=5)
    return problems.noh(32, geo_digits=5)


@pytest.mark.parametrize("case,cycles", [("sedov12", 1), ("sedov12", 200), ("noh32", 1), ("noh32", 500)])
def test_reference_binding_runs_the_library(oracle_built, lib_built, case, cycles):
    from oracle import build_ref, orc
    exe = build_ref.build_reference_lib()
    if exe is None:
        pytest.skip("the reference's sources are not on this machine")
    prob = _deck(case)
    got = orc.run_reference(prob, cycles=cycles, kind="fierro_ref_lib")
    o = orc.Oracle(prob, variant="crpow")
    o.run_cycles(cycles)
    want = o.state()
    assert got["time"] == want["time"]
    assert_bitwise(got, want, FIELDS + ("corner_force", "coords0", "sie0"), label="%s c%d binding" % (case, cycles))
    ref = orc.run_reference(prob, cycles=cycles, kind="fierro_ref")
    assert got["time"] == pytest.approx(ref["time"], rel=1e-12)
    assert_fields(got, ref, 1e-12 if cycles == 1 else 1e-9, FIELDS, label="%s c%d vs sgh_solve" % (case, cycles))
