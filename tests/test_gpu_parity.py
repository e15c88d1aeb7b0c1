"""GPU parity: the libfierro_sgh kernels (through the C ABI) against the CPU
oracle and against the reference's own outputs (golden fixtures).

Exact mode repeats the reference's arithmetic operation by operation, with a
correctly rounded pow(vol, 1/3); it is compared bit for bit with the oracle
variant that uses the same correctly rounded pow and IEEE squares, and within
the parity tolerances (1e-12 after one RK2 cycle, 1e-9 after the full run,
relative, floor 1e-3 of the field's peak) with the libm oracle and the golden
fixtures, whose pow rounding differs from correct rounding in ~0.1% of calls.
"""
import numpy as np
import pytest

from conftest import assert_bitwise, assert_fields, assert_fields_tight, field_error, load_golden

pytestmark = pytest.mark.gpu

FIELDS = ("coords", "vel", "den", "pres", "sie", "sspd", "vol")


def _cases():
    from fierro_gb300 import problems
    return {
        "sedov12": lambda: problems.sedov(12, geo_digits=5),
        "noh32": lambda: problems.noh(32, geo_digits=5),
        "sedov16_jp": lambda: problems.sedov(16, jitter=0.1, seed=7, permute=True, cycles=60),
        "noh12_jp": lambda: problems.noh(12, jitter=0.1, seed=9, permute=True, cycles=120),
    }


def _gpu_state(prob, cycles=None, stages=None, mode=0):
    from fierro_gb300 import sgh
    st0 = sgh.setup(prob)
    with sgh.SGHSolver(prob, fp_mode=mode) as s:
        s.set_state(st0)
        if stages is not None:
            s.run_stages(stages)
        else:
            s.run(cycles)
        out = s.get_state()
        t = s.time()
        en = s.energy()
    f = sgh.compared_fields(out)
    f["corner_force"] = out["corner_force"]
    f["div"] = out["elem_div"]
    f["time"] = t[0]
    f["energy"] = en
    f["coords0"] = out["node_coords"][0]
    f["sie0"] = out["elem_sie"][0]
    return f


def _oracle_state(prob, cycles=None, stages=None, variant="libm"):
    from oracle import orc
    o = orc.Oracle(prob, variant=variant)
    if stages is not None:
        o.run_stages(stages)
    else:
        o.run_cycles(cycles)
    st = o.state()
    st["energy"] = o.energy()
    return st


@pytest.mark.parametrize("case", ["sedov12", "noh32", "sedov16_jp", "noh12_jp"])
@pytest.mark.parametrize("stages", [1, 2])
def test_exact_bitwise_first_stages(oracle_built, lib_built, case, stages):
    """After one RK stage and after one full cycle every field, the corner forces
    and the divergences are bit-identical to the oracle."""
    prob = _cases()[case]()
    g = _gpu_state(prob, stages=stages)
    r = _oracle_state(prob, stages=stages)
    assert_bitwise(g, r, FIELDS + ("corner_force", "coords0", "sie0"), label="%s %d stages" % (case, stages))
    if stages == 2:
        assert_bitwise(g, r, ("div",), label=case)
        assert g["time"] == r["time"]


@pytest.mark.parametrize("case", ["sedov12", "noh32", "sedov16_jp", "noh12_jp"])
def test_exact_bitwise_full_run_crpow(oracle_built, lib_built, case):
    """Full runs are bit-identical to the oracle with correctly rounded pow."""
    prob = _cases()[case]()
    n = prob.params.cycle_stop
    g = _gpu_state(prob, cycles=n)
    r = _oracle_state(prob, cycles=n, variant="crpow")
    assert g["time"] == r["time"]
    assert_bitwise(g, r, FIELDS, label="%s full" % case)


@pytest.mark.parametrize("case", ["sedov12", "noh32", "sedov16_jp", "noh12_jp"])
def test_exact_full_run_vs_libm_oracle(oracle_built, lib_built, case):
    prob = _cases()[case]()
    n = prob.params.cycle_stop
    g = _gpu_state(prob, cycles=n)
    r = _oracle_state(prob, cycles=n)
    assert_fields(g, r, 1e-9, FIELDS, label=case)
    g1 = _gpu_state(prob, cycles=1)
    r1 = _oracle_state(prob, cycles=1)
    assert_fields(g1, r1, 1e-12, FIELDS, label=case + " 1 cycle")


@pytest.mark.parametrize("case,cycles,tol", [("sedov12", 1, 1e-12), ("sedov12", 200, 1e-9),
                                              ("noh32", 1, 1e-12), ("noh32", 500, 1e-9)])
def test_exact_vs_reference_golden(lib_built, case, cycles, tol):
    """Against the reference solver's own outputs on the shipped meshes."""
    prob = _cases()[case]()
    g = _gpu_state(prob, cycles=cycles)
    ref = load_golden("%s_c%d" % (case, cycles))
    assert g["time"] == pytest.approx(float(ref["time"]), rel=1e-12)
    assert_fields(g, ref, tol, FIELDS, label="%s c%d" % (case, cycles))


GATED = ("coords", "vel", "den", "pres", "sie")  # positions, velocities, density, pressure, energy

# The tight metric (conftest.field_error_tight: density, pressure and energy
# purely relative, so Sedov's 1e-10 background is compared at its own scale;
# positions and velocities with a floor of 1e-9 of the peak) holds the FMA mode
# to the same gates, 1e-12 after one cycle and 1e-9 after the full run, except
# where the reference's own arithmetic is ill-conditioned, bounded per deck:
#  * Noh after one cycle: the elements the shock has just reached hold
#    1e-10 + a heating increment that nearly cancels, so their energy (and
#    pressure) moves by a few 1e-12 of itself under any change of rounding
#    (measured 2.0e-12 at 32^3, 4.2e-12 at 48^3);
#  * Noh 32^3 after the full run: nodes in the stagnated core are at rest up to
#    rounding noise far below 1e-9 of the inflow speed, and the FMA mode's
#    noise differs from the exact mode's (measured 3.9e-9 against that floor).
TIGHT_ONE_CYCLE = {k: 1e-12 for k in GATED}
TIGHT_FULL = {k: 1e-9 for k in GATED}
TIGHT_BOUNDS = {("noh32", 1): {"sie": 1e-11, "pres": 1e-11}, ("noh32", 500): {"vel": 1e-8}}


@pytest.mark.parametrize("case", ["sedov12", "noh32", "sedov16_jp", "noh12_jp"])
def test_fma_mode_within_tolerance(oracle_built, lib_built, case):
    """The fused-multiply-add mode meets the parity gates on the gated fields:
    positions, velocities, density, pressure and energy within 1e-12 of the
    reference's arithmetic after one RK2 cycle and within 1e-9 after the full
    run (relative, floor 1e-3 of the field's peak).  The sums whose cancellation
    would amplify contraction (hex volume, element power, Riemann velocity, the
    energy update) stay separately rounded in this mode.  Sound speed is not a
    gated field: in Noh's barely heated elements, whose energy is ill-conditioned
    after one cycle, it stays within 2e-12."""
    prob = _cases()[case]()
    n = prob.params.cycle_stop
    g1 = _gpu_state(prob, cycles=1, mode=1)
    r1 = _oracle_state(prob, cycles=1)
    assert_fields(g1, r1, 1e-12, GATED, label=case + " fma 1 cycle")
    assert_fields(g1, r1, 2e-12, ("sspd", "vol"), label=case + " fma 1 cycle")
    assert_fields_tight(g1, r1, dict(TIGHT_ONE_CYCLE, **TIGHT_BOUNDS.get((case, 1), {})), GATED,
                        label=case + " fma 1 cycle")
    g = _gpu_state(prob, cycles=n, mode=1)
    r = _oracle_state(prob, cycles=n)
    assert_fields(g, r, 1e-9, FIELDS, label=case + " fma full")
    assert_fields_tight(g, r, dict(TIGHT_FULL, **TIGHT_BOUNDS.get((case, n), {})), GATED, label=case + " fma full")


def test_fma_mode_gates_on_the_bench_mesh_family(lib_built):
    """The benchmark's mesh family (jittered, permuted Sedov) at 64^3: the FMA
    mode against the exact mode (the reference's arithmetic, bit for bit) after
    one cycle and after 100."""
    from fierro_gb300 import problems
    prob = problems.sedov(64, jitter=0.1, seed=2024, permute=True, cycles=100)
    for cyc, tol in ((1, 1e-12), (100, 1e-9)):
        g = _gpu_state(prob, cycles=cyc, mode=1)
        r = _gpu_state(prob, cycles=cyc, mode=0)
        assert_fields(g, r, tol, GATED, label="sedov64 fma %d cycles" % cyc)
        assert g["time"] == pytest.approx(r["time"], rel=1e-13)


@pytest.mark.parametrize("case", ["sedov12", "noh32", "sedov16_jp"])
def test_total_energy_conserved(oracle_built, lib_built, case):
    """IE + KE is conserved by the compatible SGH update (sgh_solve.cpp:686-688)."""
    prob = _cases()[case]()
    from fierro_gb300 import sgh
    st0 = sgh.setup(prob)
    with sgh.SGHSolver(prob) as s:
        s.set_state(st0)
        ie0, ke0 = s.energy()
        s.run(prob.params.cycle_stop)
        ie1, ke1 = s.energy()
    te0, te1 = ie0 + ke0, ie1 + ke1
    assert abs(te1 - te0) <= 1e-12 * abs(te0), (te0, te1)
    r = _oracle_state(prob, cycles=prob.params.cycle_stop)
    assert ie1 == pytest.approx(r["energy"][0], rel=1e-12)
    assert ke1 == pytest.approx(r["energy"][1], rel=1e-9)


def test_renumbering_invariance(lib_built):
    """The same physical problem numbered two ways gives the same answer (the
    corner-force summation order follows the caller's numbering, so agreement is
    to rounding, not bitwise)."""
    from fierro_gb300 import problems
    a = problems.sedov(14, jitter=0.1, seed=21, permute=False, cycles=30)
    b = problems.sedov(14, jitter=0.1, seed=21, permute=True, cycles=30)
    ga = _gpu_state(a, cycles=30)
    gb = _gpu_state(b, cycles=30)
    # map b's node/element numbering onto a's through coordinates / centroids
    ka = np.lexsort(a.mesh.coords.T)
    kb = np.lexsort(b.mesh.coords.T)
    assert np.array_equal(a.mesh.coords[ka], b.mesh.coords[kb])
    ca = a.mesh.coords[a.mesh.nodes_in_elem].mean(axis=1)
    cb = b.mesh.coords[b.mesh.nodes_in_elem].mean(axis=1)
    ea, eb = np.lexsort(ca.T), np.lexsort(cb.T)
    na = {"coords": ga["coords"][ka], "vel": ga["vel"][ka], "den": ga["den"][ea], "sie": ga["sie"][ea],
          "pres": ga["pres"][ea]}
    nb = {"coords": gb["coords"][kb], "vel": gb["vel"][kb], "den": gb["den"][eb], "sie": gb["sie"][eb],
          "pres": gb["pres"][eb]}
    assert_fields(nb, na, 1e-11, ("coords", "vel", "den", "sie", "pres"), label="renumbered")
