"""Parity on the benchmark's own problem family: jittered (+-0.1h), permuted
Sedov (gamma 1.4, origin energy 0.2467 on [0,1.2]^3, CFL 0.4, seed 2024) and
Noh (gamma 5/3, unit inflow on [0,1]^3, CFL 0.3) at 64^3 and 48^3, against the
C restatement of the reference's algorithm (bitwise pinned to the reference's
own solver on the shipped meshes and on jittered, permuted decks).

* exact mode: every field bit for bit equal to the restatement with correctly
  rounded pow, after one RK2 cycle and after 100;
* FMA mode: within 1e-12 after one cycle and 1e-9 after 100 of the restatement
  with libm pow (the reference's own arithmetic), in both parity metrics: the
  floor-1e-3 metric and the tight one (density, pressure, energy purely
  relative, so the 1e-10 background is compared at its own scale), with one
  documented bound: Noh's energy and pressure after one cycle, 1e-11.

The bench line carries the same comparison at 120^3 against the reference's
own executable (its `parity` object).
"""
import pytest

from conftest import assert_bitwise, assert_fields, assert_fields_tight

pytestmark = pytest.mark.gpu

FIELDS = ("coords", "vel", "den", "pres", "sie", "sspd", "vol")
GATED = ("coords", "vel", "den", "pres", "sie")


def _family(name):
    from fierro_gb300 import problems
    if name == "sedov64":
        return problems.sedov(64, length=1.2, energy=0.2467, gamma=1.4, jitter=0.1, seed=2024, permute=True,
                              cycles=100)
    return problems.noh(48, length=1.0, jitter=0.1, seed=2024, permute=True, cycles=100)


def _gpu_two(prob, mode, first, total):
    """The state after `first` cycles and after `total`, from one run."""
    from fierro_gb300 import sgh
    out = []
    with sgh.SGHSolver(prob, fp_mode=mode) as s:
        s.set_state(sgh.setup(prob))
        done = 0
        for c in (first, total):
            assert s.run(c - done) == c - done
            done = c
            st = s.get_state()
            f = sgh.compared_fields(st)
            f["time"] = s.time()[0]
            f["corner_force"] = st["corner_force"]
            out.append(f)
    return out


def _oracle_two(prob, variant, first, total):
    from oracle import orc
    o = orc.Oracle(prob, variant=variant)
    out = []
    done = 0
    for c in (first, total):
        assert o.run_cycles(c - done) == c - done
        done = c
        out.append(o.state())
    return out


@pytest.mark.parametrize("family", ["sedov64", "noh48"])
def test_exact_mode_bitwise_on_the_bench_family(oracle_built, lib_built, family):
    from fierro_gb300 import sgh
    prob = _family(family)
    g1, g100 = _gpu_two(prob, sgh.FP_EXACT, 1, 100)
    r1, r100 = _oracle_two(prob, "crpow", 1, 100)
    assert_bitwise(g1, r1, FIELDS + ("corner_force",), label="%s exact 1 cycle" % family)
    assert g1["time"] == r1["time"]
    assert_bitwise(g100, r100, FIELDS, label="%s exact 100 cycles" % family)
    assert g100["time"] == r100["time"]


@pytest.mark.parametrize("family", ["sedov64", "noh48"])
def test_fma_mode_gates_on_the_bench_family(oracle_built, lib_built, family):
    from fierro_gb300 import sgh
    prob = _family(family)
    g1, g100 = _gpu_two(prob, sgh.FP_FMA, 1, 100)
    r1, r100 = _oracle_two(prob, "libm", 1, 100)
    assert_fields(g1, r1, 1e-12, GATED, label="%s fma 1 cycle" % family)
    assert_fields(g100, r100, 1e-9, GATED, label="%s fma 100 cycles" % family)
    # the tight metric after one cycle of Noh: the just-heated elements' energy
    # (1e-10 plus a nearly cancelling increment) is ill-conditioned in the
    # reference's arithmetic itself; measured 4.2e-12 at 48^3, bounded at 1e-11
    tight1 = {k: 1e-12 for k in GATED}
    if family.startswith("noh"):
        tight1.update(sie=1e-11, pres=1e-11)
    assert_fields_tight(g1, r1, tight1, GATED, label="%s fma 1 cycle" % family)
    assert_fields_tight(g100, r100, 1e-9, GATED, label="%s fma 100 cycles" % family)
    assert g100["time"] == pytest.approx(r100["time"], rel=1e-12)
