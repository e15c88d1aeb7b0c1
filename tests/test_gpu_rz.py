"""2D-RZ (num_dims == 2) on the GPU: the quad kernels against the 2D-RZ
restatement (bit for bit in exact mode) and against the reference's own runs
(tests/golden/rz_*.npz, made with num_dims = 2 on the decks of the reference's
RZ tests), energy conservation, the FMA mode, the hypo strength hook in RZ and
the refusals of inputs the reference's 2D branch mishandles."""
import importlib.util
import os

import numpy as np
import pytest

from conftest import GOLDEN, assert_bitwise, assert_fields, assert_fields_tight, load_golden

pytestmark = pytest.mark.gpu

FIELDS = ("coords", "vel", "den", "pres", "sie", "sspd", "vol")
EXTRA = ("corner_force", "div", "node_mass", "coords0", "vel0", "sie0", "stress", "stress0")
CASES = ("sedov_rz16", "noh_rz16", "noh_rz12_jp", "sedov_rz12_jp_hypo", "taylor_anvil_rz80x8_p", "sod_rz100x2_p")


def _cases():
    spec = importlib.util.spec_from_file_location("make_golden", os.path.join(GOLDEN, "make_golden.py"))
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    return mg.rz_cases()


def _gpu(prob, cycles=None, stages=None, mode=0):
    from fierro_gb300 import sgh
    st = sgh.setup(prob)
    with sgh.SGHSolver(prob, fp_mode=mode) as s:
        s.set_state(st)
        if stages is not None:
            s.run_stages(stages)
        else:
            s.run(cycles)
        out = s.get_state()
        t = s.time()
        en = s.energy()
    return {"coords": out["node_coords"][1], "vel": out["node_vel"][1], "coords0": out["node_coords"][0],
            "vel0": out["node_vel"][0], "den": out["elem_den"], "pres": out["elem_pres"],
            "sie": out["elem_sie"][1], "sie0": out["elem_sie"][0], "sspd": out["elem_sspd"],
            "vol": out["elem_vol"], "corner_force": out["corner_force"], "div": out["elem_div"],
            "node_mass": out["node_mass"], "mass": out["elem_mass"], "stress": out["elem_stress"][1],
            "stress0": out["elem_stress"][0], "time": t[0], "energy": en}


def _oracle(prob, cycles=None, stages=None, variant="crpow"):
    from oracle import orc
    o = orc.Oracle(prob, variant=variant)
    if stages is not None:
        o.run_stages(stages)
    else:
        o.run_cycles(cycles)
    st = o.state()
    st["energy"] = o.energy()
    return st


@pytest.mark.parametrize("case", CASES)
@pytest.mark.parametrize("stages", [1, 2, 3])
def test_rz_exact_bitwise_stages(oracle_built, lib_built, case, stages):
    """After 1, 2 and 3 RK stages every field, both bins, the corner forces, the
    divergence and the per-stage areal node masses (axis fix included) are
    bit-identical to the restatement."""
    prob = _cases()[case]
    g = _gpu(prob, stages=stages)
    r = _oracle(prob, stages=stages)
    assert_bitwise(g, r, FIELDS + EXTRA, label="%s %d stages" % (case, stages))


@pytest.mark.parametrize("case", CASES)
def test_rz_exact_bitwise_full_run(oracle_built, lib_built, case):
    prob = _cases()[case]
    g = _gpu(prob, cycles=prob.params.cycle_stop)
    r = _oracle(prob, cycles=prob.params.cycle_stop)
    assert g["time"] == r["time"]
    assert_bitwise(g, r, FIELDS + EXTRA, label=case)


@pytest.mark.parametrize("case", CASES)
def test_rz_exact_vs_reference_golden(lib_built, case):
    prob = _cases()[case]
    ref = load_golden("rz_" + case)
    g = _gpu(prob, cycles=prob.params.cycle_stop)
    assert g["time"] == float(ref["time"])
    assert_fields(g, ref, 1e-12, keys=FIELDS + ("node_mass",), label=case)


def test_rz_energy_conserved(oracle_built, lib_built):
    """IE + KE (KE = 1/2 sum m y |v|^2, sgh_solve.cpp:73-101) is conserved over
    200 cycles of RZ Sedov, and the GPU tallies equal the restatement's."""
    from fierro_gb300 import problems, sgh
    prob = problems.sedov_rz(24, cycles=200)
    st = sgh.setup(prob)
    with sgh.SGHSolver(prob) as s:
        s.set_state(st)
        ie0, ke0 = s.energy()
        s.run(200)
        ie1, ke1 = s.energy()
    assert ke1 > 0.1 * ie0
    assert abs((ie1 + ke1) - (ie0 + ke0)) <= 1e-12 * (ie0 + ke0)
    r = _oracle(prob, cycles=200)
    assert abs(ie1 - r["energy"][0]) <= 1e-13 * ie0 and abs(ke1 - r["energy"][1]) <= 1e-13 * ie0


@pytest.mark.parametrize("case", CASES)
def test_rz_fma_mode_within_tolerance(oracle_built, lib_built, case):
    """FMA mode in 2D-RZ: the gated fields within 1e-12 of the reference's
    arithmetic after one cycle and 1e-9 after the full run."""
    gated = ("coords", "vel", "den", "pres", "sie")
    prob = _cases()[case]
    g1 = _gpu(prob, cycles=1, mode=1)
    r1 = _oracle(prob, cycles=1)
    assert_fields(g1, r1, 1e-12, keys=gated, label="fma %s 1 cycle" % case)
    g = _gpu(prob, cycles=prob.params.cycle_stop, mode=1)
    r = _oracle(prob, cycles=prob.params.cycle_stop)
    assert_fields(g, r, 1e-9, keys=FIELDS + ("node_mass",), label="fma %s" % case)
    # the tight metric (density, pressure, energy purely relative; positions and
    # velocities with a floor of 1e-9 of the peak): the same gates, except the
    # velocity of Sod's elements at rest, rounding noise in both codes (measured
    # 5.7e-6 of the floor after 400 cycles)
    assert_fields_tight(g1, r1, 1e-12, gated, label="fma %s 1 cycle" % case)
    assert_fields_tight(g, r, {"coords": 1e-9, "vel": 2e-5 if case == "sod_rz100x2_p" else 1e-9, "den": 1e-9,
                               "pres": 1e-9, "sie": 1e-9}, gated, label="fma %s" % case)


def test_rz_timed_launches(lib_built):
    from fierro_gb300 import problems, sgh
    prob = problems.noh_rz(16, cycles=10)
    with sgh.SGHSolver(prob) as s:
        s.set_state(sgh.setup(prob))
        assert s.launches_per_cycle == 2 + 4 * prob.params.rk_num_stages
        ran, total, kms = s.run_timed(3)
        assert ran == 3 and total > 0 and len(kms) == len(s.launch_names())


def test_rz_refusals(lib_built):
    from fierro_gb300 import problems, sgh
    p = problems.with_strength(problems.sedov_rz(4, cycles=2), "hyper", 1.0)
    with pytest.raises(sgh.FierroError) as ei:
        sgh.SGHSolver(p)
    assert ei.value.code == sgh.FIERRO_ENOTSUP
    p = problems.sedov_rz(6, cycles=2)
    with sgh.SGHSolver(p) as s:
        s.set_state(sgh.setup(p))
        for call in (lambda: s.device_view(), lambda: s.set_output("/tmp"), lambda: s.adj_forward(cycles=1)):
            with pytest.raises(sgh.FierroError) as ei:
                call()
            assert ei.value.code == sgh.FIERRO_ENOTSUP


@pytest.mark.parametrize("length", [(1.2, 1.2e-4), (1.2e-4, 1.2)])
def test_rz_hoop_terms_on_thin_elements(oracle_built, lib_built, length):
    """Quads with an aspect ratio of 5000 fail the corner-area finiteness test of
    the gas force (|cross| > 1e-4 P^2), so the kernel forms Barlow's corner areas
    and the hoop terms as the reference writes them; still bit-identical."""
    from fierro_gb300 import mesh, problems
    m = mesh.quad_mesh(10, 6, length=length, jitter=0.05, seed=3)
    prob = problems.noh_rz(mesh=m, cycles=20)
    prob.params.dt_start, prob.params.dt_min = 1e-9, 1e-12
    g = _gpu(prob, cycles=20)
    r = _oracle(prob, cycles=20)
    assert np.isfinite(r["coords"]).all()
    assert_bitwise(g, r, FIELDS + EXTRA, label="thin quads %s" % (length,))


def test_rz_one_shot_solve_equals_handle(oracle_built, lib_built):
    """fierro_sgh_solve (create, upload, run, download, destroy in one call) on a
    quad mesh returns what the persistent handle computes."""
    from fierro_gb300 import sgh
    prob = _cases()["noh_rz12_jp"]
    st = sgh.setup(prob)
    host = {k: v.copy() for k, v in st.items()}
    r = sgh.sgh_solve(prob, host)
    assert r["cycles"] == prob.params.cycle_stop
    g = _gpu(prob, cycles=prob.params.cycle_stop)
    assert r["time_value"] == g["time"]
    for k, hk in (("coords", ("node_coords", 1)), ("vel", ("node_vel", 1)), ("sie", ("elem_sie", 1))):
        assert np.array_equal(host[hk[0]][hk[1]], g[k]), k
    assert np.array_equal(host["node_mass"], g["node_mass"])


def test_rz_taylor_anvil_cooling_is_reported(oracle_built, lib_built):
    """On the RZ Taylor anvil the scheme itself cools a cold element below zero
    energy near t = 1.1 (the restatement, like the reference, then produces a
    NaN sound speed); the GPU follows it bit for bit up to that cycle and the run
    call reports FIERRO_ENUMERIC instead of continuing silently."""
    from fierro_gb300 import problems, sgh
    prob = problems.taylor_anvil_rz(40, 4, seed=8, permute=True, cycles=300)
    g = _gpu(prob, cycles=160)
    r = _oracle(prob, cycles=160)
    assert_bitwise(g, r, FIELDS, label="taylor anvil rz 160")
    with sgh.SGHSolver(prob) as s:
        s.set_state(sgh.setup(prob))
        with pytest.raises(sgh.FierroError) as ei:
            s.run(300)
        assert ei.value.code == sgh.FIERRO_ENUMERIC


def test_rz_fma_mode_gates_on_the_bench_mesh_family(lib_built):
    """The RZ benchmark's mesh family (jittered, permuted RZ Sedov, source radius
    1.2/64) at 1024^2: the FMA mode against the exact mode (the reference's
    arithmetic bit for bit) after one cycle (1e-12) and after 20 (1e-9)."""
    from fierro_gb300 import problems
    prob = problems.sedov_rz(1024, jitter=0.1, seed=2024, permute=True, cycles=20, source_radius=1.2 / 64)
    for cyc, tol in ((1, 1e-12), (20, 1e-9)):
        g = _gpu(prob, cycles=cyc, mode=1)
        r = _gpu(prob, cycles=cyc, mode=0)
        assert_fields(g, r, tol, keys=("coords", "vel", "den", "pres", "sie"), label="rz1024 fma %d" % cyc)


def test_rz_staged_and_direct_transfers_agree(lib_built, monkeypatch):
    """set_state / get_state of a quad mesh through the transfer kernels (the GPU
    reading and writing the host arrays) and through pinned staging buffers give
    identical states, stress bins and state variables included."""
    from fierro_gb300 import sgh
    prob = _cases()["sedov_rz12_jp_hypo"]
    st = sgh.setup(prob)
    outs = {}
    for staged in ("0", "1"):
        monkeypatch.setenv("FIERRO_STAGED_TRANSFERS", staged)
        with sgh.SGHSolver(prob) as s:
            s.set_state({k: v.copy() for k, v in st.items()})
            s.run(7)
            outs[staged] = s.get_state()
    for k in outs["0"]:
        assert np.array_equal(outs["0"][k], outs["1"][k]), k
