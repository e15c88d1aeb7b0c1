"""The CPU oracle is pinned before it is trusted: against the reference's own
SGH solver run here (golden fixtures, and live when the reference build is
available), and against geometry identities of the hex formulas."""
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN, assert_bitwise, load_golden
from decks import THIN_SHAPES, THIN_SHAPES_RZ, thin_deck

FIELDS = ("coords", "vel", "den", "pres", "sie", "sspd", "vol")


def _problem(name):
    from fierro_gb300 import problems
    if name == "sedov12":
        return problems.sedov(12, geo_digits=5)
    return problems.noh(32, geo_digits=5)


def test_box_generator_matches_shipped_meshes():
    """The generator reproduces mesh_12x12x12.geo and mesh_Box_32.geo bit for bit
    (checksums recorded from the shipped files by tests/golden/make_golden.py)."""
    import hashlib
    from fierro_gb300 import mesh
    meta = json.load(open(os.path.join(GOLDEN, "golden.json")))
    for name, n, L in (("sedov12", 12, 1.2), ("noh32", 32, 1.0)):
        m = mesh.box_mesh(n, length=L, geo_digits=5)
        assert hashlib.sha256(m.coords.tobytes()).hexdigest() == meta[name]["coords_sha256"]
        assert hashlib.sha256(m.nodes_in_elem.astype(np.int64).tobytes()).hexdigest() == \
            meta[name]["nodes_in_elem_sha256"]


@pytest.mark.parametrize("case,cycles", [("sedov12", 1), ("sedov12", 200), ("noh32", 1), ("noh32", 500)])
def test_oracle_equals_reference_golden(oracle_built, case, cycles):
    """C restatement (libm pow, uncontracted) == the reference's own solver on the
    shipped meshes, bit for bit, after one cycle and after the full run."""
    from oracle import orc
    ref = load_golden("%s_c%d" % (case, cycles))
    o = orc.Oracle(_problem(case))
    o.run_cycles(cycles)
    st = o.state()
    assert st["time"] == float(ref["time"])
    assert_bitwise(st, ref, FIELDS + ("node_mass", "mass"), label="%s c%d" % (case, cycles))


def test_oracle_equals_reference_live_jittered(oracle_built):
    """Against the reference executable itself on a jittered, permuted mesh (the
    bench's mesh family), when the reference build is available here."""
    from fierro_gb300 import problems
    from oracle import orc
    if not orc.reference_available("fierro_ref"):
        pytest.skip("reference executable not built on this machine")
    prob = problems.sedov(10, jitter=0.1, seed=11, permute=True)
    ref = orc.run_reference(prob, cycles=40, threads=2)
    o = orc.Oracle(prob)
    o.run_cycles(40)
    assert_bitwise(o.state(), ref, FIELDS + ("corner_force", "div"), label="sedov10 jittered")


def test_crpow_variant_only_differs_through_pow(oracle_built):
    """The correctly-rounded-pow oracle equals the libm one wherever pow's
    rounding agrees; on Sedov 12^3 (200 cycles) that is everywhere."""
    from oracle import orc
    a = orc.Oracle(_problem("sedov12"), variant="libm")
    b = orc.Oracle(_problem("sedov12"), variant="crpow")
    a.run_cycles(200)
    b.run_cycles(200)
    assert_bitwise(a.state(), b.state(), FIELDS, label="libm vs crpow sedov12")


def _random_hex(rng, jitter=0.15):
    base = np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0], [0, 0, 1], [1, 0, 1], [1, 1, 1], [0, 1, 1]], float)
    return base + rng.uniform(-jitter, jitter, base.shape)


def test_geometry_identities(oracle_built):
    """geometry.cpp identities: unit-cube volume 1; sum_p B_p = 0;
    sum_p x_p (x) B_p = V I (within rounding); translation invariance."""
    from oracle import orc
    cube = _random_hex(np.random.default_rng(0), 0.0)
    x, y, z = cube.T
    assert orc.vol_hex(x, y, z) == 1.0
    B = orc.bmatrix(x, y, z)
    assert np.allclose(np.abs(B), 0.25, rtol=0, atol=1e-15)
    rng = np.random.default_rng(1)
    for _ in range(50):
        h = _random_hex(rng) * rng.uniform(0.01, 2.0)
        x, y, z = h.T
        V = orc.vol_hex(x, y, z)
        B = orc.bmatrix(x, y, z)
        assert V > 0
        assert np.max(np.abs(B.sum(axis=0))) <= 1e-14 * np.max(np.abs(B))
        M = h.T @ B  # sum_p x_p,i B_p,j
        assert np.allclose(M, V * np.eye(3), rtol=0, atol=1e-13 * V)
        t = rng.uniform(-3, 3, 3)
        x2, y2, z2 = (h + t).T
        assert abs(orc.vol_hex(x2, y2, z2) - V) <= 1e-12 * V


def _strength_cases():
    import importlib.util
    spec = importlib.util.spec_from_file_location("make_golden", os.path.join(GOLDEN, "make_golden.py"))
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    return mg.strength_cases()


@pytest.mark.parametrize("case", ["sedov8_hypo", "noh8_hyper", "sedov10_mixed"])
def test_oracle_strength_equals_reference_golden(oracle_built, case):
    """Strength models: the C restatement with the test hypo-elastic model, called
    as a hypo model (force pass) or a hyper model (state update), equals the
    reference running the same model through material_t::strength_model, bit for
    bit, including both stress bins and the state variables."""
    from oracle import orc
    prob = _strength_cases()[case]
    meta = json.load(open(os.path.join(GOLDEN, "golden.json")))["strength"][case]
    assert prob.config_text() == meta["deck"]
    ref = load_golden("strength_" + case)
    assert np.abs(ref["stress"]).max() > 1e-3  # the stress is not negligible
    o = orc.Oracle(prob)
    o.run_cycles(prob.params.cycle_stop)
    st = o.state()
    assert st["time"] == float(ref["time"])
    assert_bitwise(st, ref, FIELDS + ("corner_force", "div", "stress", "stress0", "statev"), label=case)


def test_oracle_strength_equals_reference_live(oracle_built):
    """The same against the reference executable run here, on a hyper Sedov with
    a jittered, permuted mesh, when the reference build is available."""
    from fierro_gb300 import problems
    from oracle import orc
    if not orc.reference_available("fierro_ref"):
        pytest.skip("reference executable not built on this machine")
    prob = problems.with_strength(problems.sedov(9, jitter=0.1, seed=4, permute=True, cycles=30), "hyper", 8.0)
    ref = orc.run_reference(prob, threads=2)
    o = orc.Oracle(prob)
    o.run_cycles(30)
    assert_bitwise(o.state(), ref, FIELDS + ("corner_force", "stress", "stress0"), label="sedov9 hyper")


def test_oracle_strength_needs_shear_modulus_column(oracle_built):
    from fierro_gb300 import problems
    from oracle import orc
    prob = problems.with_strength(problems.sedov(4, cycles=2), "hypo", 1.0)
    prob.num_state_vars = 3
    with pytest.raises(ValueError):
        orc.Oracle(prob)


def _rz_cases():
    import importlib.util
    spec = importlib.util.spec_from_file_location("make_golden", os.path.join(GOLDEN, "make_golden.py"))
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    return mg.rz_cases()


@pytest.mark.parametrize("case", ["sedov_rz16", "noh_rz16", "noh_rz12_jp", "sedov_rz12_jp_hypo",
                                  "taylor_anvil_rz80x8_p", "sod_rz100x2_p"])
def test_oracle_rz_equals_reference_golden(oracle_built, case):
    """2D-RZ: the C restatement of the num_dims == 2 branches (area-weighted
    force with hoop terms, RZ volume and divergence, radius-weighted energy,
    per-stage areal node mass and the axis fix) equals the reference run with
    num_dims = 2, bit for bit, including node masses and corner forces."""
    from oracle import orc
    prob = _rz_cases()[case]
    meta = json.load(open(os.path.join(GOLDEN, "golden.json")))["rz"][case]
    assert prob.config_text() == meta["deck"]
    ref = load_golden("rz_" + case)
    o = orc.Oracle(prob)
    o.run_cycles(prob.params.cycle_stop)
    st = o.state()
    assert st["time"] == float(ref["time"])
    assert_bitwise(st, ref, FIELDS + ("corner_force", "div", "node_mass", "mass", "stress", "stress0"), label=case)


def test_oracle_rz_energy_conserved(oracle_built):
    from fierro_gb300 import problems
    from oracle import orc
    o = orc.Oracle(problems.sedov_rz(16, cycles=200))
    ie0, ke0 = o.energy()
    o.run_cycles(200)
    ie1, ke1 = o.energy()
    assert ke1 > 0.1 * ie0
    assert abs((ie1 + ke1) - (ie0 + ke0)) <= 1e-12 * (ie0 + ke0)


def test_oracle_rz_refuses_reference_defects(oracle_built):
    """Inputs whose 2D branch in the reference reads or writes past an array
    (hyper strength, spherical velocity fill, z-plane or sphere boundaries) are
    refused rather than imitated."""
    from fierro_gb300 import problems
    from oracle import orc
    p = problems.with_strength(problems.sedov_rz(4, cycles=2), "hyper", 1.0)
    with pytest.raises(ValueError):
        orc.Oracle(p)
    p = problems.noh_rz(4, cycles=2)
    p.fills[0].velocity = "spherical"
    with pytest.raises(ValueError):
        orc.Oracle(p)
    p = problems.sedov_rz(4, cycles=2)
    p.boundaries.append(problems.Boundary("z_plane", 0.0, "reflected"))
    with pytest.raises(ValueError):
        orc.Oracle(p)


def _geo(name, cycles):
    import importlib.util
    spec = importlib.util.spec_from_file_location("make_golden", os.path.join(GOLDEN, "make_golden.py"))
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    return mg.geo_problem(name, cycles)


@pytest.mark.parametrize("name,cycles", [("taylor_anvil", 1), ("taylor_anvil", 300),
                                         ("triple_point", 1), ("triple_point", 400),
                                         ("sod_saltzman", 1), ("sod_saltzman", 400),
                                         ("taylor_anvil_small_rod", 1), ("taylor_anvil_small_rod", 200)])
def test_oracle_equals_reference_on_shipped_unstructured_meshes(oracle_built, name, cycles):
    """The restatement equals the reference bit for bit on two more meshes the
    reference ships: the Taylor-anvil rod (an O-grid with nodes of valence 3 and
    6, the deck of the reference's own Taylor-anvil test) and the triple-point
    box (three fills, six reflecting planes)."""
    from oracle import orc
    prob = _geo(name, cycles)
    ref = load_golden("geo_%s_c%d" % (name, cycles))
    o = orc.Oracle(prob)
    o.run_cycles(cycles)
    st = o.state()
    assert st["time"] == float(ref["time"])
    for k in ("coords", "vel", "den", "pres", "sie", "sspd", "vol", "node_mass", "mass"):
        assert np.array_equal(st[k], ref[k]), (name, cycles, k)


@pytest.mark.parametrize("kind", ["velocity", "pressure", "acceleration", "contact"])
def test_other_boundary_kinds_leave_nodes_free(oracle_built, kind):
    """A boundary set of the kinds boundary_velocity has no branch for
    (boundary.cpp:10-55; bdy_hydro_conds mesh.h:910-918) holds no velocity
    component: the reference run with such a set on the far x plane equals the
    run without it and the restatement, bit for bit."""
    import copy
    from fierro_gb300 import problems
    from oracle import orc
    prob = problems.noh(8, jitter=0.1, seed=4, permute=True, cycles=30)
    plus = copy.deepcopy(prob)
    plus.boundaries.append(problems.Boundary("x_plane", 1.0, kind))
    o = orc.Oracle(plus)
    o.run_cycles(30)
    o_plain = orc.Oracle(prob)
    o_plain.run_cycles(30)
    assert_bitwise(o.state(), o_plain.state(), FIELDS, label="restatement %s vs none" % kind)
    assert not np.any(o.get(orc.ORC_BDY_NODE_MASK) & ~o_plain.get(orc.ORC_BDY_NODE_MASK))
    if not orc.reference_available("fierro_ref"):
        pytest.skip("reference executable not built on this machine")
    ref = orc.run_reference(plus, cycles=30, threads=2)
    assert_bitwise(o.state(), ref, FIELDS + ("corner_force",), label="%s set vs reference" % kind)


@pytest.mark.parametrize("shape", THIN_SHAPES + THIN_SHAPES_RZ)
def test_oracle_equals_reference_on_thin_meshes(oracle_built, shape):
    """Meshes one element thick, down to a single element (every node on the
    surface, a lone element's limiter with no neighbour), hex and 2D-RZ: the
    restatement equals the reference executable bit for bit after 30 cycles."""
    from oracle import orc
    prob = thin_deck(shape)
    o = orc.Oracle(prob)
    o.run_cycles(30)
    if not orc.reference_available("fierro_ref"):
        pytest.skip("reference executable not built on this machine")
    ref = orc.run_reference(prob, cycles=30, threads=2)
    assert_bitwise(o.state(), ref, FIELDS + ("corner_force", "div"), label=prob.name)
