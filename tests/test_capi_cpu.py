"""C ABI checks that need no GPU: the library loads, exports every function the
public header declares, and its host-side set-up (setup.cpp:10-424) reproduces
the oracle's initial state bit for bit; invalid meshes and decks are refused
with the documented error codes."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from conftest import ROOT, assert_bitwise


def header_functions():
    src = open(os.path.join(ROOT, "include", "fierro_sgh.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:const\s+)?[A-Za-z_][A-Za-z0-9_]*\s*\**\s*(fierro_\w+)\s*\(", src, re.M)))


def test_library_exports_header(lib_built):
    from fierro_gb300 import sgh
    names = header_functions()
    assert len(names) >= 15
    missing = [n for n in names if not hasattr(sgh.lib(), n)]
    assert not missing, missing
    assert sgh.version().startswith("fierro-sgh-gb300")


@pytest.mark.parametrize("case", ["sedov12", "noh32", "sedov10_jittered_permuted"])
def test_host_setup_matches_oracle(lib_built, oracle_built, case):
    from fierro_gb300 import problems, sgh
    from oracle import orc
    prob = {"sedov12": lambda: problems.sedov(12, geo_digits=5),
            "noh32": lambda: problems.noh(32, geo_digits=5),
            "sedov10_jittered_permuted": lambda: problems.sedov(10, jitter=0.1, seed=3, permute=True)}[case]()
    st = sgh.setup(prob)
    o = orc.Oracle(prob)
    ref = o.state()
    got = {"coords": st["node_coords"][1], "vel": st["node_vel"][1], "den": st["elem_den"],
           "pres": st["elem_pres"], "sie": st["elem_sie"][1], "sspd": st["elem_sspd"], "vol": st["elem_vol"],
           "mass": st["elem_mass"], "node_mass": st["node_mass"], "coords0": st["node_coords"][0]}
    assert_bitwise(got, ref, list(got), label=case)
    # boundary node masks equal the oracle's per-set node lists
    assert np.all(st["elem_statev"][:, 0] == prob.materials[0].gamma)


def _deck():
    from fierro_gb300 import problems
    return problems.sedov(4)


def _setup_rc(prob, mutate_mesh=None, mutate_mat=None):
    from fierro_gb300 import sgh
    nie = np.ascontiguousarray(prob.mesh.nodes_in_elem, dtype=np.uint64).copy()
    xyz = np.ascontiguousarray(prob.mesh.coords, dtype=np.float64).copy()
    if mutate_mesh:
        mutate_mesh(nie, xyz)
    m = sgh.Mesh(prob.mesh.num_nodes, prob.mesh.num_elems, nie.ctypes.data, xyz.ctypes.data)
    mats = sgh.c_materials(prob)
    if mutate_mat:
        mutate_mat(mats)
    st = sgh.empty_state(prob.mesh.num_nodes, prob.mesh.num_elems, prob.num_state_vars)
    sv = np.ascontiguousarray(prob.state_vars())
    rc = sgh.lib().fierro_sgh_setup(C.byref(m), mats, len(prob.materials), sv.ctypes.data, prob.num_state_vars,
                                    sgh.c_fills(prob), len(prob.fills), sgh.c_boundaries(prob),
                                    len(prob.boundaries), C.byref(sgh.c_state(st)))
    return rc, sgh.lib().fierro_last_error().decode()


def test_setup_rejects_corrupt_meshes(lib_built):
    from fierro_gb300 import sgh
    prob = _deck()
    assert _setup_rc(prob)[0] == sgh.FIERRO_OK

    def out_of_range(nie, xyz):
        nie[3, 2] = prob.mesh.num_nodes + 5

    def duplicate(nie, xyz):
        nie[0, 1] = nie[0, 0]

    def nan_coord(nie, xyz):
        xyz[7, 1] = np.nan

    def inverted(nie, xyz):
        nie[5, :] = nie[5, [4, 5, 6, 7, 0, 1, 2, 3]]

    for fn, code in ((out_of_range, sgh.FIERRO_EINVAL), (duplicate, sgh.FIERRO_EINVAL),
                     (nan_coord, sgh.FIERRO_EINVAL), (inverted, sgh.FIERRO_ENUMERIC)):
        rc, msg = _setup_rc(prob, mutate_mesh=fn)
        assert rc == code, (fn.__name__, rc, msg)
        assert msg


def test_setup_rejects_bad_mesh_headers(lib_built):
    """Empty meshes, fewer nodes than one element needs, an unknown dimension and
    meshes past the 32-bit device index range are refused from the header alone
    (the arrays are not read)."""
    from fierro_gb300 import sgh
    prob = _deck()
    nie = np.ascontiguousarray(prob.mesh.nodes_in_elem, dtype=np.uint64).copy()
    xyz = np.ascontiguousarray(prob.mesh.coords, dtype=np.float64).copy()
    st = sgh.empty_state(prob.mesh.num_nodes, prob.mesh.num_elems, prob.num_state_vars)
    sv = np.ascontiguousarray(prob.state_vars())
    cases = [(prob.mesh.num_nodes, 0, 0, "at least one element"),
             (7, 1, 0, "at least one element"),
             (prob.mesh.num_nodes, prob.mesh.num_elems, 1, "num_dims"),
             (prob.mesh.num_nodes, 2 ** 28, 0, "32-bit"),
             (2 ** 31, prob.mesh.num_elems, 0, "32-bit")]
    for nn, ne, dims, text in cases:
        m = sgh.Mesh(nn, ne, nie.ctypes.data, xyz.ctypes.data, dims)
        rc = sgh.lib().fierro_sgh_setup(C.byref(m), sgh.c_materials(prob), len(prob.materials), sv.ctypes.data,
                                        prob.num_state_vars, sgh.c_fills(prob), len(prob.fills),
                                        sgh.c_boundaries(prob), len(prob.boundaries), C.byref(sgh.c_state(st)))
        msg = sgh.lib().fierro_last_error().decode()
        assert rc == sgh.FIERRO_EINVAL and text in msg, (nn, ne, dims, rc, msg)
    m = sgh.Mesh(prob.mesh.num_nodes, prob.mesh.num_elems, None, xyz.ctypes.data, 0)
    rc = sgh.lib().fierro_sgh_setup(C.byref(m), sgh.c_materials(prob), len(prob.materials), sv.ctypes.data,
                                    prob.num_state_vars, sgh.c_fills(prob), len(prob.fills),
                                    sgh.c_boundaries(prob), len(prob.boundaries), C.byref(sgh.c_state(st)))
    assert rc == sgh.FIERRO_EINVAL and "NULL" in sgh.lib().fierro_last_error().decode()


def test_setup_rejects_unsupported_models(lib_built):
    from fierro_gb300 import sgh
    prob = _deck()

    def eos(mats):
        mats[0].eos_model = 1

    def unknown_strength(mats):
        mats[0].strength_type = 3

    rc, msg = _setup_rc(prob, mutate_mat=eos)
    assert rc == sgh.FIERRO_ENOTSUP and "EOS" in msg
    rc, msg = _setup_rc(prob, mutate_mat=unknown_strength)
    assert rc == sgh.FIERRO_EINVAL and "strength_type" in msg


@pytest.mark.parametrize("kind", ["hypo", "hyper"])
def test_setup_with_strength_material(lib_built, oracle_built, kind):
    """setup (setup.cpp:10-424) with a strength material: stress zero, the state
    variables (shear modulus in statev(3)) copied from the material, the rest as
    without strength; equal to the C restatement's setup."""
    from fierro_gb300 import sgh
    from oracle import orc
    prob = _deck()
    prob.materials[0].strength = kind
    prob.materials[0].shear_modulus = 2.5
    st = sgh.setup(prob)
    assert np.all(st["elem_stress"] == 0.0)
    assert np.all(st["elem_statev"][:, 3] == 2.5)
    o = orc.Oracle(prob)
    r = o.state()
    np.testing.assert_array_equal(st["elem_statev"], r["statev"])
    np.testing.assert_array_equal(st["elem_sie"][1], r["sie"])
    np.testing.assert_array_equal(st["elem_pres"], r["pres"])


def test_reflected_bc_needs_plane(lib_built):
    from fierro_gb300 import problems, sgh
    prob = _deck()
    prob.boundaries = [problems.Boundary("sphere", 0.5, "reflected")]
    with pytest.raises(sgh.FierroError) as ei:
        sgh.setup(prob)
    assert ei.value.code == sgh.FIERRO_EINVAL


def test_handle_without_gpu_reports_error(lib_built):
    """Creating a device handle where no GPU is visible fails with an error code
    (no CPU fallback, no crash)."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is visible")
    from fierro_gb300 import sgh
    with pytest.raises(sgh.FierroError) as ei:
        sgh.SGHSolver(_deck())
    assert ei.value.code in (sgh.FIERRO_ECUDA, sgh.FIERRO_ENOMEM)


@pytest.mark.parametrize("case", ["sedov_rz12", "noh_rz10_jp"])
def test_rz_setup_matches_oracle(lib_built, oracle_built, case):
    """setup with num_dims == 2: RZ volumes, fills, radial velocities, boundary
    conditions and the areal node masses from Barlow's corner areas equal the
    2D-RZ restatement bit for bit."""
    from fierro_gb300 import problems, sgh
    from oracle import orc
    prob = {"sedov_rz12": lambda: problems.sedov_rz(12),
            "noh_rz10_jp": lambda: problems.noh_rz(10, jitter=0.1, seed=4, permute=True)}[case]()
    st = sgh.setup(prob)
    ref = orc.Oracle(prob).state()
    got = {"coords": st["node_coords"][1], "vel": st["node_vel"][1], "den": st["elem_den"],
           "pres": st["elem_pres"], "sie": st["elem_sie"][1], "sspd": st["elem_sspd"], "vol": st["elem_vol"],
           "mass": st["elem_mass"], "node_mass": st["node_mass"], "coords0": st["node_coords"][0]}
    assert_bitwise(got, ref, list(got), label=case)


def test_rz_setup_rejects_reference_defects(lib_built):
    from fierro_gb300 import problems, sgh
    p = problems.noh_rz(4)
    p.fills[0].velocity = "spherical"
    with pytest.raises(sgh.FierroError) as ei:
        sgh.setup(p)
    assert ei.value.code == sgh.FIERRO_ENOTSUP
    p = problems.sedov_rz(4)
    p.boundaries.append(problems.Boundary("z_plane", 0.0, "reflected"))
    with pytest.raises(sgh.FierroError) as ei:
        sgh.setup(p)
    assert ei.value.code == sgh.FIERRO_EINVAL


@pytest.mark.parametrize("dims", [3, 2])
def test_host_setup_random_decks(lib_built, oracle_built, dims):
    """Host set-up of seeded random decks (uneven boxes, several materials, box /
    sphere / cylinder fills, cartesian / radial / spherical velocities, fixed and
    reflecting planes) equals the restatement's set-up bit for bit."""
    from decks import random_deck
    from fierro_gb300 import sgh
    from oracle import orc
    for seed in range(24):
        prob = random_deck(seed, dims)
        st = sgh.setup(prob)
        r = orc.Oracle(prob).state()
        got = {"coords": st["node_coords"][1], "vel": st["node_vel"][1], "den": st["elem_den"],
               "pres": st["elem_pres"], "sie": st["elem_sie"][1], "sspd": st["elem_sspd"], "vol": st["elem_vol"],
               "mass": st["elem_mass"], "node_mass": st["node_mass"]}
        assert_bitwise(got, r, list(got), label="%s" % prob.name)


def test_host_setup_thin_meshes(lib_built, oracle_built):
    """Host set-up of boxes one element thick, down to one element (hex and
    2D-RZ), equals the restatement's set-up bit for bit."""
    from decks import THIN_SHAPES, THIN_SHAPES_RZ, thin_deck
    from fierro_gb300 import sgh
    from oracle import orc
    for shape in THIN_SHAPES + THIN_SHAPES_RZ:
        prob = thin_deck(shape)
        st = sgh.setup(prob)
        r = orc.Oracle(prob).state()
        got = {"coords": st["node_coords"][1], "vel": st["node_vel"][1], "den": st["elem_den"],
               "pres": st["elem_pres"], "sie": st["elem_sie"][1], "sspd": st["elem_sspd"], "vol": st["elem_vol"],
               "mass": st["elem_mass"], "node_mass": st["node_mass"]}
        assert_bitwise(got, r, list(got), label=prob.name)


def test_integration_notes_show_the_compiled_binding():
    """The sgh_solve replacement shown in INTEGRATION.md section 1 is the text
    that tests/test_gpu_binding.py compiles into the reference's driver
    (oracle/ref/fierro_sgh_call.inc), so the documented binding is the tested one."""
    import re
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    with open(os.path.join(root, "INTEGRATION.md")) as f:
        doc = f.read()
    sec = doc[doc.index("## 1."):doc.index("## 2.")]
    blocks = re.findall(r"```cpp\n(.*?)```\n", sec, flags=re.S)
    with open(os.path.join(root, "oracle", "ref", "fierro_sgh_call.inc")) as f:
        inc = f.read()
    assert blocks and blocks[0] == inc
