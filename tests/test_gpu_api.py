"""GPU checks of the C ABI's behaviour: one-shot sgh_solve equals the handle path,
graph replay equals stage stepping and event-timed runs, state round trips,
stopping at time_final, and error reporting (including a device-detected
inverted element, after which the context stays usable)."""
import numpy as np
import pytest

from conftest import assert_bitwise

pytestmark = pytest.mark.gpu

FIELDS = ("coords", "vel", "den", "pres", "sie", "sspd", "vol")


def _prob():
    from fierro_gb300 import problems
    return problems.sedov(10, jitter=0.1, seed=4, permute=True, cycles=25)


def test_set_get_roundtrip(lib_built):
    from fierro_gb300 import sgh
    prob = _prob()
    st = sgh.setup(prob)
    with sgh.SGHSolver(prob) as s:
        s.set_state(st)
        back = s.get_state()
    for k in ("node_coords", "node_vel", "node_mass", "elem_den", "elem_pres", "elem_sspd", "elem_sie",
              "elem_vol", "elem_mass"):
        assert np.array_equal(back[k], st[k]), k


def test_one_shot_solve_equals_handle(lib_built):
    from fierro_gb300 import sgh
    prob = _prob()
    st = sgh.setup(prob)
    one = {k: v.copy() for k, v in st.items()}
    info = sgh.sgh_solve(prob, one, cycle_stop=25)
    with sgh.SGHSolver(prob) as s:
        s.set_state(st)
        assert s.run(25) == 25
        h = s.get_state()
        t = s.time()
    assert info["cycles"] == 25 and info["time_value"] == t[0]
    a, b = sgh.compared_fields(one), sgh.compared_fields(h)
    assert_bitwise(a, b, FIELDS)
    assert np.array_equal(one["corner_force"], h["corner_force"])


def test_graph_stage_and_timed_paths_agree(lib_built):
    from fierro_gb300 import sgh
    prob = _prob()
    st = sgh.setup(prob)
    outs = []
    for how in ("graph", "stages", "timed"):
        with sgh.SGHSolver(prob) as s:
            s.set_state(st)
            if how == "graph":
                s.run(7)
            elif how == "stages":
                s.run_stages(14)
            else:
                ran, tot, kms = s.run_timed(7)
                assert ran == 7 and tot > 0 and len(kms) == s.launches_per_cycle
            outs.append(sgh.compared_fields(s.get_state()))
            assert s.time()[3] == 7
    assert_bitwise(outs[0], outs[1], FIELDS, "graph vs stages")
    assert_bitwise(outs[0], outs[2], FIELDS, "graph vs timed")


def test_stops_at_time_final(lib_built, oracle_built):
    from fierro_gb300 import problems, sgh
    from oracle import orc
    prob = problems.noh(8, cycles=10 ** 6)
    prob.params.time_final = 0.05
    st = sgh.setup(prob)
    with sgh.SGHSolver(prob) as s:
        s.set_state(st)
        ran = s.run(2000)
        t = s.time()
        out = sgh.compared_fields(s.get_state())
    o = orc.Oracle(prob, variant="crpow")
    n = o.run_cycles(2000)
    assert ran == n and t[0] == 0.05 == o.time()[0]
    assert_bitwise(out, o.state(), FIELDS, "noh8 to time_final")


def test_error_codes(lib_built):
    from fierro_gb300 import sgh
    prob = _prob()
    st = sgh.setup(prob)
    with sgh.SGHSolver(prob) as s:
        with pytest.raises(sgh.FierroError) as ei:
            s.run(1)  # before set_state
        assert ei.value.code == sgh.FIERRO_EINVAL
        bad = {k: v.copy() for k, v in st.items()}
        bad["elem_vol"][3] = -1.0
        with pytest.raises(sgh.FierroError) as ei:
            s.set_state(bad)
        assert ei.value.code == sgh.FIERRO_ENUMERIC
        bad = {k: v.copy() for k, v in st.items()}
        bad["elem_stress"][1, 2, 0, 1] = 1.0
        with pytest.raises(sgh.FierroError) as ei:
            s.set_state(bad)
        assert ei.value.code == sgh.FIERRO_ENOTSUP
        bad = {k: v.copy() for k, v in st.items()}
        bad["elem_mat_id"][0] = 7
        with pytest.raises(sgh.FierroError) as ei:
            s.set_state(bad)
        assert ei.value.code == sgh.FIERRO_EINVAL


def test_device_detects_inverted_element_and_recovers(lib_built):
    """A velocity field that crushes one element inverts it within a cycle: the
    element kernel flags it, run() returns ENUMERIC, and the same handle then
    runs a valid state normally (the status is a flag, never a trap)."""
    from fierro_gb300 import sgh
    prob = _prob()
    prob.params.dt_start = 1e-2
    prob.params.dt_min = 1e-2
    st = sgh.setup(prob)
    bad = {k: v.copy() for k, v in st.items()}
    e = 200
    nodes = prob.mesh.nodes_in_elem[e]
    cen = prob.mesh.coords[nodes].mean(axis=0)
    for n in nodes:
        bad["node_vel"][1, n] = -500.0 * (prob.mesh.coords[n] - cen)
    with sgh.SGHSolver(prob) as s:
        s.set_state(bad)
        with pytest.raises(sgh.FierroError) as ei:
            s.run(3)
        assert ei.value.code == sgh.FIERRO_ENUMERIC
        s.set_state(st)
        assert s.run(2) == 2
        out = s.get_state()
        assert np.all(out["elem_vol"] > 0)


def test_direct_and_staged_transfers_agree(lib_built, monkeypatch):
    """The GPU-side transfer (kernels reading and writing the caller's host
    arrays) and the staged transfer (host permutation through pinned buffers)
    give the same device state, the same results and the same validation
    errors."""
    from fierro_gb300 import sgh
    prob = _prob()
    st = sgh.setup(prob)
    outs = []
    for staged in ("0", "1"):
        monkeypatch.setenv("FIERRO_STAGED_TRANSFERS", staged)
        with sgh.SGHSolver(prob) as s:
            s.set_state(st)
            s.run(6)
            outs.append(s.get_state())
            bad = {k: v.copy() for k, v in st.items()}
            bad["elem_vol"][5] = float("nan")
            with pytest.raises(sgh.FierroError) as ei:
                s.set_state(bad)
            assert ei.value.code == sgh.FIERRO_ENUMERIC and "element 5" in str(ei.value)
            bad = {k: v.copy() for k, v in st.items()}
            bad["node_mass"][9] = 0.0
            with pytest.raises(sgh.FierroError) as ei:
                s.set_state(bad)
            assert ei.value.code == sgh.FIERRO_EINVAL and "node 9" in str(ei.value)
    for k in outs[0]:
        assert np.array_equal(outs[0][k], outs[1][k]), k


def test_device_topology_rejects_corrupt_meshes(lib_built, monkeypatch):
    """Handle creation validates the mesh on the GPU (direct host access) and on
    the host (staged builder) alike: out-of-range node ids, repeated nodes in an
    element and non-finite coordinates are refused with the caller's index."""
    import copy
    from fierro_gb300 import sgh
    for staged in ("0", "1"):
        monkeypatch.setenv("FIERRO_STAGED_TRANSFERS", staged)
        prob = _prob()
        cases = []
        p = copy.deepcopy(prob)
        p.mesh.nodes_in_elem[17, 3] = p.mesh.num_nodes + 5
        cases.append((p, "element 17"))
        p = copy.deepcopy(prob)
        p.mesh.nodes_in_elem[23, 6] = p.mesh.nodes_in_elem[23, 1]
        cases.append((p, "element 23"))
        p = copy.deepcopy(prob)
        p.mesh.coords[11, 2] = float("inf")
        cases.append((p, "coordinate at %d" % (11 * 3 + 2)))
        for p, where in cases:
            with pytest.raises(sgh.FierroError) as ei:
                sgh.SGHSolver(p)
            assert ei.value.code == sgh.FIERRO_EINVAL and where in str(ei.value), (staged, str(ei.value))


def _mixed_deck():
    """Box / sphere / cylinder fills in sequence (later fills overwrite), three
    velocity kinds, reflected planes and fixed curved surfaces."""
    from fierro_gb300 import problems
    from fierro_gb300.problems import Boundary, Fill, Material, Params, Problem
    from fierro_gb300.mesh import box_mesh
    m = box_mesh(11, length=1.0, jitter=0.1, seed=9, permute=True, name="mixed")
    fills = [Fill("global", 0, den=1.0, sie=1e-10),
             Fill("box", 1, x1=0.0, x2=0.35, y1=0.0, y2=0.35, z1=0.0, z2=0.35, den=2.0, sie=3.0),
             Fill("sphere", 0, radius1=0.3, radius2=0.6, velocity="spherical", speed=-0.7, den=1.5, sie=0.2),
             Fill("cylinder", 1, radius1=0.0, radius2=0.25, velocity="radial", speed=0.4, den=0.8, sie=1.0),
             Fill("box", 0, x1=0.6, x2=1.0, y1=0.6, y2=1.0, z1=0.0, z2=1.0, velocity="cartesian", u=0.1, v=-0.2,
                  w=0.3, den=1.1, sie=0.5)]
    mats = [Material(gamma=1.4), Material(gamma=5.0 / 3.0, q1=1.2, q2ex=0.5)]
    bcs = [Boundary("x_plane", 0.0, "reflected"), Boundary("y_plane", 0.0, "reflected"),
           Boundary("sphere", 1.0, "fixed"), Boundary("cylinder", 0.9, "fixed")]
    return Problem("mixed", m, mats, fills, bcs, Params(cycle_stop=10))


def test_gpu_setup_equals_host_setup(lib_built, monkeypatch):
    """fierro_sgh_setup on the GPU (kernels reading the mesh in place) writes the
    same initial state, bit for bit, as the host set-up."""
    from fierro_gb300 import problems, sgh
    decks = [_prob(), problems.noh(9, jitter=0.1, seed=2, permute=True), _mixed_deck()]
    for prob in decks:
        monkeypatch.setenv("FIERRO_STAGED_TRANSFERS", "0")
        a = sgh.setup(prob)
        monkeypatch.setenv("FIERRO_STAGED_TRANSFERS", "1")
        b = sgh.setup(prob)
        for k in a:
            assert np.array_equal(a[k], b[k]), (prob.name, k)
    # and the mixed deck runs through the device topology and transfers
    monkeypatch.setenv("FIERRO_STAGED_TRANSFERS", "0")
    prob = _mixed_deck()
    with sgh.SGHSolver(prob) as s:
        s.set_state(sgh.setup(prob))
        assert s.run(10) == 10


def test_device_view_is_zero_copy_torch(lib_built):
    """fierro_sgh_device_view through DLPack: torch tensors over the handle's own
    memory, equal (through the renumbering maps) to get_state."""
    torch = pytest.importorskip("torch")
    from fierro_gb300 import sgh
    prob = _prob()
    st = sgh.setup(prob)
    with sgh.SGHSolver(prob) as s:
        s.set_state(st)
        s.run(5)
        host = s.get_state()
        v = s.device_view()
        n2e = v["node_int2ext"].long().cpu().numpy()
        e2e = v["elem_int2ext"].long().cpu().numpy()
        assert np.array_equal(v["x"].cpu().numpy(), host["node_coords"][1][n2e, 0])
        assert np.array_equal(v["w"].cpu().numpy(), host["node_vel"][1][n2e, 2])
        assert np.array_equal(v["sie"].cpu().numpy(), host["elem_sie"][1][e2e])
        assert np.array_equal(v["den"].cpu().numpy(), host["elem_den"][e2e])
        cf = v["corner_force"].cpu().numpy()  # [lid*3+dim][e]
        assert np.array_equal(cf.T.reshape(-1, 8, 3), host["corner_force"].reshape(-1, 8, 3)[e2e])
        assert np.array_equal(v["node_ext2int"].long().cpu().numpy()[n2e], np.arange(prob.mesh.num_nodes))
        # zero copy: a second view aliases the same memory
        assert s.device_view()["den"].data_ptr() == v["den"].data_ptr()


@pytest.mark.parametrize("kind", ["velocity", "contact"])
def test_other_boundary_kinds_leave_nodes_free(oracle_built, lib_built, kind):
    """Boundary sets of the kinds the reference's boundary_velocity has no
    branch for run as the reference runs them, holding no velocity component:
    bit for bit the same run as without the set, and as the restatement."""
    import copy
    from fierro_gb300 import problems, sgh
    from oracle import orc
    prob = problems.noh(8, jitter=0.1, seed=4, permute=True, cycles=30)
    plus = copy.deepcopy(prob)
    plus.boundaries.append(problems.Boundary("x_plane", 1.0, kind))
    got = {}
    for name, p in (("plus", plus), ("plain", prob)):
        with sgh.SGHSolver(p) as s:
            s.set_state(sgh.setup(p))
            s.run(30)
            got[name] = sgh.compared_fields(s.get_state())
    fields = ("coords", "vel", "den", "pres", "sie", "sspd", "vol")
    for k in fields:
        assert np.array_equal(got["plus"][k], got["plain"][k]), k
    o = orc.Oracle(plus, variant="crpow")
    o.run_cycles(30)
    ref = o.state()
    for k in fields:
        assert np.array_equal(got["plus"][k], ref[k]), k


def _shifted_like(a: np.ndarray, shift: int) -> np.ndarray:
    """A C-contiguous float64 array shaped like `a` whose data starts `shift`
    bytes into a fresh buffer (shift 8: 8- but not 16-byte aligned)."""
    raw = np.zeros(a.nbytes + 64, dtype=np.uint8)
    base = (-raw.ctypes.data) % 16 + shift
    return np.frombuffer(raw.data, dtype=a.dtype, count=a.size, offset=base).reshape(a.shape)


@pytest.mark.parametrize("strength", [False, True])
def test_download_into_unevenly_aligned_host_arrays(lib_built, strength):
    """get_state writes the node, corner-force and stress rows with 16-byte
    stores where the host address allows: host arrays that start 8 bytes off a
    16-byte boundary (odd and even node and element counts) receive the same
    values as 16-byte aligned ones."""
    from fierro_gb300 import problems, sgh
    for n in (9, 10):
        prob = problems.sedov_mixed_strength(n, cycles=6) if strength else \
            problems.sedov(n, jitter=0.1, seed=4, permute=True, cycles=6)
        st = sgh.setup(prob)
        with sgh.SGHSolver(prob) as s:
            s.set_state(st)
            s.run(6)
            ref = s.get_state()
            for shift in (8, 0):
                out = {k: (_shifted_like(v, shift) if v.dtype == np.float64 else v.copy()) for k, v in ref.items()}
                for k in out:
                    if out[k].dtype == np.float64:
                        # the written fields start as NaN; the state variables as the handle holds them
                        out[k][...] = ref[k] if k == "elem_statev" else np.nan
                s.get_state(out)
                for k in ref:
                    assert np.array_equal(out[k], ref[k]), (n, shift, k)
