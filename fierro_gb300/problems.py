"""Problem decks: the material / fill / boundary / control records the SGH
solver's ``input()`` produces (Explicit-Lagrange-Kokkos/SGH_solver/input.cpp:50-653),
as plain data, plus builders for the benchmark problems (Sedov and Noh on box
meshes).  The same deck drives the GB300 library, the CPU oracle and the
reference oracle build, so all three see identical inputs.
"""
from __future__ import annotations

from dataclasses import dataclass, field
from typing import List

import numpy as np

from .mesh import HexMesh, box_mesh, hex_volumes, quad_mesh

# region::vol_tag (mesh.h:824-830)
REGION = {"global": 0, "box": 1, "cylinder": 2, "sphere": 3}
# init_conds::init_velocity_conds (mesh.h:839-852)
VELOCITY = {"cartesian": 0, "radial": 1, "spherical": 2, "radial_linear": 3,
            "spherical_linear": 4, "tg_vortex": 5}
# bdy::bdy_tag and bdy::bdy_hydro_conds (mesh.h:897-918)
SURFACE = {"x_plane": 0, "y_plane": 1, "z_plane": 2, "cylinder": 3, "sphere": 4}
# bdy_hydro_conds (mesh.h:910-918); boundary_velocity (boundary.cpp:10-55) acts on
# fixed and reflected sets only, the other kinds leave their nodes free
HYDRO_BC = {"fixed": 0, "reflected": 1, "velocity": 2, "pressure": 3, "acceleration": 4, "contact": 5}
# model::strength_tag (state.h:103-113)
STRENGTH = {"none": 0, "hypo": 1, "hyper": 2}


@dataclass
class Material:
    """material_t (state.h:130-178) with its model state variables:
    statev(0) = gamma, statev(1) = minimum sound speed, statev(2) = c_v,
    statev(3) = the shear modulus read by the shipped strength model.
    ``strength`` is the strength_type: "none", "hypo" (stress updated in the
    force pass) or "hyper" (updated in the state pass)."""
    q1: float = 1.0
    q1ex: float = 1.0
    q2: float = 1.3333
    q2ex: float = 0.0
    gamma: float = 5.0 / 3.0
    csmin: float = 1.0e-14
    cv: float = 1.0
    strength: str = "none"
    shear_modulus: float = 0.0

    @property
    def strength_type(self) -> int:
        return STRENGTH[self.strength]

    def state_vars(self, n: int) -> List[float]:
        sv = [self.gamma, self.csmin, self.cv, self.shear_modulus] + [0.0] * max(0, n - 4)
        return sv[:n]


@dataclass
class Fill:
    """mat_fill_t (mesh.h:858-890)."""
    volume: str = "global"
    mat_id: int = 0
    x1: float = 0.0
    x2: float = 0.0
    y1: float = 0.0
    y2: float = 0.0
    z1: float = 0.0
    z2: float = 0.0
    radius1: float = 0.0
    radius2: float = 0.0
    velocity: str = "cartesian"
    u: float = 0.0
    v: float = 0.0
    w: float = 0.0
    speed: float = 0.0
    sie: float = 0.0
    den: float = 1.0


@dataclass
class Boundary:
    """boundary_t (mesh.h:924-935)."""
    surface: str = "x_plane"
    value: float = 0.0
    hydro_bc: str = "reflected"


@dataclass
class Params:
    """The scalar controls of sgh_solve (mesh.h:1175-1208) with the reference
    defaults (driver.cpp:35-62, input.cpp:73-82)."""
    time_final: float = 1.0e16
    dt_max: float = 1.0e-2
    dt_min: float = 1.0e-8
    dt_cfl: float = 0.4
    dt_start: float = 1.0e-5
    graphics_dt_ival: float = 1.0e8
    graphics_cyc_ival: int = 1000000
    cycle_stop: int = 100
    rk_num_stages: int = 2
    fuzz: float = 1.0e-16
    tiny: float = 1.0e-12
    small: float = 1.0e-8


@dataclass
class Problem:
    name: str
    mesh: HexMesh
    materials: List[Material]
    fills: List[Fill]
    boundaries: List[Boundary]
    params: Params
    num_state_vars: int = 6
    info: dict = field(default_factory=dict)

    def state_vars(self) -> np.ndarray:
        return np.array([m.state_vars(self.num_state_vars) for m in self.materials], dtype=np.float64)

    def config_text(self) -> str:
        """The deck in the text format read by the reference oracle's input()."""
        p = self.params
        out = [
            "dt_start %r" % p.dt_start, "time_final %r" % p.time_final, "dt_max %r" % p.dt_max,
            "dt_min %r" % p.dt_min, "dt_cfl %r" % p.dt_cfl, "graphics_dt_ival %r" % p.graphics_dt_ival,
            "graphics_cyc_ival %d" % p.graphics_cyc_ival, "cycle_stop %d" % p.cycle_stop,
            "rk_num_stages %d" % p.rk_num_stages, "num_state_vars %d" % self.num_state_vars,
        ]
        if self.mesh.dims == 2:
            out.append("num_dims 2")
        for m in self.materials:
            sv = " ".join(repr(float(v)) for v in m.state_vars(self.num_state_vars))
            out.append("material %r %r %r %r %s" % (m.q1, m.q1ex, m.q2, m.q2ex, sv))
        for f in self.fills:
            vals = [REGION[f.volume], f.mat_id, f.x1, f.x2, f.y1, f.y2, f.z1, f.z2, f.radius1,
                    f.radius2, VELOCITY[f.velocity], f.u, f.v, f.w, f.speed, f.sie, f.den]
            out.append("fill " + " ".join(repr(float(v)) for v in vals))
        for b in self.boundaries:
            out.append("bc %d %r %d" % (SURFACE[b.surface], float(b.value), HYDRO_BC[b.hydro_bc]))
        for i, m in enumerate(self.materials):
            if m.strength_type:
                out.append("strength %d %d" % (i, m.strength_type))
        return "\n".join(out) + "\n"


def _planes_at_zero(kind="reflected"):
    return [Boundary("x_plane", 0.0, kind), Boundary("y_plane", 0.0, kind), Boundary("z_plane", 0.0, kind)]


def sedov(n: int = 12, length: float = 1.2, energy: float = 0.2467, gamma: float = 1.4,
          cycles: int = 200, jitter: float = 0.0, seed: int = 0, permute: bool = False,
          geo_digits: int | None = None, mesh: HexMesh | None = None, cfl: float = 0.4) -> Problem:
    """Sedov 3D blast: rho=1, sie=1e-10, u=0 everywhere; the element at the origin
    corner holds total energy `energy` (sie = energy / (rho V)); reflecting planes
    x=y=z=0.  Defaults are the 12^3 Sedov case on [0,1.2]^3."""
    if mesh is None:
        mesh = box_mesh(n, length=length, jitter=jitter, seed=seed, permute=permute,
                        geo_digits=geo_digits, name="sedov%d" % n)
    h = length / n
    # the origin-corner element is the one element holding the node at the origin
    n0 = int(np.argmin(np.einsum("ij,ij->i", mesh.coords, mesh.coords)))
    origin = np.nonzero(np.any(mesh.nodes_in_elem == n0, axis=1))[0]
    assert origin.size == 1, "origin element not unique"
    e0 = int(origin[0])
    v0 = float(hex_volumes(mesh.coords, mesh.nodes_in_elem[e0:e0 + 1])[0])
    sie0 = energy / (1.0 * v0)
    fills = [
        Fill("global", 0, den=1.0, sie=1.0e-10, velocity="cartesian"),
        Fill("box", 0, x1=0.0, x2=h, y1=0.0, y2=h, z1=0.0, z2=h, den=1.0, sie=sie0, velocity="cartesian"),
    ]
    params = Params(time_final=1.0, dt_cfl=cfl, cycle_stop=cycles)
    mat = Material(q1=1.0, q1ex=1.0, q2=1.3333, q2ex=0.0, gamma=gamma, csmin=1.0e-14, cv=1.0)
    return Problem("sedov", mesh, [mat], fills, _planes_at_zero(), params,
                   info={"origin_elem": e0, "origin_sie": sie0, "h": h})


def noh(n: int = 32, length: float = 1.0, gamma: float = 5.0 / 3.0, speed: float = -1.0,
        cycles: int = 500, jitter: float = 0.0, seed: int = 0, permute: bool = False,
        geo_digits: int | None = None, mesh: HexMesh | None = None, cfl: float = 0.3) -> Problem:
    """Noh 3D implosion: rho=1, sie=1e-10, node velocity = speed * r/|r| (zero at the
    origin), symmetry planes x=y=z=0, MARS q1=1, q2=1.3333, q1ex=1, q2ex=0."""
    if mesh is None:
        mesh = box_mesh(n, length=length, jitter=jitter, seed=seed, permute=permute,
                        geo_digits=geo_digits, name="noh%d" % n)
    fills = [Fill("global", 0, den=1.0, sie=1.0e-10, velocity="spherical", speed=speed)]
    params = Params(time_final=0.6, dt_cfl=cfl, cycle_stop=cycles)
    mat = Material(q1=1.0, q1ex=1.0, q2=1.3333, q2ex=0.0, gamma=gamma, csmin=1.0e-14, cv=1.0)
    return Problem("noh", mesh, [mat], fills, _planes_at_zero(), params)


def taylor_anvil(mesh: HexMesh, cycles: int = 300) -> Problem:
    """Taylor anvil 3D, the deck of the reference's own test
    (tests-for-Explicit-Lagrange-Kokkos/input_for_TaylorAnvil3D_test.cpp:112-160,
    mesh Explicit-Lagrange/meshes/mesh_z_taylorAnvil.geo, a quarter rod on an
    O-grid): gamma 5/3 gas, rho=1, sie=1e-9, every node moving at w=-1 into the
    reflecting plane z=0, symmetry planes x=0 and y=0; time_final 25."""
    fills = [Fill("global", 0, den=1.0, sie=1.0e-9, velocity="cartesian", u=0.0, v=0.0, w=-1.0)]
    params = Params(time_final=25.0, dt_cfl=0.4, cycle_stop=cycles)
    mat = Material(q1=1.0, q1ex=1.0, q2=1.3333, q2ex=0.0, gamma=5.0 / 3.0, csmin=1.0e-14, cv=1.0)
    return Problem("taylor_anvil", mesh, [mat], fills, _planes_at_zero(), params)


def triple_point(mesh: HexMesh, cycles: int = 400) -> Problem:
    """Triple point, the deck of the reference's input.cpp:482-593: gamma 5/3,
    rho=1 / sie=2.5 everywhere, then the box x in [1, 7], y in [0, 1.5] at rho=1,
    sie=0.25 and the box x in [1, 7], y in [1.5, 3] at rho=0.1, sie=2.5 (the
    deck's three fills; its num_fills of 2 would drop the third); reflecting planes
    on the six faces of the mesh's bounding box (the deck's x plane sits at 6.0,
    "some meshes are 7 and others are 6": the far planes here are the mesh's own
    extents); time_final 4."""
    lo, hi = mesh.coords.min(axis=0), mesh.coords.max(axis=0)
    fills = [
        Fill("global", 0, den=1.0, sie=2.5, velocity="cartesian"),
        Fill("box", 0, x1=1.0, x2=7.0, y1=0.0, y2=1.5, z1=0.0, z2=1.0, den=1.0, sie=0.25, velocity="cartesian"),
        Fill("box", 0, x1=1.0, x2=7.0, y1=1.5, y2=3.0, z1=0.0, z2=1.0, den=0.1, sie=2.5, velocity="cartesian"),
    ]
    bcs = [Boundary("x_plane", float(lo[0])), Boundary("y_plane", float(lo[1])), Boundary("z_plane", float(lo[2])),
           Boundary("x_plane", float(hi[0])), Boundary("y_plane", float(hi[1])), Boundary("z_plane", float(hi[2]))]
    params = Params(time_final=4.0, dt_cfl=0.4, cycle_stop=cycles)
    mat = Material(q1=1.0, q1ex=1.0, q2=1.3333, q2ex=0.0, gamma=5.0 / 3.0, csmin=1.0e-14, cv=1.0)
    return Problem("triple_point", mesh, [mat], fills, bcs, params)


def taylor_anvil_rz(nx: int = 40, ny: int = 4, length=(38.1, 3.81), cycles: int = 300, jitter: float = 0.0,
                    seed: int = 0, permute: bool = False, mesh: HexMesh | None = None) -> Problem:
    """2D-RZ Taylor anvil, the deck of the reference's own test
    (tests-for-Explicit-Lagrange-Kokkos/input_for_TaylorAnvilRZ_test.cpp:112-151;
    its mesh_taylorAnvil_2D_RZ.geo is not in the tree, so the rod is an nx x ny
    quad mesh with the 3D rod's length and radius, x axial, y radial): gamma 5/3
    gas, rho=1, sie=1e-9, every node moving at u=-1 into the reflecting plane
    x=0, the axis y=0 reflecting; time_final 25."""
    if mesh is None:
        mesh = quad_mesh(nx, ny, length=length, jitter=jitter, seed=seed, permute=permute,
                         name="taylor_anvil_rz%dx%d" % (nx, ny))
    fills = [Fill("global", 0, den=1.0, sie=1.0e-9, velocity="cartesian", u=-1.0, v=0.0)]
    params = Params(time_final=25.0, dt_cfl=0.4, cycle_stop=cycles)
    mat = Material(q1=1.0, q1ex=1.0, q2=1.3333, q2ex=0.0, gamma=5.0 / 3.0, csmin=1.0e-14, cv=1.0)
    bcs = [Boundary("x_plane", 0.0, "reflected"), Boundary("y_plane", 0.0, "reflected")]
    return Problem("taylor_anvil_rz", mesh, [mat], fills, bcs, params)


def sod_rz(nx: int = 100, ny: int = 2, cycles: int = 400, jitter: float = 0.0, seed: int = 0,
           permute: bool = False, mesh: HexMesh | None = None) -> Problem:
    """Sod shock tube along the axis in 2D-RZ, the SodZ deck of the reference's
    input.cpp:393-478: gamma 1.4, rho=1 and sie=2.5 everywhere, then rho=0.125 (same
    sie) in the box x in [0.5, 1]; reflecting planes x=0, y=0, x=1 and y=0.1 on an
    nx x ny quad mesh of [0, 1] x [0, 0.1] (x axial, y radial); time_final 0.2."""
    if mesh is None:
        mesh = quad_mesh(nx, ny, length=(1.0, 0.1), jitter=jitter, seed=seed, permute=permute,
                         name="sod_rz%dx%d" % (nx, ny))
    fills = [
        Fill("global", 0, den=1.0, sie=2.5, velocity="cartesian"),
        Fill("box", 0, x1=0.5, x2=1.0, y1=0.0, y2=1.0, z1=0.0, z2=1.0, den=0.125, sie=2.5, velocity="cartesian"),
    ]
    params = Params(time_final=0.2, dt_cfl=0.4, cycle_stop=cycles)
    mat = Material(q1=1.0, q1ex=1.0, q2=1.3333, q2ex=0.0, gamma=1.4, csmin=1.0e-14, cv=1.0)
    bcs = [Boundary("x_plane", 0.0, "reflected"), Boundary("y_plane", 0.0, "reflected"),
           Boundary("x_plane", 1.0, "reflected"), Boundary("y_plane", 0.1, "reflected")]
    return Problem("sod_rz", mesh, [mat], fills, bcs, params)


def sod_3d(mesh: HexMesh, cycles: int = 400) -> Problem:
    """Sod shock tube along x on a hex mesh of [0, 1] x [0, w] x [0, w]: the values
    of the SodZ deck (input.cpp:393-478: gamma 1.4, rho=1 and sie=2.5, then rho=0.125
    in x in [0.5, 1]) in 3D, with reflecting planes on the six faces of the mesh's
    bounding box; time_final 0.2.  On the reference's skewed Saltzman mesh
    (Explicit-Lagrange/meshes/mesh_Saltzman.geo) it exercises non-orthogonal hexes."""
    lo, hi = mesh.coords.min(axis=0), mesh.coords.max(axis=0)
    fills = [
        Fill("global", 0, den=1.0, sie=2.5, velocity="cartesian"),
        Fill("box", 0, x1=0.5, x2=1.0, y1=float(lo[1]), y2=float(hi[1]), z1=float(lo[2]), z2=float(hi[2]),
             den=0.125, sie=2.5, velocity="cartesian"),
    ]
    bcs = [Boundary("x_plane", float(lo[0])), Boundary("y_plane", float(lo[1])), Boundary("z_plane", float(lo[2])),
           Boundary("x_plane", float(hi[0])), Boundary("y_plane", float(hi[1])), Boundary("z_plane", float(hi[2]))]
    params = Params(time_final=0.2, dt_cfl=0.4, cycle_stop=cycles)
    mat = Material(q1=1.0, q1ex=1.0, q2=1.3333, q2ex=0.0, gamma=1.4, csmin=1.0e-14, cv=1.0)
    return Problem("sod_3d", mesh, [mat], fills, bcs, params)


def with_strength(problem: Problem, kind: str = "hypo", shear_modulus: float = 1.0) -> Problem:
    """The deck with every material given a strength model: ``kind`` is "hypo" or
    "hyper" (strength_type 1 or 2) and the shipped linear hypo-elastic model
    reads its shear modulus from statev(3)."""
    for m in problem.materials:
        m.strength = kind
        m.shear_modulus = shear_modulus
    problem.name = "%s_%s" % (problem.name, kind)
    return problem


def sedov_mixed_strength(n: int = 10, shear_modulus: float = 5.0, cycles: int = 50, jitter: float = 0.1,
                         seed: int = 5, permute: bool = True, length: float = 1.2) -> Problem:
    """Sedov with three materials: the gas without strength everywhere, a hypo
    material in the slab z < length/2 (it also holds the blast element) and a
    hyper material in the block x > length/2, z > length/2."""
    p = sedov(n, length=length, cycles=cycles, jitter=jitter, seed=seed, permute=permute)
    base = p.materials[0]
    mk = lambda kind: Material(q1=base.q1, q1ex=base.q1ex, q2=base.q2, q2ex=base.q2ex, gamma=base.gamma,
                               csmin=base.csmin, cv=base.cv, strength=kind, shear_modulus=shear_modulus)
    p.materials = [base, mk("hypo"), mk("hyper")]
    half = 0.5 * length
    glob, blast = p.fills
    p.fills = [glob,
               Fill("box", 1, x1=0.0, x2=length, y1=0.0, y2=length, z1=0.0, z2=half, den=1.0, sie=1.0e-10),
               Fill("box", 2, x1=half, x2=length, y1=0.0, y2=length, z1=half, z2=length, den=1.0, sie=1.0e-10),
               Fill(blast.volume, 1, x1=blast.x1, x2=blast.x2, y1=blast.y1, y2=blast.y2, z1=blast.z1, z2=blast.z2,
                    den=blast.den, sie=blast.sie, velocity=blast.velocity)]
    p.name = "sedov_mixed_strength"
    return p


def sedov_rz(n: int = 32, length: float = 1.2, energy: float = 0.49339, gamma: float = 5.0 / 3.0,
             cycles: int = 200, jitter: float = 0.0, seed: int = 0, permute: bool = False,
             mesh: HexMesh | None = None, cfl: float = 0.4, source_radius: float | None = None) -> Problem:
    """2D-RZ Sedov blast, the deck of the reference's RZ test
    (tests-for-Explicit-Lagrange-Kokkos/input_for_SedovRZ_test.cpp): n x n quads on
    [0, length]^2 (x axial, y radial), gamma 5/3, rho 1, sie 1e-10, a sphere of
    radius r (length/n, as the test's 1.2/64 on its 64 x 64 mesh, unless
    source_radius is given) at the origin holding sie = 0.5 energy / (rho pi r^3),
    four reflecting planes."""
    if mesh is None:
        mesh = quad_mesh(n, length=length, jitter=jitter, seed=seed, permute=permute, name="sedov_rz%d" % n)
    r2 = length / n if source_radius is None else float(source_radius)
    vol = 3.141592653589793 * (r2 ** 3 - 0.0 ** 3)
    fills = [
        Fill("global", 0, den=1.0, sie=1.0e-10, velocity="cartesian"),
        Fill("sphere", 0, radius1=0.0, radius2=r2, den=1.0, sie=0.5 * energy / (1.0 * vol), velocity="cartesian"),
    ]
    params = Params(time_final=1.0, dt_cfl=cfl, cycle_stop=cycles, graphics_dt_ival=1.0e8)
    mat = Material(q1=1.0, q1ex=1.0, q2=1.3333, q2ex=0.0, gamma=gamma, csmin=1.0e-14, cv=1.0)
    bcs = [Boundary("x_plane", 0.0, "reflected"), Boundary("y_plane", 0.0, "reflected"),
           Boundary("x_plane", length, "reflected"), Boundary("y_plane", length, "reflected")]
    return Problem("sedov_rz", mesh, [mat], fills, bcs, params, info={"h": length / n})


def noh_rz(n: int = 32, length: float = 1.0, gamma: float = 5.0 / 3.0, speed: float = -1.0,
           cycles: int = 300, jitter: float = 0.0, seed: int = 0, permute: bool = False,
           mesh: HexMesh | None = None, cfl: float = 0.4) -> Problem:
    """2D-RZ Noh implosion, the deck of the reference's RZ test
    (tests-for-Explicit-Lagrange-Kokkos/input_for_NohRZ_test.cpp): n x n quads on
    [0, length]^2, gamma 5/3, rho 1, sie 1e-9, velocity speed * (x, y)/|(x, y)|,
    reflecting planes x = 0 and y = 0 (the axis)."""
    if mesh is None:
        mesh = quad_mesh(n, length=length, jitter=jitter, seed=seed, permute=permute, name="noh_rz%d" % n)
    fills = [Fill("global", 0, den=1.0, sie=1.0e-9, velocity="radial", speed=speed)]
    params = Params(time_final=0.6, dt_cfl=cfl, cycle_stop=cycles)
    mat = Material(q1=1.0, q1ex=1.0, q2=1.3333, q2ex=0.0, gamma=gamma, csmin=1.0e-14, cv=1.0)
    bcs = [Boundary("x_plane", 0.0, "reflected"), Boundary("y_plane", 0.0, "reflected")]
    return Problem("noh_rz", mesh, [mat], fills, bcs, params)
