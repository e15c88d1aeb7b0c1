"""Seeded random problem decks for the parity tests (test infrastructure):
hex and 2D-RZ box meshes of uneven sizes and lengths, jittered or not, permuted
or not; one to three materials with random viscosity coefficients and gamma;
global, box, sphere and cylinder fills with cartesian, radial and (hex only)
spherical velocities; reflecting and fixed planes at either end; one to three
RK stages; 10 to 40 cycles."""
import numpy as np


def random_deck(seed: int, dims: int):
    from fierro_gb300 import mesh
    from fierro_gb300.problems import Boundary, Fill, Material, Params, Problem
    rng = np.random.default_rng(seed)
    if dims == 3:
        n = rng.integers(3, 9, size=3)
        L = rng.uniform(0.5, 2.0, size=3)
        m = mesh.box_mesh(int(n[0]), int(n[1]), int(n[2]), length=tuple(L), jitter=float(rng.uniform(0, 0.2)),
                          seed=int(seed), permute=bool(rng.integers(0, 2)))
    else:
        n = rng.integers(3, 12, size=2)
        L = rng.uniform(0.5, 2.0, size=2)
        m = mesh.quad_mesh(int(n[0]), int(n[1]), length=tuple(L), jitter=float(rng.uniform(0, 0.2)),
                           seed=int(seed), permute=bool(rng.integers(0, 2)))
    nmat = int(rng.integers(1, 4))
    mats = [Material(q1=float(rng.uniform(0.5, 1.5)), q1ex=float(rng.uniform(0.5, 1.5)),
                     q2=float(rng.uniform(0.5, 2.0)), q2ex=float(rng.uniform(0.0, 0.5)),
                     gamma=float(rng.uniform(1.2, 1.8)), csmin=1e-14) for _ in range(nmat)]
    fills = [Fill("global", 0, den=float(rng.uniform(0.5, 2)), sie=float(rng.uniform(1e-3, 1e-1)))]
    vel_kinds = ["cartesian", "radial"] + (["spherical"] if dims == 3 else [])
    for _ in range(int(rng.integers(1, 4))):
        vol = ["box", "sphere", "cylinder"][int(rng.integers(0, 3))]
        f = Fill(vol, int(rng.integers(0, nmat)), den=float(rng.uniform(0.5, 3)), sie=float(rng.uniform(0.01, 2.0)),
                 velocity=vel_kinds[int(rng.integers(0, len(vel_kinds)))])
        f.x1, f.x2 = (float(v) for v in sorted(rng.uniform(0, L[0], 2)))
        f.y1, f.y2 = (float(v) for v in sorted(rng.uniform(0, L[1], 2)))
        f.z1, f.z2 = (float(v) for v in sorted(rng.uniform(0, L[2], 2))) if dims == 3 else (-1.0, 1.0)
        f.radius1, f.radius2 = 0.0, float(rng.uniform(0.1, 1.0))
        f.u, f.v, f.w = (float(x) for x in rng.uniform(-0.3, 0.3, 3))
        f.speed = float(rng.uniform(-0.3, 0.3))
        fills.append(f)
    bcs = []
    planes = ["x_plane", "y_plane"] + (["z_plane"] if dims == 3 else [])
    for i, pl in enumerate(planes):
        if rng.integers(0, 2):
            bcs.append(Boundary(pl, 0.0, "reflected"))
        if rng.integers(0, 3) == 0:
            bcs.append(Boundary(pl, float(L[i]), "fixed" if rng.integers(0, 2) else "reflected"))
    params = Params(time_final=float(rng.uniform(0.05, 1.0)), dt_cfl=float(rng.uniform(0.2, 0.5)),
                    cycle_stop=int(rng.integers(10, 40)), rk_num_stages=int(rng.integers(1, 4)))
    return Problem("fuzz%d_%dd" % (seed, dims), m, mats, fills, bcs, params)


# Meshes one element thick in some direction, down to a single element: every
# node lies on the box's surface, the limiter of a lone element has no
# neighbour, and the Morton order and the patch tagging see degenerate extents.
THIN_SHAPES = [(1, 1, 1), (1, 1, 5), (1, 4, 3), (2, 1, 1), (7, 1, 1)]
THIN_SHAPES_RZ = [(1, 1), (1, 5), (6, 1), (2, 1)]


def thin_deck(shape, seed: int = 5, cycles: int = 30):
    """A jittered, permuted box (hex, or 2D-RZ quads for a two-entry shape) of
    `shape` elements with a hot, moving block in one corner, a reflecting plane
    at the origin (x = 0 for hexes, the axis y = 0 for quads) and a fixed plane
    at a far face (z for hexes, x for quads)."""
    from fierro_gb300 import mesh
    from fierro_gb300.problems import Boundary, Fill, Material, Params, Problem
    rng = np.random.default_rng(seed)
    dims = len(shape)
    L = tuple(float(v) for v in rng.uniform(0.5, 1.5, dims))
    if dims == 3:
        m = mesh.box_mesh(*shape, length=L, jitter=0.1, seed=seed, permute=True)
    else:
        m = mesh.quad_mesh(*shape, length=L, jitter=0.1, seed=seed, permute=True)
    mats = [Material(q1=1.0, q1ex=1.33, q2=1.0, q2ex=1.33, gamma=1.4, csmin=1e-14)]
    hot = Fill("box", 0, den=2.0, sie=1.0, velocity="cartesian")
    hot.x1, hot.x2 = 0.0, 0.6 * L[0]
    hot.y1, hot.y2 = 0.0, 0.6 * L[1]
    hot.z1, hot.z2 = (0.0, 0.6 * L[2]) if dims == 3 else (-1.0, 1.0)
    hot.u, hot.v, hot.w = 0.1, -0.05, 0.2 if dims == 3 else 0.0
    if dims == 3:
        bcs = [Boundary("x_plane", 0.0, "reflected"), Boundary("z_plane", L[2], "fixed")]
    else:
        bcs = [Boundary("y_plane", 0.0, "reflected"), Boundary("x_plane", L[0], "fixed")]
    return Problem("thin" + "x".join(str(n) for n in shape), m, mats, [Fill("global", 0, den=1.0, sie=1e-3), hot],
                   bcs, Params(cycle_stop=cycles))
