"""Hex and quad meshes for the SGH solver: structured box generation (optionally
jittered and randomly renumbered from a seed), an EnSight Gold ``.geo`` reader,
and the binary mesh format read by the reference oracle harness.

Meshes follow the reference's conventions (Explicit-Lagrange-Kokkos/SGH_solver):
``coords`` is ``[num_nodes][3]`` float64 and ``nodes_in_elem`` is ``[num_elems][8]``
0-based with the hex node ordering of mesh.h:15-45 (nodes 0-3 counter-clockwise on
the k face, 4-7 above them).  Box meshes number nodes with i fastest, then j, then
k, exactly like the shipped ``mesh_12x12x12.geo`` / ``mesh_Box_32.geo``.  2D-RZ
meshes have ``coords`` ``[num_nodes][2]`` (x = axial, y = radial) and quads
``[num_elems][4]`` counter-clockwise (0 at (i, j), 1 at (i+1, j), 2 at
(i+1, j+1), 3 at (i, j+1); sgh_solve.cpp:513-519).
"""
from __future__ import annotations

import struct
from dataclasses import dataclass

import numpy as np

_MASK64 = np.uint64(0xFFFFFFFFFFFFFFFF)


def splitmix64(x: np.ndarray) -> np.ndarray:
    """Vectorised splitmix64 finaliser (Steele/Lea/Flood), uint64 -> uint64.
    Used instead of numpy's generators so the stream is identical on every
    machine and numpy version."""
    z = (x.astype(np.uint64) + np.uint64(0x9E3779B97F4A7C15)) & _MASK64
    z = ((z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)) & _MASK64
    z = ((z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)) & _MASK64
    return z ^ (z >> np.uint64(31))


def uniform01(seed: int, stream: int, n: int) -> np.ndarray:
    """n doubles in [0, 1) from counter-based splitmix64(seed, stream, i)."""
    base = splitmix64(np.array([seed * 0x100000001B3 + stream], dtype=np.uint64))[0]
    with np.errstate(over="ignore"):
        ctr = np.arange(n, dtype=np.uint64) + base
    bits = splitmix64(ctr) >> np.uint64(11)
    return bits.astype(np.float64) * (1.0 / 9007199254740992.0)


@dataclass
class HexMesh:
    coords: np.ndarray         # [Nn][3] float64
    nodes_in_elem: np.ndarray  # [Ne][8] int64
    name: str = ""

    @property
    def num_nodes(self) -> int:
        return int(self.coords.shape[0])

    @property
    def num_elems(self) -> int:
        return int(self.nodes_in_elem.shape[0])

    @property
    def dims(self) -> int:
        """3 for hex meshes, 2 for 2D-RZ quad meshes."""
        return int(self.coords.shape[1])


def box_mesh(nx: int, ny: int | None = None, nz: int | None = None, length=(1.0, 1.0, 1.0),
             jitter: float = 0.0, seed: int = 0, permute: bool = False,
             geo_digits: int | None = None, name: str = "") -> HexMesh:
    """Uniform nx*ny*nz hex mesh of the box [0,Lx]x[0,Ly]x[0,Lz].

    jitter: interior nodes move by U(-jitter*h, +jitter*h) per axis (h = cell size
        along that axis); nodes on the box faces keep their coordinate on the
        face-normal axes so boundary-plane tagging (tolerance 1e-7) still holds.
    permute: renumber elements and nodes by seeded random permutations.
    geo_digits: round coordinates through '%.{d}e' text, reproducing the values a
        .geo file printed with that many digits holds (5 for the shipped meshes).
    """
    ny = nx if ny is None else ny
    nz = nx if nz is None else nz
    if np.isscalar(length):
        length = (float(length),) * 3
    Lx, Ly, Lz = (float(v) for v in length)
    hx, hy, hz = Lx / nx, Ly / ny, Lz / nz
    i = np.arange(nx + 1, dtype=np.float64)
    j = np.arange(ny + 1, dtype=np.float64)
    k = np.arange(nz + 1, dtype=np.float64)
    xs, ys, zs = i * hx, j * hy, k * hz
    if geo_digits is not None:
        fmt = "%.{}e".format(geo_digits)
        xs = np.array([float(fmt % v) for v in xs])
        ys = np.array([float(fmt % v) for v in ys])
        zs = np.array([float(fmt % v) for v in zs])
    Z, Y, X = np.meshgrid(zs, ys, xs, indexing="ij")
    coords = np.stack([X.ravel(), Y.ravel(), Z.ravel()], axis=1)
    nn = coords.shape[0]
    if jitter:
        K, J, I = np.meshgrid(np.arange(nz + 1), np.arange(ny + 1), np.arange(nx + 1), indexing="ij")
        I, J, K = I.ravel(), J.ravel(), K.ravel()
        for ax, (idx, nmax, h) in enumerate(((I, nx, hx), (J, ny, hy), (K, nz, hz))):
            interior = (I > 0) & (I < nx) & (J > 0) & (J < ny) & (K > 0) & (K < nz)
            r = uniform01(seed, 1 + ax, nn)
            delta = (2.0 * r - 1.0) * jitter * h
            coords[:, ax] = np.where(interior, coords[:, ax] + delta, coords[:, ax])
    # element connectivity, i fastest (EnSight box ordering)
    ek, ej, ei = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    ei, ej, ek = ei.ravel(), ej.ravel(), ek.ravel()

    def nid(a, b, c):
        return a + (nx + 1) * (b + (ny + 1) * c)

    nie = np.stack([
        nid(ei, ej, ek), nid(ei + 1, ej, ek), nid(ei + 1, ej + 1, ek), nid(ei, ej + 1, ek),
        nid(ei, ej, ek + 1), nid(ei + 1, ej, ek + 1), nid(ei + 1, ej + 1, ek + 1), nid(ei, ej + 1, ek + 1),
    ], axis=1).astype(np.int64)
    if permute:
        ne = nie.shape[0]
        eperm = np.argsort(splitmix64(np.arange(ne, dtype=np.uint64) + np.uint64(seed * 7919 + 11)), kind="stable")
        nperm = np.argsort(splitmix64(np.arange(nn, dtype=np.uint64) + np.uint64(seed * 104729 + 13)), kind="stable")
        # new node id of old node o is inv[o]
        inv = np.empty(nn, dtype=np.int64)
        inv[nperm] = np.arange(nn, dtype=np.int64)
        coords = coords[nperm]
        nie = inv[nie[eperm]]
    return HexMesh(np.ascontiguousarray(coords), np.ascontiguousarray(nie), name=name)


def quad_mesh(nx: int, ny: int | None = None, length=(1.0, 1.0), jitter: float = 0.0, seed: int = 0,
              permute: bool = False, origin=(0.0, 0.0), name: str = "") -> HexMesh:
    """Uniform nx*ny quad mesh of [x0, x0+Lx] x [y0, y0+Ly] for the 2D-RZ path
    (x axial, y radial).  jitter and permute as in box_mesh: interior nodes move
    by U(-jitter*h, +jitter*h) per axis, boundary nodes keep their coordinate on
    the edge-normal axis."""
    ny = nx if ny is None else ny
    if np.isscalar(length):
        length = (float(length),) * 2
    Lx, Ly = (float(v) for v in length)
    hx, hy = Lx / nx, Ly / ny
    xs = origin[0] + np.arange(nx + 1, dtype=np.float64) * hx
    ys = origin[1] + np.arange(ny + 1, dtype=np.float64) * hy
    Y, X = np.meshgrid(ys, xs, indexing="ij")
    coords = np.stack([X.ravel(), Y.ravel()], axis=1)
    nn = coords.shape[0]
    if jitter:
        J, I = np.meshgrid(np.arange(ny + 1), np.arange(nx + 1), indexing="ij")
        I, J = I.ravel(), J.ravel()
        interior = (I > 0) & (I < nx) & (J > 0) & (J < ny)
        for ax, h in enumerate((hx, hy)):
            r = uniform01(seed, 1 + ax, nn)
            coords[:, ax] = np.where(interior, coords[:, ax] + (2.0 * r - 1.0) * jitter * h, coords[:, ax])
    ej, ei = np.meshgrid(np.arange(ny), np.arange(nx), indexing="ij")
    ei, ej = ei.ravel(), ej.ravel()

    def nid(a, b):
        return a + (nx + 1) * b

    nie = np.stack([nid(ei, ej), nid(ei + 1, ej), nid(ei + 1, ej + 1), nid(ei, ej + 1)], axis=1).astype(np.int64)
    if permute:
        ne = nie.shape[0]
        eperm = np.argsort(splitmix64(np.arange(ne, dtype=np.uint64) + np.uint64(seed * 7919 + 11)), kind="stable")
        nperm = np.argsort(splitmix64(np.arange(nn, dtype=np.uint64) + np.uint64(seed * 104729 + 13)), kind="stable")
        inv = np.empty(nn, dtype=np.int64)
        inv[nperm] = np.arange(nn, dtype=np.int64)
        coords = coords[nperm]
        nie = inv[nie[eperm]]
    return HexMesh(np.ascontiguousarray(coords), np.ascontiguousarray(nie), name=name)


def quad_rz_volumes(coords: np.ndarray, nodes_in_elem: np.ndarray) -> np.ndarray:
    """Volume per radian of quads revolved about the x axis (Pappus: area times
    centroid radius), for problem set-up values only."""
    x = coords[nodes_in_elem][:, :, 0]
    y = coords[nodes_in_elem][:, :, 1]
    a = 0.5 * (x * np.roll(y, -1, axis=1) - np.roll(x, -1, axis=1) * y).sum(axis=1)
    cy = ((y + np.roll(y, -1, axis=1)) * (x * np.roll(y, -1, axis=1) - np.roll(x, -1, axis=1) * y)).sum(axis=1)
    return cy / 6.0


def read_geo(path: str) -> HexMesh:
    """EnSight Gold .geo reader for single-part hexa8 meshes, with the reference's
    conventions (read_mesh.cpp:12-147: 8 header lines, node count, x[], y[], z[],
    a 'hexa8' line, element count, 1-based connectivity)."""
    with open(path, "r") as f:
        lines = f.read().split("\n")
    pos = 8
    nn = int(lines[pos].split()[0])
    pos += 1
    vals = np.array([float(lines[pos + t].split()[0]) for t in range(3 * nn)])
    pos += 3 * nn
    while "hexa8" not in lines[pos]:
        pos += 1
    pos += 1
    ne = int(lines[pos].split()[0])
    pos += 1
    conn = np.array([[int(v) for v in lines[pos + e].split()] for e in range(ne)], dtype=np.int64) - 1
    coords = np.stack([vals[:nn], vals[nn:2 * nn], vals[2 * nn:]], axis=1)
    return HexMesh(coords, conn, name=path)


def write_mesh_bin(path: str, mesh: HexMesh) -> None:
    """Binary mesh read by the reference oracle's mesh reader:
    'FSGHMESH', u64 Nn, u64 Ne, f64 x[Nn], y[Nn] (and z[Nn] for hexes),
    u64 nodes_in_elem[Ne][8 or 4]."""
    with open(path, "wb") as f:
        f.write(b"FSGHMESH")
        f.write(struct.pack("<QQ", mesh.num_nodes, mesh.num_elems))
        for d in range(mesh.dims):
            f.write(np.ascontiguousarray(mesh.coords[:, d], dtype="<f8").tobytes())
        f.write(np.ascontiguousarray(mesh.nodes_in_elem, dtype="<u8").tobytes())


def hex_volumes(coords: np.ndarray, nodes_in_elem: np.ndarray) -> np.ndarray:
    """Exact trilinear hex volume by the divergence theorem, V = (1/3) sum over
    the six bilinear faces of centroid . vector-area (exact for bilinear faces).
    Used for problem set-up values only; the solver computes volumes itself."""
    x = coords[nodes_in_elem]  # [Ne][8][3]
    faces = [(0, 4, 7, 3), (1, 2, 6, 5), (0, 1, 5, 4), (2, 3, 7, 6), (0, 3, 2, 1), (4, 5, 6, 7)]
    vol = np.zeros(x.shape[0])
    for a, b, c, d in faces:
        pa, pb, pc, pd = x[:, a], x[:, b], x[:, c], x[:, d]
        area2 = np.cross(pc - pa, pd - pb)  # 2 * vector area (bilinear face)
        cen = 0.25 * (pa + pb + pc + pd)
        vol += np.einsum("ij,ij->i", cen, area2)
    return vol / 6.0
