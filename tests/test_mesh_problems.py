"""Mesh generation and problem decks (CPU)."""
import numpy as np

from fierro_gb300 import mesh, problems


def test_jitter_moves_only_interior_nodes_within_bound():
    n, L = 9, 1.2
    m0 = mesh.box_mesh(n, length=L)
    m1 = mesh.box_mesh(n, length=L, jitter=0.1, seed=5)
    h = L / n
    d = m1.coords - m0.coords
    assert np.all(np.abs(d) <= 0.1 * h + 1e-15)
    on_face = np.any((np.abs(m0.coords) < 1e-12) | (np.abs(m0.coords - L) < 1e-12), axis=1)
    assert np.all(d[on_face] == 0.0)
    assert np.count_nonzero(d[~on_face]) > 0.9 * d[~on_face].size
    assert np.array_equal(m1.coords, mesh.box_mesh(n, length=L, jitter=0.1, seed=5).coords)
    assert not np.array_equal(m1.coords, mesh.box_mesh(n, length=L, jitter=0.1, seed=6).coords)


def test_permutation_is_a_relabelling():
    a = mesh.box_mesh(6, length=1.0, jitter=0.1, seed=2)
    b = mesh.box_mesh(6, length=1.0, jitter=0.1, seed=2, permute=True)
    assert sorted(map(tuple, a.coords.tolist())) == sorted(map(tuple, b.coords.tolist()))
    va = np.sort(mesh.hex_volumes(a.coords, a.nodes_in_elem))
    vb = np.sort(mesh.hex_volumes(b.coords, b.nodes_in_elem))
    assert np.allclose(va, vb, rtol=1e-14, atol=0)
    assert np.all(vb > 0)
    assert len(np.unique(b.nodes_in_elem)) == b.num_nodes


def test_splitmix_stream_is_fixed():
    # a change of the generator would silently change every seeded mesh
    u = mesh.uniform01(2024, 1, 4)
    assert np.all((u >= 0) & (u < 1))
    assert np.array_equal(u, mesh.uniform01(2024, 1, 4))
    assert mesh.splitmix64(np.array([0], dtype=np.uint64))[0] == np.uint64(0xE220A8397B1DCDAF)


def test_sedov_deck_origin_energy():
    p = problems.sedov(8, jitter=0.1, seed=1, permute=True)
    e0 = p.info["origin_elem"]
    v0 = mesh.hex_volumes(p.mesh.coords, p.mesh.nodes_in_elem[e0:e0 + 1])[0]
    assert abs(p.info["origin_sie"] * v0 - 0.2467) < 1e-15
    txt = p.config_text()
    assert "fill 1.0 0.0 0.0" in txt and txt.count("\nbc ") == 3


def test_hex_volume_of_box():
    m = mesh.box_mesh(3, length=(1.0, 2.0, 3.0))
    assert np.allclose(mesh.hex_volumes(m.coords, m.nodes_in_elem), 2.0 / 9.0 * 3.0 / 3.0, rtol=1e-14)
