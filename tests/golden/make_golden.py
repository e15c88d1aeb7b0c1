"""Generates the golden fixtures in this directory from the reference itself.

The reference's own SGH solver (Explicit-Lagrange-Kokkos/SGH_solver, compiled
unmodified by oracle/build_ref.py with its own EnSight reader, uncontracted
floating point) is run on the meshes the reference ships
(Explicit-Lagrange/meshes/mesh_12x12x12.geo and mesh_Box_32.geo) with the Sedov
and Noh decks of fierro_gb300.problems, and its states after one cycle and after
the full run are stored as float64 .npz files.  Also stored: checksums of the
shipped meshes, so the box generator can be checked without the reference tree.

2D-RZ cases (rz_*.npz) run the reference with num_dims = 2 on quad meshes from
the generator, the decks of the reference's own RZ tests
(tests-for-Explicit-Lagrange-Kokkos/input_for_{Sedov,Noh}RZ_test.cpp).

Strength-model cases (strength_*.npz) run the reference with the test strength
model of oracle/ref/ref_user_mat.cpp assigned through material_t::strength_model,
on meshes from the box generator, and also store the stress bins and the
element state variables.

Unstructured-mesh cases (geo_*.npz) run the reference, with its own EnSight
reader, on two more meshes it ships: mesh_z_taylorAnvil.geo (a quarter rod on an
O-grid, nodes of valence 3 and 6) with the deck of its Taylor-anvil test
(tests-for-Explicit-Lagrange-Kokkos/input_for_TaylorAnvil3D_test.cpp), and
mesh_triple_30x18.geo with the triple-point deck of input.cpp, and the skewed
Saltzman mesh (mesh_Saltzman.geo) with the SodZ values in 3D, and the small
O-grid rod mesh-TA-rod.geo with the Taylor-anvil deck.  These fixtures
also carry the mesh (geo_<case>_mesh.npz: coordinates and 0-based connectivity
as read from the .geo), so the tests run without the reference tree.

Run from the repository root (needs the reference tree):
    python tests/golden/make_golden.py [boxes strength rz geo rz:<case> geo:<case>]   (default: all)
"""
import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

# The reference checkout: FIERRO_REFERENCE_ROOT, else the read-only mount of
# the machine the fixtures were made on.
MESHES = os.path.join(os.environ.get("FIERRO_REFERENCE_ROOT", "/root/reference"), "Explicit-Lagrange", "meshes")
FIELDS = ("coords", "vel", "den", "pres", "sie", "sspd", "vol")


def digest(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


STRENGTH_FIELDS = ("stress", "stress0", "statev", "corner_force", "div")


def strength_cases():
    """The strength-model decks (also used by the tests, which import this)."""
    from fierro_gb300 import problems
    return {
        "sedov8_hypo": problems.with_strength(problems.sedov(8, cycles=40), "hypo", 10.0),
        "noh8_hyper": problems.with_strength(problems.noh(8, cycles=60), "hyper", 0.05),
        "sedov10_mixed": problems.sedov_mixed_strength(10, shear_modulus=5.0, cycles=50),
    }


def rz_cases():
    """The 2D-RZ decks (num_dims 2; also used by the tests, which import this)."""
    from fierro_gb300 import problems
    return {
        "sedov_rz16": problems.sedov_rz(16, cycles=200),
        "noh_rz16": problems.noh_rz(16, cycles=200),
        "noh_rz12_jp": problems.noh_rz(12, jitter=0.1, seed=5, permute=True, cycles=80),
        "sedov_rz12_jp_hypo": problems.with_strength(
            problems.sedov_rz(12, jitter=0.1, seed=2, permute=True, cycles=60), "hypo", 10.0),
        # 150 cycles (t = 0.93): the scheme itself (reference and restatement alike)
        # drives a cold element's energy negative near t = 1.1-1.3 on this deck
        "taylor_anvil_rz80x8_p": problems.taylor_anvil_rz(80, 8, seed=8, permute=True, cycles=150),
        "sod_rz100x2_p": problems.sod_rz(100, 2, seed=4, permute=True, cycles=400),
    }


def geo_cases():
    """Decks on shipped unstructured meshes: name -> (.geo file, deck builder, cycle counts)."""
    from fierro_gb300 import problems
    return {
        "taylor_anvil": ("mesh_z_taylorAnvil.geo", problems.taylor_anvil, [1, 300]),
        "triple_point": ("mesh_triple_30x18.geo", problems.triple_point, [1, 400]),
        "sod_saltzman": ("mesh_Saltzman.geo", problems.sod_3d, [1, 400]),
        "taylor_anvil_small_rod": ("mesh-TA-rod.geo", problems.taylor_anvil, [1, 200]),
    }


def geo_problem(name: str, cycles: int):
    """The deck of a geo case on the mesh stored beside the fixtures."""
    from fierro_gb300 import mesh
    m = np.load(os.path.join(HERE, "geo_%s_mesh.npz" % name))
    hm = mesh.HexMesh(np.array(m["coords"]), np.array(m["nodes_in_elem"], dtype=np.int64), name=name)
    return geo_cases()[name][1](hm, cycles=cycles)


def make_geo(meta, names=None):
    from fierro_gb300 import mesh
    from oracle import orc
    meta.setdefault("geo", {})
    for name, (geo, builder, cycles) in geo_cases().items():
        if names and name not in names:
            continue
        path = os.path.join(MESHES, geo)
        g = mesh.read_geo(path)
        fn = os.path.join(HERE, "geo_%s_mesh.npz" % name)
        np.savez_compressed(fn, coords=g.coords, nodes_in_elem=g.nodes_in_elem.astype(np.int32))
        meta["geo"][name] = {"geo": geo, "mesh_file": os.path.basename(fn), "num_nodes": g.num_nodes,
                             "num_elems": g.num_elems, "coords_sha256": digest(g.coords)}
        for c in cycles:
            prob = builder(g, cycles=c)
            st = orc.run_reference(prob, cycles=c, kind="fierro_ref_geo", geo_path=path, threads=1)
            out = {k: st[k] for k in FIELDS}
            out["time"] = np.array(st["time"])
            out["node_mass"] = st["node_mass"]
            out["mass"] = st["mass"]
            fo = os.path.join(HERE, "geo_%s_c%d.npz" % (name, c))
            np.savez_compressed(fo, **out)
            meta["geo"][name]["c%d" % c] = {"file": os.path.basename(fo), "time": float(st["time"]),
                                            "deck": prob.config_text()}
            print(fo, os.path.getsize(fo))


def make_boxes(meta):
    from fierro_gb300 import mesh, problems
    from oracle import orc
    cases = [
        ("sedov12", "mesh_12x12x12.geo", problems.sedov(12, geo_digits=5), [1, 200]),
        ("noh32", "mesh_Box_32.geo", problems.noh(32, geo_digits=5), [1, 500]),
    ]
    for name, geo, prob, cycles in cases:
        path = os.path.join(MESHES, geo)
        g = mesh.read_geo(path)
        meta[name] = {"geo": geo, "coords_sha256": digest(g.coords),
                      "nodes_in_elem_sha256": digest(g.nodes_in_elem.astype(np.int64)),
                      "num_nodes": g.num_nodes, "num_elems": g.num_elems, "deck": prob.config_text()}
        for c in cycles:
            st = orc.run_reference(prob, cycles=c, kind="fierro_ref_geo", geo_path=path, threads=1)
            out = {k: st[k] for k in FIELDS}
            out["time"] = np.array(st["time"])
            out["node_mass"] = st["node_mass"]
            out["mass"] = st["mass"]
            fn = os.path.join(HERE, "%s_c%d.npz" % (name, c))
            np.savez_compressed(fn, **out)
            meta[name]["c%d" % c] = {"file": os.path.basename(fn), "time": float(st["time"])}
            print(fn, os.path.getsize(fn))


def make_strength(meta):
    from oracle import orc
    meta["strength"] = {}
    for name, prob in strength_cases().items():
        st = orc.run_reference(prob, threads=1)
        out = {k: st[k] for k in FIELDS + STRENGTH_FIELDS}
        out["time"] = np.array(st["time"])
        fn = os.path.join(HERE, "strength_%s.npz" % name)
        np.savez_compressed(fn, **out)
        meta["strength"][name] = {"file": os.path.basename(fn), "time": float(st["time"]),
                                  "cycles": prob.params.cycle_stop, "deck": prob.config_text()}
        print(fn, os.path.getsize(fn))


def make_rz(meta, names=None):
    from oracle import orc
    meta.setdefault("rz", {})
    for name, prob in rz_cases().items():
        if names and name not in names:
            continue
        st = orc.run_reference(prob, threads=1)
        out = {k: st[k] for k in FIELDS + STRENGTH_FIELDS + ("node_mass", "mass")}
        out["time"] = np.array(st["time"])
        fn = os.path.join(HERE, "rz_%s.npz" % name)
        np.savez_compressed(fn, **out)
        meta["rz"][name] = {"file": os.path.basename(fn), "time": float(st["time"]),
                            "cycles": prob.params.cycle_stop, "deck": prob.config_text()}
        print(fn, os.path.getsize(fn))


def main(groups=("boxes", "strength", "rz", "geo")):
    from oracle import build_ref
    build_ref.build_reference()
    meta_path = os.path.join(HERE, "golden.json")
    meta = json.load(open(meta_path)) if os.path.exists(meta_path) else {}
    makers = {"boxes": make_boxes, "strength": make_strength, "rz": make_rz, "geo": make_geo}
    for g in groups:
        if g.startswith("rz:"):  # one 2D-RZ case by name
            make_rz(meta, names=[g[3:]])
        elif g.startswith("geo:"):  # one shipped-mesh case by name
            make_geo(meta, names=[g[4:]])
        else:
            makers[g](meta)
    with open(meta_path, "w") as f:
        json.dump(meta, f, indent=1, sort_keys=True)


if __name__ == "__main__":
    main(tuple(sys.argv[1:]) or ("boxes", "strength", "rz", "geo"))
