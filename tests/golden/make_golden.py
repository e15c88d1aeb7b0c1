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

Run from the repository root (needs the reference tree):
    python tests/golden/make_golden.py
"""
import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

MESHES = "/root/reference/Explicit-Lagrange/meshes"
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
    }


def main():
    from fierro_gb300 import mesh, problems
    from oracle import build_ref, orc
    build_ref.build_reference()
    cases = [
        ("sedov12", "mesh_12x12x12.geo", problems.sedov(12, geo_digits=5), [1, 200]),
        ("noh32", "mesh_Box_32.geo", problems.noh(32, geo_digits=5), [1, 500]),
    ]
    meta = {}
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
    meta["rz"] = {}
    for name, prob in rz_cases().items():
        st = orc.run_reference(prob, threads=1)
        out = {k: st[k] for k in FIELDS + STRENGTH_FIELDS + ("node_mass", "mass")}
        out["time"] = np.array(st["time"])
        fn = os.path.join(HERE, "rz_%s.npz" % name)
        np.savez_compressed(fn, **out)
        meta["rz"][name] = {"file": os.path.basename(fn), "time": float(st["time"]),
                            "cycles": prob.params.cycle_stop, "deck": prob.config_text()}
        print(fn, os.path.getsize(fn))
    with open(os.path.join(HERE, "golden.json"), "w") as f:
        json.dump(meta, f, indent=1, sort_keys=True)


if __name__ == "__main__":
    main()
