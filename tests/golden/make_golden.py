"""Generates the golden fixtures in this directory from the reference itself.

The reference's own SGH solver (Explicit-Lagrange-Kokkos/SGH_solver, compiled
unmodified by oracle/build_ref.py with its own EnSight reader, uncontracted
floating point) is run on the meshes the reference ships
(Explicit-Lagrange/meshes/mesh_12x12x12.geo and mesh_Box_32.geo) with the Sedov
and Noh decks of fierro_gb300.problems, and its states after one cycle and after
the full run are stored as float64 .npz files.  Also stored: checksums of the
shipped meshes, so the box generator can be checked without the reference tree.

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
    with open(os.path.join(HERE, "golden.json"), "w") as f:
        json.dump(meta, f, indent=1, sort_keys=True)


if __name__ == "__main__":
    main()
