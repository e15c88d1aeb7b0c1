"""Build recipe for the oracle side (test infrastructure only).

Products, all written only under oracle/_ref/ (git-ignored):

* liborc_sgh.so, liborc_sgh_crpow.so -- the plain-C restatement in oracle/sgh_oracle.c
  and its 2D-RZ counterpart oracle/sgh_oracle_rz.c (libm pow, and a correctly
  rounded pow variant of the 3D Mach detector), compiled with
  -ffp-contract=off so its doubles follow the reference's uncontracted evaluation.
* fierro_ref / fierro_ref_geo / fierro_ref_fast / fierro_ref_out -- the reference's own SGH solver
  (Explicit-Lagrange-Kokkos/SGH_solver/*.cpp, unmodified) compiled with g++ -fopenmp
  against the project-written MATAR/Kokkos stand-in oracle/compat/matar.h, with
  input.cpp, the mesh reader and the driver replaced by the files in oracle/ref/,
  and a test strength model (oracle/ref/ref_user_mat.cpp) that decks can assign to a
  material through the reference's strength_model pointer.
  fierro_ref_geo links the reference's own EnSight reader (read_mesh.cpp);
  fierro_ref reads binary meshes; fierro_ref_fast is fierro_ref with the compiler's
  default floating-point contraction (used for timing only); fierro_ref_out links
  the reference's outputs.cpp and writes its EnSight / state files (the checker
  of the library's graphics dumps).

The reference sources are compiled where they lie when the reference tree is
present.  They are also staged into oracle/_ref/src/ (git-ignored) so that a
machine without the reference tree, but with a copy of this working directory,
can rebuild the same executables for its own CPU architecture.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
STAGE = os.path.join(OUT, "src")
# The reference checkout: FIERRO_REFERENCE_ROOT, else the read-only mount of
# this build machine.
REF_ROOT = os.environ.get("FIERRO_REFERENCE_ROOT", "/root/reference")
REF_SGH = os.path.join(REF_ROOT, "Explicit-Lagrange-Kokkos", "SGH_solver")

REF_UNITS = [
    "sgh_solve.cpp", "setup.cpp", "geometry.cpp", "momentum.cpp", "force_sgh.cpp",
    "energy_sgh.cpp", "properties.cpp", "eos.cpp", "boundary.cpp", "time_integration.cpp",
    "user_mat.cpp", "user_mat_init.cpp",
]
REF_HEADERS = ["mesh.h", "state.h"]
REF_GEO_READER = "read_mesh.cpp"
REF_OUTPUTS = "outputs.cpp"


def _run(cmd):
    p = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if p.returncode != 0:
        raise RuntimeError("command failed: %s\n%s" % (" ".join(cmd), p.stdout))
    return p.stdout


def _newer(target, deps):
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(d) <= t for d in deps if os.path.exists(d))


def build_oracle_lib(verbose=False):
    """Compile oracle/sgh_oracle.c into oracle/_ref/liborc_sgh.so (libm pow, as the
    reference) and oracle/_ref/liborc_sgh_crpow.so (correctly rounded pow)."""
    os.makedirs(OUT, exist_ok=True)
    src = os.path.join(HERE, "sgh_oracle.c")
    src_rz = os.path.join(HERE, "sgh_oracle_rz.c")
    hdr = os.path.join(HERE, "sgh_oracle.h")
    libs = {"liborc_sgh.so": [], "liborc_sgh_crpow.so": ["-DORC_CR_POW"]}
    for name, extra in libs.items():
        lib = os.path.join(OUT, name)
        if not _newer(lib, [src, src_rz, hdr, __file__]):
            _run(["gcc", "-O2", "-std=c11", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off"] + extra +
                 ["-o", lib, src, src_rz, "-lm"])
    return os.path.join(OUT, "liborc_sgh.so")


def _source_dir():
    if os.path.isdir(REF_SGH):
        os.makedirs(STAGE, exist_ok=True)
        for f in REF_UNITS + REF_HEADERS + [REF_GEO_READER, REF_OUTPUTS]:
            dst = os.path.join(STAGE, f)
            srcf = os.path.join(REF_SGH, f)
            if not os.path.exists(dst) or os.path.getmtime(dst) < os.path.getmtime(srcf):
                shutil.copy2(srcf, dst)
                os.chmod(dst, 0o644)
        return REF_SGH
    if os.path.isdir(STAGE) and all(os.path.exists(os.path.join(STAGE, f)) for f in REF_UNITS):
        return STAGE
    return None


def build_reference(verbose=False, jobs=None):
    """Compile the reference SGH solver executables.  Returns a dict of paths, or
    None when neither the reference tree nor a staged copy is available."""
    src_dir = _source_dir()
    if src_dir is None:
        return None
    os.makedirs(os.path.join(OUT, "obj"), exist_ok=True)
    compat = os.path.join(HERE, "compat")
    ref_dir = os.path.join(HERE, "ref")
    base = ["g++", "-std=c++17", "-O3", "-fopenmp", "-w", "-I", compat, "-I", src_dir]
    variants = {"exact": ["-ffp-contract=off"], "fast": []}
    units = [(os.path.join(src_dir, u), u) for u in REF_UNITS + [REF_GEO_READER]]
    units += [(os.path.join(ref_dir, u), u) for u in
              ["ref_input.cpp", "ref_harness.cpp", "ref_read_mesh_bin.cpp", "ref_user_mat.cpp"]]
    headers = [os.path.join(src_dir, h) for h in REF_HEADERS] + [os.path.join(compat, "matar.h")]

    jobs_list = []
    for var, flags in variants.items():
        for path, name in units:
            obj = os.path.join(OUT, "obj", "%s.%s.o" % (name, var))
            if not _newer(obj, [path] + headers + [__file__]):
                jobs_list.append(base + flags + ["-c", path, "-o", obj])
    # the graphics-dump variant: the reference's own outputs.cpp, harness without its no-op
    # (outputs.cpp gets <string> through the Kokkos headers in its own build)
    out_units = [(os.path.join(src_dir, REF_OUTPUTS), REF_OUTPUTS, ["-include", "string"]),
                 (os.path.join(ref_dir, "ref_harness.cpp"), "ref_harness_out.cpp", ["-DFIERRO_REF_REAL_OUTPUTS"])]
    for path, name, extra in out_units:
        obj = os.path.join(OUT, "obj", "%s.exact.o" % name)
        if os.path.exists(path) and not _newer(obj, [path] + headers + [__file__]):
            jobs_list.append(base + variants["exact"] + extra + ["-c", path, "-o", obj])
    with ThreadPoolExecutor(max_workers=jobs or os.cpu_count() or 4) as ex:
        list(ex.map(_run, jobs_list))

    def objs(var, reader):
        names = REF_UNITS + [reader, "ref_input.cpp", "ref_harness.cpp", "ref_user_mat.cpp"]
        return [os.path.join(OUT, "obj", "%s.%s.o" % (n, var)) for n in names]

    out_objs = [o for o in objs("exact", "ref_read_mesh_bin.cpp") if not o.endswith("ref_harness.cpp.exact.o")]
    out_objs += [os.path.join(OUT, "obj", "%s.exact.o" % n) for n in (REF_OUTPUTS, "ref_harness_out.cpp")]
    out = {
        "fierro_ref_out": (out_objs, "exact"),
        "fierro_ref": (objs("exact", "ref_read_mesh_bin.cpp"), "exact"),
        "fierro_ref_geo": (objs("exact", REF_GEO_READER), "exact"),
        "fierro_ref_fast": (objs("fast", "ref_read_mesh_bin.cpp"), "fast"),
    }
    paths = {}
    for exe, (ob, _) in out.items():
        target = os.path.join(OUT, exe)
        if not _newer(target, ob):
            _run(["g++", "-fopenmp", "-o", target] + ob + ["-lm"])
        paths[exe] = target
    return paths


def build_reference_lib(verbose=False):
    """fierro_ref_lib: the reference's driver sequence (ref_harness.cpp) with its
    sgh_solve call replaced by the reference-side binding of the GB300 library
    (oracle/ref/fierro_sgh_call.inc, the snippet of the integration notes),
    linked against fierro_gb300/libfierro_sgh.so.  Needs the reference objects
    (build_reference) and the library.  Returns the executable's path, or None
    when the reference sources are unavailable."""
    paths = build_reference()
    if paths is None:
        return None
    root = os.path.dirname(HERE)
    libdir = os.path.join(root, "fierro_gb300")
    lib = os.path.join(libdir, "libfierro_sgh.so")
    if not os.path.exists(lib):
        raise FileNotFoundError(lib)
    src_dir = _source_dir()
    compat = os.path.join(HERE, "compat")
    ref_dir = os.path.join(HERE, "ref")
    harness = os.path.join(ref_dir, "ref_harness.cpp")
    snippet = os.path.join(ref_dir, "fierro_sgh_call.inc")
    header = os.path.join(root, "include", "fierro_sgh.h")
    obj = os.path.join(OUT, "obj", "ref_harness_lib.cpp.exact.o")
    deps = [harness, snippet, header, os.path.join(compat, "matar.h"), __file__] + \
        [os.path.join(src_dir, h) for h in REF_HEADERS]
    if not _newer(obj, deps):
        _run(["g++", "-std=c++17", "-O3", "-fopenmp", "-w", "-ffp-contract=off", "-DFIERRO_REF_CALL_LIBRARY",
              "-I", compat, "-I", src_dir, "-I", ref_dir, "-I", os.path.join(root, "include"),
              "-c", harness, "-o", obj])
    names = REF_UNITS + ["ref_read_mesh_bin.cpp", "ref_input.cpp", "ref_user_mat.cpp"]
    objs = [os.path.join(OUT, "obj", "%s.exact.o" % n) for n in names] + [obj]
    target = os.path.join(OUT, "fierro_ref_lib")
    if not _newer(target, objs + [lib]):
        _run(["g++", "-fopenmp", "-o", target] + objs +
             ["-L", libdir, "-lfierro_sgh", "-Wl,-rpath," + libdir, "-lm"])
    return target


def main():
    lib = build_oracle_lib()
    print("oracle lib:", lib)
    paths = build_reference()
    print("reference:", paths if paths else "unavailable (no reference sources)")


if __name__ == "__main__":
    sys.exit(main())
