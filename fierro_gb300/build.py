"""Builds libfierro_sgh.so in-tree (fierro_gb300/libfierro_sgh.so) for sm_103a.

Translation units:
  csrc/sgh_kernels.cu  twice: exact arithmetic (-DFIERRO_FMA=0 --fmad=false) and
                       fused multiply-add (-DFIERRO_FMA=1 --fmad=true)
  csrc/sgh_rz_kernels.cu the 2D-RZ quad kernels, twice in the same two modes
  csrc/sgh_rz.cpp      2D-RZ topology, set-up, transfers and stage launches (g++)
  csrc/sgh_host.cpp    mesh topology, Morton renumbering, set-up (g++, OpenMP,
                       -ffp-contract=off so set-up doubles are uncontracted)
  csrc/sgh_capi.cpp    the C ABI (g++)
  csrc/sgh_batch.cpp   the batched-ensemble C ABI (g++)
  csrc/sgh_xfer.cu     host<->device state transfer kernels (GPU reads/writes host arrays)
  csrc/sgh_topo.cu     mesh topology on the GPU (renumbering, CSRs, boundary masks; --fmad=false)
  csrc/sgh_setup.cu    the initial state on the GPU for fierro_sgh_setup (--fmad=false)
  csrc/sgh_adjoint.cu  discrete-adjoint kernels (--fmad=false, like the exact mode)
  csrc/sgh_adjoint.cpp the adjoint's checkpointing, replay and reverse schedule (g++)
  csrc/sgh_output.cpp  graphics dumps: snapshot ring, writer thread, reference file formats (g++)
  csrc/sgh_calib.cu    FP64 throughput calibration for the roofline
  csrc/sgh_noalloc.cu  energy tallies with static scratch (no allocation)
  csrc/sgh_validate.cu device-topology invariant checks (fierro_sgh_validate)
All compile in parallel; a unit is rebuilt only when it or a header changed.
"""
from __future__ import annotations

import glob
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(ROOT, "include")
OBJ = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libfierro_sgh.so")
CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA_HOME, "bin", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _run(cmd):
    p = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if p.returncode != 0:
        raise RuntimeError("build step failed:\n%s\n%s" % (" ".join(cmd), p.stdout))
    return p.stdout


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, force: bool = False, ptxas_info: bool = False) -> str:
    os.makedirs(OBJ, exist_ok=True)
    headers = glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh")) + \
        [os.path.join(INCLUDE, "fierro_sgh.h"), os.path.abspath(__file__)]
    inc = ["-I", INCLUDE, "-I", CSRC]
    nvcc_common = [NVCC] + ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC"] + inc
    if ptxas_info:
        nvcc_common += ["-Xptxas", "-v"]
    kern = os.path.join(CSRC, "sgh_kernels.cu")
    rzk = os.path.join(CSRC, "sgh_rz_kernels.cu")
    # FIERRO_KERNEL_NVCC_FLAGS: extra nvcc flags for the cycle kernels (e.g. the
    # launch-bounds hooks -DFIERRO_ELEM_MIN_BLOCKS=3, or -DFIERRO_LIBRARY_ROOTS);
    # a change of them rebuilds those objects
    kflags = os.environ.get("FIERRO_KERNEL_NVCC_FLAGS", "").split()
    stamp = os.path.join(OBJ, "kernel_flags.txt")
    old_flags = open(stamp).read() if os.path.exists(stamp) else ""
    if old_flags != " ".join(kflags):
        for o in ("sgh_kernels_exact.o", "sgh_kernels_fma.o"):
            if os.path.exists(os.path.join(OBJ, o)):
                os.remove(os.path.join(OBJ, o))
        with open(stamp, "w") as f:
            f.write(" ".join(kflags))
    units = [
        (os.path.join(OBJ, "sgh_kernels_exact.o"),
         nvcc_common + kflags + ["-DFIERRO_FMA=0", "--fmad=false", "-c", kern], [kern]),
        (os.path.join(OBJ, "sgh_kernels_fma.o"),
         nvcc_common + kflags + ["-DFIERRO_FMA=1", "--fmad=true", "-c", kern], [kern]),
        (os.path.join(OBJ, "sgh_rz_kernels_exact.o"),
         nvcc_common + ["-DFIERRO_FMA=0", "--fmad=false", "-c", rzk], [rzk]),
        (os.path.join(OBJ, "sgh_rz_kernels_fma.o"),
         nvcc_common + ["-DFIERRO_FMA=1", "--fmad=true", "-c", rzk], [rzk]),
    ]
    calib = os.path.join(CSRC, "sgh_calib.cu")
    units.append((os.path.join(OBJ, "sgh_calib.o"), nvcc_common + ["-c", calib], [calib]))
    topo = os.path.join(CSRC, "sgh_topo.cu")
    units.append((os.path.join(OBJ, "sgh_topo.o"), nvcc_common + ["--fmad=false", "-c", topo], [topo]))
    setupk = os.path.join(CSRC, "sgh_setup.cu")
    units.append((os.path.join(OBJ, "sgh_setup.o"),
                  nvcc_common + ["--fmad=false", "-Xcompiler", "-fopenmp", "-c", setupk], [setupk]))
    xfer = os.path.join(CSRC, "sgh_xfer.cu")
    units.append((os.path.join(OBJ, "sgh_xfer.o"), nvcc_common + ["--fmad=false", "-c", xfer], [xfer]))
    adjk = os.path.join(CSRC, "sgh_adjoint.cu")
    units.append((os.path.join(OBJ, "sgh_adjoint_k.o"), nvcc_common + ["--fmad=false", "-c", adjk], [adjk]))
    val = os.path.join(CSRC, "sgh_validate.cu")
    units.append((os.path.join(OBJ, "sgh_validate.o"), nvcc_common + ["-c", val], [val]))
    noalloc = os.path.join(CSRC, "sgh_noalloc.cu")
    units.append((os.path.join(OBJ, "sgh_noalloc.o"), nvcc_common + ["-c", noalloc], [noalloc]))
    gxx = ["g++", "-O2", "-std=c++17", "-fPIC", "-fopenmp", "-ffp-contract=off", "-Wall", "-Wno-unknown-pragmas",
           "-I", os.path.join(CUDA_HOME, "include")] + inc
    for name in ("sgh_host.cpp", "sgh_capi.cpp", "sgh_batch.cpp", "sgh_adjoint.cpp", "sgh_output.cpp", "sgh_rz.cpp"):
        src = os.path.join(CSRC, name)
        units.append((os.path.join(OBJ, name.replace(".cpp", ".o")), gxx + ["-c", src], [src]))
    jobs = []
    for obj, cmd, srcs in units:
        if force or ptxas_info or _stale(obj, srcs + headers):
            jobs.append(cmd + ["-o", obj])
    outputs = []
    if jobs:
        with ThreadPoolExecutor(max_workers=len(jobs)) as ex:
            outputs = list(ex.map(_run, jobs))
    objs = [u[0] for u in units]
    if force or _stale(LIB, objs):
        _run([NVCC] + ARCH + ["-shared", "-o", LIB] + objs + ["-Xcompiler", "-fopenmp", "-lgomp"])
    if verbose or ptxas_info:
        for o in outputs:
            if o.strip():
                print(o)
    return LIB


if __name__ == "__main__":
    build(verbose=True, force="--force" in sys.argv, ptxas_info="--ptxas" in sys.argv)
    print(LIB)
