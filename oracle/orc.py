"""Python access to the CPU oracle (test infrastructure only).

* ``Oracle`` -- ctypes wrapper over oracle/_ref/liborc_sgh.so, the C restatement.
* ``run_reference`` -- runs the reference's own SGH solver built by
  oracle/build_ref.py on a problem deck and returns its final state.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this.
"""
from __future__ import annotations

import ctypes as C
import os
import re
import struct
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(HERE, "_ref")

ORC_NODE_COORDS, ORC_NODE_VEL, ORC_NODE_MASS, ORC_ELEM_DEN, ORC_ELEM_PRES, ORC_ELEM_STRESS, \
    ORC_ELEM_SSPD, ORC_ELEM_SIE, ORC_ELEM_VOL, ORC_ELEM_DIV, ORC_ELEM_MASS, ORC_ELEM_MAT_ID, \
    ORC_ELEM_STATEV, ORC_CORNER_FORCE, ORC_BDY_NODE_MASK = range(15)


class OrcMaterial(C.Structure):
    _fields_ = [("eos_model", C.c_int), ("strength_type", C.c_int), ("q1", C.c_double),
                ("q1ex", C.c_double), ("q2", C.c_double), ("q2ex", C.c_double)]


class OrcBoundary(C.Structure):
    _fields_ = [("surface", C.c_int), ("value", C.c_double), ("hydro_bc", C.c_int)]


class OrcFill(C.Structure):
    _fields_ = [("volume", C.c_int), ("mat_id", C.c_int)] + \
        [(k, C.c_double) for k in ("x1", "x2", "y1", "y2", "z1", "z2", "radius1", "radius2")] + \
        [("velocity", C.c_int)] + [(k, C.c_double) for k in ("u", "v", "w", "speed", "sie", "den")]


class OrcParams(C.Structure):
    _fields_ = [(k, C.c_double) for k in ("time_final", "dt_max", "dt_min", "dt_cfl", "dt_start",
                                          "graphics_dt_ival")] + \
        [(k, C.c_int64) for k in ("graphics_cyc_ival", "cycle_stop", "rk_num_stages")] + \
        [(k, C.c_double) for k in ("fuzz", "tiny", "small")]


_libs = {}
VARIANTS = {"libm": "liborc_sgh.so", "crpow": "liborc_sgh_crpow.so"}


def lib(variant: str = "libm"):
    """The oracle library: 'libm' calls libm pow like the reference; 'crpow' uses
    a correctly rounded pow(vol, 1/3) (see oracle/sgh_oracle.c)."""
    if variant not in _libs:
        path = os.path.join(REF_DIR, VARIANTS[variant])
        if not os.path.exists(path):
            from oracle import build_ref
            build_ref.build_oracle_lib()
        _lib = C.CDLL(path)
        _lib.orc_create.restype = C.c_void_p
        _lib.orc_create.argtypes = [C.c_int64, C.c_int64, C.c_void_p, C.c_void_p]
        _lib.orc_destroy.argtypes = [C.c_void_p]
        _lib.orc_set_materials.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.c_void_p]
        _lib.orc_set_boundaries.argtypes = [C.c_void_p, C.c_int, C.c_void_p]
        _lib.orc_setup.argtypes = [C.c_void_p, C.c_int, C.c_void_p]
        _lib.orc_init_time.argtypes = [C.c_void_p, C.c_void_p]
        _lib.orc_run_cycles.restype = C.c_int64
        _lib.orc_run_cycles.argtypes = [C.c_void_p, C.c_void_p, C.c_int64]
        _lib.orc_run_stages.restype = C.c_int64
        _lib.orc_run_stages.argtypes = [C.c_void_p, C.c_void_p, C.c_int64]
        _lib.orc_energy.argtypes = [C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_double)]
        _lib.orc_time.argtypes = [C.c_void_p] + [C.POINTER(C.c_double)] * 3 + [C.POINTER(C.c_int64)]
        _lib.orc_get.restype = C.c_int64
        _lib.orc_get.argtypes = [C.c_void_p, C.c_int, C.c_void_p]
        _lib.orc_set.restype = C.c_int64
        _lib.orc_set.argtypes = [C.c_void_p, C.c_int, C.c_void_p]
        _lib.orc_bmatrix.argtypes = [C.c_void_p] * 4
        _lib.orc_vol_hex.restype = C.c_double
        _lib.orc_vol_hex.argtypes = [C.c_void_p] * 3
        # the 2D-RZ restatement (oracle/sgh_oracle_rz.c): the same calls with orc_rz_
        for name in ("create", "destroy", "set_materials", "set_boundaries", "setup", "init_time",
                     "run_cycles", "run_stages", "energy", "time", "get", "set"):
            f3, f2 = getattr(_lib, "orc_" + name), getattr(_lib, "orc_rz_" + name)
            f2.restype, f2.argtypes = f3.restype, f3.argtypes
        _lib.orc_rz_bmatrix.argtypes = [C.c_void_p] * 3
        _lib.orc_rz_vol_quad.restype = C.c_double
        _lib.orc_rz_vol_quad.argtypes = [C.c_void_p] * 2
        _lib.orc_rz_area_quad.restype = C.c_double
        _lib.orc_rz_area_quad.argtypes = [C.c_void_p] * 2
        _lib.orc_rz_corner_areas.argtypes = [C.c_void_p] * 3
        _libs[variant] = _lib
    return _libs[variant]


def make_params(p) -> OrcParams:
    return OrcParams(p.time_final, p.dt_max, p.dt_min, p.dt_cfl, p.dt_start, p.graphics_dt_ival,
                     p.graphics_cyc_ival, p.cycle_stop, p.rk_num_stages, p.fuzz, p.tiny, p.small)


class Oracle:
    """One problem instance in the C restatement (3D hex, or 2D-RZ quad meshes
    through the orc_rz_ calls)."""

    def __init__(self, problem, setup=True, variant: str = "libm"):
        from fierro_gb300.problems import REGION, VELOCITY, SURFACE, HYDRO_BC
        self.variant = variant
        m = problem.mesh
        self.dims = m.dims
        self._p = "orc_rz_" if self.dims == 2 else "orc_"
        self.nn, self.ne = m.num_nodes, m.num_elems
        self._nie = np.ascontiguousarray(m.nodes_in_elem, dtype=np.int64)
        self._xyz = np.ascontiguousarray(m.coords, dtype=np.float64)
        self.h = self._f("create")(self.nn, self.ne, self._nie.ctypes.data, self._xyz.ctypes.data)
        if not self.h:
            raise ValueError("oracle rejected the mesh")
        mats = (OrcMaterial * len(problem.materials))(
            *[OrcMaterial(0, q.strength_type, q.q1, q.q1ex, q.q2, q.q2ex) for q in problem.materials])
        sv = np.ascontiguousarray(problem.state_vars())
        if self._f("set_materials")(self.h, len(problem.materials), mats, problem.num_state_vars, sv.ctypes.data):
            raise ValueError("oracle rejected the materials")
        nb = len(problem.boundaries)
        bcs = (OrcBoundary * max(nb, 1))(*[OrcBoundary(SURFACE[b.surface], b.value, HYDRO_BC[b.hydro_bc])
                                           for b in problem.boundaries])
        if self._f("set_boundaries")(self.h, nb, bcs):
            raise ValueError("oracle rejected the boundaries")
        self.params = make_params(problem.params)
        if setup:
            fl = problem.fills
            fills = (OrcFill * max(len(fl), 1))(*[OrcFill(
                REGION[f.volume], f.mat_id, f.x1, f.x2, f.y1, f.y2, f.z1, f.z2, f.radius1, f.radius2,
                VELOCITY[f.velocity], f.u, f.v, f.w, f.speed, f.sie, f.den) for f in fl])
            if self._f("setup")(self.h, len(fl), fills):
                raise ValueError("oracle setup failed")
        self._f("init_time")(self.h, C.byref(self.params))

    def _L(self):
        return lib(self.variant)

    def _f(self, name):
        return getattr(self._L(), self._p + name)

    def __del__(self):
        if getattr(self, "h", None):
            self._f("destroy")(self.h)
            self.h = None

    def run_cycles(self, n: int) -> int:
        return int(self._f("run_cycles")(self.h, C.byref(self.params), n))

    def run_stages(self, n: int) -> int:
        return int(self._f("run_stages")(self.h, C.byref(self.params), n))

    def get(self, which: int) -> np.ndarray:
        n = self._f("get")(self.h, which, None) if which != ORC_BDY_NODE_MASK else self.nn
        dt = np.int32 if which == ORC_BDY_NODE_MASK else (np.int64 if which == ORC_ELEM_MAT_ID else np.float64)
        out = np.empty(n, dtype=dt)
        self._f("get")(self.h, which, out.ctypes.data)
        return out

    def set(self, which: int, arr: np.ndarray) -> None:
        a = np.ascontiguousarray(arr)
        self._f("set")(self.h, which, a.ctypes.data)

    def energy(self):
        ie, ke = C.c_double(), C.c_double()
        self._f("energy")(self.h, C.byref(ie), C.byref(ke))
        return ie.value, ke.value

    def time(self):
        t, dt, gt, cyc = C.c_double(), C.c_double(), C.c_double(), C.c_int64()
        self._f("time")(self.h, C.byref(t), C.byref(dt), C.byref(gt), C.byref(cyc))
        return t.value, dt.value, gt.value, cyc.value

    def state(self) -> dict:
        """The compared fields: bin-1 node coords/vel, elem den/pres/sie/sspd/vol,
        stress, plus both bins, node mass, corner forces and state variables."""
        nn, ne, D = self.nn, self.ne, self.dims
        x = self.get(ORC_NODE_COORDS).reshape(2, nn, D)
        v = self.get(ORC_NODE_VEL).reshape(2, nn, D)
        sie = self.get(ORC_ELEM_SIE).reshape(2, ne)
        stress = self.get(ORC_ELEM_STRESS).reshape(2, ne, 3, 3)
        return {
            "stress": stress[1].copy(), "stress0": stress[0].copy(),
            "statev": self.get(ORC_ELEM_STATEV).reshape(ne, -1),
            "coords": x[1].copy(), "vel": v[1].copy(), "coords0": x[0].copy(), "vel0": v[0].copy(),
            "den": self.get(ORC_ELEM_DEN), "pres": self.get(ORC_ELEM_PRES), "sie": sie[1].copy(),
            "sie0": sie[0].copy(), "sspd": self.get(ORC_ELEM_SSPD), "vol": self.get(ORC_ELEM_VOL),
            "div": self.get(ORC_ELEM_DIV), "mass": self.get(ORC_ELEM_MASS),
            "node_mass": self.get(ORC_NODE_MASS),
            "corner_force": self.get(ORC_CORNER_FORCE).reshape(ne * 2 ** D, D),
            "time": self.time()[0],
        }


def bmatrix(x, y, z):
    B = np.empty((8, 3))
    xs, ys, zs = (np.ascontiguousarray(a, dtype=np.float64) for a in (x, y, z))
    lib().orc_bmatrix(xs.ctypes.data, ys.ctypes.data, zs.ctypes.data, B.ctypes.data)
    return B


def vol_hex(x, y, z):
    xs, ys, zs = (np.ascontiguousarray(a, dtype=np.float64) for a in (x, y, z))
    return lib().orc_vol_hex(xs.ctypes.data, ys.ctypes.data, zs.ctypes.data)


# --------------------------------------------------------------------------- reference
def reference_available(kind: str = "fierro_ref") -> bool:
    return os.path.exists(os.path.join(REF_DIR, kind))


def read_state_dump(path: str, dims: int = 3) -> dict:
    with open(path, "rb") as f:
        buf = f.read()
    assert buf[:8] == b"FSGHSTAT"
    nn, ne = struct.unpack("<QQ", buf[8:24])
    D, npe = dims, 2 ** dims
    a = np.frombuffer(buf, dtype="<f8", offset=24)
    pos = 0

    def take(n):
        nonlocal pos
        out = a[pos:pos + n]
        pos += n
        return out.copy()

    t = take(1)[0]
    x = take(2 * nn * D).reshape(2, nn, D)
    v = take(2 * nn * D).reshape(2, nn, D)
    nm = take(nn)
    den, pres, sspd = take(ne), take(ne), take(ne)
    sie = take(2 * ne).reshape(2, ne)
    vol, div, mass = take(ne), take(ne), take(ne)
    cf = take(npe * ne * D).reshape(npe * ne, D)
    out = {"coords": x[1], "vel": v[1], "coords0": x[0], "vel0": v[0], "den": den, "pres": pres,
           "sie": sie[1], "sie0": sie[0], "sspd": sspd, "vol": vol, "div": div, "mass": mass,
           "node_mass": nm, "corner_force": cf, "time": t}
    if a.size >= pos + 2 * ne * 9 + 1:
        stress = take(2 * ne * 9).reshape(2, ne, 3, 3)
        (nsv,) = struct.unpack("<Q", buf[24 + 8 * pos:32 + 8 * pos])
        pos += 1
        out["stress"], out["stress0"] = stress[1], stress[0]
        out["statev"] = take(ne * nsv).reshape(ne, nsv)
    return out


def run_reference(problem, cycles: int | None = None, kind: str = "fierro_ref", threads: int | None = None,
                  geo_path: str | None = None, workdir: str | None = None, warmup: int = 0,
                  cwd: str | None = None) -> dict:
    """Run the reference executable on the deck; returns the final state plus
    'calc_seconds' (the reference's own cycle-loop timer, sgh_solve.cpp:637-641).
    kind='fierro_ref_out' also writes the reference's graphics dumps into `cwd`."""
    from fierro_gb300.mesh import write_mesh_bin
    import copy
    prob = copy.deepcopy(problem)
    if cycles is not None:
        prob.params.cycle_stop = int(cycles)
    exe = os.path.join(REF_DIR, kind)
    if not os.path.exists(exe):
        raise FileNotFoundError(exe)
    with tempfile.TemporaryDirectory(dir=workdir) as td:
        cfg = os.path.join(td, "deck.txt")
        with open(cfg, "w") as f:
            f.write(prob.config_text())
        if geo_path is not None:
            mesh_path = geo_path
        else:
            mesh_path = os.path.join(td, "mesh.bin")
            write_mesh_bin(mesh_path, prob.mesh)
        out = os.path.join(td, "state.bin")
        env = dict(os.environ)
        if threads:
            env["OMP_NUM_THREADS"] = str(threads)
        if warmup:
            env["FIERRO_REF_WARMUP"] = str(int(warmup))
        env.setdefault("OMP_PROC_BIND", "spread")
        env.setdefault("OMP_PLACES", "cores")
        p = subprocess.run([exe, cfg, mesh_path, out], stdout=subprocess.PIPE, stderr=subprocess.STDOUT,
                           text=True, env=env, cwd=cwd)
        if p.returncode != 0:
            raise RuntimeError("reference run failed:\n" + p.stdout[-4000:])
        st = read_state_dump(out, prob.mesh.dims)
    ms = re.findall(r"Calculation time in seconds:\s*([0-9.eE+-]+)", p.stdout)
    st["calc_seconds"] = float(ms[-1]) if ms else float("nan")
    m = re.search(r"Setup time in seconds:\s*([0-9.eE+-]+)", p.stdout)
    st["setup_seconds"] = float(m.group(1)) if m else float("nan")
    st["stdout"] = p.stdout
    return st


def density_mismatch_forward(dm, variant: str = "libm"):
    """J of a fierro_gb300.adjoint.DensityMismatch computed by the C restatement
    (the reference's algorithm) instead of the GPU: a callable (sie0, gamma) -> J
    for dm.fd(..., forward=...), the check of the adjoint against central
    differences of the reference's forward."""
    from fierro_gb300.adjoint import eos_state

    def f(sie0, gamma):
        o = Oracle(dm.problem, variant=variant)
        st = eos_state(dm.state0, np.asarray(sie0, dtype=np.float64),
                       np.broadcast_to(np.asarray(gamma, dtype=np.float64), dm.sie0.shape).copy())
        o.set(ORC_ELEM_SIE, st["elem_sie"])
        o.set(ORC_ELEM_PRES, st["elem_pres"])
        o.set(ORC_ELEM_SSPD, st["elem_sspd"])
        o.set(ORC_ELEM_STATEV, st["elem_statev"])
        o.run_cycles(dm.cycles)
        return dm.value(o.get(ORC_ELEM_DEN))

    return f
