"""Python mirror of the SGH solver interface over the libfierro_sgh C ABI.

The names and argument meanings follow Explicit-Lagrange-Kokkos/SGH_solver:
``setup`` (setup.cpp:10-424) builds the initial state, ``sgh_solve``
(sgh_solve.cpp:8-692) runs the cycle loop, and ``SGHSolver`` is the persistent
device-resident handle.  State travels as a dict of numpy arrays in the
reference layouts (see include/fierro_sgh.h).

There is no CPU fallback: importing this module loads the CUDA library and
every call runs on the GPU; a missing library raises ImportError.
"""
from __future__ import annotations

import ctypes as C
import os
from typing import Dict, Optional

import numpy as np

from .problems import HYDRO_BC, REGION, SURFACE, VELOCITY, Problem

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libfierro_sgh.so")

FIERRO_OK, FIERRO_EINVAL, FIERRO_ENOMEM, FIERRO_ECUDA, FIERRO_ENUMERIC, FIERRO_ETIMEDOUT, FIERRO_ENOTSUP = range(7)
FP_EXACT, FP_FMA = 0, 1
ADJ_BRANCHES_OFF, ADJ_BRANCHES_RECORD, ADJ_BRANCHES_FREEZE = 0, 1, 2
HEALTH_BAD_VOLUME, HEALTH_BAD_STATE, HEALTH_DT_FLOOR = 1, 2, 4
OUTPUT_ENSIGHT, OUTPUT_STATE = 1, 2
_ERRNAMES = {1: "EINVAL", 2: "ENOMEM", 3: "ECUDA", 4: "ENUMERIC", 5: "ETIMEDOUT", 6: "ENOTSUP"}


class FierroError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__("fierro %s: %s" % (_ERRNAMES.get(code, str(code)), msg))
        self.code = code


class Material(C.Structure):
    _fields_ = [("eos_model", C.c_int), ("strength_type", C.c_int), ("q1", C.c_double),
                ("q1ex", C.c_double), ("q2", C.c_double), ("q2ex", C.c_double)]


class Boundary(C.Structure):
    _fields_ = [("surface", C.c_int), ("value", C.c_double), ("hydro_bc", C.c_int)]


class MatFill(C.Structure):
    _fields_ = [("volume", C.c_int), ("mat_id", C.c_int)] + \
        [(k, C.c_double) for k in ("x1", "x2", "y1", "y2", "z1", "z2", "radius1", "radius2")] + \
        [("velocity", C.c_int)] + [(k, C.c_double) for k in ("u", "v", "w", "speed", "sie", "den")]


class Params(C.Structure):
    _fields_ = [(k, C.c_double) for k in ("time_final", "dt_max", "dt_min", "dt_cfl", "dt_start",
                                          "graphics_dt_ival")] + \
        [(k, C.c_int64) for k in ("graphics_cyc_ival", "cycle_stop", "rk_num_stages")] + \
        [(k, C.c_double) for k in ("fuzz", "tiny", "small")]


class Mesh(C.Structure):
    _fields_ = [("num_nodes", C.c_int64), ("num_elems", C.c_int64), ("nodes_in_elem", C.c_void_p),
                ("coords", C.c_void_p), ("num_dims", C.c_int64)]


class State(C.Structure):
    _fields_ = [(k, C.c_void_p) for k in (
        "node_coords", "node_vel", "node_mass", "elem_den", "elem_pres", "elem_stress", "elem_sspd",
        "elem_sie", "elem_vol", "elem_div", "elem_mass", "elem_mat_id", "elem_statev", "corner_force")] + \
        [("num_state_vars", C.c_int64)]


def _load():
    if not os.path.exists(LIB_PATH):
        raise ImportError("libfierro_sgh.so is not built (run __graft_entry__.build()); "
                          "the SGH path has no CPU fallback")
    lib = C.CDLL(LIB_PATH)
    vp, i64, dbl = C.c_void_p, C.c_int64, C.c_double
    lib.fierro_last_error.restype = C.c_char_p
    lib.fierro_version.restype = C.c_char_p
    lib.fierro_sgh_setup.argtypes = [vp, vp, i64, vp, i64, vp, i64, vp, i64, vp]
    lib.fierro_sgh_solve.argtypes = [vp, vp, i64, vp, i64, vp, C.POINTER(dbl), dbl, dbl, dbl, dbl,
                                     C.POINTER(dbl), i64, dbl, i64, i64, dbl, dbl, dbl, dbl, C.c_int,
                                     C.POINTER(i64)]
    lib.fierro_sgh_create.argtypes = [vp, vp, i64, vp, i64, vp, C.c_int, vp, C.POINTER(vp)]
    lib.fierro_sgh_destroy.argtypes = [vp]
    lib.fierro_sgh_set_state.argtypes = [vp, vp]
    lib.fierro_sgh_get_state.argtypes = [vp, vp]
    lib.fierro_sgh_enqueue_cycles.argtypes = [vp, i64]
    lib.fierro_sgh_run.argtypes = [vp, i64, C.POINTER(i64)]
    lib.fierro_sgh_run_stages.argtypes = [vp, i64]
    lib.fierro_sgh_synchronize.argtypes = [vp]
    lib.fierro_sgh_time.argtypes = [vp, C.POINTER(dbl), C.POINTER(dbl), C.POINTER(dbl), C.POINTER(i64)]
    lib.fierro_sgh_energy.argtypes = [vp, C.POINTER(dbl), C.POINTER(dbl)]
    lib.fierro_sgh_launches_per_cycle.argtypes = [vp]
    lib.fierro_sgh_launches_per_cycle.restype = i64
    lib.fierro_sgh_device_bytes.argtypes = [vp]
    lib.fierro_sgh_device_bytes.restype = i64
    lib.fierro_sgh_run_timed.argtypes = [vp, i64, vp, C.POINTER(C.c_float), C.POINTER(i64)]
    lib.fierro_measure_fp64_rate.argtypes = [C.POINTER(dbl)]
    lib.fierro_fp64_stream_rate.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.POINTER(dbl)]
    lib.fierro_root_check.argtypes = [C.c_int, C.c_int, C.c_longlong, C.c_ulonglong, C.c_int, C.c_int,
                                      C.POINTER(C.c_ulonglong)]
    lib.fierro_batch_create.argtypes = [vp, i64, C.c_int, vp, C.POINTER(vp)]
    lib.fierro_batch_destroy.argtypes = [vp]
    lib.fierro_batch_set_state.argtypes = [vp, i64, vp]
    lib.fierro_batch_get_state.argtypes = [vp, i64, vp]
    lib.fierro_batch_run.argtypes = [vp, i64]
    lib.fierro_batch_time.argtypes = [vp, i64, C.POINTER(dbl), C.POINTER(dbl), C.POINTER(i64)]
    lib.fierro_batch_num_instances.argtypes = [vp]
    lib.fierro_batch_num_instances.restype = i64
    lib.fierro_batch_device_bytes.argtypes = [vp]
    lib.fierro_batch_device_bytes.restype = i64
    lib.fierro_batch_set_shape.argtypes = [vp, vp]
    lib.fierro_batch_get_shape.argtypes = [vp, vp]
    lib.fierro_batch_autotune.argtypes = [vp, i64, vp]
    lib.fierro_batch_tune_log.argtypes = [vp, vp, vp, i64, C.POINTER(i64)]
    lib.fierro_sgh_device_view.argtypes = [vp, vp]
    lib.fierro_sgh_set_output.argtypes = [vp, C.c_char_p, C.c_int, C.c_int]
    lib.fierro_sgh_flush_output.argtypes = [vp, C.POINTER(i64)]
    lib.fierro_adj_forward.argtypes = [vp, vp, vp, i64, i64, C.POINTER(i64)]
    lib.fierro_adj_backward.argtypes = [vp, vp, vp, vp, vp]
    lib.fierro_adj_verify.argtypes = [vp, C.c_int]
    lib.fierro_adj_stats.argtypes = [vp, C.POINTER(i64), i64]
    lib.fierro_adj_release.argtypes = [vp]
    lib.fierro_adj_branches.argtypes = [vp, C.c_int]
    lib.fierro_sgh_checkpoint.argtypes = [vp, C.c_char_p]
    lib.fierro_sgh_restart.argtypes = [vp, C.c_char_p]
    lib.fierro_sgh_validate.argtypes = [vp]
    lib.fierro_sgh_status.argtypes = [vp, C.POINTER(C.c_uint32)]
    return lib


_lib = _load()


def lib():
    return _lib


def _check(rc: int):
    if rc != FIERRO_OK:
        raise FierroError(rc, _lib.fierro_last_error().decode())


def version() -> str:
    return _lib.fierro_version().decode()


# ---------------------------------------------------------------- deck conversion
def c_mesh(mesh) -> tuple:
    nie = np.ascontiguousarray(mesh.nodes_in_elem, dtype=np.uint64)
    xyz = np.ascontiguousarray(mesh.coords, dtype=np.float64)
    m = Mesh(mesh.num_nodes, mesh.num_elems, nie.ctypes.data, xyz.ctypes.data, mesh.dims)
    return m, (nie, xyz)


def c_materials(problem: Problem):
    mats = problem.materials
    return (Material * len(mats))(*[Material(0, q.strength_type, q.q1, q.q1ex, q.q2, q.q2ex) for q in mats])


def c_boundaries(problem: Problem):
    bl = problem.boundaries
    return (Boundary * max(len(bl), 1))(*[Boundary(SURFACE[b.surface], b.value, HYDRO_BC[b.hydro_bc])
                                          for b in bl])


def c_fills(problem: Problem):
    fl = problem.fills
    return (MatFill * max(len(fl), 1))(*[MatFill(
        REGION[f.volume], f.mat_id, f.x1, f.x2, f.y1, f.y2, f.z1, f.z2, f.radius1, f.radius2,
        VELOCITY[f.velocity], f.u, f.v, f.w, f.speed, f.sie, f.den) for f in fl])


def c_params(problem: Problem) -> Params:
    p = problem.params
    return Params(p.time_final, p.dt_max, p.dt_min, p.dt_cfl, p.dt_start, p.graphics_dt_ival,
                  p.graphics_cyc_ival, p.cycle_stop, p.rk_num_stages, p.fuzz, p.tiny, p.small)


def empty_state(nn: int, ne: int, nsv: int = 6, pinned: bool = False, dims: int = 3) -> Dict[str, np.ndarray]:
    """Host arrays for one state in the reference layouts (dims 2: the 2D-RZ
    layouts with two components per node and four corners per element)."""
    D, npe = dims, 2 ** dims
    return {
        "node_coords": np.zeros((2, nn, D)), "node_vel": np.zeros((2, nn, D)), "node_mass": np.zeros(nn),
        "elem_den": np.zeros(ne), "elem_pres": np.zeros(ne), "elem_stress": np.zeros((2, ne, 3, 3)),
        "elem_sspd": np.zeros(ne), "elem_sie": np.zeros((2, ne)), "elem_vol": np.zeros(ne),
        "elem_div": np.zeros(ne), "elem_mass": np.zeros(ne), "elem_mat_id": np.zeros(ne, dtype=np.uint64),
        "elem_statev": np.zeros((ne, nsv)), "corner_force": np.zeros((npe * ne, D)),
    }


def c_state(st: Dict[str, np.ndarray]) -> State:
    s = State()
    for k, _ in State._fields_[:-1]:
        a = st.get(k)
        if a is not None:
            assert a.flags["C_CONTIGUOUS"], k
            setattr(s, k, a.ctypes.data)
    s.num_state_vars = st["elem_statev"].shape[1]
    return s


def setup(problem: Problem) -> Dict[str, np.ndarray]:
    """setup (setup.cpp:10-424) on the host: the initial state of a problem deck."""
    m, keep = c_mesh(problem.mesh)
    st = empty_state(problem.mesh.num_nodes, problem.mesh.num_elems, problem.num_state_vars,
                     dims=problem.mesh.dims)
    sv = np.ascontiguousarray(problem.state_vars())
    _check(_lib.fierro_sgh_setup(C.byref(m), c_materials(problem), len(problem.materials), sv.ctypes.data,
                                 problem.num_state_vars, c_fills(problem), len(problem.fills),
                                 c_boundaries(problem), len(problem.boundaries), C.byref(c_state(st))))
    return st


def sgh_solve(problem: Problem, state: Dict[str, np.ndarray], cycle_stop: Optional[int] = None,
              time_value: float = 0.0, fp_mode: int = FP_EXACT) -> dict:
    """sgh_solve (sgh_solve.cpp:8-692) over host arrays: uploads, runs the cycle
    loop on the GPU and writes the final state back into `state` (in place).
    Returns time_value, graphics_time and the number of cycles run."""
    p = problem.params
    m, keep = c_mesh(problem.mesh)
    tv = C.c_double(time_value)
    gt = C.c_double(p.graphics_dt_ival)
    ran = C.c_int64(0)
    ncyc = p.cycle_stop if cycle_stop is None else cycle_stop
    _check(_lib.fierro_sgh_solve(C.byref(m), c_materials(problem), len(problem.materials), c_boundaries(problem),
                                 len(problem.boundaries), C.byref(c_state(state)), C.byref(tv), p.time_final,
                                 p.dt_max, p.dt_min, p.dt_cfl, C.byref(gt), p.graphics_cyc_ival,
                                 p.graphics_dt_ival, ncyc, p.rk_num_stages, p.dt_start, p.fuzz, p.tiny,
                                 p.small, fp_mode, C.byref(ran)))
    return {"time_value": tv.value, "graphics_time": gt.value, "cycles": ran.value}


class SGHSolver:
    """Persistent device-resident SGH solver for one mesh."""

    def __init__(self, problem: Problem, fp_mode: int = FP_EXACT, stream: int | None = None):
        self.problem = problem
        self.nn, self.ne = problem.mesh.num_nodes, problem.mesh.num_elems
        self.nsv = problem.num_state_vars
        m, self._keep = c_mesh(problem.mesh)
        self._params = c_params(problem)
        h = C.c_void_p()
        _check(_lib.fierro_sgh_create(C.byref(m), c_materials(problem), len(problem.materials),
                                      c_boundaries(problem), len(problem.boundaries), C.byref(self._params),
                                      fp_mode, C.c_void_p(stream) if stream else None, C.byref(h)))
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            _lib.fierro_sgh_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def set_state(self, st: Dict[str, np.ndarray]):
        _check(_lib.fierro_sgh_set_state(self.h, C.byref(c_state(st))))

    def get_state(self, st: Optional[Dict[str, np.ndarray]] = None) -> Dict[str, np.ndarray]:
        if st is None:
            st = empty_state(self.nn, self.ne, self.nsv, dims=self.problem.mesh.dims)
        _check(_lib.fierro_sgh_get_state(self.h, C.byref(c_state(st))))
        return st

    def run(self, cycles: int) -> int:
        ran = C.c_int64(0)
        _check(_lib.fierro_sgh_run(self.h, cycles, C.byref(ran)))
        return ran.value

    def run_timed(self, cycles: int):
        """Runs `cycles` cycles with an event after every launch; returns
        (cycles_run, total_ms, per-launch-slot ms summed over cycles)."""
        L = self.launches_per_cycle
        kms = (C.c_float * L)()
        tot = C.c_float(0)
        ran = C.c_int64(0)
        _check(_lib.fierro_sgh_run_timed(self.h, cycles, kms, C.byref(tot), C.byref(ran)))
        return ran.value, tot.value, list(kms)

    def launch_names(self):
        S = self.problem.params.rk_num_stages
        stage = ("k_force", "k_node", "k_axis", "k_elem") if self.problem.mesh.dims == 2 else \
            ("k_force", "k_node", "k_elem")
        return ["k_dt"] + [n for s in range(S) for n in stage] + ["k_end"]

    def enqueue(self, cycles: int):
        _check(_lib.fierro_sgh_enqueue_cycles(self.h, cycles))

    def synchronize(self):
        _check(_lib.fierro_sgh_synchronize(self.h))

    def run_stages(self, stages: int):
        _check(_lib.fierro_sgh_run_stages(self.h, stages))

    def time(self):
        t, dt, gt, cyc = C.c_double(), C.c_double(), C.c_double(), C.c_int64()
        _check(_lib.fierro_sgh_time(self.h, C.byref(t), C.byref(dt), C.byref(gt), C.byref(cyc)))
        return t.value, dt.value, gt.value, cyc.value

    def energy(self):
        ie, ke = C.c_double(), C.c_double()
        _check(_lib.fierro_sgh_energy(self.h, C.byref(ie), C.byref(ke)))
        return ie.value, ke.value

    def checkpoint(self, path: str):
        """fierro_sgh_checkpoint: the loop state at this cycle boundary, to a file."""
        _check(_lib.fierro_sgh_checkpoint(self.h, os.fsencode(path)))

    def status(self) -> int:
        """fierro_sgh_status: the run's health word (HEALTH_* bits)."""
        f = C.c_uint32(0)
        _check(_lib.fierro_sgh_status(self.h, C.byref(f)))
        return f.value

    def validate(self):
        """fierro_sgh_validate: the device topology's invariants, checked on the GPU."""
        _check(_lib.fierro_sgh_validate(self.h))

    def restart(self, path: str):
        """fierro_sgh_restart: continue from a checkpoint of the same problem."""
        _check(_lib.fierro_sgh_restart(self.h, os.fsencode(path)))

    @property
    def launches_per_cycle(self) -> int:
        return int(_lib.fierro_sgh_launches_per_cycle(self.h))

    @property
    def device_bytes(self) -> int:
        return int(_lib.fierro_sgh_device_bytes(self.h))

    def set_output(self, directory: Optional[str], ensight: bool = True, state: bool = True, slots: int = 4):
        """Graphics dumps of write_outputs (EnSight Gold and the element state
        text) under `directory`, written by the handle's writer thread while the
        cycles run; None turns them off."""
        what = (OUTPUT_ENSIGHT if ensight else 0) | (OUTPUT_STATE if state else 0)
        _check(_lib.fierro_sgh_set_output(self.h, None if directory is None else directory.encode(),
                                          what if directory is not None else 0, slots))

    def flush_output(self) -> int:
        """Waits for the dumps taken so far; returns how many were written since set_state."""
        n = C.c_int64(0)
        _check(_lib.fierro_sgh_flush_output(self.h, C.byref(n)))
        return n.value

    def device_view(self) -> Dict[str, object]:
        """The device-resident state as torch tensors over the library's memory
        (no copy), in the device numbering, with the int32 renumbering maps
        (caller id = node_int2ext[device id]).  Valid until the next call that runs
        cycles or uploads a state."""
        import torch
        from torch.utils.dlpack import from_dlpack
        v = DeviceView()
        _check(_lib.fierro_sgh_device_view(self.h, C.byref(v)))
        dev = torch.cuda.current_device()
        nn, ne = v.num_nodes, v.num_elems
        out = {}
        for k in ("x", "y", "z", "u", "v", "w", "node_mass"):
            out[k] = from_dlpack(_dlpack_capsule(getattr(v, k), (nn,), 2, 64, dev))
        for k in ("den", "pres", "sspd", "sie", "vol", "mass", "div"):
            out[k] = from_dlpack(_dlpack_capsule(getattr(v, k), (ne,), 2, 64, dev))
        out["corner_force"] = from_dlpack(_dlpack_capsule(v.corner_force, (24, ne), 2, 64, dev))
        for k, n in (("node_int2ext", nn), ("elem_int2ext", ne), ("node_ext2int", nn), ("elem_ext2int", ne)):
            out[k] = from_dlpack(_dlpack_capsule(getattr(v, k), (n,), 0, 32, dev))
        return out

    def adj_forward(self, sie0=None, gamma=None, cycles: int = 1, ckpt_every: int = 20) -> int:
        """fierro_adj_forward: replace the current state's sie (and per-element gamma)
        by the parameters, recompute pressure and sound speed, run `cycles` cycles
        keeping checkpoints every `ckpt_every`.  Returns the cycles run."""
        s0 = _f64(sie0, (self.ne,))
        g0 = _f64(gamma, (self.ne,)) if gamma is None or np.ndim(gamma) else np.full(self.ne, float(gamma))
        ran = C.c_int64(0)
        _check(_lib.fierro_adj_forward(self.h, None if s0 is None else s0.ctypes.data,
                                       None if g0 is None else g0.ctypes.data, cycles, ckpt_every, C.byref(ran)))
        return ran.value


    def adj_backward(self, den=None, pres=None, sie=None, sspd=None, vol=None, coords=None, vel=None):
        """fierro_adj_backward: adjoints of the final state's fields in, returns
        (d/d sie0 [Ne], d/d gamma per element [Ne], d/d initial velocity [Nn,3])."""
        keep = {k: _f64(v) for k, v in dict(den=den, pres=pres, sie=sie, sspd=sspd, vol=vol, coords=coords,
                                             vel=vel).items()}
        seed = AdjSeed(*[None if keep[k] is None else keep[k].ctypes.data for k, _ in AdjSeed._fields_])
        sb, gb, vb = np.empty(self.ne), np.empty(self.ne), np.empty((self.nn, 3))
        _check(_lib.fierro_adj_backward(self.h, C.byref(seed), sb.ctypes.data, gb.ctypes.data, vb.ctypes.data))
        return sb, gb, vb


    def adj_verify(self, enable: bool = True):
        _check(_lib.fierro_adj_verify(self.h, 1 if enable else 0))


    def adj_stats(self) -> dict:
        out = (C.c_int64 * len(ADJ_STATS))()
        _check(_lib.fierro_adj_stats(self.h, out, len(ADJ_STATS)))
        return dict(zip(ADJ_STATS, list(out)))


    def adj_release(self):
        _check(_lib.fierro_adj_release(self.h))

    def adj_branches(self, mode: int):
        """fierro_adj_branches: ADJ_BRANCHES_RECORD makes the next adj_forward calls
        record the forward's branch decisions; ADJ_BRANCHES_FREEZE runs later
        adj_forward calls with the recorded decisions (the frozen-branch forward);
        ADJ_BRANCHES_OFF returns to plain forwards."""
        _check(_lib.fierro_adj_branches(self.h, int(mode)))


class DeviceView(C.Structure):
    _fields_ = [("num_nodes", C.c_int64), ("num_elems", C.c_int64)] + \
        [(k, C.c_void_p) for k in ("x", "y", "z", "u", "v", "w", "node_mass", "den", "pres", "sspd", "sie", "vol",
                                   "mass", "div", "corner_force", "node_int2ext", "elem_int2ext", "node_ext2int",
                                   "elem_ext2int", "stream")]


# ---- DLPack (zero-copy hand-over of device arrays to torch) -------------------
class _DLDevice(C.Structure):
    _fields_ = [("device_type", C.c_int32), ("device_id", C.c_int32)]


class _DLDataType(C.Structure):
    _fields_ = [("code", C.c_uint8), ("bits", C.c_uint8), ("lanes", C.c_uint16)]


class _DLTensor(C.Structure):
    _fields_ = [("data", C.c_void_p), ("device", _DLDevice), ("ndim", C.c_int32), ("dtype", _DLDataType),
                ("shape", C.POINTER(C.c_int64)), ("strides", C.POINTER(C.c_int64)), ("byte_offset", C.c_uint64)]


class _DLManagedTensor(C.Structure):
    pass


_DLDeleter = C.CFUNCTYPE(None, C.POINTER(_DLManagedTensor))
_DLManagedTensor._fields_ = [("dl_tensor", _DLTensor), ("manager_ctx", C.c_void_p), ("deleter", _DLDeleter)]
_dl_alive = {}  # managed tensors handed out and not yet released by their consumer


@_DLDeleter
def _dl_release(mt):
    _dl_alive.pop(C.addressof(mt.contents), None)


def _dlpack_capsule(ptr: int, shape, code: int, bits: int, device: int):
    """A 'dltensor' capsule over device memory the library owns (the deleter only
    drops the descriptor; the memory stays with the handle)."""
    shp = (C.c_int64 * len(shape))(*shape)
    mt = _DLManagedTensor()
    mt.dl_tensor = _DLTensor(C.c_void_p(ptr), _DLDevice(2, device), len(shape), _DLDataType(code, bits, 1),
                             C.cast(shp, C.POINTER(C.c_int64)), None, 0)
    mt.manager_ctx = None
    mt.deleter = _dl_release
    _dl_alive[C.addressof(mt)] = (mt, shp)
    new = C.pythonapi.PyCapsule_New
    new.restype = C.py_object
    new.argtypes = [C.c_void_p, C.c_char_p, C.c_void_p]
    return new(C.addressof(mt), b"dltensor", None)


class AdjSeed(C.Structure):
    _fields_ = [(k, C.c_void_p) for k in ("den", "pres", "sie", "sspd", "vol", "coords", "vel")]


ADJ_STATS = ("cycles", "ckpt_every", "segments", "tape_bytes", "ckpt_bytes", "device_bytes", "force_mismatches",
             "status", "dt_cfl_cycles", "dt_growth_cycles", "dt_other_cycles")


def _f64(a, shape=None):
    if a is None:
        return None
    a = np.ascontiguousarray(a, dtype=np.float64)
    if shape is not None and a.size != int(np.prod(shape)):
        raise ValueError("expected %s values, got %d" % (shape, a.size))
    return a


class BatchShape(C.Structure):
    _fields_ = [("force_block", C.c_int), ("node_block", C.c_int), ("elem_block", C.c_int),
                ("persistent", C.c_int), ("fused_stage", C.c_int)]

    def as_tuple(self):
        return (self.force_block, self.node_block, self.elem_block, self.persistent, self.fused_stage)


class BatchInstance(C.Structure):
    _fields_ = [("mesh", Mesh), ("materials", C.c_void_p), ("num_materials", C.c_int64), ("boundaries", C.c_void_p),
                ("num_bcs", C.c_int64), ("params", Params)]


class Batch:
    """Batched ensemble: many independent problems advanced together, one launch
    per kernel per cycle for all of them (fierro_batch_* in the C ABI)."""

    def __init__(self, problems, fp_mode: int = FP_EXACT, stream: int | None = None):
        self.problems = list(problems)
        n = len(self.problems)
        self._keep = []
        arr = (BatchInstance * n)()
        for i, p in enumerate(self.problems):
            m, keep = c_mesh(p.mesh)
            mats, bcs = c_materials(p), c_boundaries(p)
            self._keep += [keep, mats, bcs]
            arr[i] = BatchInstance(m, C.cast(mats, C.c_void_p), len(p.materials), C.cast(bcs, C.c_void_p),
                                   len(p.boundaries), c_params(p))
        self._arr = arr
        h = C.c_void_p()
        _check(_lib.fierro_batch_create(arr, n, fp_mode, C.c_void_p(stream) if stream else None, C.byref(h)))
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            _lib.fierro_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __len__(self):
        return len(self.problems)

    def set_state(self, i: int, st: Dict[str, np.ndarray]):
        _check(_lib.fierro_batch_set_state(self.h, i, C.byref(c_state(st))))

    def get_state(self, i: int) -> Dict[str, np.ndarray]:
        p = self.problems[i]
        st = empty_state(p.mesh.num_nodes, p.mesh.num_elems, p.num_state_vars)
        _check(_lib.fierro_batch_get_state(self.h, i, C.byref(c_state(st))))
        return st

    def run(self, cycles: int):
        _check(_lib.fierro_batch_run(self.h, cycles))

    def time(self, i: int):
        t, dt, cyc = C.c_double(), C.c_double(), C.c_int64()
        _check(_lib.fierro_batch_time(self.h, i, C.byref(t), C.byref(dt), C.byref(cyc)))
        return t.value, dt.value, cyc.value

    @property
    def device_bytes(self) -> int:
        return int(_lib.fierro_batch_device_bytes(self.h))

    def set_shape(self, force_block: int = 128, node_block: int = 256, elem_block: int = 128, persistent: int = 0,
                  fused_stage: int = 0):
        """fierro_batch_set_shape: threads per block of the force, node and element
        passes, the persistent grid (fills of the SMs, 0 = one block per tile) and
        the fused stage (1: one cooperative launch per RK stage)."""
        _check(_lib.fierro_batch_set_shape(self.h, C.byref(BatchShape(force_block, node_block, elem_block,
                                                                      persistent, fused_stage))))

    def shape(self):
        sh = BatchShape()
        _check(_lib.fierro_batch_get_shape(self.h, C.byref(sh)))
        return sh.as_tuple()

    def autotune(self, cycles: int = 3):
        """fierro_batch_autotune: times the candidate shapes from the uploaded state
        and keeps the fastest; returns (chosen shape, [(shape, ms per cycle), ...])."""
        sh = BatchShape()
        _check(_lib.fierro_batch_autotune(self.h, int(cycles), C.byref(sh)))
        cap = 64
        shapes, ms, n = (BatchShape * cap)(), (C.c_double * cap)(), C.c_int64()
        _check(_lib.fierro_batch_tune_log(self.h, shapes, ms, cap, C.byref(n)))
        return sh.as_tuple(), [(shapes[i].as_tuple(), ms[i]) for i in range(min(n.value, cap))]


def fp64_stream_rate(chains: int, op: int = 0, threads: int = 256, blocks_per_sm: int = 4) -> float:
    """fierro_fp64_stream_rate: FP64 operations per second of a pure stream of
    `chains` independent chains per thread (op 0 fma, 1 add, 2 mul)."""
    r = C.c_double()
    _check(_lib.fierro_fp64_stream_rate(int(chains), int(op), int(threads), int(blocks_per_sm), C.byref(r)))
    return r.value


def root_check(fp_mode: int, which: int, n: int, seed: int = 1, lo_exp: int = -1022, hi_exp: int = 1023) -> dict:
    """fierro_root_check: the mode's square root, cube root, quotient or
    reciprocal (which 0..3) against the CUDA library's on n inputs (eight special
    values, then seeded doubles with exponents in [lo_exp, hi_exp]); which 4..6:
    square roots, quotients and reciprocals next to rounding boundaries."""
    out = (C.c_ulonglong * 3)()
    _check(_lib.fierro_root_check(int(fp_mode), int(which), int(n), int(seed), int(lo_exp), int(hi_exp), out))
    return {"n": int(n), "differing": int(out[0]), "max_ulp": int(out[1]), "above_one_ulp": int(out[2])}


def measure_fp64_rate() -> float:
    """Measured FP64 fused-multiply-add rate of the current GPU (FMA/s)."""
    r = C.c_double(0)
    _check(_lib.fierro_measure_fp64_rate(C.byref(r)))
    return r.value


def compared_fields(st: Dict[str, np.ndarray]) -> Dict[str, np.ndarray]:
    """The fields parity is judged on (bin 1 = current values), as flat arrays."""
    return {"coords": st["node_coords"][1], "vel": st["node_vel"][1], "den": st["elem_den"],
            "pres": st["elem_pres"], "sie": st["elem_sie"][1], "sspd": st["elem_sspd"], "vol": st["elem_vol"]}
