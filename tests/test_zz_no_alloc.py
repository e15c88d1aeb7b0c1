"""The allocation-free energy tally, called through the C ABI, against the
handle's fierro_sgh_energy.

fierro_energy_tally_noalloc serves callers that cannot call cudaMalloc when they
need the tallies (a driver capturing its time step into a CUDA graph, or a code
whose device memory all belongs to its own arena): it keeps its per-block
partial sums in a static device array instead of allocating.  This file runs
last so a failure here never hides the other tests; it passes alone in a fresh
process as well as after them.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _noalloc(lib):
    f = lib.fierro_energy_tally_noalloc
    f.restype = C.c_int
    f.argtypes = [C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64,
                  C.c_void_p, C.c_void_p]
    return f


def test_noalloc_tally_matches_handle_energy(lib_built):
    import torch
    from fierro_gb300 import problems, sgh
    prob = problems.sedov(18, jitter=0.1, seed=5, permute=True, cycles=40)
    tally = _noalloc(sgh.lib())
    stream = torch.cuda.current_stream()
    out = torch.full((2,), float("nan"), dtype=torch.float64, device="cuda")
    with sgh.SGHSolver(prob) as s:
        s.set_state(sgh.setup(prob))
        for cycles in (7, 25):  # two calls in a row, on two different states
            s.run(cycles)
            ie_ref, ke_ref = s.energy()
            st = s.get_state()
            dev = {k: torch.from_numpy(np.ascontiguousarray(a)).cuda() for k, a in (
                ("mass", st["elem_mass"]), ("sie", st["elem_sie"][1]), ("node_mass", st["node_mass"]),
                ("u", st["node_vel"][1][:, 0]), ("v", st["node_vel"][1][:, 1]), ("w", st["node_vel"][1][:, 2]))}
            torch.cuda.synchronize()
            rc = tally(dev["mass"].data_ptr(), dev["sie"].data_ptr(), s.ne, dev["node_mass"].data_ptr(),
                       dev["u"].data_ptr(), dev["v"].data_ptr(), dev["w"].data_ptr(), s.nn, out.data_ptr(),
                       stream.cuda_stream)
            assert rc == sgh.FIERRO_OK, sgh.lib().fierro_last_error()
            torch.cuda.synchronize()
            ie, ke = (float(x) for x in out.cpu())
            assert ie == pytest.approx(ie_ref, rel=1e-12, abs=0)
            assert ke == pytest.approx(ke_ref, rel=1e-12, abs=0)
            out.fill_(float("nan"))


def test_noalloc_tally_rejects_oversize(lib_built):
    from fierro_gb300 import sgh
    tally = _noalloc(sgh.lib())
    rc = tally(None, None, (1 << 30) + 1, None, None, None, None, 0, None, None)
    assert rc == sgh.FIERRO_EINVAL
    assert "maximum" in sgh.lib().fierro_last_error().decode()


def _tally_inputs(s):
    """The arrays the tally reads, from a handle's current state (host copies),
    with the handle's own tallies."""
    st = s.get_state()
    arrs = {"mass": st["elem_mass"], "sie": st["elem_sie"][1], "node_mass": st["node_mass"],
            "u": st["node_vel"][1][:, 0], "v": st["node_vel"][1][:, 1], "w": st["node_vel"][1][:, 2]}
    return s.energy(), {k: np.ascontiguousarray(a, dtype=np.float64) for k, a in arrs.items()}


def test_noalloc_tally_captured_in_a_cuda_graph(lib_built):
    """The case the entry point exists for: a caller captures its time step,
    diagnostics included, into a CUDA graph and may not allocate meanwhile.  After
    one plain call, the tally is captured in global capture mode, in which a
    device allocation would fail and invalidate the capture, and the graph is
    replayed on two different states.  The device's free memory does not move
    across the plain call or the replays.  (Across the capture itself it does:
    instantiating any graph takes device memory of its own, 2 MiB here.)"""
    import torch
    from fierro_gb300 import problems, sgh
    prob = problems.sedov(18, jitter=0.1, seed=5, permute=True, cycles=40)
    tally = _noalloc(sgh.lib())
    cases = []
    with sgh.SGHSolver(prob) as s:
        s.set_state(sgh.setup(prob))
        for cycles in (4, 13):
            s.run(cycles)
            cases.append(_tally_inputs(s))
    names = ("mass", "sie", "node_mass", "u", "v", "w")
    buf = {k: torch.empty(len(cases[0][1][k]), dtype=torch.float64, device="cuda") for k in names}
    out = torch.full((2,), float("nan"), dtype=torch.float64, device="cuda")
    ne, nn = len(cases[0][1]["mass"]), len(cases[0][1]["u"])
    side = torch.cuda.Stream()

    def load(arrs):
        for k in names:
            buf[k].copy_(torch.from_numpy(arrs[k]))
        out.fill_(float("nan"))
        torch.cuda.synchronize()

    def call(stream_handle):
        return tally(buf["mass"].data_ptr(), buf["sie"].data_ptr(), ne, buf["node_mass"].data_ptr(),
                     buf["u"].data_ptr(), buf["v"].data_ptr(), buf["w"].data_ptr(), nn, out.data_ptr(),
                     stream_handle)

    def check(ref):
        ie, ke = (float(x) for x in out.cpu())
        assert ie == pytest.approx(ref[0], rel=1e-12, abs=0)
        assert ke == pytest.approx(ref[1], rel=1e-12, abs=0)

    load(cases[1][1])
    free0 = torch.cuda.mem_get_info()[0]
    assert call(side.cuda_stream) == sgh.FIERRO_OK, sgh.lib().fierro_last_error()
    side.synchronize()
    assert torch.cuda.mem_get_info()[0] == free0
    check(cases[1][0])

    g = torch.cuda.CUDAGraph()
    torch.cuda.synchronize()
    with torch.cuda.graph(g, stream=side):
        rc = call(torch.cuda.current_stream().cuda_stream)
    assert rc == sgh.FIERRO_OK, sgh.lib().fierro_last_error()
    torch.cuda.synchronize()
    for ref, arrs in cases:  # two replays in a row, on two different states
        load(arrs)
        free2 = torch.cuda.mem_get_info()[0]
        g.replay()
        torch.cuda.synchronize()
        assert torch.cuda.mem_get_info()[0] == free2
        check(ref)
    del g


class _Driver:
    """The few CUDA driver calls the second-context test needs (ctypes on libcuda)."""

    def __init__(self):
        cu = C.CDLL("libcuda.so.1")
        self.cu = cu
        for name, args in (("cuInit", [C.c_uint]), ("cuDeviceGet", [C.POINTER(C.c_int), C.c_int]),
                           ("cuCtxCreate_v2", [C.POINTER(C.c_void_p), C.c_uint, C.c_int]),
                           ("cuCtxPushCurrent_v2", [C.c_void_p]),
                           ("cuCtxPopCurrent_v2", [C.POINTER(C.c_void_p)]),
                           ("cuCtxDestroy_v2", [C.c_void_p]), ("cuCtxSynchronize", []),
                           ("cuMemAlloc_v2", [C.POINTER(C.c_uint64), C.c_size_t]),
                           ("cuMemFree_v2", [C.c_uint64]),
                           ("cuMemcpyHtoD_v2", [C.c_uint64, C.c_void_p, C.c_size_t]),
                           ("cuMemcpyDtoH_v2", [C.c_void_p, C.c_uint64, C.c_size_t])):
            f = getattr(cu, name)
            f.restype = C.c_int
            f.argtypes = args

    def ok(self, rc, what):
        assert rc == 0, "%s returned CUresult %d" % (what, rc)


def test_noalloc_tally_in_a_second_context(lib_built):
    """A caller with a driver context of its own on the same device (cuCtxCreate)
    and the primary context, used alternately: each context holds its own copy
    of the static scratch array, and every call uses the copy of the context
    current at the call (a copy cached from the other context would not even be
    mapped there).  The tallies are right in both contexts, twice each."""
    import torch
    from fierro_gb300 import problems, sgh
    prob = problems.sedov(18, jitter=0.1, seed=5, permute=True, cycles=40)
    tally = _noalloc(sgh.lib())
    cases = []
    with sgh.SGHSolver(prob) as s:
        s.set_state(sgh.setup(prob))
        for cycles in (6, 17):
            s.run(cycles)
            cases.append(_tally_inputs(s))
    names = ("mass", "sie", "node_mass", "u", "v", "w")
    ne, nn = len(cases[0][1]["mass"]), len(cases[0][1]["u"])
    torch.cuda.synchronize()

    # primary context (torch's): device tensors and the stream of torch
    prim = {k: torch.empty(len(cases[0][1][k]), dtype=torch.float64, device="cuda") for k in names}
    prim_out = torch.empty(2, dtype=torch.float64, device="cuda")

    def run_primary(ref, arrs):
        for k in names:
            prim[k].copy_(torch.from_numpy(arrs[k]))
        prim_out.fill_(float("nan"))
        torch.cuda.synchronize()
        rc = tally(prim["mass"].data_ptr(), prim["sie"].data_ptr(), ne, prim["node_mass"].data_ptr(),
                   prim["u"].data_ptr(), prim["v"].data_ptr(), prim["w"].data_ptr(), nn, prim_out.data_ptr(),
                   torch.cuda.current_stream().cuda_stream)
        assert rc == sgh.FIERRO_OK, sgh.lib().fierro_last_error()
        torch.cuda.synchronize()
        ie, ke = (float(x) for x in prim_out.cpu())
        assert ie == pytest.approx(ref[0], rel=1e-12, abs=0)
        assert ke == pytest.approx(ref[1], rel=1e-12, abs=0)

    d = _Driver()
    d.ok(d.cu.cuInit(0), "cuInit")
    dev = C.c_int()
    d.ok(d.cu.cuDeviceGet(C.byref(dev), torch.cuda.current_device()), "cuDeviceGet")
    ctx = C.c_void_p()
    d.ok(d.cu.cuCtxCreate_v2(C.byref(ctx), 0, dev), "cuCtxCreate")  # pushes it as current
    ptrs = {}
    try:
        for k in names + ("out",):
            p = C.c_uint64()
            d.ok(d.cu.cuMemAlloc_v2(C.byref(p), 8 * (2 if k == "out" else len(cases[0][1][k]))), "cuMemAlloc")
            ptrs[k] = p.value
        popped = C.c_void_p()
        d.ok(d.cu.cuCtxPopCurrent_v2(C.byref(popped)), "cuCtxPopCurrent")

        def run_second(ref, arrs):
            d.ok(d.cu.cuCtxPushCurrent_v2(ctx), "cuCtxPushCurrent")
            try:
                for k in names:
                    d.ok(d.cu.cuMemcpyHtoD_v2(ptrs[k], arrs[k].ctypes.data, arrs[k].nbytes), "cuMemcpyHtoD")
                nan2 = np.full(2, np.nan)
                d.ok(d.cu.cuMemcpyHtoD_v2(ptrs["out"], nan2.ctypes.data, 16), "cuMemcpyHtoD")
                rc = tally(ptrs["mass"], ptrs["sie"], ne, ptrs["node_mass"], ptrs["u"], ptrs["v"], ptrs["w"], nn,
                           ptrs["out"], None)
                assert rc == sgh.FIERRO_OK, sgh.lib().fierro_last_error()
                d.ok(d.cu.cuCtxSynchronize(), "cuCtxSynchronize")
                got = np.empty(2)
                d.ok(d.cu.cuMemcpyDtoH_v2(got.ctypes.data, ptrs["out"], 16), "cuMemcpyDtoH")
            finally:
                d.ok(d.cu.cuCtxPopCurrent_v2(C.byref(popped)), "cuCtxPopCurrent")
            assert got[0] == pytest.approx(ref[0], rel=1e-12, abs=0)
            assert got[1] == pytest.approx(ref[1], rel=1e-12, abs=0)

        for ref, arrs in cases:  # alternate: primary, second, primary, second
            run_primary(ref, arrs)
            run_second(ref, arrs)
    finally:
        d.cu.cuCtxPushCurrent_v2(ctx)
        for p in ptrs.values():
            d.cu.cuMemFree_v2(p)
        d.cu.cuCtxDestroy_v2(ctx)  # also pops it from this thread's stack
    torch.cuda.synchronize()
