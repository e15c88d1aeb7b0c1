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
