"""Failure detection without a GPU fault: the device health word, the device
topology checker, and host-injected allocation failures.  Nothing here traps,
faults or hangs the GPU: failures are made on the host (an impossible dt floor,
an allocation budget) and read back as status words and error codes."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_dt_floor_is_reported_not_fatal(lib_built):
    """With dt_min above every CFL step the reference's clamp raises dt to dt_min
    (time_integration.cpp:131-135); the run goes on, and the health word says so."""
    from fierro_gb300 import problems, sgh
    prob = problems.sedov(8, cycles=5)
    with sgh.SGHSolver(prob) as s:
        s.set_state(sgh.setup(prob))
        s.run(3)
        assert s.status() == 0
    prob.params.dt_min = 1e-2
    prob.params.dt_start = 1e-2
    with sgh.SGHSolver(prob) as s:
        s.set_state(sgh.setup(prob))
        try:
            s.run(3)
        except sgh.FierroError:
            pass  # the oversized steps may invert elements, which is reported separately
        assert s.status() & sgh.HEALTH_DT_FLOOR


def test_inverted_element_sets_bad_volume(lib_built):
    from fierro_gb300 import problems, sgh
    prob = problems.sedov(6, cycles=5)
    st = sgh.setup(prob)
    st["node_vel"][1][:, 0] = np.where(st["node_coords"][1][:, 0] > 0.5, -1.0e5, 1.0e5)
    with sgh.SGHSolver(prob) as s:
        s.set_state(st)
        with pytest.raises(sgh.FierroError) as ei:
            s.run(4)
        assert ei.value.code == sgh.FIERRO_ENUMERIC
        assert s.status() & sgh.HEALTH_BAD_VOLUME


@pytest.mark.parametrize("case", ["sedov10_jp", "sedov10_jp_staged", "noh_rz12_jp", "sedov_rz9"])
def test_device_topology_invariants(lib_built, monkeypatch, case):
    from fierro_gb300 import problems, sgh
    if case.endswith("staged"):
        monkeypatch.setenv("FIERRO_STAGED_TRANSFERS", "1")
    prob = {"sedov10_jp": lambda: problems.sedov(10, jitter=0.1, seed=3, permute=True),
            "sedov10_jp_staged": lambda: problems.sedov(10, jitter=0.1, seed=3, permute=True),
            "noh_rz12_jp": lambda: problems.noh_rz(12, jitter=0.1, seed=5, permute=True),
            "sedov_rz9": lambda: problems.sedov_rz(9)}[case]()
    with sgh.SGHSolver(prob) as s:
        s.validate()


@pytest.mark.parametrize("limit", [0, 1, 7, 20])
def test_injected_allocation_failure(lib_built, monkeypatch, limit):
    """Allocation n+1 fails: creation returns FIERRO_ENOMEM and releases what it
    had; a handle created afterwards runs normally."""
    from fierro_gb300 import problems, sgh
    prob = problems.sedov(6, cycles=3)
    monkeypatch.setenv("FIERRO_FAIL_ALLOC_AFTER", str(limit))
    with pytest.raises(sgh.FierroError) as ei:
        sgh.SGHSolver(prob)
    assert ei.value.code == sgh.FIERRO_ENOMEM and "injected" in str(ei.value)
    monkeypatch.delenv("FIERRO_FAIL_ALLOC_AFTER")
    with sgh.SGHSolver(prob) as s:
        s.set_state(sgh.setup(prob))
        assert s.run(3) == 3


def test_fp64_rate_probes(lib_built):
    """The FP64 roof the bench reports against: the calibration rate and the pure
    FP64 stream of fierro_fp64_stream_rate agree (both measure the same pipe), and
    the stream rejects shapes it does not run."""
    from fierro_gb300 import sgh
    calib = sgh.measure_fp64_rate()
    stream = sgh.fp64_stream_rate(8, 0, 256, 8)
    assert calib > 1e11 and stream > 1e11
    assert abs(stream - calib) <= 0.05 * calib, (stream, calib)
    assert sgh.fp64_stream_rate(8, 1, 256, 4) > 0.8 * stream  # DADD at the DFMA rate
    for bad in ((3, 0, 256, 4), (8, 3, 256, 4), (8, 0, 100, 4), (8, 0, 256, 0)):
        with pytest.raises(sgh.FierroError) as ei:
            sgh.fp64_stream_rate(*bad)
        assert ei.value.code == sgh.FIERRO_EINVAL


def test_mode_roots_against_library(lib_built):
    """The arithmetic modes' square roots, cube roots, quotients and reciprocals
    against the CUDA library's.  Exact mode: bit for bit (its Newton square
    roots and quotients are correctly rounded, with the library's operation
    where the remainder test cannot decide), also on arguments whose result lies
    within a tiny fraction of an ulp of a rounding boundary.  FMA mode: square
    and cube roots within one ulp over the whole exponent range and over the
    range the cycle feeds them, the square root nearly always equal; quotients
    and reciprocals equal to the IEEE ones but within one ulp next to a
    rounding boundary."""
    from fierro_gb300 import sgh
    n = 1 << 26
    for lo, hi in ((-1022, 1023), (-90, 8)):
        for which in (0, 1, 2, 3):
            r = sgh.root_check(sgh.FP_EXACT, which, n, seed=3 + which, lo_exp=lo, hi_exp=hi)
            assert r["differing"] == 0, (which, lo, r)
        s = sgh.root_check(sgh.FP_FMA, 0, n, seed=11, lo_exp=lo, hi_exp=hi)
        assert s["max_ulp"] <= 1 and s["above_one_ulp"] == 0 and s["differing"] <= 1e-5 * n, s
        c = sgh.root_check(sgh.FP_FMA, 1, n, seed=12, lo_exp=lo, hi_exp=hi)
        assert c["max_ulp"] <= 1 and c["above_one_ulp"] == 0 and c["differing"] <= 0.15 * n, c
        for which in (2, 3):
            q = sgh.root_check(sgh.FP_FMA, which, n, seed=13 + which, lo_exp=lo, hi_exp=hi)
            assert q["differing"] == 0, (which, lo, q)
    for which in (4, 5, 6):
        r = sgh.root_check(sgh.FP_EXACT, which, 1 << 24, seed=21 + which)
        assert r["differing"] == 0, (which, r)
        f = sgh.root_check(sgh.FP_FMA, which, 1 << 24, seed=21 + which)
        assert f["max_ulp"] <= 1, (which, f)
    # the adjoint's reciprocal and reciprocal square root: within 2^11 ulps (~2^-42;
    # measured at most 361 and 349 ulps)
    for which in (7, 8):
        for mode in (sgh.FP_EXACT, sgh.FP_FMA):
            f = sgh.root_check(mode, which, 1 << 24, seed=31 + which, lo_exp=-240, hi_exp=240)
            assert f["max_ulp"] <= 2048, (which, mode, f)
    for bad in ((2, 0, 64), (1, 9, 64), (1, 0, 4)):
        with pytest.raises(sgh.FierroError) as ei:
            sgh.root_check(*bad)
        assert ei.value.code == sgh.FIERRO_EINVAL
