"""Batched ensemble against separate single-problem runs: every instance of a
mixed batch (Sedov and Noh, different sizes, gammas, CFL numbers, renumbered
meshes, one instance that stops early at its own time_final) matches a
separate fierro_sgh handle bit for bit, in both arithmetic modes."""
import numpy as np
import pytest

from conftest import assert_bitwise

pytestmark = pytest.mark.gpu

FIELDS = ("coords", "vel", "den", "pres", "sie", "sspd", "vol")


def _problems():
    from fierro_gb300 import problems
    ps = [
        problems.sedov(8, cycles=40),
        problems.noh(10, jitter=0.1, seed=3, permute=True, cycles=40),
        problems.sedov(13, length=1.0, energy=1.7, gamma=1.6, jitter=0.1, seed=5, permute=True, cycles=40),
        problems.noh(9, speed=-0.7, gamma=1.3, cycles=40),
        problems.sedov(5, energy=0.05, gamma=1.25, cfl=0.3, cycles=40),
        problems.noh(7, jitter=0.05, seed=8, cycles=40),
    ]
    ps[3].params.time_final = 0.004  # stops before 40 cycles
    return ps


@pytest.mark.parametrize("mode", [0, 1])
def test_batch_equals_single_runs(lib_built, mode):
    from fierro_gb300 import sgh
    ps = _problems()
    states = [sgh.setup(p) for p in ps]
    with sgh.Batch(ps, fp_mode=mode) as b:
        for i, st in enumerate(states):
            b.set_state(i, st)
        b.run(25)
        b.run(15)
        got = [b.get_state(i) for i in range(len(ps))]
        times = [b.time(i) for i in range(len(ps))]
    stopped_early = False
    for i, p in enumerate(ps):
        with sgh.SGHSolver(p, fp_mode=mode) as s:
            s.set_state(states[i])
            ran = s.run(40)
            ref = s.get_state()
            t = s.time()
        assert times[i][2] == ran and times[i][0] == t[0], (i, times[i], t)
        stopped_early |= ran < 40
        assert_bitwise(sgh.compared_fields(got[i]), sgh.compared_fields(ref), FIELDS, label="instance %d" % i)
        assert np.array_equal(got[i]["elem_div"], ref["elem_div"])
    assert stopped_early


def test_batch_rejects_mismatched_controls(lib_built):
    from fierro_gb300 import sgh
    ps = _problems()[:2]
    ps[1].params.rk_num_stages = 1
    with pytest.raises(sgh.FierroError) as ei:
        sgh.Batch(ps)
    assert ei.value.code == sgh.FIERRO_EINVAL


@pytest.mark.parametrize("mode", ["fma", "exact"])
@pytest.mark.parametrize("shape", [(32, 64, 32, 0, 0), (64, 512, 64, 2, 0), (128, 256, 128, 1, 0),
                                   (128, 256, 128, 0, 1), (128, 256, 32, 0, 1)])
def test_launch_shape_does_not_change_results(lib_built, shape, mode):
    """Every launch shape (threads per block of the three passes, persistent grid
    or not, the fused stage: one cooperative launch per RK stage with grid
    barriers) gives the default shape's results bit for bit, in both modes."""
    from fierro_gb300 import sgh
    ps = _problems()
    states = [sgh.setup(p) for p in ps]
    out = {}
    for sh in ((128, 256, 128, 0, 0), shape):
        with sgh.Batch(ps, fp_mode=sgh.FP_FMA if mode == "fma" else sgh.FP_EXACT) as b:
            b.set_shape(*sh)
            assert b.shape() == sh
            for i, st in enumerate(states):
                b.set_state(i, st)
            b.run(30)
            out[sh] = ([sgh.compared_fields(b.get_state(i)) for i in range(len(ps))],
                       [b.time(i) for i in range(len(ps))])
    ref, got = out[(128, 256, 128, 0, 0)], out[shape]
    assert ref[1] == got[1]
    for i in range(len(ps)):
        assert_bitwise(got[0][i], ref[0][i], FIELDS, label="instance %d shape %s" % (i, shape))


def test_autotune_keeps_the_uploaded_state_and_the_results(lib_built):
    """fierro_batch_autotune times the candidate shapes from the uploaded state,
    restores it and keeps the fastest; the run that follows equals a run with the
    default shape bit for bit, and the log holds every timed candidate."""
    from fierro_gb300 import sgh
    ps = _problems()
    states = [sgh.setup(p) for p in ps]
    with sgh.Batch(ps) as b:
        for i, st in enumerate(states):
            b.set_state(i, st)
        b.run(20)
        ref = [sgh.compared_fields(b.get_state(i)) for i in range(len(ps))]
    with sgh.Batch(ps) as b:
        for i, st in enumerate(states):
            b.set_state(i, st)
        chosen, log = b.autotune(cycles=2)
        assert len(log) >= 10 and all(ms > 0 for _, ms in log)
        assert any(sh[4] == 1 for sh, _ in log)  # the fused stage was timed
        assert chosen == min(log, key=lambda r: r[1])[0] and b.shape() == chosen
        b.run(20)
        for i in range(len(ps)):
            assert_bitwise(sgh.compared_fields(b.get_state(i)), ref[i], FIELDS, label="instance %d" % i)
        with pytest.raises(sgh.FierroError):
            b.autotune(cycles=2)  # after the first run
        with pytest.raises(sgh.FierroError):
            b.set_shape(64, 256, 128, 0)
    with sgh.Batch(ps[:1]) as b:
        with pytest.raises(sgh.FierroError):
            b.set_shape(48, 256, 128, 0)  # not a power of two
        with pytest.raises(sgh.FierroError):
            b.set_shape(128, 256, 128, 0, 2)  # fused_stage is 0 or 1
        with pytest.raises(sgh.FierroError):
            b.autotune(cycles=2)  # no state yet


def test_fused_stage_barrier_wait_is_bounded(lib_built, monkeypatch):
    """The fused stage's grid barrier waits a bounded time.  Launched with four
    times the blocks that can be resident and without the cooperative attribute
    (FIERRO_FUSED_OVERSUBSCRIBE, a host-side test hook), the barrier cannot
    complete: every block's wait runs out, the launch ends, and
    fierro_batch_run returns FIERRO_ETIMEDOUT.  A batch made without the hook
    then runs the fused stage normally."""
    import time
    from fierro_gb300 import sgh
    ps = _problems()[:2]
    states = [sgh.setup(p) for p in ps]
    monkeypatch.setenv("FIERRO_FUSED_OVERSUBSCRIBE", "4")
    with sgh.Batch(ps) as b:
        b.set_shape(128, 256, 128, 0, 1)
        for i, st in enumerate(states):
            b.set_state(i, st)
        t0 = time.perf_counter()
        with pytest.raises(sgh.FierroError) as ei:
            b.run(1)
        assert ei.value.code == sgh.FIERRO_ETIMEDOUT
        assert time.perf_counter() - t0 < 120.0
    monkeypatch.delenv("FIERRO_FUSED_OVERSUBSCRIBE")
    with sgh.Batch(ps) as b:
        b.set_shape(128, 256, 128, 0, 1)
        for i, st in enumerate(states):
            b.set_state(i, st)
        b.run(3)
