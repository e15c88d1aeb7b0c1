"""Checkpoint / restart: a loop stopped at a cycle boundary, written out and
loaded into a fresh handle continues bit for bit as the uninterrupted loop does
(state, both bins, corner forces, divergence, time, dt, cycle count, energies),
on hex and 2D-RZ meshes, with and without a strength model and in both
topology builders; a checkpoint of another problem is refused."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _problems():
    from fierro_gb300 import problems
    return {
        "sedov10_jp": lambda: problems.sedov(10, jitter=0.1, seed=3, permute=True, cycles=60),
        "sedov8_hypo": lambda: problems.with_strength(problems.sedov(8, cycles=60), "hypo", 10.0),
        "noh_rz12_jp": lambda: problems.noh_rz(12, jitter=0.1, seed=5, permute=True, cycles=60),
    }


def _snapshot(s):
    out = s.get_state()
    snap = {k: v.copy() for k, v in out.items()}
    snap["time"] = np.array(s.time())
    snap["energy"] = np.array(s.energy())
    return snap


@pytest.mark.parametrize("case", ["sedov10_jp", "sedov8_hypo", "noh_rz12_jp"])
@pytest.mark.parametrize("staged", [False, True])
def test_restart_continues_bit_for_bit(lib_built, tmp_path, monkeypatch, case, staged):
    from fierro_gb300 import sgh
    if staged:
        monkeypatch.setenv("FIERRO_STAGED_TRANSFERS", "1")
    prob = _problems()[case]()
    st = sgh.setup(prob)
    path = str(tmp_path / "loop.ckpt")
    with sgh.SGHSolver(prob) as a:
        a.set_state(st)
        a.run(17)
        a.checkpoint(path)
        a.run(23)
        want = _snapshot(a)
    with sgh.SGHSolver(prob) as b:
        b.restart(path)
        assert b.time()[3] == 17
        b.run(23)
        got = _snapshot(b)
    for k in want:
        assert np.array_equal(got[k], want[k]), k


def test_restart_refuses_other_problems(lib_built, tmp_path):
    from fierro_gb300 import problems, sgh
    p1 = problems.sedov(8, cycles=10)
    path = str(tmp_path / "a.ckpt")
    with sgh.SGHSolver(p1) as a:
        a.set_state(sgh.setup(p1))
        a.run(3)
        a.checkpoint(path)
        a.run_stages(1)
        with pytest.raises(sgh.FierroError) as ei:
            a.checkpoint(str(tmp_path / "mid.ckpt"))
        assert ei.value.code == sgh.FIERRO_EINVAL
    for other in (problems.sedov(9, cycles=10), problems.sedov(8, jitter=0.05, seed=1, cycles=10)):
        with sgh.SGHSolver(other) as b:
            with pytest.raises(sgh.FierroError) as ei:
                b.restart(path)
            assert ei.value.code == sgh.FIERRO_EINVAL
    (tmp_path / "junk.ckpt").write_bytes(b"not a checkpoint")
    with sgh.SGHSolver(p1) as c:
        with pytest.raises(sgh.FierroError) as ei:
            c.restart(str(tmp_path / "junk.ckpt"))
        assert ei.value.code == sgh.FIERRO_EINVAL


@pytest.mark.parametrize("case", ["sedov10_jp", "sedov8_hypo"])
def test_refused_restart_leaves_the_handle_runnable(lib_built, tmp_path, case):
    """A checkpoint that is refused (another deck, a corrupt state-variable count,
    a truncated file, trailing bytes) changes nothing in the handle: its state,
    time and energies stay as they were and the loop continues bit for bit as an
    uninterrupted one."""
    import struct
    from fierro_gb300 import problems, sgh
    prob = _problems()[case]()
    st = sgh.setup(prob)
    good = tmp_path / "good.ckpt"
    with sgh.SGHSolver(prob) as w:
        w.set_state(st)
        w.run(9)
        w.checkpoint(str(good))
    raw = good.read_bytes()
    bad = {}
    nsv_off = 8 + 4 + 4 + 8 + 8  # magic, version, dims, nn, ne
    for name, nsv in (("huge_nsv", 1 << 40), ("negative_nsv", -3), ("other_nsv", 7)):
        bad[name] = raw[:nsv_off] + struct.pack("<q", nsv) + raw[nsv_off + 8:]
    bad["truncated"] = raw[:len(raw) - 8]
    bad["trailing"] = raw + b"\0"
    other = problems.sedov(10, jitter=0.1, seed=4, permute=True, cycles=60)
    p_other = tmp_path / "other.ckpt"
    if case == "sedov10_jp":
        with sgh.SGHSolver(other) as o:
            o.set_state(sgh.setup(other))
            o.run(2)
            o.checkpoint(str(p_other))
        bad["other_deck"] = p_other.read_bytes()
    with sgh.SGHSolver(prob) as ref:
        ref.set_state(st)
        ref.run(5 + 11)
        want = _snapshot(ref)
    with sgh.SGHSolver(prob) as a:
        a.set_state(st)
        a.run(5)
        before = _snapshot(a)
        for name, data in bad.items():
            path = tmp_path / (name + ".ckpt")
            path.write_bytes(data)
            with pytest.raises(sgh.FierroError) as ei:
                a.restart(str(path))
            assert ei.value.code == sgh.FIERRO_EINVAL, name
            now = _snapshot(a)
            for k in before:
                assert np.array_equal(now[k], before[k]), (name, k)
        a.run(11)
        got = _snapshot(a)
    for k in want:
        assert np.array_equal(got[k], want[k]), k
