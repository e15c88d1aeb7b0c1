"""One handle per host thread: handles own their stream, graphs and device
memory and share no globals, so two handles driven from two threads at once
give the results each gives alone, and the error text is per thread."""
import threading

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _decks():
    from fierro_gb300 import problems
    return [problems.sedov(10, jitter=0.1, seed=3, permute=True, cycles=40),
            problems.noh(12, jitter=0.05, seed=4, permute=True, cycles=40)]


def _run(prob, out, key, mode):
    from fierro_gb300 import sgh
    st = sgh.setup(prob)
    with sgh.SGHSolver(prob, fp_mode=mode) as s:
        s.set_state(st)
        for _ in range(4):
            s.run(10)
        out[key] = (s.get_state(), s.time()[0])


@pytest.mark.parametrize("mode", [0, 1])
def test_two_handles_two_threads(lib_built, mode):
    decks = _decks()
    alone = {}
    for i, p in enumerate(decks):
        _run(p, alone, i, mode)
    together = {}
    errors = []

    def worker(i):
        try:
            _run(decks[i], together, i, mode)
        except Exception as exc:  # reported by the main thread
            errors.append(exc)

    threads = [threading.Thread(target=worker, args=(i,)) for i in range(len(decks))]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    assert not errors, errors
    for i in range(len(decks)):
        a, b = alone[i], together[i]
        assert a[1] == b[1]
        for k in ("node_coords", "node_vel", "elem_sie", "elem_den", "elem_pres", "elem_sspd", "elem_vol"):
            assert np.array_equal(a[0][k], b[0][k]), (i, k)


def test_error_text_is_per_thread(lib_built):
    """A failing call on one thread leaves another thread's last error alone."""
    from fierro_gb300 import problems, sgh
    prob = problems.sedov(6, cycles=5)
    seen = {}
    go = threading.Event()

    def failing():
        with sgh.SGHSolver(prob) as s:
            rc = sgh.lib().fierro_sgh_run(s.h, 1, None)  # no state uploaded yet
            seen["fail"] = (rc, sgh.lib().fierro_last_error().decode())
        go.set()

    def succeeding():
        with sgh.SGHSolver(prob) as s:
            s.set_state(sgh.setup(prob))
            go.wait(timeout=60)
            s.run(2)
            seen["ok"] = sgh.lib().fierro_last_error().decode()

    ta, tb = threading.Thread(target=failing), threading.Thread(target=succeeding)
    tb.start()
    ta.start()
    ta.join()
    tb.join()
    assert seen["fail"][0] == sgh.FIERRO_EINVAL and "set_state" in seen["fail"][1]
    assert seen["ok"] == ""
