"""Graphics dumps (write_outputs, outputs.cpp:10-506) written by the handle's
writer thread equal, file for file and byte for byte, the files the reference's
own outputs.cpp writes for the same deck (oracle/_ref/fierro_ref_out): EnSight
Gold case / geometry / variable files and the element state text, at the
reference's write events (t = 0, every graphics_cyc_ival cycles, graphics_time,
time_final)."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _tree(root):
    out = {}
    for d, _, files in os.walk(root):
        for f in files:
            path = os.path.join(d, f)
            out[os.path.relpath(path, root)] = open(path, "rb").read()
    return out


def _compare(prob, cycles, tmp_path, slots=3):
    from oracle import orc
    from fierro_gb300 import sgh
    if not orc.reference_available("fierro_ref_out"):
        pytest.skip("reference output build unavailable")
    ref_dir = tmp_path / "ref"
    ours = tmp_path / "ours"
    ref_dir.mkdir()
    orc.run_reference(prob, cycles=cycles, kind="fierro_ref_out", cwd=str(ref_dir))
    st = sgh.setup(prob)
    with sgh.SGHSolver(prob) as s:
        s.set_output(str(ours), ensight=True, state=True, slots=slots)
        s.set_state(st)
        s.run(cycles)
        n = s.flush_output()
    a, b = _tree(str(ref_dir)), _tree(str(ours))
    assert sorted(a) == sorted(b)
    bad = [k for k in a if a[k] != b[k]]
    assert not bad, bad[:5]
    return n


def test_cycle_interval_dumps_match_reference(lib_built, oracle_built, tmp_path):
    from fierro_gb300 import problems
    p = problems.sedov(8, jitter=0.1, seed=3, permute=True, cycles=20)
    p.params.graphics_cyc_ival = 7
    assert _compare(p, 20, tmp_path) == 3


def test_time_interval_and_final_dumps_match_reference(lib_built, oracle_built, tmp_path):
    from fierro_gb300 import problems
    p = problems.noh(8, jitter=0.05, seed=4, permute=True, cycles=2000)
    p.params.graphics_dt_ival = 0.01
    p.params.time_final = 0.035
    # ring smaller than the number of dumps: the run waits for the writer
    assert _compare(p, 2000, tmp_path, slots=2) >= 4


def test_output_off_and_restart_numbering(lib_built, tmp_path):
    from fierro_gb300 import problems, sgh
    p = problems.sedov(6, cycles=10)
    p.params.graphics_cyc_ival = 5
    st = sgh.setup(p)
    with sgh.SGHSolver(p) as s:
        s.set_output(str(tmp_path / "o"), ensight=False, state=True)
        s.set_state(st)
        s.run(10)
        assert s.flush_output() == 3  # t = 0, cycles 4 and 9
        s.set_state(st)               # a new series
        s.run(4)
        assert s.flush_output() == 1
        s.set_output(None)
        s.run(5)
        assert s.flush_output() == 0
