"""Discrete adjoint of the SGH cycle loop (fierro_adj_forward / fierro_adj_backward).

The gradient of J = sum_e M_e (rho_e - rho_target_e)^2 with respect to the
per-element initial sie and gamma is checked against central finite differences
(step 1e-6 along seeded directions, relative tolerance 1e-6):
  * of the GPU forward (the plain cycle graphs), and
  * of the CPU oracle's forward (the reference's algorithm, pinned bit for bit
    to the reference's own build).
The replay that feeds the reverse pass must reproduce the forward bit for bit
(recomputed corner forces and time steps), and the gradient must not depend on
the checkpoint interval.  The deck is a jittered Sedov mesh: on the perfectly
symmetric uniform mesh the CFL minimum and the limiter's neighbour minimum are
exact ties between mirror-image elements, where J has no derivative."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-6


def _case(n=12, cycles=100, k=13, jitter=0.1):
    from fierro_gb300 import adjoint, problems
    target = adjoint.sedov_target(n, cycles, jitter=jitter, seed=7)
    p = problems.sedov(n, jitter=jitter, seed=7, cycles=cycles)
    return adjoint.DensityMismatch(p, target, cycles, ckpt_every=k)


def _directional(sb, gb, d_sie, d_g):
    return float(np.dot(sb, d_sie) + np.sum(gb) * d_g)


def test_replay_is_bit_identical(lib_built):
    dm = _case()
    J = dm.forward()
    dm.solver.adj_verify(True)
    seed = 2.0 * dm.mass * (dm.last_den - dm.target)
    dm.solver.adj_backward(den=seed)
    st = dm.solver.adj_stats()
    assert st["force_mismatches"] == 0 and st["status"] == 0, st
    assert st["cycles"] == 100 and st["segments"] == 8
    # both time-step regimes are reversed: growth-capped early cycles, CFL-limited later
    assert st["dt_cfl_cycles"] > 0 and st["dt_growth_cycles"] > 0, st
    assert J > 0


def test_gradient_matches_gpu_finite_differences(lib_built):
    dm = _case()
    J, sb, gb, vb = dm.gradient()
    for d_sie, d_g in dm.directions(4, seed=1):
        ad = _directional(sb, gb, d_sie, d_g)
        fd = dm.fd(d_sie, d_g)
        assert abs(fd - ad) <= TOL * abs(fd), (fd, ad, abs(fd - ad) / abs(fd))
    # each parameter block alone
    d_sie, _ = dm.directions(1, seed=2)[0]
    assert abs(dm.fd(d_sie, 0.0) - np.dot(sb, d_sie)) <= TOL * abs(np.dot(sb, d_sie))
    assert abs(dm.fd(0 * d_sie, 1.0) - np.sum(gb)) <= TOL * abs(np.sum(gb))


def test_gradient_matches_oracle_finite_differences(lib_built, oracle_built):
    dm = _case()
    J, sb, gb, vb = dm.gradient()
    from oracle import orc
    f = orc.density_mismatch_forward(dm)
    assert abs(f(dm.sie0, dm.gamma0) - J) <= 1e-9 * J
    for d_sie, d_g in dm.directions(3, seed=3):
        ad = _directional(sb, gb, d_sie, d_g)
        fd = dm.fd(d_sie, d_g, forward=f)
        assert abs(fd - ad) <= TOL * abs(fd), (fd, ad, abs(fd - ad) / abs(fd))


def test_checkpoint_interval_does_not_change_the_gradient(lib_built):
    dm = _case(cycles=24)
    ref = None
    for k in (1, 5, 24, 100):
        dm.ckpt_every = k
        J, sb, gb, vb = dm.gradient()
        if ref is None:
            ref = (sb, gb, vb)
        else:
            assert np.array_equal(sb, ref[0]) and np.array_equal(gb, ref[1]) and np.array_equal(vb, ref[2]), k


def test_velocity_gradient_noh(lib_built):
    """d J / d initial node velocity on a jittered Noh deck, against central
    differences of the GPU forward along seeded velocity directions (the held
    components at the symmetry planes stay zero)."""
    from fierro_gb300 import adjoint, problems, sgh
    cycles = 30
    p = problems.noh(8, jitter=0.1, seed=5, cycles=cycles)
    st0 = sgh.setup(p)
    with sgh.SGHSolver(p) as s:
        s.set_state(st0)
        s.run(cycles)
        target = s.get_state()["elem_den"] * 0.9
    dm = adjoint.DensityMismatch(p, target, cycles, ckpt_every=8)
    J, sb, gb, vb = dm.gradient()
    rng = np.random.default_rng(4)
    v0 = dm.state0["node_vel"][1].copy()
    held = (v0 == 0.0)  # symmetry planes and the origin
    for _ in range(2):
        dv = rng.uniform(-1.0, 1.0, v0.shape)
        dv[held] = 0.0
        ad = float(np.sum(vb * dv))
        vals = []
        for sgn in (1.0, -1.0):
            st = {k: a.copy() for k, a in dm.state0.items()}
            st["node_vel"][:] = (v0 + sgn * 1e-6 * dv)[None]
            dm.solver.set_state(st)
            dm.solver.adj_forward(None, None, cycles, 8)
            vals.append(dm.value(dm.solver.get_state()["elem_den"]))
        fd = (vals[0] - vals[1]) / 2e-6
        assert abs(fd - ad) <= TOL * abs(fd), (fd, ad)


def test_autograd_function(lib_built):
    torch = pytest.importorskip("torch")
    from fierro_gb300 import adjoint
    dm = _case(cycles=20, k=6)
    sie0 = torch.tensor(dm.sie0, requires_grad=True)
    gamma = torch.tensor(float(dm.gamma0[0]), dtype=torch.float64, requires_grad=True)
    den, pres, sie = adjoint.SGHFunction.apply(sie0, gamma, dm.solver, dm.state0, dm.cycles, dm.ckpt_every)
    J = torch.sum(torch.from_numpy(dm.mass) * (den - torch.from_numpy(dm.target)) ** 2)
    J.backward()
    J2, sb, gb, vb = dm.gradient()
    assert abs(float(J) - J2) <= 1e-14 * J2
    assert np.array_equal(sie0.grad.numpy(), sb)
    assert abs(float(gamma.grad) - float(np.sum(gb))) <= 1e-12 * abs(float(np.sum(gb)))


def test_adjoint_rejects_fma_mode_and_bad_calls(lib_built):
    from fierro_gb300 import problems, sgh
    p = problems.sedov(4, cycles=5)
    st = sgh.setup(p)
    with sgh.SGHSolver(p, fp_mode=sgh.FP_FMA) as s:
        s.set_state(st)
        with pytest.raises(sgh.FierroError) as ei:
            s.adj_forward(None, None, 5, 2)
        assert ei.value.code == sgh.FIERRO_ENOTSUP
    with sgh.SGHSolver(p) as s:
        s.set_state(st)
        with pytest.raises(sgh.FierroError):
            s.adj_backward(den=np.ones(p.mesh.num_elems))
        s.adj_forward(None, None, 5, 2)
        s.run(1)  # the state moved on: backward must refuse
        with pytest.raises(sgh.FierroError):
            s.adj_backward(den=np.ones(p.mesh.num_elems))


def test_frozen_forward_reproduces_the_recorded_run(lib_built):
    """The frozen-branch forward on the recorded parameters is the recorded run
    bit for bit (state, time, J), and recording changes neither the forward nor
    the gradient."""
    from fierro_gb300 import sgh
    dm = _case()
    J, sb, gb, vb = dm.gradient()
    want = dm.solver.get_state()
    t_want = dm.solver.time()
    Jr, sbr, gbr, vbr = dm.gradient_frozen()
    assert Jr == J and np.array_equal(sbr, sb) and np.array_equal(gbr, gb) and np.array_equal(vbr, vb)
    Jf = dm.forward()
    got = dm.solver.get_state()
    assert Jf == J
    g, w = sgh.compared_fields(got), sgh.compared_fields(want)
    for k in w:
        assert np.array_equal(g[k], w[k]), k
    assert dm.solver.time() == t_want
    # no backward after a frozen forward, and a cycle count other than the recorded one is refused
    with pytest.raises(sgh.FierroError):
        dm.solver.adj_backward(den=np.ones(dm.problem.mesh.num_elems))
    dm.solver.set_state(dm.state0)
    with pytest.raises(sgh.FierroError) as ei:
        dm.solver.adj_forward(None, None, dm.cycles + 1, dm.ckpt_every)
    assert ei.value.code == sgh.FIERRO_EINVAL
    dm.unfreeze()
    assert dm.forward() == J


def test_gradient_matches_frozen_branch_differences(lib_built):
    """Central differences (step 1e-6) of the frozen-branch forward against the
    adjoint, 12^3 jittered Sedov, 100 cycles, four seeded directions."""
    dm = _case()
    J, sb, gb, vb = dm.gradient_frozen()
    for d_sie, d_g in dm.directions(4, seed=11):
        ad = _directional(sb, gb, d_sie, d_g)
        fd = dm.fd(d_sie, d_g, h=1e-6)
        assert abs(fd - ad) <= TOL * abs(fd), (fd, ad, abs(fd - ad) / abs(fd))
    dm.unfreeze()



def test_config5_gradient_within_1e6_of_frozen_branch_differences(lib_built):
    """The discrete-adjoint configuration at its own size: jittered Sedov 64^3
    (262,144 elements), 400 RK2 cycles, checkpoint every 20 cycles, J against
    the origin-energy-0.3 target.  The gradient in sie0 and gamma against central
    differences at step 1e-6 of the frozen-branch forward along four of the
    seeded directions (relative sie0 perturbations U(-1,1) and a gamma shift
    U(-1,1)), each within 1e-6 relative with the five-point stencil.  The
    frozen forward is smooth (J minus its tangent is a clean quadratic along a
    direction), so the three-point stencil's error is its truncation term
    h^2 J3 / 6, a few 1e-6 at this step on this deck: it must fall by ~4x when
    the step halves, the signature of truncation rather than of a wrong
    derivative."""
    from fierro_gb300 import adjoint, problems
    n, cycles = 64, 400
    target = adjoint.sedov_target(n, cycles, jitter=0.1, seed=7)
    dm = adjoint.DensityMismatch(problems.sedov(n, jitter=0.1, seed=7, cycles=cycles), target, cycles,
                                 ckpt_every=20)
    J, sb, gb, vb = dm.gradient_frozen()
    assert J > 0
    dirs = dm.directions(16, seed=2024)
    for d_sie, d_g in dirs[:4]:
        ad = _directional(sb, gb, d_sie, d_g)
        fd3, fd5 = dm.fd5(d_sie, d_g, h=1e-6)
        assert abs(fd5 - ad) <= TOL * abs(fd5), (fd5, ad, abs(fd5 - ad) / abs(fd5))
    d_sie, d_g = dirs[0]
    ad = _directional(sb, gb, d_sie, d_g)
    e1 = abs(dm.fd(d_sie, d_g, h=1e-6) - ad)
    e2 = abs(dm.fd(d_sie, d_g, h=5e-7) - ad)
    assert 3.0 <= e1 / e2 <= 5.0, (e1, e2)
    dm.unfreeze()
    dm.solver.close()
