"""Failure detection, provoked from the host (no GPU fault): each check the kernels make
turns into a status and a readable message, nothing is written out of bounds, and the
context goes on stepping after the state is reset.

* more colloids reaching one cell than the fluid-to-colloid table holds -> MPCD_ERR_CAPACITY
* a cell holding more particles than max_per_cell allows -> MPCD_ERR_CAPACITY
* a fluid velocity beyond the range of the exact cell sums -> MPCD_ERR_RANGE
* a weight copy of the closure's network kernel that never arrives: its bounded waits give
  up, the step reports it and leaves the colloid state as it was
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _kw(**over):
    m = 335.1
    kw = dict(n_sub=10, ndt=0.1, kbt=1.0, kbt1=1.0, mass_fl=1.0, mass_colloid=m, sig_colloid=4.0, eps=1.0,
              sigma=4.0, I_colloid=0.4 * m * 4.0, v0=0.01, theta_deg=90.0, Dr=0.001, seed=17)
    kw.update(over)
    return kw


def _fresh(L=10, dens=10, Nc=3, **over):
    import brownian_gb300 as bg
    sim = bg.Simulation(L, L ** 3 * dens, Nc, **_kw(**over))
    sim.initialize(bg.INIT_REFERENCE)
    return sim, sim.get_state()


def _recovers(sim, good):
    """after the failure: the good state back, the set-up again, and steps that succeed"""
    sim.set_state(*[good[k] for k in ("pos_fl", "vel_fl", "pos_colloid", "vel_colloid", "ang_vel_colloid", "ra")])
    sim.setup()
    sim.step(2)
    d = sim.diag()
    assert np.isfinite(d["ke_fluid"]) and abs(d["temperature_fluid"] - 1.0) < 0.2


def test_cell_table_overflow_is_reported():
    import brownian_gb300 as bg
    m = 10 * 4.0 / 3.0 * np.pi * 0.4 ** 3
    sim, good = _fresh(Nc=18, v0=0.0, sig_colloid=0.8, sigma=0.8, mass_colloid=m, I_colloid=0.4 * m * 0.16)
    bad = {k: v.copy() for k, v in good.items()}
    # 18 small spheres around one point: every one reaches the same cells (16 per cell fit)
    rng = np.random.default_rng(0)
    bad["pos_colloid"] = 5.5 + rng.uniform(-0.05, 0.05, (18, 3))
    sim.set_state(*[bad[k] for k in ("pos_fl", "vel_fl", "pos_colloid", "vel_colloid", "ang_vel_colloid", "ra")])
    with pytest.raises(bg.MPCDError) as e:
        sim.setup()
    assert e.value.code == bg.ERR_CAPACITY
    assert "table" in str(e.value)
    _recovers(sim, good)
    sim.close()


def test_cell_occupancy_overflow_is_reported():
    import brownian_gb300 as bg
    sim, good = _fresh(Nc=2, max_per_cell=40)
    bad = {k: v.copy() for k, v in good.items()}
    bad["pos_fl"][:50] = [7.5, 7.5, 7.5]  # 50 particles at one point: in one cell whatever the grid shift
    sim.set_state(*[bad[k] for k in ("pos_fl", "vel_fl", "pos_colloid", "vel_colloid", "ang_vel_colloid", "ra")])
    sim.setup()
    with pytest.raises(bg.MPCDError) as e:
        sim.step(1)
    assert e.value.code == bg.ERR_CAPACITY
    assert "max_per_cell" in str(e.value)
    _recovers(sim, good)
    sim.close()


def test_velocity_out_of_range_is_reported():
    import brownian_gb300 as bg
    sim, good = _fresh(Nc=2)
    bad = {k: v.copy() for k, v in good.items()}
    bad["vel_fl"][123] = [500.0, 0.0, 0.0]  # far beyond 24 thermal speeds
    sim.set_state(*[bad[k] for k in ("pos_fl", "vel_fl", "pos_colloid", "vel_colloid", "ang_vel_colloid", "ra")])
    with pytest.raises(bg.MPCDError) as e:
        sim.setup()
    assert e.value.code == bg.ERR_RANGE
    assert "vmax" in str(e.value)
    _recovers(sim, good)
    sim.close()


def test_surrogate_weight_copy_that_never_arrives():
    import brownian_gb300 as bg
    from brownian_gb300 import closure
    L, nc = 30, 64
    M = bg.displaced_mass(2.0, 10)
    p = bg.make_params(L, 1, nc, n_sub=10, mass_colloid=M, sig_colloid=4.0, sigma=4.0, I_colloid=0.4 * M * 4.0,
                       v0=0.05, theta_deg=90.0, Dr=0.001, seed=9)
    net = closure.Network(max_batch=1024)
    net.set_normalisation(np.zeros(81), np.ones(81), np.zeros(6), np.full(6, 0.05))
    net.set_params(np.zeros(net.n_params))
    sur = closure.Surrogate(p, net)
    rng = np.random.default_rng(3)
    pos = np.stack(np.meshgrid(*[np.arange(4) * 7.0 + 2.0] * 3), -1).reshape(-1, 3)[:nc]
    vel = rng.normal(0, 0.05, (nc, 3))
    w = rng.normal(0, 0.02, (nc, 3))
    ra = rng.normal(0, 1, (nc, 3))
    ra /= np.linalg.norm(ra, axis=1, keepdims=True)
    sur.set_state(pos, vel, w, ra)
    sur.step(2)
    before = sur.get_state()
    sur.set_fault(10)
    with pytest.raises(bg.MPCDError) as e:
        sur.step(3)
    assert e.value.code == bg.ERR_CUDA
    assert "did not arrive" in str(e.value)
    after = sur.get_state()
    for k in before:
        assert np.array_equal(before[k], after[k]), k  # the failing steps left the state alone
    with pytest.raises(bg.MPCDError):
        sur.set_fault(3)  # a chunk the producer loop does not issue
    sur.set_fault(-1)
    sur.step(2)
    st = sur.get_state()
    assert all(np.all(np.isfinite(v)) for v in st.values())
    assert not np.array_equal(st["pos_colloid"], before["pos_colloid"])
    sur.close()
    net.close()


def test_closure_training_product_that_never_completes():
    """The tcgen05 layer products of training wait for their results with a bound; with the
    test hook they issue nothing, every wait runs out, and the call fails with its status and
    message; cleared, the next call runs."""
    import torch

    import brownian_gb300 as bg
    from brownian_gb300 import closure
    rng = np.random.default_rng(4)
    net = closure.Network(max_batch=512, seed=4)
    net.set_normalisation(np.zeros(81), np.ones(81), np.zeros(6), np.ones(6))
    x = torch.from_numpy(rng.normal(0, 1, (300, 81)).astype(np.float32)).cuda()
    y = torch.from_numpy(rng.normal(0, 1, (300, 6)).astype(np.float32)).cuda()
    l0, g0 = net.grad(x.data_ptr(), y.data_ptr(), 300)
    net.set_fault(True)
    with pytest.raises(bg.MPCDError) as e:
        net.grad(x.data_ptr(), y.data_ptr(), 300)
    assert e.value.code == bg.ERR_CUDA
    assert "time limit" in str(e.value)
    net.set_fault(False)
    l1, g1 = net.grad(x.data_ptr(), y.data_ptr(), 300)
    assert np.isfinite(l1) and abs(l1 - l0) <= 1e-6 * abs(l0)
    assert np.array_equal(np.isfinite(g1), np.ones_like(g1, dtype=bool))
    net.close()
