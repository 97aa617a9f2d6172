"""Device trajectories: frames recorded on the GPU against the host copies of the same
states, and the GPU statistics against numpy (closure.msd / closure.autocorr)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

KW = dict(n_sub=10, ndt=0.1, kbt=1.0, kbt1=1.0, mass_fl=1.0, mass_colloid=335.1, sig_colloid=4.0, eps=1.0,
          sigma=4.0, I_colloid=0.4 * 335.1 * 4.0, v0=0.05, theta_deg=90.0, Dr=0.001, seed=5)


def _rel(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def test_traj_from_simulation(tmp_path):
    import brownian_gb300 as bg
    from brownian_gb300 import closure
    L, Nc, steps = 16, 6, 40
    sim = bg.Simulation(L, L ** 3 * 10, Nc, **KW)
    sim.initialize(bg.INIT_PHYSICAL)
    sim.setup()
    tr = bg.Trajectory(Nc, steps + 1, L)
    X, V, R = [], [], []
    for s in range(steps + 1):
        if s:
            sim.step(1)
        tr.record(sim)
        c = sim.get_colloids()
        X.append(c["pos_colloid"]); V.append(c["vel_colloid"]); R.append(c["ra"])
    X, V, R = np.array(X), np.array(V), np.array(R)
    U = closure.unwrap(X, float(L))
    gU, gV, gR = tr.read()
    assert tr.frames == steps + 1
    # (the device adds each increment to the previous frame, closure.unwrap adds the summed
    # increments to the first: the same numbers to rounding)
    assert _rel(gU, U) < 1e-13 and np.array_equal(gV, V) and np.array_equal(gR, R)
    lags = dict(msd_lags=(1, 2, 5, 10, 40, 41), vacf_lags=(0, 1, 3, 10), oacf_lags=(0, 5, 20))
    st = tr.analyse(**lags)
    assert _rel(st["msd"][:5], closure.msd(gU, lags["msd_lags"][:5])) < 1e-12
    assert np.isnan(st["msd"][5])  # no two frames 41 apart
    assert _rel(st["vacf"], closure.autocorr(V, lags["vacf_lags"])) < 1e-12
    assert _rel(st["oacf"], closure.autocorr(R, lags["oacf_lags"])) < 1e-12
    p = tmp_path / "sim.bgbtraj"
    tr.write(p, dt_frame=0.1)
    d = bg.read_trajectory(p)
    assert np.array_equal(d["pos"], gU) and np.array_equal(d["vel"], gV) and np.array_equal(d["ra"], gR)
    assert np.array_equal(d["box"], [L, L, L]) and d["dt_frame"] == 0.1
    with pytest.raises(bg.MPCDError):  # full
        tr.record(sim)
    tr.close()
    sim.close()


def test_traj_from_surrogate():
    import brownian_gb300 as bg
    from brownian_gb300 import closure
    Nc, L = 8, 20
    net = closure.Network(max_batch=1024)
    net.set_normalisation(np.zeros(81), np.ones(81), np.zeros(6), np.full(6, 0.05))
    net.set_params(np.zeros(net.n_params))
    p = bg.make_params(L, 1, Nc, n_sub=10, mass_colloid=335.1, sig_colloid=4.0, sigma=4.0,
                       I_colloid=0.4 * 335.1 * 4.0, v0=0.05, theta_deg=90.0, Dr=0.001, seed=2, precision=bg.FP32C)
    sur = closure.Surrogate(p, net)
    g = np.stack(np.meshgrid(*[np.arange(0, L - 4, 9.0)] * 3), -1).reshape(-1, 3)[:Nc] + 2
    rng = np.random.default_rng(0)
    sur.set_state(g, rng.normal(0, 0.05, (Nc, 3)), np.zeros((Nc, 3)), np.tile([1.0, 0, 0], (Nc, 1)))
    tr = bg.Trajectory(Nc, 30, L)
    X, V, R = [], [], []
    for s in range(30):
        if s:
            sur.step(1)
        tr.record(sur)
        st = sur.get_state()
        X.append(st["pos_colloid"]); V.append(st["vel_colloid"]); R.append(st["ra"])
    gU, gV, gR = tr.read()
    assert _rel(gU, closure.unwrap(np.array(X), float(L))) < 1e-13
    assert np.array_equal(gV, np.array(V)) and np.array_equal(gR, np.array(R))
    tr.close()
    sur.close()
    net.close()
