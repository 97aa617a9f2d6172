"""Colloid-only dynamics with the closure: the GPU feature kernel gives the
network inputs of brownian_gb300.closure.features, and the step runs."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _params(L, nc):
    import brownian_gb300 as bg
    M = bg.displaced_mass(2.0, 10)
    return bg.make_params(L, 1, nc, n_sub=10, mass_colloid=M, sig_colloid=4.0, sigma=4.0, I_colloid=0.4 * M * 4.0,
                          v0=0.05, theta_deg=90.0, Dr=0.001, seed=9)


def _state(L, nc, seed):
    rng = np.random.default_rng(seed)
    pos = []
    while len(pos) < nc:  # random sequential placement with centre distance >= 4.2
        x = rng.uniform(0, L, 3)
        if all(np.linalg.norm((x - y) - L * np.round((x - y) / L)) >= 4.2 for y in pos):
            pos.append(x)
    pos = np.array(pos)
    vel = rng.normal(0, 0.05, (nc, 3))
    w = rng.normal(0, 0.02, (nc, 3))
    ra = rng.normal(0, 1, (nc, 3))
    ra /= np.linalg.norm(ra, axis=1, keepdims=True)
    return pos, vel, w, ra


def test_feature_kernel_matches_numpy_features():
    from brownian_gb300 import closure
    L, nc = 30, 150
    net = closure.Network(max_batch=1024)
    sur = closure.Surrogate(_params(L, nc), net)
    pos, vel, w, ra = _state(L, nc, 1)
    sur.set_state(pos, vel, w, ra)
    got = sur.features()
    st = sur.get_state()  # positions as the GPU holds them (FP32, wrapped)
    ref = closure.features(st, L, 2.0)
    assert np.allclose(got, ref, atol=2e-5), np.max(np.abs(got - ref))
    sur.close()
    net.close()


def test_surrogate_steps_stay_finite_and_move():
    from brownian_gb300 import closure
    L, nc = 30, 150
    net = closure.Network(max_batch=1024)
    net.set_normalisation(np.zeros(81), np.ones(81), np.zeros(6), np.full(6, 0.05))
    net.set_params(np.zeros(net.n_params))  # mean 0, standard deviation 0.05 in every direction
    sur = closure.Surrogate(_params(L, nc), net)
    pos, vel, w, ra = _state(L, nc, 2)
    sur.set_state(pos, vel, w, ra)
    sur.step(50)
    st = sur.get_state()
    for k, v in st.items():
        assert np.all(np.isfinite(v)), k
    assert np.allclose(np.linalg.norm(st["ra"], axis=1), 1.0, atol=1e-4)
    d = st["pos_colloid"] - pos
    d -= L * np.round(d / L)
    assert np.mean(np.linalg.norm(d, axis=1)) > 0.05
    # the inputs the step left for the next one are the features of the new state
    fused = sur.features(recompute=False)
    fresh = sur.features(recompute=True)
    assert np.allclose(fused, fresh, atol=2e-5), np.max(np.abs(fused - fresh))
    sur.close()
    net.close()
