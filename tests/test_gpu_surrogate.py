"""Colloid-only dynamics with the closure: the GPU feature kernels give the
network inputs of brownian_gb300.closure.features, the network inside the step
gives the outputs of mpcd_mlp_forward on the same inputs bit for bit, and the
step runs."""
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
    pos = np.empty((nc, 3))
    n = 0
    while n < nc:  # random sequential placement with centre distance >= 4.2
        x = rng.uniform(0, L, 3)
        d = pos[:n] - x
        d -= L * np.round(d / L)
        if n == 0 or np.min(np.sum(d * d, axis=1)) >= 4.2 ** 2:
            pos[n] = x
            n += 1
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
    sur.step(49)
    before = sur.features(recompute=True)
    sur.step(1)
    st = sur.get_state()
    for k, v in st.items():
        assert np.all(np.isfinite(v)), k
    assert np.allclose(np.linalg.norm(st["ra"], axis=1), 1.0, atol=1e-4)
    d = st["pos_colloid"] - pos
    d -= L * np.round(d / L)
    assert np.mean(np.linalg.norm(d, axis=1)) > 0.05
    # the inputs the last step fed its network are the features of the state before it
    fused = sur.features(recompute=False)
    assert np.array_equal(fused, before), np.max(np.abs(fused - before))
    sur.close()
    net.close()


@pytest.mark.parametrize("nc", [150, 700])
def test_step_network_matches_mlp_forward(nc):
    import torch

    from brownian_gb300 import closure
    L = 30 if nc == 150 else 52
    rng = np.random.default_rng(nc)
    net = closure.Network(max_batch=1024, seed=4)
    net.set_params(rng.normal(0, 0.06, net.n_params).astype(np.float32))
    net.set_normalisation(rng.normal(0, 0.2, 81).astype(np.float32), rng.uniform(0.5, 2, 81).astype(np.float32),
                          rng.normal(0, 0.1, 6).astype(np.float32), rng.uniform(5, 20, 6).astype(np.float32))
    sur = closure.Surrogate(_params(L, nc), net)
    sur.set_state(*_state(L, nc, 5))
    sur.step(3)
    x = sur.features(recompute=False)
    got = sur.outputs()
    xd = torch.from_numpy(x).cuda()
    od = torch.empty((nc, 12), dtype=torch.float32, device="cuda")
    net.forward(xd.data_ptr(), od.data_ptr(), nc)
    torch.cuda.synchronize()
    ref = od.cpu().numpy()
    assert np.all(np.isfinite(got))
    assert np.array_equal(got, ref), np.max(np.abs(got - ref))
    sur.close()
    net.close()


def test_cluster_substeps_above_1024_colloids():
    """More than 1024 colloids: the substeps run in a cluster of 8 blocks.  The step stays finite,
    the next step's network inputs are the features of the state it left (numpy restatement),
    and the force partners cover every pair within the WCA cutoff."""
    from brownian_gb300 import closure
    L, nc = 60, 1200
    net = closure.Network(max_batch=64, seed=2)
    rng = np.random.default_rng(7)
    net.set_params(rng.normal(0, 0.05, net.n_params).astype(np.float32))
    net.set_normalisation(np.zeros(81), np.ones(81), np.zeros(6), np.full(6, 0.5))
    sur = closure.Surrogate(_params(L, nc), net)
    sur.set_state(*_state(L, nc, 11))
    sur.step(20)
    st = sur.get_state()
    for k, v in st.items():
        assert np.all(np.isfinite(v)), k
    sur.step(1)
    fused = sur.features(recompute=False)
    ref = closure.features(st, L, 2.0)
    assert np.allclose(fused, ref, atol=2e-5), np.max(np.abs(fused - ref))
    assert sur.fast_steps() == 0
    sur.close()
    net.close()
