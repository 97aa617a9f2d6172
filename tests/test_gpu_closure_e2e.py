"""The learned closure end to end at a small size: samples from the exact collision
kernel, training on the GPU, and what the trained network gains over the method
without it (colloid-only dynamics with no fluid exchange) and over its own mean without
the learned variance, measured against full MPCD."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _p(L, nc, v0, seed):
    import brownian_gb300 as bg
    M = bg.displaced_mass(2.0, 10)
    return bg.make_params(L, L ** 3 * 10, nc, n_sub=10, mass_colloid=M, sig_colloid=4.0, sigma=4.0,
                          I_colloid=0.4 * M * 4.0, v0=v0, theta_deg=90.0, Dr=0.001, seed=seed, precision=bg.FP32C)


def test_trained_closure_beats_no_closure():
    from brownian_gb300 import closure
    X, Y = closure.generate_gpu([_p(24, 40, v0, 5 + i) for i, v0 in enumerate((0.0, 0.05, 0.1))], steps=300)
    perm = np.random.default_rng(0).permutation(X.shape[0])
    X, Y = X[perm], Y[perm]
    n = X.shape[0]
    cut = int(0.9 * n)
    net = closure.Network(max_batch=2048, seed=1)
    net.fit_normalisation(X[:cut], Y[:cut])
    closure.train(net, X[:cut], Y[:cut], epochs=25, batch=1024, lr=1e-3)
    held = closure.nll(net, X[cut:], Y[cut:])
    free = closure.free_nll(Y[:cut], Y[cut:])  # without the network
    assert held < free - 0.2, (held, free)
    res = closure.compare(_p(24, 40, 0.05, 42), net, steps=400, lags=(5, 20, 50), blocks=2)
    rel = res["rel_diff_vs_full"]
    d_c = abs(rel["closure"]["msd"][1])
    d_n = abs(rel["no_closure"]["msd"][1])
    assert d_c < d_n, rel
    # the learned variance matters: with the network's mean only the colloids lose the
    # fluctuations of the fluid and their kinetic energy (VACF at lag 0) falls well below
    # the full method's, which the closure with its variance keeps
    v_c = abs(rel["closure"]["vacf"][0])
    v_m = abs(rel["mean_only"]["vacf"][0])
    assert v_c < v_m, rel
    # the trained closure's colloids never outrun the force-partner skin
    assert res["fast_steps"]["closure"] == 0, res["fast_steps"]
    net.close()
