"""updown_velocity (cpp/run.cpp:28-50) on the GPU against the CPU oracle.

FP64 form: the GPU and the oracle run the same steps from the same state, then
both evaluate the routine: the per-colloid counts of the run() shell and the inner
shell are equal, the velocity sums and the routine's own outputs agree to 1e-9
relative (the oracle sums in neighbour-list order, the GPU exactly).  FP32 form:
the kernel's counts and sums against a numpy restatement on the GPU's own state.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

KW = dict(n_sub=10, ndt=0.1, kbt=1.0, kbt1=1.0, mass_fl=1.0, mass_colloid=335.1, sig_colloid=4.0, eps=1.0,
          sigma=4.0, I_colloid=0.4 * 335.1 * 4.0, v0=0.01, theta_deg=90.0, Dr=0.001, seed=3)


def _rel(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def _pair(L, N, Nc):
    import brownian_gb300 as bg
    from oracle import oracle as O
    o = O.Oracle(L=L, n_fluid=N, n_colloid=Nc, rng_mode=O.RNG_KEYED, **KW)
    o.initialize_colloid()
    o.initialize_fluid()
    o.tumble()
    st = o.state()
    sim = bg.Simulation(L, N, Nc, **KW)
    sim.set_state(st["pos_fl"], st["vel_fl"], st["pos_colloid"], st["vel_colloid"], st["ang_vel_colloid"], st["ra"])
    o.setup()
    sim.setup()
    return o, sim


@pytest.mark.parametrize("steps", [0, 3])
def test_updown_fp64_matches_oracle(steps):
    o, sim = _pair(12, 12 ** 3 * 10, 4)
    sim.step(steps)
    o.run_steps(steps)
    g, r = sim.updown_velocity(), o.updown_velocity()
    assert np.array_equal(g["cnt"], r["cnt"]) and np.array_equal(g["up_cnt"], r["up_cnt"])
    assert np.all(g["cnt"] > 0) and np.all(g["up_cnt"] > 0)
    assert _rel(g["vel_sum"], r["vel_sum"]) < 1e-9
    assert _rel(g["up_vel_sum"], r["up_vel_sum"]) < 1e-9
    assert _rel(g["reference"]["vel"], r["vel"]) < 1e-9
    assert _rel(g["reference"]["up_vel"], r["up_vel"]) < 1e-9
    sim.close()
    o.close()


def _box_rule(cell_p, cell_c, L):
    """the 342 boxes around the colloid's box (own box excluded), cpp/neighbour_list.cpp:12-25"""
    d = (cell_p - cell_c) % L
    near = np.all((d <= 3) | (d >= L - 3), axis=-1)
    return near & np.any(cell_p != cell_c, axis=-1)


def test_updown_fp32c_against_numpy():
    import brownian_gb300 as bg
    L, N, Nc = 16, 16 ** 3 * 10, 6
    sim = bg.Simulation(L, N, Nc, precision=bg.FP32C, **KW)
    sim.initialize(bg.INIT_PHYSICAL)
    sim.setup()
    sim.step(4)
    g = sim.updown_velocity()
    st = sim.get_state()
    x, v = st["pos_fl"], st["vel_fl"]
    X, V = st["pos_colloid"], st["vel_colloid"]
    cp = np.floor(x).astype(np.int64) % L
    rs2, ru2 = (KW["sigma"] * 0.5 + 0.5) ** 2, (KW["sigma"] * 0.5 + 0.1) ** 2
    for j in range(Nc):
        cc = np.floor(X[j]).astype(np.int64) % L
        r = x - X[j]
        r -= L * np.round(r / L)
        r2 = np.sum(r * r, axis=1)
        rear = (r @ V[j]) <= 0
        ok = _box_rule(cp, cc, L) & rear
        sh, up = ok & (r2 <= rs2), ok & (r2 <= ru2)
        # a particle within 1e-9 of a threshold could fall either side in FP32 positions
        assert abs(int(sh.sum()) - int(g["cnt"][j])) <= 1 and abs(int(up.sum()) - int(g["up_cnt"][j])) <= 1
        if sh.sum() == g["cnt"][j]:
            assert np.allclose(v[sh].sum(axis=0), g["vel_sum"][j], rtol=1e-6, atol=1e-9)
    sim.close()
