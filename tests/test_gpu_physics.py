"""The corrected collision rules (physics = PHYSICS_FIXED): a colloid's own box among its
candidate boxes and both tangential Gaussian components of the wall reflection.

Against the oracle run with the same rules (FP64, states within 1e-10 relative, as the
reference mode).  Small spheres (radius 0.5) make the own-box rule matter: the box holding a
sphere's centre then reaches outside the sphere, and under the reference's rules fluid there
is never tested against it.  (Over longer runs such fluid ends deep inside a light sphere and
its next collision trips the library's displacement check; the corrected rules avoid that.)"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

KW = dict(n_sub=10, ndt=0.1, kbt=1.0, kbt1=1.0, mass_fl=1.0, mass_colloid=5.24, sig_colloid=1.0, eps=1.0,
          sigma=1.0, I_colloid=0.4 * 5.24 * 0.25, v0=0.01, theta_deg=90.0, Dr=0.001, seed=9)


def _rel(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def _pair(physics, L=10, N=10000, Nc=6, **over):
    import brownian_gb300 as bg
    from oracle import oracle as O
    kw = dict(KW, **over)
    o = O.Oracle(L=L, n_fluid=N, n_colloid=Nc, rng_mode=O.RNG_KEYED, physics=physics, **kw)
    o.initialize_colloid()
    o.initialize_fluid()
    o.tumble()
    st = o.state()
    sim = bg.Simulation(L, N, Nc, physics=physics, **kw)
    sim.set_state(st["pos_fl"], st["vel_fl"], st["pos_colloid"], st["vel_colloid"], st["ang_vel_colloid"], st["ra"])
    o.setup()
    sim.setup()
    return o, sim


@pytest.mark.parametrize("physics", [0, 1])
def test_rules_match_oracle(physics):
    o, sim = _pair(physics)
    sim.step(5)
    o.run_steps(5)
    g = sim.get_state()
    for k in ("pos_fl", "vel_fl", "pos_colloid", "vel_colloid", "ang_vel_colloid", "ra"):
        assert _rel(g[k], o.get(k)) < 1e-10, k
    sim.close()
    o.close()


def test_fixed_rules_fp32c_run():
    import brownian_gb300 as bg
    sim = bg.Simulation(16, 16 ** 3 * 10, 8, precision=bg.FP32C, physics=bg.PHYSICS_FIXED, **KW)
    sim.initialize(bg.INIT_PHYSICAL)
    sim.setup()
    sim.step(20)
    d = sim.diag()
    assert 0.9 < d["temperature_fluid"] < 1.1 and d["events"] > 0
    sim.close()
