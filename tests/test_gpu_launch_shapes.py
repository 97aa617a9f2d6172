"""Launch shapes of a single system (mpcd_set_launch) leave the same bits: the event pass's and
the colloid finish's grids and blocks, the side work's threads per colloid, the free-flight
pass's grid and the substep it follows; every sum is exact and every draw keyed."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _sim(prec):
    import brownian_gb300 as bg
    M = bg.displaced_mass(2.0, 10)
    sim = bg.Simulation(16, 16 ** 3 * 10, 8, n_sub=10, mass_colloid=M, sig_colloid=4.0, sigma=4.0,
                        I_colloid=0.4 * M * 4.0, v0=0.05, theta_deg=90.0, Dr=0.001, seed=11, precision=prec,
                        sort_every=3)
    sim.initialize(bg.INIT_PHYSICAL)
    sim.setup()
    return sim


@pytest.mark.parametrize("form", ["fp64", "fp32c"])
def test_launch_shapes_leave_the_same_bits(form):
    import brownian_gb300 as bg
    prec = bg.FP64 if form == "fp64" else bg.FP32C
    a, b = _sim(prec), _sim(prec)
    a.step(4)
    b.set_launch(bg.LAUNCH_EVENTS, 40, 64)
    b.set_launch(bg.LAUNCH_FIN, 20, 64)
    b.set_launch(bg.LAUNCH_AUX, 1, 256)
    b.set_launch(bg.LAUNCH_FREE, 100, 3)
    b.step(2)
    b.set_launch(bg.LAUNCH_FREE, 700, 0)
    b.step(2)
    sa, sb = a.get_state(), b.get_state()
    for k in sa:
        assert np.array_equal(sa[k], sb[k]), k
    with pytest.raises(bg.MPCDError):
        b.set_launch(bg.LAUNCH_FREE, 100, 10)  # the substep it follows: 0..n_sub-1
    a.close()
    b.close()
