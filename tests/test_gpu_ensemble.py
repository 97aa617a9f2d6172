"""Batched ensemble: systems of different sizes, colloid counts and activities
stepped together (one launch per stage) give, bit for bit, what each gives
stepped alone, for any launch shape of the batched step."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SYSTEMS = [(10, 3, 0.0), (12, 0, 0.05), (14, 5, 0.02), (16, 4, 0.1)]  # box, colloids, v0


def _params(i, L, nc, v0):
    import brownian_gb300 as bg
    M = bg.displaced_mass(2.0, 10)
    return bg.make_params(L, L ** 3 * 10, nc, n_sub=10, mass_colloid=M, sig_colloid=4.0, sigma=4.0,
                          I_colloid=0.4 * M * 4.0, v0=v0, theta_deg=90.0, Dr=0.001, seed=100 + i,
                          precision=bg.FP32C, sort_every=2)


def _single(p):
    import brownian_gb300 as bg
    kw = {k: getattr(p, k) for k, _ in bg.Params._fields_ if k not in ("Lx", "Ly", "Lz", "n_fluid", "n_colloid")}
    return bg.Simulation(p.Lx, p.n_fluid, p.n_colloid, **kw)


def test_ensemble_matches_systems_stepped_alone():
    import brownian_gb300 as bg
    params = [_params(i, *s) for i, s in enumerate(SYSTEMS)]
    ens = bg.Ensemble(params)
    singles = [_single(p) for p in params]
    for s in list(ens) + singles:
        s.initialize(bg.INIT_PHYSICAL)
        s.setup()
    ens.step(5)
    for s in singles:
        s.step(5)
    for r, (a, b) in enumerate(zip(ens, singles)):
        ga, gb = a.get_state(), b.get_state()
        for k in ga:
            assert np.array_equal(ga[k], gb[k]), (r, k)
        assert a.step_count == b.step_count == 5
    # other launch shapes of the batched step: the same bits
    ens.set_launch(bg.ENS_EVENTS, 7, 32)
    ens.set_launch(bg.ENS_RUN, 1, 32)
    ens.set_launch(bg.ENS_FIN, 1, 64)
    ens.set_launch(bg.ENS_AUX, 1, 256)
    ens.step(3)
    for s in singles:
        s.step(3)
    for r, (a, b) in enumerate(zip(ens, singles)):
        ga, gb = a.get_state(), b.get_state()
        for k in ga:
            assert np.array_equal(ga[k], gb[k]), (r, k)
    d = ens[2].diag()
    assert abs(d["temperature_fluid"] - 1.0) < 0.05
    ens.close()


def test_ensemble_schedules_leave_the_same_bits():
    """The batched free-flight schedule, the batched per-substep schedule and each system
    stepped alone on the per-substep schedule, switched between steps (sort steps among
    them), leave the same bits."""
    import brownian_gb300 as bg
    systems = SYSTEMS + [(12, 8, 0.08)]
    params = [_params(i, *s) for i, s in enumerate(systems)]
    ens = bg.Ensemble(params)
    assert ens.flight
    singles = [_single(p) for p in params]
    for s in list(ens) + singles:
        s.initialize(bg.INIT_PHYSICAL)
        s.setup()
    for s in singles:
        s.set_flight(False)
    for on, k in ((True, 3), (False, 2), (True, 4)):
        ens.set_flight(on)
        ens.step(k)
        for s in singles:
            s.step(k)
        for r, (a, b) in enumerate(zip(ens, singles)):
            ga, gb = a.get_state(), b.get_state()
            for key in ga:
                assert np.array_equal(ga[key], gb[key]), (on, r, key)
    # particles were near in every system with colloids; in the one without, only the rare
    # particle faster than the flight table allows
    near = [s.flight_near() for s in ens]
    assert near[1] < 20 and all(n > 100 for i, n in enumerate(near) if i != 1), near
    ens.close()


def test_ensemble_rejects_mixed_forms():
    import brownian_gb300 as bg
    p = [_params(0, 10, 2, 0.0), _params(1, 10, 2, 0.0)]
    p[1].precision = bg.FP64
    with pytest.raises(bg.MPCDError):
        bg.Ensemble(p)
