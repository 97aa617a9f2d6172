"""GPU path against the CPU oracle on the benchmarked systems and over long runs.

* the 64^3 system (2,621,440 fluid particles, 500 colloids of radius 2, WCA sigma 4,
  v0 0.01, Dr 0.001, SRD angle 90 degrees, 10 substeps): three steps from one state,
  FP64 states within 1e-10 relative and the next SRD binning bit for bit;
* the large system's physics at a reduced box (SRD angle 130 degrees, colloid radius 3,
  WCA sigma 6, colloid mass the displaced fluid mass, 20 substeps, v0 0.02, Dr 0.0005),
  with colloid pairs placed inside the WCA cutoff: five steps, same bars;
* the 20^3 system (80,000 fluid particles, 20 colloids, seed 0) for 1,000 steps on both
  sides from the same keyed initial state, the GPU in either form: total momentum, fluid
  temperature, colloid MSD and velocity autocorrelation compared within their statistical
  errors;
* mpcd_diag against the oracle's diagnostics (the sums of cpp/active_brownian.cpp:39-55);
* mpcd_initialize against the oracle's keyed initialisation (cpp/initialize.cpp:31-83,
  cpp/run.cpp:3-8), and the physical initial state checked statistically.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RTOL = 1e-10
STATE = ("pos_fl", "vel_fl", "pos_colloid", "vel_colloid", "ang_vel_colloid", "ra")


def displaced(radius, density=10.0):
    return density * 4.0 / 3.0 * np.pi * radius ** 3


def kw_cfg1(**over):
    m = displaced(2.0)
    kw = dict(n_sub=10, ndt=0.1, kbt=1.0, kbt1=1.0, mass_fl=1.0, mass_colloid=m, sig_colloid=4.0, eps=1.0,
              sigma=4.0, I_colloid=0.4 * m * 4.0, v0=0.01, theta_deg=90.0, Dr=0.001, seed=1)
    kw.update(over)
    return kw


def kw_cfg3(**over):
    m = displaced(3.0)
    kw = dict(n_sub=20, ndt=0.1, kbt=1.0, kbt1=1.0, mass_fl=1.0, mass_colloid=m, sig_colloid=6.0, eps=1.0,
              sigma=6.0, I_colloid=0.4 * m * 9.0, v0=0.02, theta_deg=130.0, Dr=0.0005, seed=7)
    kw.update(over)
    return kw


def relerr(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def assert_states_close(sim, o, rtol=RTOL):
    g = sim.get_state()
    errs = {k: relerr(g[k], o.get(k)) for k in STATE}
    bad = {k: e for k, e in errs.items() if not e <= rtol}
    assert not bad, f"relative errors above {rtol}: {bad}"
    return errs


def assert_next_binning_equal(sim, o):
    cell_gpu, occ_gpu, shift_gpu = sim.rotation_binning()
    o.nn = o.nn + 1
    o.rotation_mpcd()
    cell_ref, occ_ref = o.binning(0)
    assert np.array_equal(shift_gpu, o.shift())
    assert np.array_equal(cell_gpu, cell_ref)
    assert np.array_equal(occ_gpu, occ_ref)


def oracle_from(st, L, N, Nc, kw):
    from oracle import oracle as O
    o = O.Oracle(L=L, n_fluid=N, n_colloid=Nc, rng_mode=O.RNG_KEYED, **kw)
    for k in STATE:
        o.set(k, st[k])
    return o


def test_64cube_500_colloids_three_steps_match_oracle():
    """The bench workload: GPU-initialised state (the oracle would take minutes to place
    2.6 M particles around 500 spheres), copied to the oracle; three steps (the first with
    the counting sort by cell); states to 1e-10 relative; the following binning bit for bit."""
    import brownian_gb300 as bg
    L, N, Nc = 64, 64 ** 3 * 10, 500
    kw = kw_cfg1()
    sim = bg.Simulation(L, N, Nc, **kw)
    sim.initialize(bg.INIT_REFERENCE)
    st = sim.get_state()
    # both sides from the same doubles (the device keeps displacements v dt)
    sim.set_state(*[st[k] for k in STATE])
    o = oracle_from(st, L, N, Nc, kw)
    sim.setup()
    o.setup()
    assert np.array_equal(sim.get_state()["f"], o.get("f"))
    sim.step(3)
    o.run_steps(3)
    errs = assert_states_close(sim, o)
    assert max(errs.values()) < RTOL
    assert_next_binning_equal(sim, o)
    # the step exercised the wall collisions and run()'s rear shells
    d = sim.diag()
    assert d["events"] > 0 and d["shell_records"] > 0
    sim.close()
    o.close()


def crafted_pairs_28():
    """16 colloids of radius 3 in a 28^3 box: eight pairs 6.4 apart (inside the WCA cutoff
    2^(1/6) 6 = 6.73), the pairs at least 7.6 apart from each other."""
    pos = []
    for y in (4.0, 18.0):
        for z in (5.0, 19.0):
            for x in (3.0, 17.0):
                pos.append([x, y, z])
                pos.append([x + 6.4, y + 0.3, z - 0.2])
    return np.array(pos)


def test_large_system_physics_match_oracle():
    """SRD angle 130 degrees, radius 3, WCA sigma 6, displaced mass, 20 substeps, v0 0.02,
    Dr 0.0005 (the 128^3 system's physics) in a 28^3 box, FP64, five steps."""
    import brownian_gb300 as bg
    from oracle import oracle as O
    L, N, Nc = 28, 28 ** 3 * 10, 16
    kw = kw_cfg3()
    o = O.Oracle(L=L, n_fluid=N, n_colloid=Nc, rng_mode=O.RNG_KEYED, **kw)
    o.initialize_colloid()
    o.set("pos_colloid", crafted_pairs_28())
    o.initialize_fluid()
    o.tumble()
    st = o.state()
    sim = bg.Simulation(L, N, Nc, **kw)
    sim.set_state(*[st[k] for k in STATE])
    o.setup()
    sim.setup()
    f = sim.get_state()["f"]
    assert np.count_nonzero(np.abs(f).sum(1)) == 16  # every colloid feels its partner
    assert np.array_equal(f, o.get("f"))
    for _ in range(5):
        sim.step(1)
        o.run_steps(1)
        assert_states_close(sim, o)
    assert_next_binning_equal(sim, o)
    sim.close()
    o.close()


def _series_stats(x, nblocks=10):
    """Mean and standard error of a time series from block averages."""
    b = np.array_split(np.asarray(x), nblocks)
    m = np.array([v.mean() for v in b])
    return float(m.mean()), float(m.std(ddof=1) / np.sqrt(nblocks))


def _msd_vacf(U, V, lags):
    """MSD and VACF per lag averaged over time origins, and their standard errors over
    colloids (each colloid's time average is one sample)."""
    out = {}
    for lag in lags:
        d = U[lag:] - U[:-lag] if lag else np.zeros_like(U)
        msd_c = (d * d).sum(2).mean(0)
        vac_c = (V[lag:] * V[:len(V) - lag]).sum(2).mean(0)
        n = msd_c.size
        out[lag] = (msd_c.mean(), msd_c.std(ddof=1) / np.sqrt(n), vac_c.mean(), vac_c.std(ddof=1) / np.sqrt(n))
    return out


@pytest.mark.parametrize("precision", ["fp64", "fp32c"])
def test_1000_steps_20cube_statistics_match_oracle(precision):
    """20^3, 80,000 fluid particles, 20 colloids of radius 2, seed 0, 1,000 steps on both
    sides from the oracle's keyed initial state, the GPU in the FP64 form and in the
    FP32-compensated form (each against the FP64 oracle).  Bars (stated): per-step total momentum
    equal to the oracle's within 1e-12 of sum |p| while the colloid trajectories agree to
    1e-10, else a drift of the oracle's order (the reference itself does not conserve
    momentum: a colloid whose rear shell is empty takes run()'s kick M v0 alone); block-averaged
    fluid temperature within 4 combined standard errors (10 blocks of 100 steps); colloid
    MSD and VACF at lags 0-100 steps within 4 combined standard errors (over colloids)."""
    import brownian_gb300 as bg
    from oracle import oracle as O
    L, N, Nc, steps = 20, 80000, 20, 1000
    kw = kw_cfg1(seed=0)
    o = O.Oracle(L=L, n_fluid=N, n_colloid=Nc, rng_mode=O.RNG_KEYED, **kw)
    o.initialize_colloid()
    o.initialize_fluid()
    o.tumble()
    st = o.state()
    prec = bg.FP64 if precision == "fp64" else bg.FP32C
    sim = bg.Simulation(L, N, Nc, precision=prec, **kw)
    sim.set_state(*[st[k] for k in STATE])
    o.setup()
    sim.setup()
    box = np.array([L, L, L], dtype=float)
    rec = {s: dict(P=[], T=[], X=[], V=[]) for s in ("gpu", "orc")}
    sum_p = None
    for t in range(steps + 1):
        if t:
            sim.step(1)
            o.run_steps(1)
        d = sim.diag()
        od = o.diag()
        sum_p = od[8] if sum_p is None else sum_p
        c = sim.get_colloids()
        rec["gpu"]["P"].append(np.array(d["momentum"]))
        rec["gpu"]["T"].append(d["temperature_fluid"])
        rec["gpu"]["X"].append(c["pos_colloid"])
        rec["gpu"]["V"].append(c["vel_colloid"])
        rec["orc"]["P"].append(od[5:8].copy())
        rec["orc"]["T"].append(2.0 * od[0] / (3.0 * N) / kw["kbt"])
        rec["orc"]["X"].append(o.get("pos_colloid"))
        rec["orc"]["V"].append(o.get("vel_colloid"))
    # unwrapped colloid positions
    U = {}
    for s in rec:
        X = np.array(rec[s]["X"])
        dX = X[1:] - X[:-1]
        dX -= box * np.round(dX / box)
        U[s] = np.concatenate([X[:1], X[:1] + np.cumsum(dX, axis=0)])
        rec[s]["V"] = np.array(rec[s]["V"])
    dev = float(np.max(np.abs(U["gpu"] - U["orc"])))
    Pg, Po = np.array(rec["gpu"]["P"]), np.array(rec["orc"]["P"])
    drift_g = np.max(np.abs(Pg - Pg[0]))
    drift_o = np.max(np.abs(Po - Po[0]))
    if dev < 1e-10:
        assert np.max(np.abs(Pg - Po)) <= 1e-12 * sum_p, (dev, np.max(np.abs(Pg - Po)), sum_p)
    else:
        kick = kw["mass_colloid"] * kw["v0"]
        assert drift_g <= 10.0 * max(drift_o, kick), (dev, drift_g, drift_o)
    tg, eg = _series_stats(rec["gpu"]["T"][1:])
    to, eo = _series_stats(rec["orc"]["T"][1:])
    assert abs(tg - to) <= 4.0 * np.hypot(eg, eo) + 1e-12, (tg, eg, to, eo)
    lags = (0, 1, 5, 10, 50, 100)
    sg = _msd_vacf(U["gpu"], rec["gpu"]["V"], lags)
    so = _msd_vacf(U["orc"], rec["orc"]["V"], lags)
    for lag in lags:
        mg, emg, vg, evg = sg[lag]
        mo, emo, vo, evo = so[lag]
        assert abs(mg - mo) <= 4.0 * np.hypot(emg, emo) + 1e-12 * max(mo, 1.0), (lag, mg, mo, emg, emo)
        assert abs(vg - vo) <= 4.0 * np.hypot(evg, evo) + 1e-12, (lag, vg, vo, evg, evo)
    sim.close()
    o.close()


@pytest.mark.parametrize("steps", [0, 3])
def test_diag_matches_oracle_diagnostics(steps):
    """mpcd_diag against the oracle's sums: kinetic energies, angular kinetic energy, WCA
    potential and energy within 1e-10 relative, total momentum within 1e-12 of sum |p|."""
    import brownian_gb300 as bg
    from oracle import oracle as O
    L, N, Nc = 12, 17280, 5
    kw = kw_cfg1(seed=9, v0=0.03)
    o = O.Oracle(L=L, n_fluid=N, n_colloid=Nc, rng_mode=O.RNG_KEYED, **kw)
    o.initialize_colloid()
    o.set("pos_colloid", np.array([[2.0, 2.0, 2.0], [6.3, 2.1, 1.9], [2.2, 6.25, 2.05], [6.2, 6.4, 6.3],
                                   [9.1, 9.0, 9.2]]))
    o.initialize_fluid()
    o.tumble()
    st = o.state()
    sim = bg.Simulation(L, N, Nc, **kw)
    sim.set_state(*[st[k] for k in STATE])
    o.setup()
    sim.setup()
    if steps:
        sim.step(steps)
        o.run_steps(steps)
    d = sim.diag()
    od = o.diag()
    assert od[3] > 0  # pairs inside the cutoff
    for i, k in enumerate(("ke_fluid", "ke_colloid", "ang_ke_colloid", "potential_colloid", "energy_colloid")):
        assert abs(d[k] - od[i]) <= RTOL * abs(od[i]), (k, d[k], od[i])
    assert np.max(np.abs(np.array(d["momentum"]) - od[5:8])) <= 1e-12 * od[8]
    assert abs(d["temperature_fluid"] - 2.0 * od[0] / (3.0 * N)) <= RTOL
    sim.close()
    o.close()


def test_initialize_reference_matches_oracle():
    """mpcd_initialize(MPCD_INIT_REFERENCE) draws what the oracle's keyed initialize_colloid,
    initialize_fluid and tumble draw: positions and orientations bit for bit, velocities
    within 1e-13 (the mean removed after a sum in another order)."""
    import brownian_gb300 as bg
    from oracle import oracle as O
    L, N, Nc = 16, 16 ** 3 * 10, 8
    kw = kw_cfg1(seed=21)
    o = O.Oracle(L=L, n_fluid=N, n_colloid=Nc, rng_mode=O.RNG_KEYED, **kw)
    o.initialize_colloid()
    o.initialize_fluid()
    o.tumble()
    sim = bg.Simulation(L, N, Nc, **kw)
    sim.initialize(bg.INIT_REFERENCE)
    g = sim.get_state()
    for k in ("pos_fl", "pos_colloid", "ra", "vel_colloid", "ang_vel_colloid"):
        assert np.array_equal(g[k], o.get(k)), k
    assert relerr(g["vel_fl"], o.get("vel_fl")) <= 1e-13
    # the reference's rules: colloids 1.3 sig_colloid apart, fluid outside the spheres
    X = g["pos_colloid"]
    dd = X[:, None] - X[None]
    dd -= L * np.round(dd / L)
    r = np.sqrt((dd ** 2).sum(2)) + np.eye(Nc) * 1e9
    assert r.min() >= 1.3 * kw["sig_colloid"]
    sim.close()
    o.close()


def test_initialize_physical_statistics():
    """MPCD_INIT_PHYSICAL: no two colloids closer than diameter + gap, no fluid inside a
    sphere, Maxwell-Boltzmann velocities (per-component variance kT/m within 5 standard
    errors, kurtosis 3 within 5 standard errors), zero net momentum, unit orientations."""
    import brownian_gb300 as bg
    L, N, Nc = 24, 24 ** 3 * 10, 30
    kw = kw_cfg1(seed=4)
    sim = bg.Simulation(L, N, Nc, init_gap=0.5, **kw)
    sim.initialize(bg.INIT_PHYSICAL)
    g = sim.get_state()
    X, x = g["pos_colloid"], g["pos_fl"]
    dd = X[:, None] - X[None]
    dd -= L * np.round(dd / L)
    r = np.sqrt((dd ** 2).sum(2)) + np.eye(Nc) * 1e9
    assert r.min() >= kw["sigma"] + 0.5
    for j in range(Nc):
        e = x - X[j]
        e -= L * np.round(e / L)
        assert np.sqrt((e ** 2).sum(1)).min() >= kw["sigma"] / 2
    v = g["vel_fl"]
    assert np.all(np.abs(v.sum(0)) <= 1e-10 * np.abs(v).sum())
    var = v.var(0)
    assert np.all(np.abs(var - 1.0) < 5.0 * np.sqrt(2.0 / N)), var
    kurt = (v ** 4).mean(0) / var ** 2
    assert np.all(np.abs(kurt - 3.0) < 5.0 * np.sqrt(24.0 / N)), kurt
    V = g["vel_colloid"]
    assert np.all(np.abs(V.sum(0)) <= 1e-12 * max(np.abs(V).sum(), 1e-300))
    ra = g["ra"]
    assert np.allclose((ra ** 2).sum(1), 1.0, atol=1e-12)
    sim.close()
