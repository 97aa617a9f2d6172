"""The FP32-compensated form (precision=FP32C) on the GPU.

Its fluid is integer cell + FP32 offset with FP32 velocities, so it is not
bit-comparable to the reference; it is checked against the FP64 form started
from the same state with the same keyed draws (one step apart, almost every
particle agrees to FP32 rounding), for exact momentum bookkeeping, thermostat
temperature, order independence of the counting sort, and the state round trip.
"""
import numpy as np
import pytest

from test_gpu_parity import _kw

pytestmark = pytest.mark.gpu


def make_pair32(L, N, Nc, sort_every=0, **over):
    """An FP64 and an FP32C system set from the same oracle-initialised state."""
    import brownian_gb300 as bg
    from oracle import oracle as O
    kw = _kw(**over)
    o = O.Oracle(L=L, n_fluid=N, n_colloid=Nc, rng_mode=O.RNG_KEYED, **kw)
    o.initialize_colloid()
    o.initialize_fluid()
    o.tumble()
    st = o.state()
    out = []
    for prec in (bg.FP64, bg.FP32C):
        sim = bg.Simulation(L, N, Nc, sort_every=sort_every, precision=prec, **kw)
        sim.set_state(st["pos_fl"], st["vel_fl"], st["pos_colloid"], st["vel_colloid"], st["ang_vel_colloid"],
                      st["ra"])
        sim.setup()
        out.append(sim)
    return st, out[0], out[1]


def min_image(d, L):
    return d - L * np.round(d / L)


def test_state_round_trip():
    st, _, s32 = make_pair32(12, 17280, 3)
    g = s32.get_state()
    dpos = min_image(g["pos_fl"] - st["pos_fl"], 12.0)
    assert np.max(np.abs(dpos)) <= 2.0 ** -23
    assert np.array_equal(g["vel_fl"], st["vel_fl"].astype(np.float32).astype(np.float64))
    for k in ("pos_colloid", "vel_colloid", "ang_vel_colloid", "ra"):
        assert np.array_equal(g[k], st[k]), k


def test_one_step_agrees_with_fp64():
    _, s64, s32 = make_pair32(20, 80000, 20)
    s64.step(1)
    s32.step(1)
    a, b = s64.get_state(), s32.get_state()
    dv = np.max(np.abs(a["vel_fl"] - b["vel_fl"]), axis=1)
    dx = np.max(np.abs(min_image(a["pos_fl"] - b["pos_fl"], 20.0)), axis=1)
    # a particle can take the other branch only at a cell face or a sphere surface
    assert np.mean(dv > 1e-4) < 1e-3, np.sort(dv)[-20:]
    assert np.mean(dx > 1e-5) < 1e-3, np.sort(dx)[-20:]
    assert np.quantile(dv, 0.99) < 1e-5
    for k in ("pos_colloid", "ra"):
        assert np.max(np.abs(min_image(a[k] - b[k], 20.0))) < 1e-4, k
    rel = np.linalg.norm(a["vel_colloid"] - b["vel_colloid"]) / np.linalg.norm(a["vel_colloid"])
    assert rel < 2e-2, rel


def test_one_step_agrees_with_oracle():
    """The FP32-compensated step against the FP64 oracle from the same state with the same
    keyed draws: the error of every observable of one step, stated as a bar."""
    import brownian_gb300 as bg
    from oracle import oracle as O
    L, N, Nc = 20, 80000, 20
    kw = _kw()
    o = O.Oracle(L=L, n_fluid=N, n_colloid=Nc, rng_mode=O.RNG_KEYED, **kw)
    o.initialize_colloid()
    o.initialize_fluid()
    o.tumble()
    st = o.state()
    sim = bg.Simulation(L, N, Nc, precision=bg.FP32C, **kw)
    sim.set_state(st["pos_fl"], st["vel_fl"], st["pos_colloid"], st["vel_colloid"], st["ang_vel_colloid"],
                  st["ra"])
    sim.setup()
    o.setup()
    sim.step(1)
    o.run_steps(1)
    g = sim.get_state()
    dv = np.max(np.abs(g["vel_fl"] - o.get("vel_fl")), axis=1)
    dx = np.max(np.abs(min_image(g["pos_fl"] - o.get("pos_fl"), float(L))), axis=1)
    # FP32 rounding of a thermal velocity (|v| ~ 1) is 6e-8; a particle at a cell face or a
    # sphere surface can take the other branch
    assert np.quantile(dv, 0.99) < 1e-5
    assert np.mean(dv > 1e-4) < 1e-3
    assert np.mean(dx > 1e-5) < 1e-3
    for k in ("pos_colloid", "ra"):
        assert np.max(np.abs(min_image(g[k] - o.get(k), float(L)))) < 1e-4, k
    rel = np.linalg.norm(g["vel_colloid"] - o.get("vel_colloid")) / np.linalg.norm(o.get("vel_colloid"))
    assert rel < 2e-2, rel
    # the cell occupancies of the next binning: a particle changes cell only at a face
    _, occ_gpu, shift_gpu = sim.rotation_binning()
    o.nn = o.nn + 1
    o.rotation_mpcd()
    _, occ_ref = o.binning(0)
    assert np.array_equal(shift_gpu, o.shift())
    assert np.sum(np.abs(occ_gpu.astype(np.int64) - occ_ref)) <= 1e-3 * N
    sim.close()
    o.close()


def test_momentum_and_temperature():
    _, _, s32 = make_pair32(12, 17280, 5)
    d0 = s32.diag()
    s32.step(50)
    d1 = s32.diag()
    scale = 17280 * 1.6  # sum |p_i| of a thermal fluid at kT = m = 1
    drift = np.max(np.abs(np.array(d1["momentum"]) - np.array(d0["momentum"])))
    assert drift / scale < 1e-6, drift
    assert abs(d1["temperature_fluid"] - 1.0) < 0.05
    assert d1["events"] > 0


def test_counting_sort_is_order_independent():
    """A sort every step and no sort at all give the same bits: every sum is exact
    and every draw is keyed by particle id."""
    _, _, a = make_pair32(10, 10000, 3, sort_every=1)
    _, _, b = make_pair32(10, 10000, 3, sort_every=-1)
    a.step(5)
    b.step(5)
    sa, sb = a.get_state(), b.get_state()
    for k in sa:
        assert np.array_equal(sa[k], sb[k]), k


def test_routine_calls_equal_fused_step_fp32c():
    _, _, a = make_pair32(10, 8000, 3)
    _, _, b = make_pair32(10, 8000, 3)
    a.step(2)
    for _ in range(2):
        b.rotation_mpcd()
        b.run()
        for l in range(1, 11):
            b.substep(l)
    sa, sb = a.get_state(), b.get_state()
    for k in sa:
        assert np.array_equal(sa[k], sb[k]), k


@pytest.mark.parametrize("sort_every", [-1, 3])
def test_free_flight_schedule_gives_the_same_bits(sort_every):
    """The free-flight schedule (the rotation pass streams the particles no colloid can
    reach through the whole step and bins them; the substep passes walk the near list)
    against the same steps without it: every array bit for bit after six steps of a 24^3
    system with 20 active colloids, with steps that sort in between (those run without the
    schedule) and without."""
    _, _, a = make_pair32(24, 138240, 20, sort_every=sort_every, v0=0.05)
    _, _, b = make_pair32(24, 138240, 20, sort_every=sort_every, v0=0.05)
    b.set_flight(False)
    near = []
    for _ in range(6):
        a.step(1)
        b.step(1)
        near.append(a.flight_near())
    sa, sb = a.get_state(), b.get_state()
    for k in sa:
        assert np.array_equal(sa[k], sb[k]), k
    da, db = a.diag(), b.diag()
    assert da["events"] == db["events"] > 0
    assert da["shell_records"] == db["shell_records"] > 0
    # some particles near the colloids, most in free flight
    assert 0 < max(near) < 0.6 * 138240, near
    ca, oa, _ = a.rotation_binning()
    cb, ob, _ = b.rotation_binning()
    assert np.array_equal(ca, cb) and np.array_equal(oa, ob)
    # a step routine by routine after them (it reads the cell tables the last free-flight
    # step left for the next step's first substeps)
    for sim in (a, b):
        sim.rotation_mpcd()
        sim.run()
        for l in range(1, 11):
            sim.substep(l)
    sa, sb = a.get_state(), b.get_state()
    for k in sa:
        assert np.array_equal(sa[k], sb[k]), k


def test_free_flight_without_colloids():
    """No colloids: every particle is in free flight, one pass per step; the same bits."""
    import brownian_gb300 as bg
    sims = []
    for _ in range(2):
        sim = bg.Simulation(12, 17280, 0, precision=bg.FP32C, **_kw())
        sim.initialize(bg.INIT_PHYSICAL)
        sim.setup()
        sims.append(sim)
    a, b = sims
    b.set_flight(False)
    a.step(4)
    b.step(4)
    assert a.flight_near() == 0
    sa, sb = a.get_state(), b.get_state()
    for k in ("pos_fl", "vel_fl"):
        assert np.array_equal(sa[k], sb[k]), k


def test_strongly_active_colloids_stay_in_range():
    """v0 = 0.1: run() can give a rear-shell particle the colloid's whole kick M v0 / m
    (a shell of one particle when another colloid blocks the rear); the default speed
    bound and cell-table reach follow from that (this system once overran them at step 80)."""
    import brownian_gb300 as bg
    M = bg.displaced_mass(2.0, 10)
    sim = bg.Simulation(64, 64 ** 3 * 10, 500, n_sub=10, mass_colloid=M, sig_colloid=4.0, sigma=4.0,
                        I_colloid=0.4 * M * 4.0, v0=0.1, theta_deg=90.0, Dr=0.001, seed=14, precision=bg.FP32C)
    sim.initialize(bg.INIT_PHYSICAL)
    sim.setup()
    sim.step(150)
    d = sim.diag()
    # the active kicks feed energy that the cell thermostat removes only at the next rotation
    assert 0.9 < d["temperature_fluid"] < 1.2
    sim.close()
