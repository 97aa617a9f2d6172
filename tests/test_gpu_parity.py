"""GPU path against the CPU oracle (keyed Philox draws on both sides).

Bit-exact: cell numbers and per-cell occupancy of the SRD binning, the grid
shift, the WCA forces.  FP64 states: within 1e-10 relative over 100 steps (the
paths differ only in summation order and in libm versus CUDA transcendentals,
differences of a few ulp per step).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RTOL = 1e-10


def _kw(**over):
    kw = dict(n_sub=10, ndt=0.1, kbt=1.0, kbt1=1.0, mass_fl=1.0, mass_colloid=335.1, sig_colloid=4.0, eps=1.0,
              sigma=4.0, I_colloid=0.4 * 335.1 * 4.0, v0=0.01, theta_deg=90.0, Dr=0.001, seed=3)
    kw.update(over)
    return kw


def make_pair(L, N, Nc, crafted=None, sort_every=0, **over):
    import brownian_gb300 as bg
    from oracle import oracle as O
    kw = _kw(**over)
    o = O.Oracle(L=L, n_fluid=N, n_colloid=Nc, rng_mode=O.RNG_KEYED, **kw)
    o.initialize_colloid()
    o.initialize_fluid()
    o.tumble()
    if crafted is not None:
        crafted(o)
    st = o.state()
    sim = bg.Simulation(L, N, Nc, sort_every=sort_every, **kw)
    sim.set_state(st["pos_fl"], st["vel_fl"], st["pos_colloid"], st["vel_colloid"], st["ang_vel_colloid"], st["ra"])
    o.setup()
    sim.setup()
    return o, sim


def relerr(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def assert_close(sim, o, rtol=RTOL, keys=("pos_fl", "vel_fl", "pos_colloid", "vel_colloid", "ang_vel_colloid", "ra")):
    g = sim.get_state()
    errs = {k: relerr(g[k], o.get(k)) for k in keys}
    bad = {k: e for k, e in errs.items() if not e <= rtol}
    assert not bad, f"relative errors above {rtol}: {bad}"
    return errs


def test_initial_binning_bit_exact():
    o, sim = make_pair(12, 12 * 12 * 12 * 10, 4)
    # the setup pass binned for step 1; the oracle bins inside rotation_mpcd
    cell_gpu, occ_gpu, shift_gpu = sim.rotation_binning()
    o.nn = 1
    o.rotation_mpcd()
    cell_ref, occ_ref = o.binning(0)
    assert np.array_equal(shift_gpu, o.shift())
    assert np.array_equal(cell_gpu, cell_ref)
    assert np.array_equal(occ_gpu, occ_ref)


def test_setup_forces_bit_exact():
    def crafted(o):
        o.set("pos_colloid", np.array([[2.0, 2.0, 2.0], [6.3, 2.1, 1.9], [2.2, 6.25, 2.05], [6.2, 6.4, 6.3],
                                       [4.1, 4.0, 6.2]]))
    o, sim = make_pair(12, 3456, 5, crafted=crafted)
    g = sim.get_state()
    assert np.any(g["f"] != 0)
    assert np.array_equal(g["f"], o.get("f"))


@pytest.mark.parametrize("steps,sort_every", [(1, 0), (5, 0), (5, 1), (5, -1)])
def test_steps_match_oracle_small(steps, sort_every):
    """sort_every: 0 the default period, 1 a counting sort by cell every step, -1 never"""
    o, sim = make_pair(10, 10000, 3, sort_every=sort_every)
    sim.step(steps)
    o.run_steps(steps)
    assert_close(sim, o)


def test_100_steps_match_oracle_cfg0_like():
    # the 20^3, density-10, 20-colloid system at 100 steps
    o, sim = make_pair(20, 80000, 20)
    for _ in range(4):
        sim.step(25)
        o.run_steps(25)
        errs = assert_close(sim, o)
    cell_gpu, occ_gpu, _ = sim.rotation_binning()
    o2 = o  # the next rotation's binning must agree bit for bit as well
    o2.nn = o2.nn + 1
    o2.rotation_mpcd()
    cell_ref, occ_ref = o2.binning(0)
    assert np.array_equal(cell_gpu, cell_ref)
    assert np.array_equal(occ_gpu, occ_ref)


def test_routine_calls_equal_fused_step():
    """rotation_mpcd, run, substep 1..n called one by one give the fused graph's bits."""
    o, a = make_pair(10, 8000, 3)
    _, b = make_pair(10, 8000, 3)
    a.step(3)
    for _ in range(3):
        b.rotation_mpcd()
        b.run()
        for l in range(1, 11):
            b.substep(l)
    sa, sb = a.get_state(), b.get_state()
    for k in sa:
        assert np.array_equal(sa[k], sb[k]), k
    assert a.step_count == b.step_count == 3


@pytest.mark.parametrize("sort_every", [-1, 3])
def test_free_flight_schedule_gives_the_same_bits(sort_every):
    """The free-flight schedule (the particles no colloid can reach in a step streamed
    through all its substeps by one pass beside the near particles' substeps) against the
    same steps without it: every array bit for bit after six steps of a 24^3 system with 20
    active colloids, and the next binning."""
    _, a = make_pair(24, 138240, 20, sort_every=sort_every, v0=0.05)
    _, b = make_pair(24, 138240, 20, sort_every=sort_every, v0=0.05)
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
    assert 0 < max(near) < 0.6 * 138240, near
    ca, oa, ra = a.rotation_binning()
    cb, ob, rb = b.rotation_binning()
    assert np.array_equal(ca, cb) and np.array_equal(oa, ob) and np.array_equal(ra, rb)
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


def test_runs_are_deterministic():
    _, a = make_pair(12, 17280, 5)
    _, b = make_pair(12, 17280, 5)
    a.step(10)
    b.step(10)
    sa, sb = a.get_state(), b.get_state()
    for k in sa:
        assert np.array_equal(sa[k], sb[k]), k
    # the same state into caller-provided page-locked buffers
    import torch
    out = {k: torch.empty(v.shape, dtype=torch.float64).pin_memory().numpy() for k, v in sa.items()}
    got = b.get_state(out=out)
    for k in sa:
        assert got[k] is out[k] and np.array_equal(out[k], sa[k]), k
    with pytest.raises(ValueError):
        b.get_state(out=dict(out, pos_fl=np.empty((3, 3))))
    ro = np.zeros_like(out["f"])
    ro.flags.writeable = False
    with pytest.raises(ValueError):
        b.get_state(out=dict(out, f=ro))


def test_momentum_conserved():
    o, sim = make_pair(12, 17280, 5)
    d0 = sim.diag()
    sim.step(50)
    d1 = sim.diag()
    scale = 17280 * 1.6  # sum |p_i| of a thermal fluid at kT = m = 1
    drift = np.max(np.abs(np.array(d1["momentum"]) - np.array(d0["momentum"])))
    assert drift / scale < 1e-12, drift
    assert abs(d1["temperature_fluid"] - 1.0) < 0.05


def test_shell_counts_match_oracle():
    o, sim = make_pair(12, 17280, 5, v0=0.05)
    sim.rotation_mpcd()
    sim.run()
    o.nn = 1
    o.rotation_mpcd()
    o.run()
    assert np.array_equal(sim.shell_count(), o.shell_count())
