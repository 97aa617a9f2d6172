"""The substep routines one by one (mpcd_update_pos_md ... mpcd_update_velocity_colloid)
against the oracle's routine of the same name, each compared right after it runs:

* states within 1e-10 relative (the paths differ in summation order and libm);
* the colloid pair list of neighbour_list_md, and the box binning (per particle box,
  per box occupancy) and per-colloid candidate counts of neighbour_list_mpcd, exactly;
* the routines called in the reference's order give the fused mpcd_step's bits, and
  calls out of that order are refused.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RTOL = 1e-10

# what each routine changes, compared after it (cpp/parameters.hpp:12-14)
WRITES = {
    "update_pos_md": ("pos_colloid",),
    "neighbour_list_md": (),
    "update_pos_mpcd": ("pos_fl",),
    "neighbour_list_mpcd": (),
    "fluid_colloid_collision": ("pos_fl", "vel_fl", "vel_colloid", "ang_vel_colloid"),
    "update_activity_direction": ("ra",),
    "compute_force_md": ("f",),
    "update_velocity_colloid": ("vel_colloid",),
}
STATE = ("pos_fl", "vel_fl", "pos_colloid", "vel_colloid", "ang_vel_colloid", "ra")


def _kw(**over):
    m = 335.1
    kw = dict(n_sub=10, ndt=0.1, kbt=1.0, kbt1=1.0, mass_fl=1.0, mass_colloid=m, sig_colloid=4.0, eps=1.0,
              sigma=4.0, I_colloid=0.4 * m * 4.0, v0=0.03, theta_deg=90.0, Dr=0.001, seed=13)
    kw.update(over)
    return kw


# six colloids in a 14^3 box: two pairs inside the WCA cutoff (4.49), the rest within the
# pair-list radius 3 sig_colloid = 12 of several others
PAIRS = np.array([[2.0, 2.0, 2.0], [6.3, 2.1, 1.9], [2.2, 6.25, 2.05], [9.0, 9.5, 9.2], [9.3, 9.4, 13.5],
                  [2.5, 10.0, 7.0]])


def make_pair(L=14, dens=10, Nc=6, crafted=PAIRS, **over):
    import brownian_gb300 as bg
    from oracle import oracle as O
    kw = _kw(**over)
    N = L ** 3 * dens
    o = O.Oracle(L=L, n_fluid=N, n_colloid=Nc, rng_mode=O.RNG_KEYED, **kw)
    o.initialize_colloid()
    if crafted is not None:
        o.set("pos_colloid", crafted[:Nc])
    o.initialize_fluid()
    o.tumble()
    st = o.state()
    sim = bg.Simulation(L, N, Nc, **kw)
    sim.set_state(*[st[k] for k in STATE])
    o.setup()
    sim.setup()
    return o, sim


def relerr(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def test_each_routine_matches_its_oracle_routine():
    o, sim = make_pair()
    for step in range(2):
        o.nn = o.nn + 1
        o.rotation_mpcd()
        o.run()
        sim.rotation_mpcd()
        sim.run()
        for l in range(1, 11):
            o.begin_substep(l)
            for name, keys in WRITES.items():
                getattr(sim, name)()
                getattr(o, name)()
                g = sim.get_state()
                for k in keys:
                    e = relerr(g[k], o.get(k))
                    assert e <= RTOL, (step, l, name, k, e)
                if name == "neighbour_list_md":
                    ref = o.neighbour_md()
                    got = sim.neighbour_md()
                    assert sum(len(x) for x in ref) > 0
                    for i in range(sim.Nc):
                        assert np.array_equal(got[i], ref[i]), (step, l, i)
                if name == "neighbour_list_mpcd":
                    cell_of, occ, nn = sim.box_binning()
                    cref, oref = o.binning(1)
                    assert np.array_equal(cell_of, cref), (step, l)
                    assert np.array_equal(occ, oref), (step, l)
                    assert np.array_equal(nn, [len(x) for x in o.neigh_fl()]), (step, l)
                if name == "compute_force_md":
                    assert o.potential() > 0
                    d = sim.diag()
                    assert abs(d["potential_colloid"] - o.potential()) <= RTOL * o.potential()
    # the whole state after two steps
    g = sim.get_state()
    for k in STATE:
        assert relerr(g[k], o.get(k)) <= RTOL, k
    sim.close()
    o.close()


def test_routines_give_the_fused_steps_bits():
    """Three steps routine by routine, and three with substeps alternating between
    mpcd_substep and the eight routines, equal three mpcd_step steps bit for bit (the
    first step sorts the fluid by cell), and leave the same next SRD binning."""
    _, a = make_pair()
    _, b = make_pair()
    _, c = make_pair()
    a.step(3)
    for _ in range(3):
        b.rotation_mpcd()
        b.run()
        c.rotation_mpcd()
        c.run()
        for l in range(1, 11):
            b.substep_routines()
            if l % 2:
                c.substep(l)
            else:
                c.substep_routines()
    sa = a.get_state()
    for other in (b, c):
        so = other.get_state()
        for k in sa:
            assert np.array_equal(sa[k], so[k]), k
        assert other.step_count == 3
        for x, y in zip(a.rotation_binning(), other.rotation_binning()):
            assert np.array_equal(x, y)
    # and the fused step continues from a routine-driven one
    a.step(2)
    b.step(2)
    sa, sb = a.get_state(), b.get_state()
    for k in sa:
        assert np.array_equal(sa[k], sb[k]), k


def test_pair_list_of_a_large_box_matches_oracle():
    """500 colloids in the 64^3 box: the bucketed pair list equals the reference's
    O(Nc^2) list exactly."""
    import brownian_gb300 as bg
    from oracle import oracle as O
    L, N, Nc = 64, 20000, 500
    kw = _kw(seed=3)
    sim = bg.Simulation(L, N, Nc, **kw)
    sim.initialize(bg.INIT_REFERENCE)
    sim.setup()
    sim.rotation_mpcd()
    sim.run()
    sim.update_pos_md()
    sim.neighbour_list_md()
    o = O.Oracle(L=L, n_fluid=N, n_colloid=Nc, rng_mode=O.RNG_KEYED, **kw)
    o.set("pos_colloid", sim.get_colloids()["pos_colloid"])
    o.neighbour_list_md()
    ref = o.neighbour_md()
    got = sim.neighbour_md()
    assert sum(len(x) for x in ref) > 500
    for i in range(Nc):
        assert np.array_equal(got[i], ref[i]), i
    sim.close()
    o.close()


def test_routine_order_is_enforced():
    import brownian_gb300 as bg
    _, sim = make_pair(L=10, Nc=3)
    with pytest.raises(bg.MPCDError) as e:
        sim.update_pos_md()  # before rotation_mpcd and run
    assert e.value.code == bg.ERR_STATE
    sim.rotation_mpcd()
    sim.run()
    with pytest.raises(bg.MPCDError) as e:
        sim.neighbour_list_md()  # update_pos_md opens the substep
    assert e.value.code == bg.ERR_STATE and "update_pos_md" in str(e.value)
    sim.update_pos_md()
    with pytest.raises(bg.MPCDError):
        sim.update_pos_mpcd()  # neighbour_list_md comes first
    with pytest.raises(bg.MPCDError):
        sim.substep(1)  # the open substep is closed by update_velocity_colloid
    for n in bg.SUBSTEP_ROUTINES[1:]:
        getattr(sim, n)()
    sim.substep(2)  # the fused substep continues the sequence
    sim.close()


def test_fp32c_form_refuses_the_routines():
    import brownian_gb300 as bg
    sim = bg.Simulation(10, 10000, 2, precision=bg.FP32C, **_kw())
    sim.initialize(bg.INIT_REFERENCE)
    sim.setup()
    sim.rotation_mpcd()
    sim.run()
    with pytest.raises(bg.MPCDError) as e:
        sim.update_pos_md()
    assert e.value.code == bg.ERR_STATE
    sim.close()
