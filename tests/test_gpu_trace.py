"""The traced step: a real step (the same bits as an untraced one), with every launch's
start and end on the graph's own timeline."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _sim(prec):
    import brownian_gb300 as bg
    M = bg.displaced_mass(2.0, 10)
    sim = bg.Simulation(16, 16 ** 3 * 10, 8, n_sub=10, mass_colloid=M, sig_colloid=4.0, sigma=4.0,
                        I_colloid=0.4 * M * 4.0, v0=0.05, theta_deg=90.0, Dr=0.001, seed=7, precision=prec)
    sim.initialize(bg.INIT_PHYSICAL)
    sim.setup()
    return sim


@pytest.mark.parametrize("form", ["fp64", "fp32c"])
def test_trace_step_is_a_step_with_a_timeline(form):
    import brownian_gb300 as bg
    prec = bg.FP64 if form == "fp64" else bg.FP32C
    a, b = _sim(prec), _sim(prec)
    a.step(2)
    l0 = a.launch_count
    a.step(1)
    per_step = a.launch_count - l0
    tr = a.trace_step()
    b.step(4)
    sa, sb = a.get_state(), b.get_state()
    for k in sa:
        assert np.array_equal(sa[k], sb[k]), k
    assert a.step_count == b.step_count == 4
    assert len(tr) == per_step, (len(tr), per_step)
    names = {n for n, _, _ in tr}
    assert {"k_cell_prep", "k_rotate_classify", "k_free_flight", "k_stream_near", "k_fin", "k_end_step"} <= names
    assert all(0.0 <= t0 <= t1 for _, t0, t1 in tr)
    # the end of the step comes last
    end = [t1 for n, _, t1 in tr if n == "k_end_step"][0]
    assert end >= max(t1 for _, _, t1 in tr) - 1e-9
    a.close()
    b.close()
