"""mpcd_fluid_sums_noalloc: the fluid momentum and kinetic energy for callers
that cannot allocate device memory (their GPU memory belongs to their own pool,
or an allocation's device synchronisation would stall their pipeline).

The entry point works on the caller's own device arrays and keeps its partial
sums in a fixed array inside the library.  Checked through the C ABI against
the fluid part of mpcd_diag on two calls in a row (the second on a later state,
so a stale partial from the first call would show), and for its size limit.
This file is collected last so that a run stopping at the first failure has
already run every other test.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RTOL = 1e-10


def _sums(vel, n, mass, out, stream):
    import brownian_gb300 as bg
    return bg.lib().mpcd_fluid_sums_noalloc(C.c_void_p(vel), n, mass, C.c_void_p(out), C.c_void_p(stream))


def test_noalloc_sums_match_diag_on_two_calls():
    import torch

    import brownian_gb300 as bg
    L, N, Nc, mass = 12, 17280, 5, 1.0
    sim = bg.Simulation(L, N, Nc, mass_fl=mass, mass_colloid=335.1, sig_colloid=4.0, sigma=4.0,
                        I_colloid=0.4 * 335.1 * 4.0, v0=0.01, theta_deg=90.0, Dr=0.001, seed=5)
    sim.initialize(bg.INIT_PHYSICAL)
    sim.setup()
    stream = torch.cuda.current_stream()
    out = torch.zeros(4, dtype=torch.float64, device="cuda")
    for call in range(2):
        if call:
            sim.step(2)
        vel = sim.get_state()["vel_fl"]
        d = sim.diag()
        v = torch.from_numpy(vel).cuda()
        out.fill_(float("nan"))
        assert _sums(v.data_ptr(), N, mass, out.data_ptr(), stream.cuda_stream) == bg.OK
        torch.cuda.synchronize()
        got = out.cpu().numpy()
        scale = mass * np.abs(vel).sum()  # the net momentum is near zero: compare against sum |p|
        assert np.all(np.abs(got[:3] - np.array(d["momentum_fluid"])) <= RTOL * scale), (call, got, d)
        assert abs(got[3] - d["ke_fluid"]) <= RTOL * d["ke_fluid"], (call, got[3], d["ke_fluid"])
    sim.close()


@pytest.mark.parametrize("n", [0, 1, 2047, 2049, 600_000])
def test_noalloc_sums_match_numpy(n):
    """Sizes that leave the last block partial and, at 600,000 particles (293 blocks of
    2,048), make the final reduction's strided loop over the block partials run more than
    once; two calls in a row, the second on other velocities."""
    import torch

    import brownian_gb300 as bg
    rng = np.random.default_rng(n + 1)
    out = torch.zeros(4, dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream()
    for call in range(2):
        vel = rng.normal(0.0, 1.0 + call, size=(max(n, 1), 3))[:n]
        v = torch.from_numpy(np.ascontiguousarray(vel)).cuda() if n else torch.zeros(3, dtype=torch.float64,
                                                                                      device="cuda")
        out.fill_(float("nan"))
        assert _sums(v.data_ptr(), n, 2.0, out.data_ptr(), stream.cuda_stream) == bg.OK
        torch.cuda.synchronize()
        got = out.cpu().numpy()
        mom = 2.0 * vel.sum(axis=0) if n else np.zeros(3)
        ke = 0.5 * 2.0 * float((vel * vel).sum()) if n else 0.0
        scale = 2.0 * np.abs(vel).sum() if n else 1.0
        assert np.all(np.abs(got[:3] - mom) <= RTOL * scale), (n, call, got, mom)
        assert abs(got[3] - ke) <= RTOL * max(ke, 1e-300), (n, call, got[3], ke)


def test_noalloc_rejects_more_than_its_maximum():
    import torch

    import brownian_gb300 as bg
    out = torch.zeros(4, dtype=torch.float64, device="cuda")
    v = torch.zeros(3, dtype=torch.float64, device="cuda")
    r = _sums(v.data_ptr(), bg.NOALLOC_MAX_PARTICLES + 1, 1.0, out.data_ptr(), 0)
    assert r == bg.ERR_CAPACITY
