"""libbrownian_shim: the reference's `void name()` routines over the C ABI.

A driver that defines the reference driver's globals and calls the routines in
its main loop's order (tests/shim/driver.cpp) must end in the same state, bit
for bit, as the same system stepped through mpcd_step.
"""
import os
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
LIB = os.path.join(ROOT, "brownian_gb300", "lib")


def test_reference_driver_through_the_shim_matches_mpcd_step(tmp_path):
    import brownian_gb300 as bg
    exe = str(tmp_path / "driver")
    subprocess.run(["g++", "-O2", "-o", exe, os.path.join(HERE, "shim", "driver.cpp"), "-L" + LIB, "-lbrownian_shim",
                    "-lbrownian_gb300", "-Wl,-rpath," + LIB], check=True)
    L, dens, Nc, steps = 16, 5, 4, 3
    N = L ** 3 * dens
    out = str(tmp_path / "state.bin")
    subprocess.run([exe, str(L), str(dens), str(Nc), str(steps), out], check=True, timeout=300)
    raw = np.fromfile(out, dtype=np.float64)
    sizes = [("pos_fl", N), ("vel_fl", N), ("pos_colloid", Nc), ("vel_colloid", Nc), ("ang_vel_colloid", Nc),
             ("ra", Nc)]
    got, o = {}, 0
    for k, n in sizes:
        got[k] = raw[o:o + 3 * n].reshape(n, 3)
        o += 3 * n
    # the driver's parameters (the reference's defaults, v0 = 0.02)
    sim = bg.Simulation(L, N, Nc, n_sub=10, kbt=1.0, kbt1=1.0, ndt=0.1, mass_fl=1.0, mass_colloid=654.1,
                        sig_colloid=5.0, eps=1.0, sigma=4.0, I_colloid=0.1 * 654.1 * 16.0, v0=0.02, theta_deg=130.0,
                        Dr=0.0, seed=77777)
    sim.initialize(bg.INIT_REFERENCE)
    sim.setup()
    sim.step(steps)
    ref = sim.get_state()
    for k, _ in sizes:
        assert np.array_equal(got[k], ref[k]), k
    assert raw[o] == sim.diag()["potential_colloid"]
