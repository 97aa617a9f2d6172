"""The trajectory file format (mpcd_traj_write) read back by brownian_gb300.read_trajectory,
on a file written here by the format's description (no GPU)."""
import numpy as np

import brownian_gb300 as bg


def test_read_trajectory_layout(tmp_path):
    rng = np.random.default_rng(1)
    nf, nc = 5, 3
    pos, vel, ra = (rng.normal(size=(nf, nc, 3)) for _ in range(3))
    p = tmp_path / "t.bgbtraj"
    with open(p, "wb") as f:
        f.write(b"BGBTRAJ1")
        f.write(np.array([1, nc, nf, 7], dtype="<i4").tobytes())
        f.write(np.array([10.0, 11.0, 12.0, 0.1], dtype="<f8").tobytes())
        for k in range(nf):
            for a in (pos, vel, ra):
                f.write(a[k].astype("<f8").tobytes())
    d = bg.read_trajectory(p)
    assert np.array_equal(d["box"], [10.0, 11.0, 12.0]) and d["dt_frame"] == 0.1
    assert np.array_equal(d["pos"], pos) and np.array_equal(d["vel"], vel) and np.array_equal(d["ra"], ra)


def test_read_trajectory_rejects_truncated(tmp_path):
    p = tmp_path / "bad.bgbtraj"
    with open(p, "wb") as f:
        f.write(b"BGBTRAJ1")
        f.write(np.array([1, 2, 3, 7], dtype="<i4").tobytes())
        f.write(np.zeros(4, dtype="<f8").tobytes())
        f.write(np.zeros(5, dtype="<f8").tobytes())
    try:
        bg.read_trajectory(p)
    except ValueError:
        return
    raise AssertionError("a truncated file was accepted")
