"""Routine-by-routine traces of the reference step — TEST INFRASTRUCTURE ONLY.

`replay(case)` drives the oracle through exactly the sequence that
oracle/ref_harness.cpp drives the reference's own cpp/ routines through
(cpp/active_brownian.cpp:14-38) and returns the same records (tag, bytes), so a
trace of the compiled reference and a trace of the oracle can be compared
record by record.  `parse_records` reads the harness's binary record stream.
"""
import hashlib
import struct

import numpy as np

from . import oracle as O


def parse_records(path):
    out = []
    with open(path, "rb") as f:
        while True:
            head = f.read(56)
            if not head:
                break
            tag = head[:48].split(b"\0", 1)[0].decode()
            (nb,) = struct.unpack("<Q", head[48:])
            out.append((tag, f.read(nb)))
    return out


def sha(b):
    return hashlib.sha256(b).hexdigest()


def make_oracle(case):
    p = dict(case["params"])
    return O.Oracle(L=p["L"], n_fluid=p["N"], n_colloid=p["Nc"], n_sub=p["n_sub"], ndt=p["ndt"], kbt=p["kbt"],
                    kbt1=p["kbt1"], mass_fl=p["mass_fl"], mass_colloid=p["M"], sig_colloid=p["sig_colloid"],
                    eps=p["eps"], sigma=p["sigma"], I_colloid=p["I"], v0=p["v0"], theta_deg=130.0,
                    rng_mode=O.RNG_SEQ, seed=p["seed"])


def _pts(a):
    return np.ascontiguousarray(a, dtype=np.float64).tobytes()


def _state(o, pre):
    recs = [(f"{pre}/{k}", _pts(o.get(k))) for k in ["pos_fl", "vel_fl", "pos_colloid", "vel_colloid",
                                                       "ang_vel_colloid", "ra", "f"]]
    recs.append((f"{pre}/potential", struct.pack("<d", o.potential())))
    return recs


def _binning(o, pre, kind):
    cell_of, occ = o.binning(kind)
    return [(f"{pre}/cell_of", cell_of.tobytes()), (f"{pre}/occupancy", occ.tobytes())]


def _neigh(o, pre):
    v = []
    for lst in o.neigh_fl():
        v.append(np.array([len(lst)], dtype=np.int32))
        v.append(lst.astype(np.int32))
    return [(f"{pre}/neigh_fl", np.concatenate(v).tobytes())]


def replay(case, nsteps=None, detail=None):
    """Records of the oracle (sequential ran() mode) for one golden case."""
    p = case["params"]
    nsteps = p["nsteps"] if nsteps is None else nsteps
    detail = p["detail"] if detail is None else detail
    o = make_oracle(case)
    recs = []
    o.initialize_colloid()
    o.initialize_fluid()
    if case.get("crafted_colloids") is not None:
        o.set("pos_colloid", np.array(case["crafted_colloids"], dtype=np.float64))
    recs += _state(o, "init")
    o.create_box()
    C = o.C
    t = np.concatenate([o.box_neighbours(b) for b in range(1, C + 1)]).astype(np.int32)
    recs.append(("setup/box_neigh", t.tobytes()))
    o.neighbour_list_mpcd()
    recs += _binning(o, "setup.nl_mpcd", 1)
    recs += _neigh(o, "setup.nl_mpcd")
    o.neighbour_list_md()
    o.compute_force_md()
    recs.append(("setup.force/f", _pts(o.get("f"))))
    recs.append(("setup.force/potential", struct.pack("<d", o.potential())))
    o.tumble()
    recs.append(("setup.tumble/ra", _pts(o.get("ra"))))
    for nn in range(1, nsteps + 1):
        s = f"s{nn}"
        d = nn <= detail
        o.nn = nn
        o.rotation_mpcd()
        if d:
            recs.append((f"{s}.rotation/vel_fl", _pts(o.get("vel_fl"))))
            recs += _binning(o, f"{s}.rotation", 0)
        o.run()
        if d:
            recs.append((f"{s}.run/vel_fl", _pts(o.get("vel_fl"))))
            recs.append((f"{s}.run/vel_colloid", _pts(o.get("vel_colloid"))))
            recs.append((f"{s}.run/shell_count", o.shell_count().tobytes()))
        for l in range(1, p["n_sub"] + 1):
            pre = f"{s}.l{l}"
            dl = d and l <= 2
            if not dl:
                o.substep(l)
                continue
            # the body of orc_substep, split to record after each routine
            o.set("old_force", o.get("f"))
            o.update_pos_md()
            recs.append((f"{pre}.pos_md/pos_colloid", _pts(o.get("pos_colloid"))))
            o.neighbour_list_md()
            o.update_pos_mpcd()
            recs.append((f"{pre}.pos_mpcd/pos_fl", _pts(o.get("pos_fl"))))
            o.neighbour_list_mpcd()
            recs += _binning(o, f"{pre}.nl_mpcd", 1)
            recs += _neigh(o, f"{pre}.nl_mpcd")
            o.fluid_colloid_collision()
            recs.append((f"{pre}.collision/pos_fl", _pts(o.get("pos_fl"))))
            recs.append((f"{pre}.collision/vel_fl", _pts(o.get("vel_fl"))))
            recs.append((f"{pre}.collision/vel_colloid", _pts(o.get("vel_colloid"))))
            recs.append((f"{pre}.collision/ang_vel_colloid", _pts(o.get("ang_vel_colloid"))))
            o.update_activity_direction()
            recs.append((f"{pre}.activity/ra", _pts(o.get("ra"))))
            o.compute_force_md()
            recs.append((f"{pre}.force/f", _pts(o.get("f"))))
            recs.append((f"{pre}.force/potential", struct.pack("<d", o.potential())))
            o.update_velocity_colloid()
            recs.append((f"{pre}.velocity/vel_colloid", _pts(o.get("vel_colloid"))))
        recs += _state(o, f"{s}.end")
    o.close()
    return recs
