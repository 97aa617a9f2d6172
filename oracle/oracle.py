"""ctypes binding of the CPU oracle (oracle/mpcd_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline leg, never by the product package.
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")

RNG_SEQ = 0
RNG_KEYED = 1

STATE_NAMES = ["pos_fl", "vel_fl", "pos_colloid", "vel_colloid", "ang_vel_colloid", "ra", "f", "old_force"]


class Params(C.Structure):
    _fields_ = [
        ("Lx", C.c_int), ("Ly", C.c_int), ("Lz", C.c_int),
        ("n_fluid", C.c_int), ("n_colloid", C.c_int), ("n_sub", C.c_int),
        ("kbt", C.c_double), ("kbt1", C.c_double), ("ndt", C.c_double),
        ("mass_fl", C.c_double), ("mass_colloid", C.c_double),
        ("sig_colloid", C.c_double), ("eps", C.c_double), ("sigma", C.c_double),
        ("I_colloid", C.c_double), ("v0", C.c_double), ("theta_deg", C.c_double), ("Dr", C.c_double),
        ("rng_mode", C.c_int), ("seed", C.c_int64), ("physics", C.c_int),
    ]


def build():
    """Compile liboracle.so (and nothing else) with the oracle's Makefile."""
    subprocess.run(["make", "-s", "-C", HERE, "all"], check=True)


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = C.CDLL(LIB_PATH)
        vp = C.c_void_p
        L.orc_create.restype = vp
        L.orc_create.argtypes = [C.POINTER(Params)]
        L.orc_destroy.argtypes = [vp]
        L.orc_error.restype = C.c_char_p
        L.orc_error.argtypes = [vp]
        for name in ["orc_initialize_colloid", "orc_initialize_fluid", "orc_create_box", "orc_neighbour_list_md",
                     "orc_neighbour_list_mpcd", "orc_rotation_mpcd", "orc_run", "orc_tumble",
                     "orc_fluid_colloid_collision", "orc_compute_force_md", "orc_update_activity_direction",
                     "orc_update_pos_md", "orc_update_pos_mpcd", "orc_update_velocity_colloid", "orc_setup",
                     "orc_step"]:
            getattr(L, name).argtypes = [vp]
            getattr(L, name).restype = C.c_int
        L.orc_substep.argtypes = [vp, C.c_int]
        L.orc_begin_substep.argtypes = [vp, C.c_int]
        L.orc_get_neighbour_md.argtypes = [vp, C.c_int, C.POINTER(C.c_int32), C.c_int]
        L.orc_run_steps.argtypes = [vp, C.c_int]
        L.orc_get_step.argtypes = [vp]
        L.orc_set_step.argtypes = [vp, C.c_int]
        L.orc_diag.argtypes = [vp, C.POINTER(C.c_double)]
        L.orc_get.argtypes = [vp, C.c_int, C.POINTER(C.c_double)]
        L.orc_set.argtypes = [vp, C.c_int, C.POINTER(C.c_double)]
        L.orc_potential.restype = C.c_double
        L.orc_potential.argtypes = [vp]
        L.orc_get_binning.argtypes = [vp, C.c_int, C.POINTER(C.c_int32), C.POINTER(C.c_int32)]
        L.orc_get_shift.argtypes = [vp, C.POINTER(C.c_double)]
        L.orc_get_neigh_fl.argtypes = [vp, C.c_int, C.POINTER(C.c_int32), C.c_int]
        L.orc_box_neighbours.argtypes = [vp, C.c_int, C.POINTER(C.c_int32)]
        L.orc_get_shell_count.argtypes = [vp, C.POINTER(C.c_int32)]
        L.orc_philox4x32_10.argtypes = [C.POINTER(C.c_uint32), C.POINTER(C.c_uint32), C.POINTER(C.c_uint32)]
        L.orc_ran_seq.restype = C.c_double
        L.orc_ran_seq.argtypes = [vp]
        L.orc_updown_velocity.argtypes = [vp, C.POINTER(C.c_double), C.POINTER(C.c_double)]
        L.orc_updown_sums.argtypes = [vp, C.POINTER(C.c_int32), C.POINTER(C.c_int32), C.POINTER(C.c_double),
                                      C.POINTER(C.c_double)]
        _lib = L
    return _lib


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _ip(a):
    return a.ctypes.data_as(C.POINTER(C.c_int32))


def philox(ctr, key):
    c = (C.c_uint32 * 4)(*ctr)
    k = (C.c_uint32 * 2)(*key)
    o = (C.c_uint32 * 4)()
    lib().orc_philox4x32_10(c, k, o)
    return list(o)


class Oracle:
    """One CPU simulation; methods are the reference routines of the same name."""

    def __init__(self, **kw):
        p = Params()
        L = kw.pop("L", None)
        if L is not None:
            kw.setdefault("Lx", L); kw.setdefault("Ly", L); kw.setdefault("Lz", L)
        defaults = dict(kbt=1.0, kbt1=1.0, ndt=0.1, mass_fl=1.0, eps=1.0, theta_deg=130.0, Dr=0.0, v0=0.0,
                        n_sub=10, rng_mode=RNG_SEQ, seed=77777)
        for k, v in defaults.items():
            kw.setdefault(k, v)
        for k, v in kw.items():
            setattr(p, k, v)
        self.p = p
        self.h = lib().orc_create(C.byref(p))
        if not self.h:
            raise MemoryError("orc_create failed")
        self.N, self.Nc = p.n_fluid, p.n_colloid
        self.C = p.Lx * p.Ly * p.Lz

    def close(self):
        if self.h:
            lib().orc_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _call(self, name, *args):
        r = getattr(lib(), "orc_" + name)(self.h, *args)
        if r:
            raise RuntimeError(f"oracle {name}: {lib().orc_error(self.h).decode()}")
        return r

    def __getattr__(self, name):
        if name in ("initialize_colloid", "initialize_fluid", "create_box", "neighbour_list_md",
                    "neighbour_list_mpcd", "rotation_mpcd", "run", "tumble", "fluid_colloid_collision",
                    "compute_force_md", "update_activity_direction", "update_pos_md", "update_pos_mpcd",
                    "update_velocity_colloid", "setup", "step"):
            return lambda: self._call(name)
        raise AttributeError(name)

    def substep(self, l):
        self._call("substep", l)

    def begin_substep(self, l):
        """substep counter l and old_force = f, what main does before update_pos_md"""
        self._call("begin_substep", l)

    def neighbour_md(self):
        """per colloid (0-based), its partners j > i of the last neighbour_list_md, 0-based"""
        out = []
        buf = np.zeros(max(self.Nc, 1), dtype=np.int32)
        for i in range(1, self.Nc + 1):
            n = lib().orc_get_neighbour_md(self.h, i, _ip(buf), buf.size)
            out.append(buf[:n].copy() - 1)
        return out

    def run_steps(self, n):
        self._call("run_steps", n)

    @property
    def nn(self):
        return lib().orc_get_step(self.h)

    @nn.setter
    def nn(self, v):
        lib().orc_set_step(self.h, v)

    def get(self, name):
        which = STATE_NAMES.index(name)
        n = self.N if which < 2 else self.Nc
        a = np.empty((n, 3), dtype=np.float64)
        if lib().orc_get(self.h, which, _dp(a)):
            raise ValueError(name)
        return a

    def set(self, name, arr):
        which = STATE_NAMES.index(name)
        a = np.ascontiguousarray(arr, dtype=np.float64)
        lib().orc_set(self.h, which, _dp(a))

    def state(self):
        return {k: self.get(k) for k in STATE_NAMES[:7]}

    def potential(self):
        return lib().orc_potential(self.h)

    def diag(self):
        o = np.zeros(9)
        lib().orc_diag(self.h, _dp(o))
        return o

    def binning(self, kind):
        cell_of = np.zeros(self.N, dtype=np.int32)
        occ = np.zeros(self.C, dtype=np.int32)
        lib().orc_get_binning(self.h, kind, _ip(cell_of), _ip(occ))
        return cell_of, occ

    def shift(self):
        o = np.zeros(3)
        lib().orc_get_shift(self.h, _dp(o))
        return o

    def neigh_fl(self):
        out = []
        buf = np.zeros(1 << 16, dtype=np.int32)
        for j in range(1, self.Nc + 1):
            n = lib().orc_get_neigh_fl(self.h, j, _ip(buf), buf.size)
            if n > buf.size:
                buf = np.zeros(n, dtype=np.int32)
                n = lib().orc_get_neigh_fl(self.h, j, _ip(buf), buf.size)
            out.append(buf[:n].copy())
        return out

    def box_neighbours(self, b):
        o = np.zeros(343, dtype=np.int32)
        n = lib().orc_box_neighbours(self.h, b, _ip(o))
        return o[:n].copy()

    def shell_count(self):
        o = np.zeros(self.Nc, dtype=np.int32)
        lib().orc_get_shell_count(self.h, _ip(o))
        return o

    def updown_velocity(self):
        """updown_velocity (cpp/run.cpp:28-50) on the current state: the neighbour lists are
        rebuilt from the current positions (neighbour_list_mpcd), then the routine runs; returns
        its per-colloid counts and velocity sums and its own outputs (vel per colloid, the single
        up_vel vector)."""
        self._call("neighbour_list_mpcd")
        n = self.Nc
        cnt, up_cnt = np.zeros(n, np.int32), np.zeros(n, np.int32)
        vs, us = np.zeros((n, 3)), np.zeros((n, 3))
        lib().orc_updown_sums(self.h, _ip(cnt), _ip(up_cnt), _dp(vs), _dp(us))
        vel, up = np.zeros((n, 3)), np.zeros(3)
        self._call("updown_velocity", _dp(vel), _dp(up))
        return dict(cnt=cnt, up_cnt=up_cnt, vel_sum=vs, up_vel_sum=us, vel=vel, up_vel=up)

    def ran(self, count):
        return np.array([lib().orc_ran_seq(self.h) for _ in range(count)])
