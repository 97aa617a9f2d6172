"""brownian_gb300: the MPCD + active-colloid time step on GB300 (sm_103a).

Python mirror of the C ABI in include/brownian_gb300.h.  `Simulation` holds one
device-resident system; its methods carry the names of the reference routines
(cpp/ of shashankgandham/brownian): initialize, setup (the prologue of main),
rotation_mpcd, run, substep, step.  `active_brownian` is the reference's main()
loop.  There is no CPU path: every call runs the sm_103a kernels of
lib/libbrownian_gb300.so, and importing the package fails if that library is
missing or cannot load.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "lib", "libbrownian_gb300.so")

OK, ERR_PARAM, ERR_CUDA, ERR_CAPACITY, ERR_RANGE, ERR_STATE, ERR_NOMEM = range(7)
FP64, FP32C = 0, 1
INIT_REFERENCE, INIT_PHYSICAL = 0, 1

# every symbol include/brownian_gb300.h declares
EXPORTS = ["mpcd_create", "mpcd_destroy", "mpcd_last_error", "mpcd_set_stream", "mpcd_set_state", "mpcd_get_state",
           "mpcd_set_step", "mpcd_get_step", "mpcd_initialize", "mpcd_setup", "mpcd_rotation_mpcd", "mpcd_run",
           "mpcd_substep", "mpcd_update_pos_md", "mpcd_neighbour_list_md", "mpcd_update_pos_mpcd",
           "mpcd_neighbour_list_mpcd", "mpcd_fluid_colloid_collision", "mpcd_update_activity_direction",
           "mpcd_compute_force_md", "mpcd_update_velocity_colloid", "mpcd_get_neighbour_md", "mpcd_get_box_binning",
           "mpcd_step", "mpcd_step_async", "mpcd_sync", "mpcd_set_flight", "mpcd_get_flight", "mpcd_diag", "mpcd_get_rotation_binning", "mpcd_get_shell_count",
           "mpcd_profile_enable", "mpcd_profile_read", "mpcd_trace_step", "mpcd_launch_count", "mpcd_set_launch",
           "mpcd_fluid_sums_noalloc", "mpcd_ensemble_create", "mpcd_ensemble_destroy", "mpcd_ensemble_last_error",
           "mpcd_ensemble_system", "mpcd_ensemble_step", "mpcd_ensemble_set_launch", "mpcd_ensemble_launch_count",
           "mpcd_ensemble_set_flight", "mpcd_ensemble_get_flight",
           "mpcd_exchange_read", "mpcd_mlp_create", "mpcd_mlp_destroy", "mpcd_mlp_last_error", "mpcd_mlp_param_count",
           "mpcd_mlp_set_normalisation", "mpcd_mlp_get_params", "mpcd_mlp_set_params", "mpcd_mlp_forward",
           "mpcd_mlp_grad", "mpcd_mlp_train_step", "mpcd_mlp_set_fault", "mpcd_surrogate_create", "mpcd_surrogate_destroy",
           "mpcd_surrogate_last_error", "mpcd_surrogate_set_state", "mpcd_surrogate_get_state",
           "mpcd_surrogate_features", "mpcd_surrogate_outputs", "mpcd_surrogate_fast_steps", "mpcd_surrogate_step",
           "mpcd_surrogate_set_fault", "mpcd_surrogate_set_noise", "mpcd_updown_velocity", "mpcd_traj_create",
           "mpcd_traj_destroy", "mpcd_traj_last_error", "mpcd_traj_frames", "mpcd_traj_reset", "mpcd_traj_record",
           "mpcd_traj_record_surrogate", "mpcd_traj_analyse", "mpcd_traj_read", "mpcd_traj_write"]
# the routines of the substep body, in the reference's order (cpp/active_brownian.cpp:28-37)
SUBSTEP_ROUTINES = ("update_pos_md", "neighbour_list_md", "update_pos_mpcd", "neighbour_list_mpcd",
                    "fluid_colloid_collision", "update_activity_direction", "compute_force_md",
                    "update_velocity_colloid")
ENS_EVENTS, ENS_RUN, ENS_FIN, ENS_AUX, ENS_FREE = 0, 1, 2, 3, 4
NOALLOC_MAX_PARTICLES = 33554432
PHYSICS_REFERENCE, PHYSICS_FIXED = 0, 1
LAUNCH_EVENTS, LAUNCH_FIN, LAUNCH_AUX, LAUNCH_FREE = 0, 1, 2, 3


class MPCDError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"[{code}] {msg}")
        self.code = code


class Params(C.Structure):
    _fields_ = [
        ("Lx", C.c_int), ("Ly", C.c_int), ("Lz", C.c_int),
        ("n_fluid", C.c_int), ("n_colloid", C.c_int), ("n_sub", C.c_int),
        ("kbt", C.c_double), ("kbt1", C.c_double), ("ndt", C.c_double),
        ("mass_fl", C.c_double), ("mass_colloid", C.c_double), ("sig_colloid", C.c_double),
        ("eps", C.c_double), ("sigma", C.c_double), ("I_colloid", C.c_double), ("v0", C.c_double),
        ("theta_deg", C.c_double), ("Dr", C.c_double), ("seed", C.c_uint64), ("precision", C.c_int),
        ("max_per_cell", C.c_int), ("vmax", C.c_double), ("init_gap", C.c_double), ("sort_every", C.c_int),
        ("physics", C.c_int),
    ]


class Diag(C.Structure):
    _fields_ = [
        ("step", C.c_int64), ("ke_fluid", C.c_double), ("ke_colloid", C.c_double),
        ("ang_ke_colloid", C.c_double), ("potential_colloid", C.c_double), ("energy_colloid", C.c_double),
        ("momentum", C.c_double * 3), ("momentum_fluid", C.c_double * 3), ("temperature_fluid", C.c_double),
        ("events", C.c_int64), ("shell_records", C.c_int64),
    ]

    def as_dict(self):
        return {k: (list(getattr(self, k)) if k.startswith("momentum") else getattr(self, k)) for k, _ in self._fields_}


_lib = None


def lib():
    """The loaded C-ABI library; raises if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} is missing: run brownian_gb300.build.build() (no CPU fallback exists)")
        L = C.CDLL(LIB_PATH)
        vp, dp, ip = C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_int32)
        L.mpcd_create.argtypes = [C.POINTER(Params), C.POINTER(vp)]
        L.mpcd_destroy.argtypes = [vp]
        L.mpcd_last_error.argtypes = [vp]
        L.mpcd_last_error.restype = C.c_char_p
        L.mpcd_set_stream.argtypes = [vp, vp]
        L.mpcd_set_state.argtypes = [vp, dp, dp, dp, dp, dp, dp]
        L.mpcd_get_state.argtypes = [vp, dp, dp, dp, dp, dp, dp, dp]
        L.mpcd_set_step.argtypes = [vp, C.c_int64]
        L.mpcd_get_step.argtypes = [vp]
        L.mpcd_get_step.restype = C.c_int64
        L.mpcd_initialize.argtypes = [vp, C.c_int]
        for n in ["mpcd_setup", "mpcd_rotation_mpcd", "mpcd_run"]:
            getattr(L, n).argtypes = [vp]
        L.mpcd_substep.argtypes = [vp, C.c_int]
        for n in SUBSTEP_ROUTINES:
            getattr(L, "mpcd_" + n).argtypes = [vp]
        L.mpcd_get_neighbour_md.argtypes = [vp, ip, ip, C.c_int]
        L.mpcd_get_box_binning.argtypes = [vp, ip, ip, ip]
        L.mpcd_step.argtypes = [vp, C.c_int]
        L.mpcd_step_async.argtypes = [vp, C.c_int]
        L.mpcd_sync.argtypes = [vp]
        L.mpcd_set_flight.argtypes = [vp, C.c_int]
        L.mpcd_get_flight.argtypes = [vp, ip]
        L.mpcd_diag.argtypes = [vp, C.POINTER(Diag)]
        L.mpcd_get_rotation_binning.argtypes = [vp, ip, ip, dp]
        L.mpcd_get_shell_count.argtypes = [vp, ip]
        L.mpcd_profile_enable.argtypes = [vp, C.c_int]
        L.mpcd_profile_read.argtypes = [vp, C.c_void_p, C.POINTER(C.c_int64), dp, C.c_int]
        L.mpcd_trace_step.argtypes = [vp, C.c_void_p, dp, dp, C.c_int]
        L.mpcd_launch_count.argtypes = [vp]
        L.mpcd_launch_count.restype = C.c_int64
        L.mpcd_set_launch.argtypes = [vp, C.c_int, C.c_int, C.c_int]
        L.mpcd_fluid_sums_noalloc.argtypes = [vp, C.c_int64, C.c_double, vp, vp]
        L.mpcd_exchange_read.argtypes = [vp, dp, C.c_int]
        L.mpcd_updown_velocity.argtypes = [vp, C.POINTER(C.c_int32), C.POINTER(C.c_int32), dp, dp]
        L.mpcd_traj_create.argtypes = [C.c_int, C.c_int, dp, C.POINTER(vp)]
        L.mpcd_traj_destroy.argtypes = [vp]
        L.mpcd_traj_last_error.argtypes = [vp]
        L.mpcd_traj_last_error.restype = C.c_char_p
        L.mpcd_traj_frames.argtypes = [vp]
        L.mpcd_traj_reset.argtypes = [vp]
        L.mpcd_traj_record.argtypes = [vp, vp]
        L.mpcd_traj_record_surrogate.argtypes = [vp, vp]
        L.mpcd_traj_analyse.argtypes = [vp, C.POINTER(C.c_int), C.c_int, dp, dp, dp]
        L.mpcd_traj_read.argtypes = [vp, C.c_int, C.c_int, dp, dp, dp]
        L.mpcd_traj_write.argtypes = [vp, C.c_char_p, C.c_double]
        L.mpcd_ensemble_create.argtypes = [C.POINTER(Params), C.c_int, C.POINTER(vp)]
        L.mpcd_ensemble_destroy.argtypes = [vp]
        L.mpcd_ensemble_last_error.argtypes = [vp]
        L.mpcd_ensemble_last_error.restype = C.c_char_p
        L.mpcd_ensemble_system.argtypes = [vp, C.c_int]
        L.mpcd_ensemble_system.restype = vp
        L.mpcd_ensemble_step.argtypes = [vp, C.c_int]
        L.mpcd_ensemble_set_launch.argtypes = [vp, C.c_int, C.c_int, C.c_int]
        L.mpcd_ensemble_launch_count.argtypes = [vp]
        L.mpcd_ensemble_launch_count.restype = C.c_int64
        L.mpcd_ensemble_set_flight.argtypes = [vp, C.c_int]
        L.mpcd_ensemble_get_flight.argtypes = [vp]
        _lib = L
    return _lib


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double)) if a is not None else None


def _f64(a, n):
    if a is None:
        return None
    a = np.ascontiguousarray(a, dtype=np.float64)
    if a.shape != (n, 3):
        raise ValueError(f"expected shape ({n}, 3), got {a.shape}")
    return a


class Trajectory:
    """Colloid frames kept on the device (mpcd_traj_*): unwrapped positions, velocities and
    orientations; `record(src)` takes a frame from a Simulation (between steps) or from a
    closure.Surrogate; `analyse` gives MSD, VACF and orientation autocorrelation per lag (in
    frames), reduced on the GPU."""

    def __init__(self, n_colloid, max_frames, box):
        L = lib()
        box = np.ascontiguousarray(np.broadcast_to(np.asarray(box, dtype=np.float64), (3,)))
        h = C.c_void_p()
        r = L.mpcd_traj_create(int(n_colloid), int(max_frames), _dp(box), C.byref(h))
        if r:
            raise MPCDError(r, "mpcd_traj_create rejected the sizes")
        self.h, self.Nc, self.box = h, int(n_colloid), box.copy()

    def _ck(self, r):
        if r:
            raise MPCDError(r, lib().mpcd_traj_last_error(self.h).decode())

    @property
    def frames(self):
        return lib().mpcd_traj_frames(self.h)

    def reset(self):
        self._ck(lib().mpcd_traj_reset(self.h))

    def record(self, src):
        if isinstance(src, Simulation):
            r = lib().mpcd_traj_record(self.h, src.h)
            if r:
                raise MPCDError(r, lib().mpcd_last_error(src.h).decode())
        else:
            self._ck(lib().mpcd_traj_record_surrogate(self.h, src.h))

    def analyse(self, msd_lags=(1, 2, 5, 10, 20, 50, 100), vacf_lags=(0, 1, 2, 5, 10, 20), oacf_lags=(0, 10, 50, 100)):
        out = {}
        for key, lags in (("msd", msd_lags), ("vacf", vacf_lags), ("oacf", oacf_lags)):
            lg = np.ascontiguousarray(lags, dtype=np.int32)
            res = [np.empty(len(lg)) for _ in range(3)]
            self._ck(lib().mpcd_traj_analyse(self.h, lg.ctypes.data_as(C.POINTER(C.c_int)), len(lg),
                                             *[_dp(a) for a in res]))
            out[key] = res[("msd", "vacf", "oacf").index(key)]
        return out

    def read(self, first=0, count=None):
        count = self.frames - first if count is None else count
        a = [np.empty((count, self.Nc, 3)) for _ in range(3)]
        self._ck(lib().mpcd_traj_read(self.h, first, count, *[_dp(x) for x in a]))
        return tuple(a)

    def write(self, path, dt_frame=1.0):
        self._ck(lib().mpcd_traj_write(self.h, os.fsencode(path), float(dt_frame)))

    def close(self):
        if self.h:
            lib().mpcd_traj_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def read_trajectory(path):
    """A trajectory file written by Trajectory.write / mpcd_traj_write: dict(box, dt_frame,
    pos, vel, ra), the arrays (n_frames, n_colloid, 3)."""
    with open(path, "rb") as f:
        if f.read(8) != b"BGBTRAJ1":
            raise ValueError(f"{path}: not a trajectory file")
        version, nc, nf, fields = np.frombuffer(f.read(16), dtype="<i4")
        if version != 1 or fields != 7:
            raise ValueError(f"{path}: unsupported version {version} / fields {fields}")
        geo = np.frombuffer(f.read(32), dtype="<f8")
        data = np.frombuffer(f.read(), dtype="<f8")
    if data.size != nf * 3 * nc * 3:
        raise ValueError(f"{path}: truncated")
    d = data.reshape(nf, 3, nc, 3)
    return dict(box=geo[:3].copy(), dt_frame=float(geo[3]), pos=d[:, 0].copy(), vel=d[:, 1].copy(), ra=d[:, 2].copy())


def displaced_mass(radius, density, mass_fl=1.0):
    """Mass of the fluid a sphere displaces (the configs' colloid mass)."""
    return density * mass_fl * 4.0 / 3.0 * np.pi * radius ** 3


def make_params(L, n_fluid, n_colloid, *, n_sub=10, kbt=1.0, kbt1=1.0, ndt=0.1, mass_fl=1.0, mass_colloid=654.1,
                sig_colloid=5.0, eps=1.0, sigma=None, I_colloid=None, v0=0.0, theta_deg=130.0, Dr=0.0, seed=77777,
                precision=FP64, max_per_cell=0, vmax=0.0, init_gap=0.5, sort_every=0, physics=0):
    """mpcd_params of one system (defaults: the reference's, cpp/active_brownian.cpp:3-7)."""
    Lx, Ly, Lz = (L, L, L) if np.isscalar(L) else L
    sigma = 0.8 * sig_colloid if sigma is None else sigma          # cpp/active_brownian.cpp:7
    I_colloid = 0.1 * mass_colloid * sigma * sigma if I_colloid is None else I_colloid
    return Params(Lx, Ly, Lz, n_fluid, n_colloid, n_sub, kbt, kbt1, ndt, mass_fl, mass_colloid, sig_colloid, eps,
                  sigma, I_colloid, v0, theta_deg, Dr, seed, precision, max_per_cell, vmax, init_gap, sort_every,
                  physics)


class Simulation:
    """One MPCD + active-colloid system resident on the GPU."""

    def __init__(self, L, n_fluid, n_colloid, **kw):
        self._adopt(make_params(L, n_fluid, n_colloid, **kw))
        h = C.c_void_p()
        r = lib().mpcd_create(C.byref(self.params), C.byref(h))
        if r:
            raise MPCDError(r, "mpcd_create rejected the parameters or could not allocate")
        self.h = h
        self._owned = True

    def _adopt(self, params):
        self.params = params
        self.N, self.Nc = params.n_fluid, params.n_colloid
        self.C = params.Lx * params.Ly * params.Lz
        self.dt = params.ndt / params.n_sub

    @classmethod
    def _view(cls, handle, params):
        """A system owned by something else (an ensemble); closing the view frees nothing."""
        s = cls.__new__(cls)
        s._adopt(params)
        s.h = C.c_void_p(handle)
        s._owned = False
        return s

    # ---------------------------------------------------------------- plumbing
    def _ck(self, r):
        if r:
            raise MPCDError(r, lib().mpcd_last_error(self.h).decode())

    def close(self):
        if getattr(self, "h", None):
            if getattr(self, "_owned", True):
                lib().mpcd_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def set_stream(self, stream_ptr):
        """Launch on an external cudaStream_t (e.g. torch.cuda.Stream().cuda_stream)."""
        self._ck(lib().mpcd_set_stream(self.h, C.c_void_p(stream_ptr)))

    # ---------------------------------------------------------------- state
    def set_state(self, pos_fl=None, vel_fl=None, pos_colloid=None, vel_colloid=None, ang_vel_colloid=None, ra=None):
        a = [_f64(pos_fl, self.N), _f64(vel_fl, self.N), _f64(pos_colloid, self.Nc), _f64(vel_colloid, self.Nc),
             _f64(ang_vel_colloid, self.Nc), _f64(ra, self.Nc)]
        self._ck(lib().mpcd_set_state(self.h, *[_dp(x) for x in a]))

    _STATE_KEYS = ("pos_fl", "vel_fl", "pos_colloid", "vel_colloid", "ang_vel_colloid", "ra", "f")

    def get_state(self, out=None):
        """The state as (n, 3) float64 arrays.  `out`: a dict of C-contiguous float64 arrays of
        those shapes to fill instead of new ones (page-locked ones make the copies direct)."""
        if out is None:
            out = {k: np.empty((self.N, 3)) for k in ("pos_fl", "vel_fl")}
            out.update({k: np.empty((self.Nc, 3)) for k in self._STATE_KEYS[2:]})
        for k in self._STATE_KEYS:
            a = out[k]
            n = self.N if k in ("pos_fl", "vel_fl") else self.Nc
            if (a.dtype != np.float64 or a.shape != (n, 3) or not a.flags["C_CONTIGUOUS"]
                    or not a.flags["WRITEABLE"]):
                raise ValueError(f"out[{k!r}] must be a writeable C-contiguous float64 array of shape ({n}, 3)")
        self._ck(lib().mpcd_get_state(self.h, *[_dp(out[k]) for k in self._STATE_KEYS]))
        return out

    def exchange(self, reset=True):
        """(Nc, 6): momentum and angular momentum the fluid gave each colloid since the last reset."""
        out = np.empty((self.Nc, 6))
        self._ck(lib().mpcd_exchange_read(self.h, _dp(out), 1 if reset else 0))
        return out

    def updown_velocity(self):
        """updown_velocity (cpp/run.cpp:28-50) on the current state.  Per colloid: `cnt`, `up_cnt`
        (rear-side fluid within sigma/2 + 0.5 and sigma/2 + 0.1), `vel_sum`, `up_vel_sum` (their
        velocity sums) and the slip velocities `vel` = vel_sum/cnt - V, `up_vel` = up_vel_sum/up_cnt
        - V (where the shell is empty, zero).  `reference` restates the routine's own arithmetic: its
        `vel` (cpp/run.cpp:48, taken only where up_cnt > 0, else the raw sum) and its `up_vel`, a
        single vector carried over the colloids (cpp/run.cpp:45-47)."""
        n = self.Nc
        cnt, up_cnt = np.zeros(n, np.int32), np.zeros(n, np.int32)
        vs, us = np.zeros((n, 3)), np.zeros((n, 3))
        self._ck(lib().mpcd_updown_velocity(self.h, cnt.ctypes.data_as(C.POINTER(C.c_int32)),
                                            up_cnt.ctypes.data_as(C.POINTER(C.c_int32)), _dp(vs), _dp(us)))
        V = self.get_colloids()["vel_colloid"]
        with np.errstate(invalid="ignore", divide="ignore"):
            vel = np.where(cnt[:, None] > 0, vs / np.maximum(cnt, 1)[:, None] - V, 0.0)
            up_vel = np.where(up_cnt[:, None] > 0, us / np.maximum(up_cnt, 1)[:, None] - V, 0.0)
        ref_vel = np.empty((n, 3))
        acc = np.zeros(3)
        for i in range(n):
            acc = acc + us[i]
            acc = acc / up_cnt[i] - V[i] if up_cnt[i] > 0 else acc
            ref_vel[i] = vs[i] / cnt[i] - V[i] if up_cnt[i] > 0 else vs[i]
        return dict(cnt=cnt, up_cnt=up_cnt, vel_sum=vs, up_vel_sum=us, vel=vel, up_vel=up_vel,
                    reference=dict(vel=ref_vel, up_vel=acc))

    def get_colloids(self):
        """The colloid arrays only (no fluid transfer)."""
        out = {k: np.empty((self.Nc, 3)) for k in ("pos_colloid", "vel_colloid", "ang_vel_colloid", "ra", "f")}
        self._ck(lib().mpcd_get_state(self.h, None, None, *[_dp(out[k]) for k in ("pos_colloid", "vel_colloid",
                                                                                 "ang_vel_colloid", "ra", "f")]))
        return out

    @property
    def step_count(self):
        return lib().mpcd_get_step(self.h)

    @step_count.setter
    def step_count(self, v):
        self._ck(lib().mpcd_set_step(self.h, v))

    # ---------------------------------------------------------------- routines
    def initialize(self, style=INIT_REFERENCE):
        self._ck(lib().mpcd_initialize(self.h, style))

    def setup(self):
        self._ck(lib().mpcd_setup(self.h))

    def rotation_mpcd(self):
        self._ck(lib().mpcd_rotation_mpcd(self.h))

    def run(self):
        self._ck(lib().mpcd_run(self.h))

    def substep(self, l):
        self._ck(lib().mpcd_substep(self.h, l))

    def update_pos_md(self):
        self._ck(lib().mpcd_update_pos_md(self.h))

    def neighbour_list_md(self):
        self._ck(lib().mpcd_neighbour_list_md(self.h))

    def update_pos_mpcd(self):
        self._ck(lib().mpcd_update_pos_mpcd(self.h))

    def neighbour_list_mpcd(self):
        self._ck(lib().mpcd_neighbour_list_mpcd(self.h))

    def fluid_colloid_collision(self):
        self._ck(lib().mpcd_fluid_colloid_collision(self.h))

    def update_activity_direction(self):
        self._ck(lib().mpcd_update_activity_direction(self.h))

    def compute_force_md(self):
        self._ck(lib().mpcd_compute_force_md(self.h))

    def update_velocity_colloid(self):
        self._ck(lib().mpcd_update_velocity_colloid(self.h))

    def substep_routines(self):
        """one substep as the eight routine calls, in the reference's order"""
        for n in SUBSTEP_ROUTINES:
            getattr(self, n)()

    def neighbour_md(self, cap=256):
        """the pair list of the last neighbour_list_md: per colloid its partners j > i (0-based)"""
        cnt = np.zeros(self.Nc, np.int32)
        lst = np.zeros((max(self.Nc, 1), cap), np.int32)
        self._ck(lib().mpcd_get_neighbour_md(self.h, cnt.ctypes.data_as(C.POINTER(C.c_int32)),
                                             lst.ctypes.data_as(C.POINTER(C.c_int32)), cap))
        return [lst[i, :min(cnt[i], cap)].copy() for i in range(self.Nc)]

    def box_binning(self):
        """the last neighbour_list_mpcd's box of each particle (1-based), occupancy of each box,
        candidate count of each colloid"""
        cell_of = np.empty(self.N, np.int32)
        occ = np.empty(self.C, np.int32)
        nn = np.empty(max(self.Nc, 1), np.int32)
        self._ck(lib().mpcd_get_box_binning(self.h, *[a.ctypes.data_as(C.POINTER(C.c_int32)) for a in (cell_of, occ, nn)]))
        return cell_of, occ, nn[:self.Nc]

    def step(self, nsteps=1):
        self._ck(lib().mpcd_step(self.h, nsteps))

    def step_async(self, nsteps=1):
        """enqueue nsteps steps without waiting; sync() waits and reports device errors"""
        self._ck(lib().mpcd_step_async(self.h, nsteps))

    def sync(self):
        self._ck(lib().mpcd_sync(self.h))

    def set_flight(self, on=True):
        """the free-flight schedule of mpcd_step (on by default; bit-identical results)"""
        self._ck(lib().mpcd_set_flight(self.h, 1 if on else 0))

    def flight_near(self):
        """near particles of the last free-flight step"""
        n = C.c_int32(0)
        self._ck(lib().mpcd_get_flight(self.h, C.byref(n)))
        return int(n.value)

    def diag(self):
        d = Diag()
        self._ck(lib().mpcd_diag(self.h, C.byref(d)))
        return d.as_dict()

    # ---------------------------------------------------------------- observables
    def rotation_binning(self):
        cell_of = np.empty(self.N, dtype=np.int32)
        occ = np.empty(self.C, dtype=np.int32)
        shift = np.empty(3)
        self._ck(lib().mpcd_get_rotation_binning(self.h, cell_of.ctypes.data_as(C.POINTER(C.c_int32)),
                                                 occ.ctypes.data_as(C.POINTER(C.c_int32)), _dp(shift)))
        return cell_of, occ, shift

    def shell_count(self):
        o = np.empty(self.Nc, dtype=np.int32)
        self._ck(lib().mpcd_get_shell_count(self.h, o.ctypes.data_as(C.POINTER(C.c_int32))))
        return o

    # ---------------------------------------------------------------- profiling
    def profile(self, on=True):
        self._ck(lib().mpcd_profile_enable(self.h, 1 if on else 0))

    def profile_read(self):
        cap = 64
        names = (C.c_char * 48 * cap)()
        launches = (C.c_int64 * cap)()
        ms = (C.c_double * cap)()
        n = lib().mpcd_profile_read(self.h, names, launches, ms, cap)
        return {bytes(names[i]).split(b"\0", 1)[0].decode(): (launches[i], ms[i]) for i in range(min(n, cap))}

    def trace_step(self, cap=1024):
        """One step (the state advances) traced: [(kernel, start_ms, end_ms)] in launch
        order, times from the step's start on the graph's own timeline."""
        names = (C.c_char * 48 * cap)()
        t0 = (C.c_double * cap)()
        t1 = (C.c_double * cap)()
        n = lib().mpcd_trace_step(self.h, names, t0, t1, cap)
        if n < 0:
            self._ck(n)
        return [(bytes(names[i]).split(b"\0", 1)[0].decode(), t0[i], t1[i]) for i in range(min(n, cap))]

    def set_launch(self, which, grid=0, block=32):
        """Launch shape of the event (LAUNCH_EVENTS) or colloid-finish (LAUNCH_FIN)
        kernel; grid 0 is the default, one block per SM (128 threads for the events,
        32 for the finish)."""
        self._ck(lib().mpcd_set_launch(self.h, which, grid, block))

    @property
    def launch_count(self):
        return lib().mpcd_launch_count(self.h)


class Ensemble:
    """Many independent FP32-compensated systems stepped together, one launch per
    stage over all of them (mpcd_ensemble_*).  `params` is a list of Params
    (make_params(..., precision=FP32C)); ens[r] is system r as a Simulation view."""

    def __init__(self, params):
        self.params = list(params)
        arr = (Params * len(self.params))(*self.params)
        h = C.c_void_p()
        r = lib().mpcd_ensemble_create(arr, len(self.params), C.byref(h))
        if r:
            raise MPCDError(r, "mpcd_ensemble_create rejected the parameters or could not allocate")
        self.h = h
        self.systems = [Simulation._view(lib().mpcd_ensemble_system(self.h, i), p) for i, p in enumerate(self.params)]

    def _ck(self, r):
        if r:
            raise MPCDError(r, lib().mpcd_ensemble_last_error(self.h).decode())

    def __len__(self):
        return len(self.systems)

    def __getitem__(self, i):
        return self.systems[i]

    def step(self, nsteps=1):
        self._ck(lib().mpcd_ensemble_step(self.h, nsteps))

    def set_launch(self, which, per_system=1, block=32):
        self._ck(lib().mpcd_ensemble_set_launch(self.h, which, per_system, block))

    def set_flight(self, on=True):
        """The batched step's schedule: free flight (default) or one pass per substep
        over every particle; both leave the same bits."""
        self._ck(lib().mpcd_ensemble_set_flight(self.h, 1 if on else 0))

    @property
    def flight(self):
        return bool(lib().mpcd_ensemble_get_flight(self.h))

    @property
    def launch_count(self):
        return lib().mpcd_ensemble_launch_count(self.h)

    def close(self):
        if getattr(self, "h", None):
            for s in self.systems:
                s.h = None
            lib().mpcd_ensemble_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def active_brownian(sim, nsteps, style=INIT_REFERENCE, diag_every=1):
    """The reference's main() (cpp/active_brownian.cpp:9-60): initialise, the
    prologue (create_box, neighbour lists, forces; tumble is part of initialize),
    then nsteps MPCD steps; returns the per-step diagnostics."""
    sim.initialize(style)
    sim.setup()
    out = []
    for s in range(nsteps):
        sim.step(1)
        if diag_every and (s + 1) % diag_every == 0:
            out.append(sim.diag())
    return out
