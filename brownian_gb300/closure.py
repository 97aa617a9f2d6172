"""The learned closure: a network that predicts, from a colloid's own motion and
its neighbourhood, the mean and spread of the momentum and angular momentum the
fluid gives it in one MPCD step, so that colloid-only runs can skip the fluid.

* `features`: the 81 inputs of each colloid (velocity, angular velocity and
  orientation; relative positions and velocities of up to 12 nearest colloids
  within three radii, nearest first, zero-padded).
* `generate`: training samples from full MPCD runs (the exact collision kernel's
  exchange record, mpcd_exchange_read), with the activity v0 swept.
* `Network`: the GPU network (csrc/mlp.cu): BF16 tensor-core forward, backward
  and Adam; `train` runs epochs of shuffled mini-batches on the GPU.

Device buffers are torch tensors (plumbing only); every operation is this
library's own kernels.
"""
import ctypes as C

import numpy as np

from . import FP32C, INIT_PHYSICAL, MPCDError, Simulation, lib

IN, OUT, NY = 81, 12, 6
K_NEAR = 12


def features(state, L, radius, k_near=K_NEAR):
    """(Nc, 81) float32 features of every colloid from a state dict (get_state or
    get_colloids): V, Omega, ra, then for the k_near nearest colloids within 3 radii
    the minimum-image relative position and the relative velocity."""
    X = np.asarray(state["pos_colloid"], dtype=np.float64)
    V = np.asarray(state["vel_colloid"], dtype=np.float64)
    W = np.asarray(state["ang_vel_colloid"], dtype=np.float64)
    ra = np.asarray(state["ra"], dtype=np.float64)
    nc = X.shape[0]
    Ls = np.array([L, L, L], dtype=np.float64) if np.isscalar(L) else np.asarray(L, dtype=np.float64)
    out = np.zeros((nc, IN), dtype=np.float32)
    out[:, 0:3], out[:, 3:6], out[:, 6:9] = V, W, ra
    if nc > 1:
        d = X[None, :, :] - X[:, None, :]
        d -= Ls * np.round(d / Ls)
        r2 = np.sum(d * d, axis=2)
        np.fill_diagonal(r2, np.inf)
        cut2 = (3.0 * radius) ** 2
        order = np.argsort(r2, axis=1, kind="stable")[:, :k_near]
        for j in range(nc):
            m = 0
            for k in order[j]:
                if r2[j, k] >= cut2:
                    break
                out[j, 9 + 6 * m:12 + 6 * m] = d[j, k]
                out[j, 12 + 6 * m:15 + 6 * m] = V[k] - V[j]
                m += 1
    return out


def generate(L, n_colloid, radius=2.0, density=10, steps=200, v0_values=(0.0, 0.025, 0.05, 0.075, 0.1), seed=0,
             warmup=20, Dr=0.001):
    """Samples (X (n, 81), Y (n, 6)) from full FP32-compensated MPCD runs of an L^3 box,
    one run per v0: features at the start of each step, the fluid's exchange over it."""
    M = density * 4.0 / 3.0 * np.pi * radius ** 3
    Xs, Ys = [], []
    for i, v0 in enumerate(v0_values):
        sim = Simulation(L, L ** 3 * density, n_colloid, n_sub=10, mass_colloid=M, sig_colloid=2 * radius,
                         sigma=2 * radius, I_colloid=0.4 * M * radius ** 2, v0=v0, theta_deg=90.0, Dr=Dr,
                         seed=seed * 1000 + i, precision=FP32C)
        sim.initialize(INIT_PHYSICAL)
        sim.setup()
        sim.step(warmup)
        sim.exchange(reset=True)
        for _ in range(steps):
            Xs.append(features(sim.get_colloids(), L, radius))
            sim.step(1)
            Ys.append(sim.exchange(reset=True).astype(np.float32))
        sim.close()
    return np.concatenate(Xs), np.concatenate(Ys)


class Network:
    """The closure network on the GPU (mpcd_mlp_*)."""

    def __init__(self, max_batch=16384, seed=0):
        L = lib()
        vp = C.c_void_p
        L.mpcd_mlp_create.argtypes = [C.c_int, C.c_uint64, C.POINTER(vp)]
        L.mpcd_mlp_destroy.argtypes = [vp]
        L.mpcd_mlp_last_error.argtypes = [vp]
        L.mpcd_mlp_last_error.restype = C.c_char_p
        L.mpcd_mlp_param_count.argtypes = [vp]
        L.mpcd_mlp_param_count.restype = C.c_int64
        fp = C.POINTER(C.c_float)
        L.mpcd_mlp_set_normalisation.argtypes = [vp, fp, fp, fp, fp]
        L.mpcd_mlp_get_params.argtypes = [vp, fp]
        L.mpcd_mlp_set_params.argtypes = [vp, fp]
        L.mpcd_mlp_forward.argtypes = [vp, vp, C.c_int, vp, vp]
        L.mpcd_mlp_grad.argtypes = [vp, vp, vp, C.c_int, fp, C.POINTER(C.c_double)]
        L.mpcd_mlp_train_step.argtypes = [vp, vp, vp, C.c_int, C.c_float, C.POINTER(C.c_double)]
        L.mpcd_mlp_set_fault.argtypes = [vp, C.c_int]
        self.max_batch = max_batch
        h = vp()
        r = L.mpcd_mlp_create(max_batch, seed, C.byref(h))
        if r:
            raise MPCDError(r, "mpcd_mlp_create failed")
        self.h = h
        self.n_params = L.mpcd_mlp_param_count(h)
        self.norm = None

    def _ck(self, r):
        if r:
            raise MPCDError(r, lib().mpcd_mlp_last_error(self.h).decode())

    @staticmethod
    def _fp(a):
        return np.ascontiguousarray(a, dtype=np.float32).ctypes.data_as(C.POINTER(C.c_float))

    def set_normalisation(self, xmean, xstd, ymean, ystd):
        self.norm = [np.ascontiguousarray(a, dtype=np.float32) for a in (xmean, xstd, ymean, ystd)]
        self._ck(lib().mpcd_mlp_set_normalisation(self.h, *[self._fp(a) for a in self.norm]))

    def fit_normalisation(self, X, Y):
        xm, xs = X.mean(axis=0), X.std(axis=0)
        xs = np.where(xs > 1e-12, xs, 0.0)  # constant (always padded) inputs are switched off
        self.set_normalisation(xm, xs, Y.mean(axis=0), np.maximum(Y.std(axis=0), 1e-12))

    def params(self):
        out = np.empty(self.n_params, dtype=np.float32)
        self._ck(lib().mpcd_mlp_get_params(self.h, out.ctypes.data_as(C.POINTER(C.c_float))))
        return out

    def set_params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32)
        self._ck(lib().mpcd_mlp_set_params(self.h, p.ctypes.data_as(C.POINTER(C.c_float))))

    def forward(self, x_dev, out_dev, rows, stream=0):
        """x_dev, out_dev: device pointers (rows x 81, rows x 12 float32)."""
        self._ck(lib().mpcd_mlp_forward(self.h, C.c_void_p(x_dev), rows, C.c_void_p(out_dev), C.c_void_p(stream)))

    def grad(self, x_dev, y_dev, rows):
        g = np.empty(self.n_params, dtype=np.float32)
        loss = C.c_double()
        self._ck(lib().mpcd_mlp_grad(self.h, C.c_void_p(x_dev), C.c_void_p(y_dev), rows,
                                     g.ctypes.data_as(C.POINTER(C.c_float)), C.byref(loss)))
        return loss.value, g

    def set_fault(self, on=True):
        """Test hook: the training products issue nothing, so their bounded waits run out."""
        self._ck(lib().mpcd_mlp_set_fault(self.h, 1 if on else 0))

    def train_step(self, x_dev, y_dev, rows, lr):
        loss = C.c_double()
        self._ck(lib().mpcd_mlp_train_step(self.h, C.c_void_p(x_dev), C.c_void_p(y_dev), rows, lr, C.byref(loss)))
        return loss.value

    def close(self):
        if getattr(self, "h", None):
            lib().mpcd_mlp_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def nll(net, X, Y):
    """Mean Gaussian negative log-likelihood of (X, Y) under the network, in chunks."""
    import torch
    Xd = torch.from_numpy(np.ascontiguousarray(X, dtype=np.float32)).cuda()
    Yd = torch.from_numpy(np.ascontiguousarray(Y, dtype=np.float32)).cuda()
    tot, n = 0.0, X.shape[0]
    for b0 in range(0, n, net.max_batch):
        rows = min(net.max_batch, n - b0)
        l, _ = net.grad(Xd[b0:].data_ptr(), Yd[b0:].data_ptr(), rows)
        tot += l * rows
    return tot / n


def free_nll(Y_train, Y):
    """The same likelihood without the network: targets as N(mean, std) of the training set."""
    ym, ys = Y_train.mean(0), Y_train.std(0)
    return float(np.mean(np.sum(0.5 * ((Y - ym) / ys) ** 2, axis=1)))


def train(net, X, Y, epochs=20, batch=4096, lr=3e-4, seed=0, log=None):
    """Adam over shuffled mini-batches on the GPU; returns the mean loss of each epoch."""
    import torch
    rng = np.random.default_rng(seed)
    Xd = torch.from_numpy(np.ascontiguousarray(X, dtype=np.float32)).cuda()
    Yd = torch.from_numpy(np.ascontiguousarray(Y, dtype=np.float32)).cuda()
    n = X.shape[0]
    losses = []
    for ep in range(epochs):
        perm = torch.from_numpy(rng.permutation(n)).cuda()
        xs, ys = Xd[perm].contiguous(), Yd[perm].contiguous()
        tot, cnt = 0.0, 0
        for b0 in range(0, n - batch + 1 if n >= batch else 1, batch):
            rows = min(batch, n - b0)
            l = net.train_step(xs[b0:].data_ptr(), ys[b0:].data_ptr(), rows, lr)
            tot += l * rows
            cnt += rows
        losses.append(tot / max(cnt, 1))
        if log:
            log(ep, losses[-1])
    return losses


class Surrogate:
    """Colloid-only dynamics with the closure network (mpcd_surrogate_*)."""

    def __init__(self, params, net):
        L = lib()
        vp, dp = C.c_void_p, C.POINTER(C.c_double)
        from . import Params
        L.mpcd_surrogate_create.argtypes = [C.POINTER(Params), vp, C.POINTER(vp)]
        L.mpcd_surrogate_destroy.argtypes = [vp]
        L.mpcd_surrogate_last_error.argtypes = [vp]
        L.mpcd_surrogate_last_error.restype = C.c_char_p
        L.mpcd_surrogate_set_state.argtypes = [vp, dp, dp, dp, dp]
        L.mpcd_surrogate_get_state.argtypes = [vp, dp, dp, dp, dp]
        L.mpcd_surrogate_features.argtypes = [vp, C.POINTER(C.c_float), C.c_int]
        L.mpcd_surrogate_step.argtypes = [vp, C.c_int]
        L.mpcd_surrogate_set_fault.argtypes = [vp, C.c_int]
        L.mpcd_surrogate_set_noise.argtypes = [vp, C.c_double]
        self.params, self.net = params, net
        self.Nc = params.n_colloid
        h = vp()
        r = L.mpcd_surrogate_create(C.byref(params), net.h, C.byref(h))
        if r:
            raise MPCDError(r, "mpcd_surrogate_create rejected the parameters")
        self.h = h

    def _ck(self, r):
        if r:
            raise MPCDError(r, lib().mpcd_surrogate_last_error(self.h).decode())

    @staticmethod
    def _dp(a):
        return a.ctypes.data_as(C.POINTER(C.c_double))

    def set_state(self, pos, vel, ang_vel, ra):
        a = [np.ascontiguousarray(x, dtype=np.float64).reshape(self.Nc, 3) for x in (pos, vel, ang_vel, ra)]
        self._ck(lib().mpcd_surrogate_set_state(self.h, *[self._dp(x) for x in a]))

    def set_fault(self, drop_chunk=-1):
        """test hook: the network kernel's producer skips weight chunk drop_chunk (-1: none)"""
        self._ck(lib().mpcd_surrogate_set_fault(self.h, int(drop_chunk)))

    def set_noise(self, scale=1.0):
        """fluctuation of the drawn exchange: 1 the network's variance, 0 the mean only"""
        self._ck(lib().mpcd_surrogate_set_noise(self.h, float(scale)))

    def get_state(self):
        out = {k: np.empty((self.Nc, 3)) for k in ("pos_colloid", "vel_colloid", "ang_vel_colloid", "ra")}
        self._ck(lib().mpcd_surrogate_get_state(self.h, *[self._dp(out[k]) for k in
                                                           ("pos_colloid", "vel_colloid", "ang_vel_colloid", "ra")]))
        return out

    def features(self, recompute=True):
        out = np.empty((self.Nc, IN), dtype=np.float32)
        self._ck(lib().mpcd_surrogate_features(self.h, out.ctypes.data_as(C.POINTER(C.c_float)), 1 if recompute else 0))
        return out

    def outputs(self):
        """The network's outputs of the last step in physical units (means 6, log-variances 6)."""
        out = np.empty((self.Nc, NY * 2), dtype=np.float32)
        f = lib().mpcd_surrogate_outputs
        f.argtypes = [C.c_void_p, C.POINTER(C.c_float)]
        self._ck(f(self.h, out.ctypes.data_as(C.POINTER(C.c_float))))
        return out

    def step(self, nsteps=1):
        self._ck(lib().mpcd_surrogate_step(self.h, nsteps))

    def fast_steps(self):
        """Steps in which some colloid moved more than half the force-partner skin."""
        f = lib().mpcd_surrogate_fast_steps
        f.argtypes = [C.c_void_p, C.POINTER(C.c_int64)]
        c = C.c_int64()
        self._ck(f(self.h, C.byref(c)))
        return c.value

    def close(self):
        if getattr(self, "h", None):
            lib().mpcd_surrogate_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ------------------------------------------------------------------ statistics

def unwrap(traj, L):
    """(T, Nc, 3) wrapped positions -> unwrapped (minimum-image increments)."""
    d = np.diff(traj, axis=0)
    d -= L * np.round(d / L)
    return np.concatenate([traj[:1], traj[:1] + np.cumsum(d, axis=0)])


def msd(U, lags):
    return np.array([np.mean(np.sum((U[lag:] - U[:-lag]) ** 2, axis=2)) for lag in lags])


def autocorr(A, lags):
    """<a(t) . a(t + lag)> over time origins and colloids."""
    return np.array([np.mean(np.sum(A[lag:] * A[:len(A) - lag], axis=2)) if lag else np.mean(np.sum(A * A, axis=2))
                     for lag in lags])


# ------------------------------------------------------------------ end to end

def _sim(p):
    from . import Params
    kw = {k: getattr(p, k) for k, _ in Params._fields_ if k not in ("Lx", "Ly", "Lz", "n_fluid", "n_colloid")}
    return Simulation(p.Lx, p.n_fluid, p.n_colloid, **kw)


def generate_gpu(params_list, steps, warmup=20, net=None):
    """Samples from full MPCD runs, one per Params: the features (computed on the GPU by
    the surrogate's feature kernel) at the start of every step and the exchange over it."""
    Xs, Ys = [], []
    feat_net = net if net is not None else Network(max_batch=max(p.n_colloid for p in params_list))
    for p in params_list:
        sim = _sim(p)
        sim.initialize(INIT_PHYSICAL)
        sim.setup()
        sim.step(warmup)
        sim.exchange(reset=True)
        feat = Surrogate(p, feat_net)
        for _ in range(steps):
            c = sim.get_colloids()
            feat.set_state(c["pos_colloid"], c["vel_colloid"], c["ang_vel_colloid"], c["ra"])
            Xs.append(feat.features())
            sim.step(1)
            Ys.append(sim.exchange(reset=True).astype(np.float32))
        feat.close()
        sim.close()
    if net is None:
        feat_net.close()
    return np.concatenate(Xs), np.concatenate(Ys)


def compare(p, net, steps, warmup=20, lags=(1, 2, 5, 10, 20, 50, 100), vlags=(0, 1, 2, 5, 10, 20),
            olags=(0, 10, 50, 100), blocks=4):
    """Full MPCD (the yardstick) against colloid-only dynamics from the same colloid state:
    the closure (the network's mean and variance), the closure's mean only (the drag without
    the fluctuations), and no fluid exchange at all.  Each run is `blocks` consecutive
    stretches of `steps` / `blocks` steps; per stretch the MSD, velocity and orientation
    autocorrelations on the GPU; reported as the mean over stretches with its standard error
    (stretches longer than the largest lag are close to independent).  Also the time per MPCD
    step of the full run and of the closure."""
    import time
    full = _sim(p)
    full.initialize(INIT_PHYSICAL)
    full.setup()
    full.step(warmup)
    c0 = full.get_colloids()
    t0 = time.perf_counter()
    full.step(20)
    full.get_colloids()
    t_full = (time.perf_counter() - t0) / 20
    L = float(p.Lx)
    lag_kw = dict(msd_lags=lags, vacf_lags=vlags, oacf_lags=olags)
    per = steps // blocks
    stats = {"full": block_stats(full, per, blocks, L, **lag_kw)}
    full.close()
    sur = Surrogate(p, net)
    sur.set_state(c0["pos_colloid"], c0["vel_colloid"], c0["ang_vel_colloid"], c0["ra"])
    sur.step(5)
    t0 = time.perf_counter()
    sur.step(100)
    t_sur = (time.perf_counter() - t0) / 100
    sur.set_state(c0["pos_colloid"], c0["vel_colloid"], c0["ang_vel_colloid"], c0["ra"])
    stats["closure"] = block_stats(sur, per, blocks, L, **lag_kw)
    fast = {"closure": sur.fast_steps()}
    sur.set_noise(0.0)
    sur.set_state(c0["pos_colloid"], c0["vel_colloid"], c0["ang_vel_colloid"], c0["ra"])
    stats["mean_only"] = block_stats(sur, per, blocks, L, **lag_kw)
    sur.close()
    none_net = Network(max_batch=p.n_colloid)
    none_net.set_normalisation(np.zeros(IN), np.ones(IN), np.zeros(NY), np.full(NY, 1e-20))
    none_net.set_params(np.zeros(none_net.n_params))
    bare = Surrogate(p, none_net)
    bare.set_state(c0["pos_colloid"], c0["vel_colloid"], c0["ang_vel_colloid"], c0["ra"])
    stats["no_closure"] = block_stats(bare, per, blocks, L, **lag_kw)
    fast["no_closure"] = bare.fast_steps()
    bare.close()
    none_net.close()
    out = {"t_full_ms": t_full * 1e3, "t_surrogate_ms": t_sur * 1e3, "speedup": t_full / t_sur}
    out["stats"] = stats
    out["fast_steps"] = fast  # steps in which a colloid outran half its force-partner skin
    out["lags"] = {"msd": list(lags), "vacf": list(vlags), "oacf": list(olags)}
    out["blocks"] = blocks
    rel, err = {}, {}
    f = stats["full"]
    for name in ("closure", "mean_only", "no_closure"):
        rel[name], err[name] = {}, {}
        for k in ("msd", "vacf", "oacf"):
            m, e = np.array(stats[name][k]), np.array(stats[name][k + "_stderr"])
            mf, ef = np.array(f[k]), np.array(f[k + "_stderr"])
            with np.errstate(divide="ignore", invalid="ignore"):
                rel[name][k] = (m / mf - 1.0).tolist()
                err[name][k] = np.sqrt((e / np.abs(mf)) ** 2 + (m * ef / mf ** 2) ** 2).tolist()
    out["rel_diff_vs_full"] = rel
    out["rel_diff_stderr"] = err
    return out


def block_stats(obj, steps, blocks, L, **lags):
    """device_stats of `blocks` consecutive stretches of `steps` steps: per quantity the mean
    over the stretches and (key + "_stderr") its standard error."""
    per = [device_stats(obj, steps, L, **lags) for _ in range(blocks)]
    out = {}
    for k in ("msd", "vacf", "oacf"):
        a = np.array([q[k] for q in per])
        out[k] = a.mean(0).tolist()
        out[k + "_stderr"] = (a.std(0, ddof=1) / np.sqrt(blocks)).tolist() if blocks > 1 else [float("nan")] * a.shape[1]
    return out


def device_stats(obj, steps, L, **lags):
    """MSD / VACF / OACF of `steps` steps of a Simulation or Surrogate, the frames kept and
    reduced on the GPU (a Trajectory; no host copy per step).  Same numbers as msd / autocorr
    on the host trajectory, to rounding."""
    from . import Trajectory
    tr = Trajectory(obj.Nc, steps + 1, L)
    try:
        tr.record(obj)
        for _ in range(steps):
            obj.step(1)
            tr.record(obj)
        return {k: v.tolist() for k, v in tr.analyse(**lags).items()}
    finally:
        tr.close()


def demo(colloids=500, fraction=0.1, steps=30, seed=5):
    """The colloid-only step with a random network (means and log-variances of order one,
    exchange standard deviation 0.5) on randomly placed colloids of radius 2: a fixed
    workload for timing and profiling the step's kernels.  Returns the state."""
    import brownian_gb300 as bg
    R = 2.0
    L = int(round((colloids * 4.0 / 3.0 * np.pi * R ** 3 / fraction) ** (1.0 / 3.0)))
    M = bg.displaced_mass(R, 10)
    p = bg.make_params(L, 1, colloids, n_sub=10, mass_colloid=M, sig_colloid=4.0, sigma=4.0, I_colloid=0.4 * M * 4.0,
                       v0=0.05, theta_deg=90.0, Dr=0.001, seed=seed)
    rng = np.random.default_rng(seed)
    pos = []
    while len(pos) < colloids:  # random sequential placement, centre distance >= 4.3
        x = rng.uniform(0, L, 3)
        if pos:
            d = np.array(pos) - x
            d -= L * np.round(d / L)
            if np.min(np.sum(d * d, axis=1)) < 4.3 ** 2:
                continue
        pos.append(x)
    vel = rng.normal(0, 0.05, (colloids, 3))
    w = rng.normal(0, 0.02, (colloids, 3))
    ra = rng.normal(0, 1, (colloids, 3))
    ra /= np.linalg.norm(ra, axis=1, keepdims=True)
    net = Network(max_batch=max(colloids, 16), seed=seed)
    net.set_params(rng.normal(0, 0.05, net.n_params).astype(np.float32))
    net.set_normalisation(rng.normal(0, 0.1, IN).astype(np.float32), rng.uniform(0.5, 2, IN).astype(np.float32),
                          np.zeros(NY, np.float32), np.full(NY, 0.5, np.float32))
    sur = Surrogate(p, net)
    try:
        sur.set_state(np.array(pos), vel, w, ra)
        sur.step(steps)
        return sur.get_state()
    finally:
        sur.close()
        net.close()


def train_demo(batch=8192, steps=20, seed=0):
    """Training steps of the network on random data of `batch` rows (timing and profiling of
    the training kernels): ms per step by CUDA events, and the FLOP rate of the layer products
    that run on the tcgen05 path (forward and backward data: 2 x batch x 589,824 FLOP a step)."""
    import torch
    rng = np.random.default_rng(seed)
    x = torch.from_numpy(rng.normal(0, 1, (batch, IN)).astype(np.float32)).cuda()
    y = torch.from_numpy(rng.normal(0, 1, (batch, NY)).astype(np.float32)).cuda()
    net = Network(max_batch=batch, seed=seed)
    try:
        net.set_normalisation(np.zeros(IN, np.float32), np.ones(IN, np.float32), np.zeros(NY, np.float32),
                              np.ones(NY, np.float32))
        for _ in range(3):
            net.train_step(x.data_ptr(), y.data_ptr(), batch, 1e-3)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(steps):
            loss = net.train_step(x.data_ptr(), y.data_ptr(), batch, 1e-3)
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / steps
        inp, h, outp = 96, 256, 16  # the padded layer widths the products run at
        flop = 2.0 * batch * (inp * h + 2 * h * h + h * outp) + 2.0 * batch * (outp * h + 2 * h * h)
        return {"batch": batch, "ms_per_step": ms, "loss": loss, "tc_flop_per_step": flop}
    finally:
        net.close()


if __name__ == "__main__":
    import argparse
    ap = argparse.ArgumentParser(description="colloid-only step with a random network, or training steps on random "
                                             "data (timing and profiling)")
    ap.add_argument("what", choices=["demo", "train"])
    ap.add_argument("--colloids", type=int, default=500)
    ap.add_argument("--fraction", type=float, default=0.1)
    ap.add_argument("--steps", type=int, default=30)
    ap.add_argument("--batch", type=int, default=8192)
    a = ap.parse_args()
    if a.what == "train":
        print("ok", train_demo(a.batch, a.steps))
    else:
        st = demo(a.colloids, a.fraction, a.steps)
        print("ok", {k: float(np.abs(v).max()) for k, v in st.items()})
