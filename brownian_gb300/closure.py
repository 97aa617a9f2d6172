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


def train(net, X, Y, epochs=20, batch=4096, lr=1e-3, seed=0, log=None):
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
