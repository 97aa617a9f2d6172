"""CPU restatement of the closure network (test infrastructure only).

The same MLP as brownian_gb300/csrc/mlp.cu (81 -> 256 -> 256 -> 256 -> 12, SiLU,
Gaussian negative log-likelihood of normalised targets) in numpy.  With
`bf16=True` every tensor the GPU stores in BF16 (normalised inputs, weights,
pre-activations, activations, output gradient, hidden gradients) is rounded to
BF16 at the same point, so the GPU's gradients can be checked tightly; with
`bf16=False` in float64 the backward pass is itself checked against finite
differences (tests/test_closure_oracle.py).
"""
import numpy as np

IN, H, OUT, NY = 81, 256, 12, 6
DIMS = [(IN, H), (H, H), (H, H), (H, OUT)]


def bf16(a):
    """Round float32 values to bfloat16 (nearest, ties to even), returned as float32."""
    a = np.ascontiguousarray(a, dtype=np.float32)
    b = a.view(np.uint32).astype(np.uint64)
    b = ((b + 0x7FFF + ((b >> 16) & 1)) >> 16) << 16
    return b.astype(np.uint32).view(np.float32)


def unflatten(p):
    """flat vector -> [(W, b)] in the order W1 [81][256], b1, ..., W4 [256][12], b4"""
    out, o = [], 0
    for k, n in DIMS:
        W = p[o:o + k * n].reshape(k, n)
        o += k * n
        b = p[o:o + n]
        o += n
        out.append((W, b))
    assert o == p.size
    return out


def param_count():
    return sum(k * n + n for k, n in DIMS)


def sig(z):
    return 1.0 / (1.0 + np.exp(-z))


def loss_and_grad(p, x, y, xmean, xstd, ymean, ystd, bf16_emul=True, dtype=np.float32):
    """Mean Gaussian NLL over the batch and its gradient w.r.t. the flat parameters."""
    r = bf16 if bf16_emul else (lambda a: np.asarray(a, dtype=dtype))
    layers = [(r(W), np.asarray(b, dtype=dtype)) for W, b in unflatten(np.asarray(p, dtype=dtype))]
    n = x.shape[0]
    xs = np.where(xstd > 0, 1.0 / np.where(xstd > 0, xstd, 1.0), 0.0).astype(dtype)
    ys = np.where(ystd > 0, 1.0 / np.where(ystd > 0, ystd, 1.0), 0.0).astype(dtype)
    a = r(np.clip((x - xmean) * xs, -6, 6))
    acts, zs = [a], []
    for l, (W, b) in enumerate(layers):
        z = a @ W + b
        if l < 3:
            zs.append(r(z))
            a = r(z * sig(z))
            acts.append(a)
        else:
            o = z
    t = (y - ymean) * ys
    mu, sraw = o[:, :NY], o[:, NY:]
    s = np.clip(sraw, -6, 6)
    e = np.exp(-s)
    d = t - mu
    loss = float(np.sum(0.5 * (d * d * e + s)) / n)
    dmu = -d * e / n
    ds = np.where(sraw == s, 0.5 * (1 - d * d * e) / n, 0.0)
    dcur = r(np.concatenate([dmu, ds], axis=1))
    grads = [None] * 4
    for l in range(3, -1, -1):
        W, _ = layers[l]
        grads[l] = (acts[l].T @ dcur, dcur.sum(axis=0))
        if l == 0:
            break
        z = zs[l - 1].astype(dtype)
        sz = sig(z)
        dcur = r((dcur @ W.T) * (sz * (1 + z * (1 - sz))))
    flat = np.concatenate([np.concatenate([gW.ravel(), gb]) for gW, gb in grads])
    return loss, flat


def forward(p, x, xmean, xstd, ymean, ystd, dtype=np.float64, bf16_emul=False):
    """Outputs in physical units: means (6) and log-variances (6).  With bf16_emul, in float32
    with every tensor the GPU stores in BF16 (normalised inputs, weights, activations) rounded
    to BF16 where it does, as loss_and_grad does."""
    if bf16_emul:
        dtype = np.float32
        r = bf16
    else:
        r = lambda a: a  # noqa: E731
    layers = [(r(np.asarray(W, dtype)), np.asarray(b, dtype)) for W, b in unflatten(np.asarray(p, dtype))]
    if bf16_emul:
        xs = np.where(xstd > 0, 1.0 / np.where(xstd > 0, xstd, 1.0), 0.0).astype(dtype)
        a = r(np.clip((np.asarray(x, dtype) - xmean) * xs, -6, 6))
    else:
        a = np.clip((x - xmean) / np.where(xstd > 0, xstd, np.inf), -6, 6)
    for l, (W, b) in enumerate(layers):
        z = a @ W + b
        a = r(z * sig(z)) if l < 3 else z
    return np.concatenate([a[:, :NY] * ystd + ymean, np.clip(a[:, NY:], -6, 6) + 2 * np.log(ystd)], axis=1)
