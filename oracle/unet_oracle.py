"""ORACLE — test infrastructure only.

numpy (float64) restatement of the learned preconditioner's U-Net
(neon_gb300/learned.py): 3x3x3 zero-padded convolutions, 2x2x2 average
pooling, nearest upsampling, ReLU, bias-free, with the same BF16 roundings of
weights, activations and backward signals as the GPU path (round-to-nearest-
even, written from the bfloat16 format) so that GPU and oracle differ only by
FP32-vs-FP64 accumulation. Used by tests to check the GPU forward pass and
gradients; never imported by the product.
"""
import numpy as np

LAYERS = [("c0a", 16, 16), ("c0b", 16, 16), ("c1a", 16, 32), ("c1b", 32, 32), ("c2a", 32, 64), ("c2b", 64, 64),
          ("c1c", 96, 32), ("c1d", 32, 32), ("c0c", 48, 16), ("c0d", 16, 16)]


def bf16(a):
    """Round float64/float32 values to the nearest bfloat16 (ties to even), returned as float64."""
    f = np.ascontiguousarray(a, np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    lsb = (u >> 16) & 1
    r = ((u + 0x7FFF + lsb) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def taps():
    return [(t // 9 - 1, (t // 3) % 3 - 1, t % 3 - 1) for t in range(27)]  # (dz, dy, dx)


def conv(x, w):
    """x [nz,ny,nx,cin], w [cout,27,cin] -> [nz,ny,nx,cout] (zero padding)."""
    nz, ny, nx, cin = x.shape
    xp = np.zeros((nz + 2, ny + 2, nx + 2, cin))
    xp[1:-1, 1:-1, 1:-1] = x
    y = np.zeros((nz, ny, nx, w.shape[0]))
    for t, (dz, dy, dx) in enumerate(taps()):
        y += xp[1 + dz:1 + dz + nz, 1 + dy:1 + dy + ny, 1 + dx:1 + dx + nx] @ w[:, t, :].T
    return y


def conv_bwd_weight(x, dy):
    """dw[co,t,ci] = sum_v dy[v,co] x[v+t,ci]."""
    nz, ny, nx, cin = x.shape
    xp = np.zeros((nz + 2, ny + 2, nx + 2, cin))
    xp[1:-1, 1:-1, 1:-1] = x
    dw = np.zeros((dy.shape[-1], 27, cin))
    D = dy.reshape(-1, dy.shape[-1])
    for t, (dz, dyy, dx) in enumerate(taps()):
        X = xp[1 + dz:1 + dz + nz, 1 + dyy:1 + dyy + ny, 1 + dx:1 + dx + nx].reshape(-1, cin)
        dw[:, t, :] = D.T @ X
    return dw


def conv_bwd_data(dy, w):
    """adjoint of conv: flipped taps, transposed channels."""
    wt = w[:, ::-1, :].transpose(2, 1, 0)  # [cin, 27, cout]
    return conv(dy, wt)


def pool(x):
    nz, ny, nx, c = x.shape
    return x.reshape(nz // 2, 2, ny // 2, 2, nx // 2, 2, c).mean(axis=(1, 3, 5))


def pool_bwd(dy):
    return np.repeat(np.repeat(np.repeat(dy, 2, 0), 2, 1), 2, 2) / 8.0


def up(x):
    return np.repeat(np.repeat(np.repeat(x, 2, 0), 2, 1), 2, 2)


def up_bwd(dy):
    nz, ny, nx, c = dy.shape
    return dy.reshape(nz // 2, 2, ny // 2, 2, nx // 2, 2, c).sum(axis=(1, 3, 5))


def relu(x):
    return np.maximum(x, 0.0)


def forward(W, r, n, rounding=True):
    """W: dict name -> [cout,27,cin] float; r: n^3 field (x fastest). Returns (z, cache)."""
    R = bf16 if rounding else (lambda a: np.asarray(a, np.float64))
    Wb = {k: R(v) for k, v in W.items()}
    sigma = np.sqrt(np.mean(np.asarray(r, np.float64) ** 2)) or 1.0
    in0 = np.zeros((n, n, n, 16))
    in0[..., 0] = R((np.asarray(r, np.float32) / np.float32(sigma)).reshape(n, n, n))
    a0 = R(relu(conv(in0, Wb["c0a"])))
    s0 = R(relu(conv(a0, Wb["c0b"])))
    p0 = R(pool(s0))
    a1 = R(relu(conv(p0, Wb["c1a"])))
    s1 = R(relu(conv(a1, Wb["c1b"])))
    p1 = R(pool(s1))
    a2 = R(relu(conv(p1, Wb["c2a"])))
    b2 = R(relu(conv(a2, Wb["c2b"])))
    cat1 = np.concatenate([up(b2), s1], axis=-1)
    d1a = R(relu(conv(cat1, Wb["c1c"])))
    d1b = R(relu(conv(d1a, Wb["c1d"])))
    cat0 = np.concatenate([up(d1b), s0], axis=-1)
    d0a = R(relu(conv(cat0, Wb["c0c"])))
    out = conv(d0a, Wb["c0d"])
    z = out[..., 0].ravel() * sigma
    cache = dict(Wb=Wb, sigma=sigma, in0=in0, a0=a0, s0=s0, p0=p0, a1=a1, s1=s1, p1=p1, a2=a2, b2=b2, cat1=cat1, d1a=d1a,
                 d1b=d1b, cat0=cat0, d0a=d0a, n=n, R=R)
    return z, cache


def backward(cache, dz):
    """dL/dW given dL/dz, mirroring the GPU's BF16 rounding of backward signals."""
    c = cache
    R, Wb, n = c["R"], c["Wb"], c["n"]
    g = {}
    gout = np.zeros((n, n, n, 16))
    gout[..., 0] = (np.asarray(dz, np.float64) * c["sigma"]).reshape(n, n, n)
    dy = R(gout)
    g["c0d"] = conv_bwd_weight(c["d0a"], dy)
    gd0a = conv_bwd_data(dy, Wb["c0d"])
    dy = R(gd0a * (c["d0a"] > 0))
    g["c0c"] = conv_bwd_weight(c["cat0"], dy)
    gcat0 = conv_bwd_data(dy, Wb["c0c"])
    g1 = up_bwd(gcat0[..., :32])
    dy = R(g1 * (c["d1b"] > 0))
    g["c1d"] = conv_bwd_weight(c["d1a"], dy)
    g1 = conv_bwd_data(dy, Wb["c1d"])
    dy = R(g1 * (c["d1a"] > 0))
    g["c1c"] = conv_bwd_weight(c["cat1"], dy)
    gcat1 = conv_bwd_data(dy, Wb["c1c"])
    g2 = up_bwd(gcat1[..., :64])
    dy = R(g2 * (c["b2"] > 0))
    g["c2b"] = conv_bwd_weight(c["a2"], dy)
    g2 = conv_bwd_data(dy, Wb["c2b"])
    dy = R(g2 * (c["a2"] > 0))
    g["c2a"] = conv_bwd_weight(c["p1"], dy)
    gp1 = conv_bwd_data(dy, Wb["c2a"])
    gs1 = gcat1[..., 64:] + pool_bwd(gp1)
    dy = R(gs1 * (c["s1"] > 0))
    g["c1b"] = conv_bwd_weight(c["a1"], dy)
    g1 = conv_bwd_data(dy, Wb["c1b"])
    dy = R(g1 * (c["a1"] > 0))
    g["c1a"] = conv_bwd_weight(c["p0"], dy)
    gp0 = conv_bwd_data(dy, Wb["c1a"])
    gs0 = gcat0[..., 32:] + pool_bwd(gp0)
    dy = R(gs0 * (c["s0"] > 0))
    g["c0b"] = conv_bwd_weight(c["a0"], dy)
    g0 = conv_bwd_data(dy, Wb["c0b"])
    dy = R(g0 * (c["a0"] > 0))
    g["c0a"] = conv_bwd_weight(c["in0"], dy)
    return g
