"""CPU restatement of the warm-start surrogate network (test infrastructure).

The U-Net of muphfasa_gb300/surrogate.py in NumPy: the same layers, weight
layout (Wt [Cout][9 Cin], tap-major), leaky ReLU slope, pooling, upsampling,
concatenation order and masked MSE loss, with its forward and backward pass
written out by hand.  With `bf16=True` it rounds to BF16 at the points where
the GPU kernels store BF16 (inputs, weights, activations, and the
pre-activation gradients fed to the GEMMs), so GPU gradients can be compared
layer by layer; with `bf16=False` it runs in float64 and is checked against
finite differences.  The network has no counterpart in the reference; only
tests import this module.
"""
from __future__ import annotations

import numpy as np

CHANS = (32, 64, 128, 256)
NAMES = ("e1a", "e1b", "e2a", "e2b", "e3a", "e3b", "e4a", "e4b", "d3a", "d3b", "d2a", "d2b", "d1a", "d1b", "head")
SLOPE = 0.1


def to_bf16(x):
    """Round float32 values to the nearest BF16 (ties to even), as float32."""
    a = np.ascontiguousarray(x, dtype=np.float32)
    b = a.view(np.uint32).astype(np.uint64)
    b = (b + 0x7FFF + ((b >> 16) & 1)) >> 16 << 16
    return b.astype(np.uint32).view(np.float32).reshape(a.shape)


class Net:
    def __init__(self, params, bf16=True):
        """params: {name: (Wt [Cout][K], bias [Cout])}."""
        self.bf16 = bf16
        self.dt = np.float32 if bf16 else np.float64
        self.p = {n: (np.asarray(w, self.dt), np.asarray(b, self.dt)) for n, (w, b) in params.items()}

    def q(self, x):
        return to_bf16(x) if self.bf16 else np.asarray(x, np.float64)

    # -- layers ---------------------------------------------------------------
    @staticmethod
    def im2col(x):
        Bn, H, W, Cc = x.shape
        xp = np.zeros((Bn, H + 2, W + 2, Cc), x.dtype)
        xp[:, 1:-1, 1:-1] = x
        cols = [xp[:, dy:dy + H, dx:dx + W] for dy in range(3) for dx in range(3)]
        return np.stack(cols, axis=3).reshape(Bn * H * W, 9 * Cc)

    @staticmethod
    def col2im(dcol, shape):
        Bn, H, W, Cc = shape
        d = dcol.reshape(Bn, H, W, 9, Cc)
        out = np.zeros((Bn, H + 2, W + 2, Cc), dcol.dtype)
        for dy in range(3):
            for dx in range(3):
                out[:, dy:dy + H, dx:dx + W] += d[:, :, :, dy * 3 + dx]
        return out[:, 1:-1, 1:-1]

    def conv_fwd(self, name, x, k3=True, act=True):
        Wt, b = self.p[name]
        Wq = self.q(Wt)
        A = self.im2col(x) if k3 else x.reshape(-1, x.shape[-1])
        y = (A.astype(np.float64) @ Wq.T.astype(np.float64)).astype(self.dt) + b
        if act:
            y = np.where(y < 0, y * self.dt(SLOPE), y)
        out = y if not act else self.q(y)
        self.cache[name] = (x, A, out, k3, act)
        return out.reshape(x.shape[:-1] + (Wt.shape[0],))

    def conv_bwd(self, name, dout, need_dx=True):
        x, A, out, k3, act = self.cache[name]
        Wt, _ = self.p[name]
        Wq = self.q(Wt)
        d = dout.reshape(-1, Wt.shape[0]).astype(self.dt)
        if act:
            d = np.where(out.reshape(d.shape) < 0, d * self.dt(SLOPE), d)
        self.grads[name] = None
        gb = d.sum(axis=0, dtype=np.float64).astype(self.dt)
        dq = self.q(d)
        gw = (dq.T.astype(np.float64) @ A.astype(np.float64)).astype(self.dt)
        self.grads[name] = (gw, gb)
        if not need_dx:
            return None
        dA = (dq.astype(np.float64) @ Wq.astype(np.float64)).astype(self.dt)
        if k3:
            return self.col2im(dA, x.shape)
        return dA.reshape(x.shape)

    def pool(self, x):
        s = x[:, 0::2, 0::2] + x[:, 0::2, 1::2]
        s = s + x[:, 1::2, 0::2]
        s = s + x[:, 1::2, 1::2]
        return self.q(self.dt(0.25) * s)

    def pool_bwd(self, d):
        return np.repeat(np.repeat(self.dt(0.25) * d, 2, axis=1), 2, axis=2)

    @staticmethod
    def up(x):
        return np.repeat(np.repeat(x, 2, axis=1), 2, axis=2)

    @staticmethod
    def up_bwd(d):
        return d[:, 0::2, 0::2] + d[:, 0::2, 1::2] + d[:, 1::2, 0::2] + d[:, 1::2, 1::2]

    # -- network --------------------------------------------------------------
    def forward(self, x):
        self.cache, self.grads = {}, {}
        c1, c2, c3, c4 = CHANS
        x = self.q(x)
        s1 = self.conv_fwd("e1b", self.conv_fwd("e1a", x))
        s2 = self.conv_fwd("e2b", self.conv_fwd("e2a", self.pool(s1)))
        s3 = self.conv_fwd("e3b", self.conv_fwd("e3a", self.pool(s2)))
        s4 = self.conv_fwd("e4b", self.conv_fwd("e4a", self.pool(s3)))
        t3 = self.conv_fwd("d3b", self.conv_fwd("d3a", np.concatenate([self.up(s4), s3], axis=-1)))
        t2 = self.conv_fwd("d2b", self.conv_fwd("d2a", np.concatenate([self.up(t3), s2], axis=-1)))
        t1 = self.conv_fwd("d1b", self.conv_fwd("d1a", np.concatenate([self.up(t2), s1], axis=-1)))
        return self.conv_fwd("head", t1, k3=False, act=False)

    def loss(self, pred, y, m):
        count = float(m.sum()) * pred.shape[-1]
        d = (pred - y) * m[..., None]
        return float((d.astype(np.float64) ** 2).sum()) / count, (2.0 / count) * d.astype(self.dt)

    def backward(self, dpred):
        c1, c2, c3, c4 = CHANS
        d = self.conv_bwd("d1b", self.conv_bwd("head", dpred))
        dcat1 = self.conv_bwd("d1a", d)
        dt2, ds1 = self.up_bwd(dcat1[..., :c2]), dcat1[..., c2:]
        dcat2 = self.conv_bwd("d2a", self.conv_bwd("d2b", dt2))
        dt3, ds2 = self.up_bwd(dcat2[..., :c3]), dcat2[..., c3:]
        dcat3 = self.conv_bwd("d3a", self.conv_bwd("d3b", dt3))
        ds4, ds3 = self.up_bwd(dcat3[..., :c4]), dcat3[..., c4:]
        dp3 = self.conv_bwd("e4a", self.conv_bwd("e4b", ds4))
        dp2 = self.conv_bwd("e3a", self.conv_bwd("e3b", ds3 + self.pool_bwd(dp3)))
        dp1 = self.conv_bwd("e2a", self.conv_bwd("e2b", ds2 + self.pool_bwd(dp2)))
        self.conv_bwd("e1a", self.conv_bwd("e1b", ds1 + self.pool_bwd(dp1)), need_dx=False)
        return self.grads


def init_params(seed=0, in_ch=8, out_ch=3):
    """Float64 parameters with the same shapes as the GPU network (for
    CPU-only checks)."""
    rng = np.random.default_rng(seed)
    c1, c2, c3, c4 = CHANS
    spec = [(in_ch, c1), (c1, c1), (c1, c2), (c2, c2), (c2, c3), (c3, c3), (c3, c4), (c4, c4),
            (c4 + c3, c3), (c3, c3), (c3 + c2, c2), (c2, c2), (c2 + c1, c1), (c1, c1)]
    p = {}
    for n, (a, b) in zip(NAMES[:-1], spec):
        p[n] = (rng.standard_normal((b, 9 * a)) * np.sqrt(2.0 / (9 * a)), 0.01 * rng.standard_normal(b))
    p["head"] = (0.1 * rng.standard_normal((out_ch, c1)) * np.sqrt(2.0 / c1), 0.01 * rng.standard_normal(out_ch))
    return p
