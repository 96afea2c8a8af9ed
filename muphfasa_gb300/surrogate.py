"""Warm-start surrogate: a 4-level convolutional U-Net (about 2M parameters,
BF16 weights and activations, FP32 accumulation and master weights) that
predicts the steady (rho, u) of a 2-D D2Q9 case from its geometry and
parameters.  No counterpart in the reference.

Everything runs on the GPU through the library's own kernels (mph_nn_*:
tensor-core GEMMs, im2col / col2im, activations, pooling, upsampling, loss,
Adam); this module only sequences them and owns the device buffers.

Layout: activations NHWC as [P][C] rows (P = batch x H x W); a 3 x 3 conv
keeps FP32 master weights Wt [Cout][9 Cin] (tap-major, channel-minor), a BF16
copy for the GEMMs, a bias, Adam moments and gradients.

  encoder  8 -> 32 -> 32 | pool | 64, 64 | pool | 128, 128 | pool | 256, 256
  decoder  up + skip -> 128, 128 | up + skip -> 64, 64 | up + skip -> 32, 32
  head     1 x 1 conv 32 -> 3 (no activation)

H and W must be multiples of 8.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import check, lib

IN_CH = 8
OUT_CH = 3
CHANS = (32, 64, 128, 256)


class Dev:
    """One device buffer (mph_nn_alloc / mph_nn_free)."""

    def __init__(self, nbytes: int):
        self.nbytes = int(nbytes)
        p = C.c_void_p()
        check(lib().mph_nn_alloc(C.c_longlong(self.nbytes), C.byref(p)))
        self.p = p

    @property
    def ptr(self):
        return self.p

    def upload(self, arr: np.ndarray):
        a = np.ascontiguousarray(arr)
        assert a.nbytes <= self.nbytes
        check(lib().mph_nn_copy(self.p, a.ctypes.data_as(C.c_void_p), C.c_longlong(a.nbytes), 0, None))

    def download(self, n: int, dtype=np.float32) -> np.ndarray:
        out = np.empty(n, dtype=dtype)
        check(lib().mph_nn_copy(out.ctypes.data_as(C.c_void_p), self.p, C.c_longlong(out.nbytes), 1, None))
        return out

    def close(self):
        if getattr(self, "p", None) is not None and self.p.value:
            lib().mph_nn_free(self.p)
        self.p = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _f32(n):
    return Dev(4 * int(n))


def _bf(n):
    return Dev(2 * int(n))


_L = None


def _lib():
    global _L
    if _L is None:
        L = lib()
        P, LL, I, F, fp = C.c_void_p, C.c_longlong, C.c_int, C.c_float, C.c_void_p
        L.mph_nn_gemm.argtypes = [I, I, I, P, LL, I, P, LL, I, fp, LL, I, P]
        L.mph_nn_im2col3.argtypes = [P, I, I, I, I, P, P]
        L.mph_nn_col2im3.argtypes = [fp, I, I, I, I, fp, P]
        L.mph_nn_bias_act.argtypes = [fp, fp, LL, I, I, P, fp, I, I, P]
        L.mph_nn_act_bwd.argtypes = [fp, I, I, P, I, I, LL, I, I, fp, P]
        L.mph_nn_colsum.argtypes = [fp, LL, I, fp, P]
        L.mph_nn_pool.argtypes = [P, I, I, I, I, P, P]
        L.mph_nn_pool_bwd.argtypes = [fp, I, I, I, I, fp, P]
        L.mph_nn_up.argtypes = [P, I, I, I, I, P, I, I, P]
        L.mph_nn_up_bwd.argtypes = [fp, I, I, I, I, I, I, fp, P]
        L.mph_nn_slice.argtypes = [I, P, I, I, LL, I, P, I, I, I, P]
        L.mph_nn_mse.argtypes = [fp, fp, fp, LL, I, F, fp, fp, I, P]
        L.mph_nn_adam.argtypes = [fp, fp, fp, fp, LL, F, F, F, F, I, F, F, P]
        L.mph_nn_sumsq.argtypes = [fp, LL, fp, I, P]
        L.mph_nn_cast.argtypes = [I, P, LL, P, P]
        L.mph_nn_fill.argtypes = [fp, LL, F, P]
        L.mph_nn_transpose.argtypes = [P, LL, I, P, P]
        L.mph_nn_wflip.argtypes = [P, I, I, P, P]
        L.mph_nn_conv3.argtypes = [P, I, I, I, I, P, I, fp, I, P]
        L.mph_nn_sync.argtypes = [P]
        L.mph_nn_gemm_mode.argtypes = [I]
        L.mph_nn_status.argtypes = [C.POINTER(C.c_int), I]
        _L = L
    return _L


class Conv:
    """3 x 3 (pad 1) or 1 x 1 convolution with bias and optional leaky ReLU.

    Every GEMM reads both operands K-contiguous (the tensor-core kernel's
    TMA copies):
      forward          Y [P][Cout]    = Xcol [P][9 Cin] . Wt^T, as an implicit
                       GEMM (mph_nn_conv3: the tap-shifted pixels of X are the A
                       tiles, no im2col) where the shapes allow
      weight gradient  gW [Cout][9 Cin] = dY^T [Cout][P] . Xcol^T [9 Cin][P]
                       (both operands transposed once per step)
      data gradient    dX [P][Cin]    = dYcol [P][9 Cout] . W2^T, with dYcol the
                       im2col of dY and W2 the weights with mirrored taps, so the
                       gradient is a 3 x 3 convolution of dY (no 9 x expanded
                       FP32 column gradient and no col2im), implicit as well."""

    def __init__(self, cin, cout, rng, k3=True, act=True):
        self.cin, self.cout, self.k3, self.act = cin, cout, k3, act
        self.K = 9 * cin if k3 else cin
        w = rng.standard_normal((cout, self.K)).astype(np.float32) * np.float32(np.sqrt(2.0 / self.K))
        if not act:
            w *= np.float32(0.1)
        self.n = cout * self.K
        self.wt, self.b = _f32(self.n), _f32(cout)
        self.wt.upload(w)
        self.b.upload(np.zeros(cout, np.float32))
        self.wt_bf = _bf(self.n)
        self.w2 = _bf(self.n) if k3 else None
        self.gw, self.gb = _f32(self.n), _f32(cout)
        self.mw, self.vw, self.mb, self.vb = _f32(self.n), _f32(self.n), _f32(cout), _f32(cout)
        L = _lib()
        for buf, n in ((self.mw, self.n), (self.vw, self.n), (self.mb, cout), (self.vb, cout)):
            check(L.mph_nn_fill(buf.ptr, n, 0.0, None))
        self.refresh()
        self.P = 0
        # whether mph_nn_conv3 takes this layer's forward / data-gradient shapes
        # (found at the first call)
        self.implicit = self.bwd_implicit = None

    def _conv3(self, x, Bn, H, W, C, wt, cout, y):
        """mph_nn_conv3 when it applies, else False (the caller uses im2col + GEMM)."""
        from . import MphError
        try:
            check(_lib().mph_nn_conv3(x.ptr, Bn, H, W, C, wt.ptr, cout, y.ptr, 0, None))
            return True
        except MphError as ex:
            if ex.code != 4:  # MPH_ERR_UNSUPPORTED
                raise
            return False

    def refresh(self):
        check(_lib().mph_nn_cast(0, self.wt.ptr, self.n, self.wt_bf.ptr, None))

    def alloc(self, P):
        if P <= self.P:
            return
        self.P = P
        self.y = _f32(P * self.cout)
        self.out = _bf(P * self.cout)
        self.dpre, self.dpre_bf = _f32(P * self.cout), _bf(P * self.cout)
        self.dpre_t, self.xcol_t = _bf(P * self.cout), _bf(P * self.K)
        self.dx = _f32(P * self.cin)
        if self.k3:
            self.xcol, self.dycol = _bf(P * self.K), _bf(P * 9 * self.cout)

    def forward(self, x: Dev, Bn, H, W, out_f32: Dev | None = None):
        L, P = _lib(), Bn * H * W
        self.alloc(P)
        self.x, self.shape = x, (Bn, H, W)
        self.fwd_implicit = False
        if self.k3 and self.implicit is not False:
            self.fwd_implicit = self._conv3(x, Bn, H, W, self.cin, self.wt_bf, self.cout, self.y)
            self.implicit = self.fwd_implicit
        if not self.fwd_implicit:
            A = x
            if self.k3:
                check(L.mph_nn_im2col3(x.ptr, Bn, H, W, self.cin, self.xcol.ptr, None))
                A = self.xcol
            check(L.mph_nn_gemm(P, self.cout, self.K, A.ptr, self.K, 0, self.wt_bf.ptr, self.K, 0, self.y.ptr,
                                self.cout, 0, None))
        check(L.mph_nn_bias_act(self.y.ptr, self.b.ptr, P, self.cout, int(self.act),
                                self.out.ptr if out_f32 is None else None,
                                out_f32.ptr if out_f32 is not None else None, self.cout, 0, None))
        return self.out

    def backward(self, dout: Dev, need_dx=True):
        L = _lib()
        Bn, H, W = self.shape
        P = Bn * H * W
        check(L.mph_nn_act_bwd(dout.ptr, self.cout, 0, self.out.ptr, self.cout, 0, P, self.cout, int(self.act),
                               self.dpre.ptr, None))
        check(L.mph_nn_colsum(self.dpre.ptr, P, self.cout, self.gb.ptr, None))
        check(L.mph_nn_cast(0, self.dpre.ptr, P * self.cout, self.dpre_bf.ptr, None))
        if self.k3 and self.fwd_implicit:  # the weight gradient needs the im2col matrix once
            check(L.mph_nn_im2col3(self.x.ptr, Bn, H, W, self.cin, self.xcol.ptr, None))
        B = self.xcol if self.k3 else self.x
        check(L.mph_nn_transpose(self.dpre_bf.ptr, P, self.cout, self.dpre_t.ptr, None))
        check(L.mph_nn_transpose(B.ptr, P, self.K, self.xcol_t.ptr, None))
        check(L.mph_nn_gemm(self.cout, self.K, P, self.dpre_t.ptr, P, 0, self.xcol_t.ptr, P, 0, self.gw.ptr,
                            self.K, 0, None))
        if not need_dx:
            return None
        if self.k3:
            check(L.mph_nn_wflip(self.wt_bf.ptr, self.cout, self.cin, self.w2.ptr, None))
            done = False
            if self.bwd_implicit is not False:
                done = self.bwd_implicit = self._conv3(self.dpre_bf, Bn, H, W, self.cout, self.w2, self.cin, self.dx)
            if not done:
                check(L.mph_nn_im2col3(self.dpre_bf.ptr, Bn, H, W, self.cout, self.dycol.ptr, None))
                check(L.mph_nn_gemm(P, self.cin, 9 * self.cout, self.dycol.ptr, 9 * self.cout, 0, self.w2.ptr,
                                    9 * self.cout, 0, self.dx.ptr, self.cin, 0, None))
        else:
            check(L.mph_nn_gemm(P, self.K, self.cout, self.dpre_bf.ptr, self.cout, 0, self.wt_bf.ptr, self.K, 1,
                                self.dx.ptr, self.K, 0, None))
        return self.dx

    def adam(self, lr, t, wd=0.0, gscale=1.0, b1=0.9, b2=0.999, eps=1e-8):
        L = _lib()
        check(L.mph_nn_adam(self.wt.ptr, self.mw.ptr, self.vw.ptr, self.gw.ptr, self.n, lr, b1, b2, eps, t, wd, gscale,
                            None))
        check(L.mph_nn_adam(self.b.ptr, self.mb.ptr, self.vb.ptr, self.gb.ptr, self.cout, lr, b1, b2, eps, t, 0.0,
                            gscale, None))
        self.refresh()

    def grad_sumsq(self, part: Dev, nblk: int, off: int = 0):
        """Block sums of the squared weight and bias gradients into
        part[off : off + 2 nblk] (no host synchronisation)."""
        L = _lib()
        base = part.ptr.value + 4 * off
        check(L.mph_nn_sumsq(self.gw.ptr, self.n, C.c_void_p(base), nblk, None))
        check(L.mph_nn_sumsq(self.gb.ptr, self.cout, C.c_void_p(base + 4 * nblk), nblk, None))

    def get(self):
        return self.wt.download(self.n).reshape(self.cout, self.K), self.b.download(self.cout)

    def set(self, wt, b):
        self.wt.upload(np.asarray(wt, np.float32).reshape(-1))
        self.b.upload(np.asarray(b, np.float32))
        self.refresh()


class UNet:
    """The 4-level U-Net.  forward() returns the FP32 prediction buffer
    [P][3]; backward(dpred) fills every layer's gw / gb."""

    NAMES = ("e1a", "e1b", "e2a", "e2b", "e3a", "e3b", "e4a", "e4b", "d3a", "d3b", "d2a", "d2b", "d1a", "d1b", "head")

    def __init__(self, seed=0):
        rng = np.random.default_rng(seed)
        c1, c2, c3, c4 = CHANS
        spec = [(IN_CH, c1), (c1, c1), (c1, c2), (c2, c2), (c2, c3), (c3, c3), (c3, c4), (c4, c4),
                (c4 + c3, c3), (c3, c3), (c3 + c2, c2), (c2, c2), (c2 + c1, c1), (c1, c1)]
        self.layers = {n: Conv(a, b, rng) for n, (a, b) in zip(self.NAMES[:-1], spec)}
        self.layers["head"] = Conv(c1, OUT_CH, rng, k3=False, act=False)
        self.shape = None
        self.t = 0

    def n_params(self):
        return sum(l.n + l.cout for l in self.layers.values())

    def _alloc(self, Bn, H, W):
        if self.shape is not None and self.shape[0] >= Bn and self.shape[1:] == (H, W):
            return
        c1, c2, c3, c4 = CHANS
        P = [Bn * (H >> s) * (W >> s) for s in range(4)]
        self.p1, self.p2, self.p3 = _bf(P[1] * c1), _bf(P[2] * c2), _bf(P[3] * c3)
        self.cat3, self.cat2, self.cat1 = _bf(P[2] * (c4 + c3)), _bf(P[1] * (c3 + c2)), _bf(P[0] * (c2 + c1))
        self.pred = _f32(P[0] * OUT_CH)
        self.dt3, self.dt2 = _f32(P[2] * c3), _f32(P[1] * c2)
        self.ds4, self.ds3, self.ds2, self.ds1 = _f32(P[3] * c4), _f32(P[2] * c3), _f32(P[1] * c2), _f32(P[0] * c1)
        self.tmp = _f32(P[0] * c1)
        self.shape = (Bn, H, W)

    def forward(self, x: Dev, Bn, H, W):
        assert H % 8 == 0 and W % 8 == 0
        self._alloc(Bn, H, W)
        Lb, l = _lib(), self.layers
        c1, c2, c3, c4 = CHANS
        dims = [(H >> s, W >> s) for s in range(4)]
        self.dims, self.Bn = dims, Bn
        Pl = [Bn * h * w for h, w in dims]
        a = l["e1a"].forward(x, Bn, *dims[0])
        s1 = l["e1b"].forward(a, Bn, *dims[0])
        check(Lb.mph_nn_pool(s1.ptr, Bn, *dims[0], c1, self.p1.ptr, None))
        a = l["e2a"].forward(self.p1, Bn, *dims[1])
        s2 = l["e2b"].forward(a, Bn, *dims[1])
        check(Lb.mph_nn_pool(s2.ptr, Bn, *dims[1], c2, self.p2.ptr, None))
        a = l["e3a"].forward(self.p2, Bn, *dims[2])
        s3 = l["e3b"].forward(a, Bn, *dims[2])
        check(Lb.mph_nn_pool(s3.ptr, Bn, *dims[2], c3, self.p3.ptr, None))
        a = l["e4a"].forward(self.p3, Bn, *dims[3])
        s4 = l["e4b"].forward(a, Bn, *dims[3])
        check(Lb.mph_nn_up(s4.ptr, Bn, *dims[3], c4, self.cat3.ptr, c4 + c3, 0, None))
        check(Lb.mph_nn_slice(0, s3.ptr, c3, 0, Pl[2], c3, self.cat3.ptr, c4 + c3, c4, 0, None))
        a = l["d3a"].forward(self.cat3, Bn, *dims[2])
        t3 = l["d3b"].forward(a, Bn, *dims[2])
        check(Lb.mph_nn_up(t3.ptr, Bn, *dims[2], c3, self.cat2.ptr, c3 + c2, 0, None))
        check(Lb.mph_nn_slice(0, s2.ptr, c2, 0, Pl[1], c2, self.cat2.ptr, c3 + c2, c3, 0, None))
        a = l["d2a"].forward(self.cat2, Bn, *dims[1])
        t2 = l["d2b"].forward(a, Bn, *dims[1])
        check(Lb.mph_nn_up(t2.ptr, Bn, *dims[1], c2, self.cat1.ptr, c2 + c1, 0, None))
        check(Lb.mph_nn_slice(0, s1.ptr, c1, 0, Pl[0], c1, self.cat1.ptr, c2 + c1, c2, 0, None))
        a = l["d1a"].forward(self.cat1, Bn, *dims[0])
        t1 = l["d1b"].forward(a, Bn, *dims[0])
        l["head"].forward(t1, Bn, *dims[0], out_f32=self.pred)
        return self.pred

    def backward(self, dpred: Dev):
        Lb, l = _lib(), self.layers
        c1, c2, c3, c4 = CHANS
        Bn, dims = self.Bn, self.dims
        Pl = [Bn * h * w for h, w in dims]
        d = l["head"].backward(dpred)
        d = l["d1b"].backward(d)
        dcat1 = l["d1a"].backward(d)
        check(Lb.mph_nn_up_bwd(dcat1.ptr, c2 + c1, 0, Bn, *dims[1], c2, self.dt2.ptr, None))
        check(Lb.mph_nn_slice(1, dcat1.ptr, c2 + c1, c2, Pl[0], c1, self.ds1.ptr, c1, 0, 0, None))
        d = l["d2b"].backward(self.dt2)
        dcat2 = l["d2a"].backward(d)
        check(Lb.mph_nn_up_bwd(dcat2.ptr, c3 + c2, 0, Bn, *dims[2], c3, self.dt3.ptr, None))
        check(Lb.mph_nn_slice(1, dcat2.ptr, c3 + c2, c3, Pl[1], c2, self.ds2.ptr, c2, 0, 0, None))
        d = l["d3b"].backward(self.dt3)
        dcat3 = l["d3a"].backward(d)
        check(Lb.mph_nn_up_bwd(dcat3.ptr, c4 + c3, 0, Bn, *dims[3], c4, self.ds4.ptr, None))
        check(Lb.mph_nn_slice(1, dcat3.ptr, c4 + c3, c4, Pl[2], c3, self.ds3.ptr, c3, 0, 0, None))
        d = l["e4b"].backward(self.ds4)
        dp3 = l["e4a"].backward(d)
        check(Lb.mph_nn_pool_bwd(dp3.ptr, Bn, *dims[2], c3, self.tmp.ptr, None))
        check(Lb.mph_nn_slice(1, self.tmp.ptr, c3, 0, Pl[2], c3, self.ds3.ptr, c3, 0, 1, None))
        d = l["e3b"].backward(self.ds3)
        dp2 = l["e3a"].backward(d)
        check(Lb.mph_nn_pool_bwd(dp2.ptr, Bn, *dims[1], c2, self.tmp.ptr, None))
        check(Lb.mph_nn_slice(1, self.tmp.ptr, c2, 0, Pl[1], c2, self.ds2.ptr, c2, 0, 1, None))
        d = l["e2b"].backward(self.ds2)
        dp1 = l["e2a"].backward(d)
        check(Lb.mph_nn_pool_bwd(dp1.ptr, Bn, *dims[0], c1, self.tmp.ptr, None))
        check(Lb.mph_nn_slice(1, self.tmp.ptr, c1, 0, Pl[0], c1, self.ds1.ptr, c1, 0, 1, None))
        d = l["e1b"].backward(self.ds1)
        l["e1a"].backward(d, need_dx=False)

    def grad_norm(self) -> float:
        """Global L2 norm of all gradients, with one download."""
        nblk, nl = 64, len(self.layers)
        if not hasattr(self, "_part"):
            self._part = _f32(2 * nblk * nl)
        for i, layer in enumerate(self.layers.values()):
            layer.grad_sumsq(self._part, nblk, 2 * nblk * i)
        return float(np.sqrt(self._part.download(2 * nblk * nl).astype(np.float64).sum()))

    def step(self, lr, wd=0.0, clip=None):
        """Adam step; with clip, gradients are scaled so their global L2 norm
        is at most clip (returns the norm before scaling)."""
        self.t += 1
        norm, gscale = None, 1.0
        if clip is not None:
            norm = self.grad_norm()
            if not np.isfinite(norm):
                return norm  # skip a non-finite step
            gscale = min(1.0, clip / max(norm, 1e-30))
        for layer in self.layers.values():
            layer.adam(lr, self.t, wd, gscale)
        return norm

    def state(self):
        return {n: l.get() for n, l in self.layers.items()}

    def load(self, state):
        for n, (w, b) in state.items():
            self.layers[n].set(w, b)


class Trainer:
    """Masked-MSE training of a UNet on host-resident (input, target, mask)
    arrays: x [S][H][W][8], y [S][H][W][3], m [S][H][W] (fluid = 1)."""

    def __init__(self, net: UNet, batch: int, H: int, W: int):
        self.net, self.batch, self.H, self.W = net, batch, H, W
        P = batch * H * W
        self.xf, self.xb = _f32(P * IN_CH), _bf(P * IN_CH)
        self.yt, self.wm = _f32(P * OUT_CH), _f32(P)
        self.dpred = _f32(P * OUT_CH)
        self.nblk = 256
        self.part = _f32(self.nblk)

    def load_batch(self, x, y=None, m=None):
        Bn = x.shape[0]
        P = Bn * self.H * self.W
        self.xf.upload(x.astype(np.float32).reshape(-1))
        check(_lib().mph_nn_cast(0, self.xf.ptr, P * IN_CH, self.xb.ptr, None))
        if y is not None:
            self.yt.upload(y.astype(np.float32).reshape(-1))
            self.wm.upload(m.astype(np.float32).reshape(-1))
        return Bn

    def loss_grad(self, Bn, count):
        P = Bn * self.H * self.W
        check(_lib().mph_nn_mse(self.net.pred.ptr, self.yt.ptr, self.wm.ptr, P, OUT_CH, 1.0 / count,
                                self.dpred.ptr, self.part.ptr, self.nblk, None))
        return float(self.part.download(self.nblk).sum()) / count

    def train_step(self, x, y, m, lr, wd=0.0, clip=1.0):
        Bn = self.load_batch(x, y, m)
        self.net.forward(self.xb, Bn, self.H, self.W)
        count = float(m.sum()) * OUT_CH
        loss = self.loss_grad(Bn, count)
        self.net.backward(self.dpred)
        self.net.step(lr, wd, clip)
        return loss

    def predict(self, x):
        Bn = self.load_batch(x)
        pred = self.net.forward(self.xb, Bn, self.H, self.W)
        return pred.download(Bn * self.H * self.W * OUT_CH).reshape(Bn, self.H, self.W, OUT_CH)
