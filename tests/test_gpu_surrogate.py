"""The surrogate's GPU kernels against the CPU restatement (oracle/nn_oracle):
the tensor-core GEMM in all four operand layouts, im2col / col2im adjointness,
and the whole U-Net's prediction and every layer's weight and bias gradient;
plus a training smoke check."""
import ctypes as C

import numpy as np
import pytest

from oracle import nn_oracle as NO

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def S(mph):
    from muphfasa_gb300 import surrogate
    return surrogate


def _bf16_dev(S, a):
    a32 = np.ascontiguousarray(a, np.float32)
    f = S._f32(a32.size)
    f.upload(a32.reshape(-1))
    b = S._bf(a32.size)
    S.check(S._lib().mph_nn_cast(0, f.ptr, a32.size, b.ptr, None))
    return b


@pytest.mark.parametrize("ta,tb", [(0, 0), (0, 1), (1, 0), (1, 1)])
def test_gemm_layouts(ta, tb, S):
    rng = np.random.default_rng(ta * 2 + tb)
    M, N, K = 77, 45, 83
    A = NO.to_bf16(rng.standard_normal((M, K)).astype(np.float32))
    B = NO.to_bf16(rng.standard_normal((K, N)).astype(np.float32))
    a_store = A.T if ta else A          # [K][M] or [M][K]
    b_store = B if tb else B.T          # [K][N] or [N][K]
    da, db = _bf16_dev(S, a_store), _bf16_dev(S, b_store)
    c = S._f32(M * N)
    S.check(S._lib().mph_nn_gemm(M, N, K, da.ptr, M if ta else K, ta, db.ptr, N if tb else K, tb, c.ptr, N, 0, None))
    got = c.download(M * N).reshape(M, N)
    ref = A.astype(np.float64) @ B.astype(np.float64)
    scale = np.abs(A).astype(np.float64) @ np.abs(B).astype(np.float64)
    assert np.all(np.abs(got - ref) <= 1e-5 * scale + 1e-6)
    # accumulate mode adds to C
    S.check(S._lib().mph_nn_gemm(M, N, K, da.ptr, M if ta else K, ta, db.ptr, N if tb else K, tb, c.ptr, N, 1, None))
    got2 = c.download(M * N).reshape(M, N)
    assert np.all(np.abs(got2 - 2 * ref) <= 2e-5 * scale + 2e-6)


@pytest.mark.parametrize("shape", [(200, 70, 100), (1024, 256, 576), (128, 64, 64), (130, 70, 32), (300, 64, 4096)])
@pytest.mark.parametrize("ta,tb", [(0, 0), (0, 1), (1, 0), (1, 1)])
def test_tcgen05_gemm_matches_mma_sync_and_numpy(ta, tb, shape, S):
    """The tensor-memory GEMMs (tcgen05.mma: cp.async pipelined, single-
    buffered, and TMA-fed where the operands are K-contiguous and aligned)
    against NumPy and against the mma.sync kernel."""
    rng = np.random.default_rng(10 + ta * 2 + tb)
    M, N, K = shape
    A = NO.to_bf16(rng.standard_normal((M, K)).astype(np.float32))
    B = NO.to_bf16(rng.standard_normal((K, N)).astype(np.float32))
    da, db = _bf16_dev(S, A.T if ta else A), _bf16_dev(S, B if tb else B.T)
    L = S._lib()
    out = {}
    try:
        for mode in (1, 2, 3, 4):
            S.check(L.mph_nn_gemm_mode(mode))
            c = S._f32(M * N)
            S.check(L.mph_nn_gemm(M, N, K, da.ptr, M if ta else K, ta, db.ptr, N if tb else K, tb, c.ptr, N, 0, None))
            out[mode] = c.download(M * N).reshape(M, N)
    finally:
        S.check(L.mph_nn_gemm_mode(0))
    flag = C.c_int(-1)
    S.check(L.mph_nn_status(C.byref(flag), 1))
    assert flag.value == 0
    ref = A.astype(np.float64) @ B.astype(np.float64)
    scale = np.abs(A).astype(np.float64) @ np.abs(B).astype(np.float64)
    for mode in (2, 3, 4):
        assert np.all(np.abs(out[mode] - ref) <= 1e-5 * scale + 1e-6), mode
        assert np.all(np.abs(out[mode] - out[1]) <= 2e-5 * scale + 2e-6), mode


def _download_bf16(S, dev, n):
    f = S._f32(n)
    S.check(S._lib().mph_nn_cast(1, dev.ptr, n, f.ptr, None))
    return f.download(n)


@pytest.mark.parametrize("rows,cols", [(1, 1), (37, 5), (4096, 288), (1000, 33), (130, 70), (2, 2), (64, 4096)])
def test_transpose_bf16(rows, cols, S):
    rng = np.random.default_rng(rows + cols)
    x = NO.to_bf16(rng.standard_normal((rows, cols)).astype(np.float32))
    dx, dy = _bf16_dev(S, x), S._bf(x.size)
    S.check(S._lib().mph_nn_transpose(dx.ptr, rows, cols, dy.ptr, None))
    assert np.array_equal(_download_bf16(S, dy, x.size).reshape(cols, rows), x.T)


@pytest.mark.parametrize("cin,cout", [(5, 3), (32, 64), (96, 32)])
def test_data_gradient_as_mirrored_convolution(cin, cout, S):
    """dX of a 3 x 3 convolution computed as the convolution of dY with the
    mirrored, channel-exchanged weights (mph_nn_wflip + im2col of dY + one
    GEMM) equals col2im of the column gradient dY . Wt within FP32 rounding."""
    rng = np.random.default_rng(cin * cout)
    Bn, H, W = 2, 8, 16
    P = Bn * H * W
    wt = NO.to_bf16(rng.standard_normal((cout, 9 * cin)).astype(np.float32))
    dy = NO.to_bf16(rng.standard_normal((P, cout)).astype(np.float32))
    L = S._lib()
    dwt, ddy = _bf16_dev(S, wt), _bf16_dev(S, dy)
    w2, dycol, dx = S._bf(wt.size), S._bf(P * 9 * cout), S._f32(P * cin)
    S.check(L.mph_nn_wflip(dwt.ptr, cout, cin, w2.ptr, None))
    w2h = _download_bf16(S, w2, wt.size).reshape(cin, 9, cout)
    assert np.array_equal(w2h, wt.reshape(cout, 9, cin)[:, ::-1, :].transpose(2, 1, 0))
    S.check(L.mph_nn_im2col3(ddy.ptr, Bn, H, W, cout, dycol.ptr, None))
    S.check(L.mph_nn_gemm(P, cin, 9 * cout, dycol.ptr, 9 * cout, 0, w2.ptr, 9 * cout, 0, dx.ptr, cin, 0, None))
    got = dx.download(P * cin).reshape(Bn, H, W, cin)
    ref = NO.Net.col2im(dy.astype(np.float64) @ wt.astype(np.float64), (Bn, H, W, cin))
    scale = NO.Net.col2im(np.abs(dy).astype(np.float64) @ np.abs(wt).astype(np.float64), (Bn, H, W, cin))
    assert np.all(np.abs(got - ref) <= 1e-5 * scale + 1e-6)


@pytest.mark.parametrize("Cc", [8, 16, 96])
def test_im2col_16_byte_path(Cc, S):
    """im2col with C a multiple of 8 (16-byte moves) against the restatement."""
    rng = np.random.default_rng(Cc)
    Bn, H, W = 2, 8, 16
    x = NO.to_bf16(rng.standard_normal((Bn, H, W, Cc)).astype(np.float32))
    dx_, col = _bf16_dev(S, x), S._bf(Bn * H * W * 9 * Cc)
    S.check(S._lib().mph_nn_im2col3(dx_.ptr, Bn, H, W, Cc, col.ptr, None))
    got = _download_bf16(S, col, Bn * H * W * 9 * Cc).reshape(Bn * H * W, 9 * Cc)
    assert np.array_equal(got, NO.Net.im2col(x))


@pytest.mark.parametrize("P,Cc", [(131072, 32), (2048, 256), (300, 64), (4096, 3), (100, 8), (5000, 96), (131072, 3)])
def test_colsum(P, Cc, S):
    rng = np.random.default_rng(P + Cc)
    x = rng.standard_normal((P, Cc)).astype(np.float32)
    dx_, out = S._f32(x.size), S._f32(Cc)
    dx_.upload(x.reshape(-1))
    S.check(S._lib().mph_nn_colsum(dx_.ptr, P, Cc, out.ptr, None))
    ref = x.astype(np.float64).sum(axis=0)
    assert np.allclose(out.download(Cc), ref, rtol=1e-5, atol=1e-5 * np.sqrt(P))


@pytest.mark.parametrize("shape", [(4096, 32, 288), (1000, 96, 864), (64, 288, 8192), (256, 3, 64), (131, 200, 72)])
def test_tma_gemm_shapes_of_the_network(shape, S):
    """The TMA-fed tcgen05 GEMM (K-contiguous operands) on the network's
    shapes: a forward convolution (N = 32), a partial last row tile and a
    128-wide column tile, a weight gradient (K = pixels, split K, M < 128), a
    3-column output and a K that is not a multiple of the 64-wide slices."""
    rng = np.random.default_rng(sum(shape))
    M, N, K = shape
    A = NO.to_bf16(rng.standard_normal((M, K)).astype(np.float32))
    B = NO.to_bf16(rng.standard_normal((K, N)).astype(np.float32))
    da, db = _bf16_dev(S, A), _bf16_dev(S, B.T)
    L = S._lib()
    c = S._f32(M * N)
    try:
        S.check(L.mph_nn_gemm_mode(4))
        S.check(L.mph_nn_gemm(M, N, K, da.ptr, K, 0, db.ptr, K, 0, c.ptr, N, 0, None))
        got = c.download(M * N).reshape(M, N)
        S.check(L.mph_nn_gemm(M, N, K, da.ptr, K, 0, db.ptr, K, 0, c.ptr, N, 1, None))
        got2 = c.download(M * N).reshape(M, N)
    finally:
        S.check(L.mph_nn_gemm_mode(0))
    flag = C.c_int(-1)
    S.check(L.mph_nn_status(C.byref(flag), 1))
    assert flag.value == 0
    ref = A.astype(np.float64) @ B.astype(np.float64)
    scale = np.abs(A).astype(np.float64) @ np.abs(B).astype(np.float64)
    assert np.all(np.abs(got - ref) <= 1e-5 * scale + 1e-6)
    assert np.all(np.abs(got2 - 2 * ref) <= 2e-5 * scale + 2e-6)


@pytest.mark.parametrize("Bn,H,W,Cc,cout", [(2, 16, 128, 32, 64), (2, 8, 64, 64, 32), (4, 16, 16, 96, 32),
                                            (1, 4, 256, 64, 128), (8, 16, 8, 128, 256), (2, 32, 32, 256, 3)])
def test_implicit_conv3_against_im2col_gemm(Bn, H, W, Cc, cout, S):
    """mph_nn_conv3 (implicit GEMM: TMA boxes of each tap's shifted pixels,
    64- or 32-channel slices, tiles of whole rows or of 128-pixel pieces of a
    row, split K on the small outputs) against the float64 product of the
    restatement's im2col with the weights, and accumulate mode."""
    rng = np.random.default_rng(Bn * H * W + Cc + cout)
    x = NO.to_bf16(rng.standard_normal((Bn, H, W, Cc)).astype(np.float32))
    wt = NO.to_bf16(rng.standard_normal((cout, 9 * Cc)).astype(np.float32))
    dx_, dw = _bf16_dev(S, x), _bf16_dev(S, wt)
    P = Bn * H * W
    y = S._f32(P * cout)
    L = S._lib()
    S.check(L.mph_nn_conv3(dx_.ptr, Bn, H, W, Cc, dw.ptr, cout, y.ptr, 0, None))
    got = y.download(P * cout).reshape(P, cout)
    S.check(L.mph_nn_conv3(dx_.ptr, Bn, H, W, Cc, dw.ptr, cout, y.ptr, 1, None))
    got2 = y.download(P * cout).reshape(P, cout)
    flag = C.c_int(-1)
    S.check(L.mph_nn_status(C.byref(flag), 1))
    assert flag.value == 0
    A = NO.Net.im2col(x).astype(np.float64)
    ref, scale = A @ wt.T.astype(np.float64), np.abs(A) @ np.abs(wt.T).astype(np.float64)
    assert np.all(np.abs(got - ref) <= 1e-5 * scale + 1e-6)
    assert np.all(np.abs(got2 - 2 * ref) <= 2e-5 * scale + 2e-6)


def test_implicit_conv3_rejects_shapes_it_cannot_tile(S, mph):
    rng = np.random.default_rng(0)
    x = _bf16_dev(S, rng.standard_normal((1, 6, 10, 8)).astype(np.float32))
    w = _bf16_dev(S, rng.standard_normal((32, 72)).astype(np.float32))
    y = S._f32(60 * 32)
    with pytest.raises(mph.MphError) as e:
        S.check(S._lib().mph_nn_conv3(x.ptr, 1, 6, 10, 8, w.ptr, 32, y.ptr, 0, None))
    assert e.value.code == 4


def test_im2col_col2im_adjoint(S):
    rng = np.random.default_rng(3)
    Bn, H, W, Cc = 2, 8, 16, 5
    x = NO.to_bf16(rng.standard_normal((Bn, H, W, Cc)).astype(np.float32))
    y = rng.standard_normal((Bn * H * W, 9 * Cc)).astype(np.float32)
    dx_, col = _bf16_dev(S, x), S._bf(y.size)
    S.check(S._lib().mph_nn_im2col3(dx_.ptr, Bn, H, W, Cc, col.ptr, None))
    colf = S._f32(y.size)
    S.check(S._lib().mph_nn_cast(1, col.ptr, y.size, colf.ptr, None))
    got_col = colf.download(y.size).reshape(y.shape)
    assert np.array_equal(got_col, NO.Net.im2col(x))
    dy, dxo = S._f32(y.size), S._f32(x.size)
    dy.upload(y.reshape(-1))
    S.check(S._lib().mph_nn_col2im3(dy.ptr, Bn, H, W, Cc, dxo.ptr, None))
    back = dxo.download(x.size).reshape(x.shape)
    assert np.allclose(back, NO.Net.col2im(y.astype(np.float64), x.shape), rtol=1e-5, atol=1e-5)
    assert np.isclose(float((got_col.astype(np.float64) * y).sum()), float((x.astype(np.float64) * back).sum()),
                      rtol=1e-5)


def test_unet_prediction_and_gradients_match_oracle(S):
    rng = np.random.default_rng(5)
    Bn, H, W = 2, 16, 16
    net = S.UNet(seed=7)
    # give the biases nonzero values so their gradients and the head matter
    for name, layer in net.layers.items():
        w, b = layer.get()
        layer.set(w, 0.05 * rng.standard_normal(b.shape))
    tr = S.Trainer(net, Bn, H, W)
    x = rng.standard_normal((Bn, H, W, S.IN_CH)).astype(np.float32)
    y = rng.standard_normal((Bn, H, W, S.OUT_CH)).astype(np.float32)
    m = (rng.random((Bn, H, W)) > 0.25).astype(np.float32)
    tr.load_batch(x, y, m)
    pred = net.forward(tr.xb, Bn, H, W)
    count = float(m.sum()) * S.OUT_CH
    loss = tr.loss_grad(Bn, count)
    net.backward(tr.dpred)
    gpu_pred = pred.download(Bn * H * W * S.OUT_CH).reshape(Bn, H, W, S.OUT_CH)

    params = net.state()
    ref = NO.Net(params, bf16=True)
    rp = ref.forward(x)
    rloss, dpred = ref.loss(rp, y, m)
    grads = ref.backward(dpred)
    exact = NO.Net(params, bf16=False)
    ep = exact.forward(x)
    eloss, edpred = exact.loss(ep, y, m)
    egrads = exact.backward(edpred)
    assert np.linalg.norm(gpu_pred - rp) <= 1e-2 * np.linalg.norm(rp)
    assert abs(loss - rloss) <= 1e-2 * rloss
    # Layer by layer: the GPU gradient against the BF16 restatement, and both
    # against the float64 restatement.  BF16 roundings (8 significant bits)
    # compound through the backward chain, so the deepest layers carry a few
    # per cent; the GPU must stay as close to float64 as the BF16 restatement.
    report = []
    for name, layer in net.layers.items():
        gw = layer.gw.download(layer.n).reshape(layer.cout, layer.K)
        gb = layer.gb.download(layer.cout)
        rw, rb = grads[name]
        xw, xb = egrads[name]
        rel = lambda a, b: float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))
        e_gpu, e_bf, e_gpu64 = rel(gw, rw), rel(rw, xw), rel(gw, xw)
        report.append((name, e_gpu, e_bf, e_gpu64, rel(gb, rb)))
    msg = "\n".join(f"{r[0]:5s} gpu-vs-bf16 {r[1]:.3e} bf16-vs-f64 {r[2]:.3e} gpu-vs-f64 {r[3]:.3e} bias {r[4]:.3e}"
                    for r in report)
    print(msg)
    for name, e_gpu, e_bf, e_gpu64, e_b in report:
        assert e_gpu < 0.1 and e_b < 0.1, msg
        assert e_gpu64 <= 2.0 * e_bf + 0.01, msg


def test_every_layer_gradient_from_its_own_operands(S):
    """Per-layer check at GEMM precision: after one backward pass of a
    4 x 32 x 32 batch (large enough for the TMA-fed GEMMs and split K), each
    layer's weight gradient and data gradient are recomputed in float64 from
    the BF16 operands the GPU used (its input activation and its upstream
    gradient dPre), and must agree to 1e-5 of the magnitude scale: a
    transposed or misplaced operand in any layer fails here."""
    rng = np.random.default_rng(11)
    Bn, H, W = 4, 32, 32
    net = S.UNet(seed=3)
    tr = S.Trainer(net, Bn, H, W)
    x = rng.standard_normal((Bn, H, W, S.IN_CH)).astype(np.float32)
    y = rng.standard_normal((Bn, H, W, S.OUT_CH)).astype(np.float32)
    m = (rng.random((Bn, H, W)) > 0.25).astype(np.float32)
    tr.load_batch(x, y, m)
    net.forward(tr.xb, Bn, H, W)
    tr.loss_grad(Bn, float(m.sum()) * S.OUT_CH)
    net.backward(tr.dpred)
    for name, layer in net.layers.items():
        lb, lh, lw = layer.shape
        P = lb * lh * lw
        xin = _download_bf16(S, layer.x, P * layer.cin).reshape(lb, lh, lw, layer.cin).astype(np.float64)
        dpre = _download_bf16(S, layer.dpre_bf, P * layer.cout).reshape(P, layer.cout).astype(np.float64)
        wt = _download_bf16(S, layer.wt_bf, layer.n).reshape(layer.cout, layer.K).astype(np.float64)
        A = NO.Net.im2col(xin) if layer.k3 else xin.reshape(P, layer.cin)
        gw = layer.gw.download(layer.n).reshape(layer.cout, layer.K)
        ref, scale = dpre.T @ A, np.abs(dpre).T @ np.abs(A)
        assert np.all(np.abs(gw - ref) <= 1e-5 * scale + 1e-7), name
        if name == "e1a":
            continue  # the first layer computes no data gradient
        dx = layer.dx.download(P * layer.cin).reshape(lb, lh, lw, layer.cin)
        if layer.k3:
            ref = NO.Net.col2im(dpre @ wt, (lb, lh, lw, layer.cin))
            scale = NO.Net.col2im(np.abs(dpre) @ np.abs(wt), (lb, lh, lw, layer.cin))
        else:
            ref = (dpre @ wt).reshape(dx.shape)
            scale = (np.abs(dpre) @ np.abs(wt)).reshape(dx.shape)
        assert np.all(np.abs(dx - ref) <= 1e-5 * scale + 1e-7), name


def test_training_reduces_loss(S):
    rng = np.random.default_rng(2)
    Bn, H, W = 4, 32, 32
    yy, xx = np.meshgrid(np.linspace(0, 1, H), np.linspace(0, 1, W), indexing="ij")
    xs, ys = [], []
    for i in range(16):
        a = rng.uniform(0.5, 1.5)
        inp = np.zeros((H, W, S.IN_CH), np.float32)
        inp[..., 0] = a
        inp[..., 6], inp[..., 7] = xx, yy
        xs.append(inp)
        ys.append(np.stack([a * np.sin(np.pi * xx), a * yy, a * xx * yy], -1).astype(np.float32))
    X, Y, M = np.stack(xs), np.stack(ys), np.ones((16, H, W), np.float32)
    net = S.UNet(seed=1)
    tr = S.Trainer(net, Bn, H, W)
    losses = []
    for it in range(60):
        k = (it * Bn) % 16
        losses.append(tr.train_step(X[k:k + Bn], Y[k:k + Bn], M[k:k + Bn], lr=1e-3))
    assert np.mean(losses[-8:]) < 0.2 * np.mean(losses[:4])
