"""GPU tests of the learned denoiser's tensor-core kernels against the CPU
oracle (oracle/denoiser_ref.py): every stored activation of the forward pass,
the network output, the loss and the parameter gradient of one
forward+backward pass, on seeded random features."""
import numpy as np
import pytest

import helios_gb300 as hx
from oracle import denoiser_ref as dr

pytestmark = pytest.mark.gpu


def _rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))


def _problem(seed, n, h, w):
    rng = np.random.default_rng(seed)
    params = dr.init_params(seed)
    params[:] += rng.normal(0, 0.02, params.shape).astype(np.float32)  # non-zero biases
    feats = np.zeros((n, h, w, dr.FEATURES), np.float32)
    feats[..., 0:3] = rng.exponential(0.5, (n, h, w, 3))
    feats[..., 4:7] = rng.uniform(0, 1, (n, h, w, 3))
    feats[..., 7] = rng.uniform(0, 1, (n, h, w))
    nrm = rng.normal(size=(n, h, w, 3))
    feats[..., 8:11] = nrm / np.linalg.norm(nrm, axis=-1, keepdims=True)
    tg = np.zeros((n, h, w, 4), np.float32)
    tg[..., 0:3] = rng.exponential(0.5, (n, h, w, 3))
    return params, feats, tg


@pytest.fixture(scope="module")
def denoiser(gpu_ctx):
    dn = hx.Denoiser(gpu_ctx)
    yield dn
    dn.close()


def test_forward_backward_matches_oracle(gpu_ctx, denoiser):
    """End to end: the oracle runs the whole network from the same inputs, so
    BF16 rounding differences propagate (ReLU masks of near-zero values can
    flip); per-tensor relative error stays at the 1e-2 level."""
    n, h, w = 2, 64, 64
    params, feats, tg = _problem(3 + h, n, h, w)
    assert denoiser.num_params == dr.num_params()
    denoiser.set_params(params)
    fb = hx.DeviceBuffer(gpu_ctx, feats.nbytes)
    tb = hx.DeviceBuffer(gpu_ctx, tg.nbytes)
    fb.upload(feats)
    tb.upload(tg)
    loss = denoiser.forward_backward(fb, tb, n, h, w)
    ref_loss, ref_grad, t = dr.loss_and_grad(params, feats, tg, rnd=True)
    # activations, layer by layer (BF16 storage: a few flips of the last bit)
    for name, _, _ in hx.DENOISER_TENSORS[:-1]:
        g = denoiser.read_tensor(name, training=True)
        assert _rel(g, t[name]) < 1e-2, (name, _rel(g, t[name]))
    y = denoiser.read_output(training=True)[..., 0:3]
    assert _rel(y, t["y"]) < 1e-2, _rel(y, t["y"])
    assert abs(loss - ref_loss) <= 1e-3 * ref_loss, (loss, ref_loss)
    # parameter gradient, per layer
    grad = denoiser.gradients()
    off = 0
    for (name, _, _, _), (ci, co) in zip(dr.LAYERS, dr.layer_shapes()):
        nw = 9 * ci * co
        gw, rw = grad[off:off + nw], ref_grad[off:off + nw]
        gb, rb = grad[off + nw:off + nw + co], ref_grad[off + nw:off + nw + co]
        assert _rel(gw, rw) < 3e-2, (name, "W", _rel(gw, rw))
        assert _rel(gb, rb) < 3e-2, (name, "b", _rel(gb, rb))
        off += nw + co
    fb.close()
    tb.close()


def _src_names(i):
    return [s for s, _ in dr.LAYERS[i][1]]


@pytest.mark.parametrize("shape", [(2, 64, 64), (1, 48, 80)])
def test_each_kernel_matches_oracle_on_device_inputs(gpu_ctx, denoiser, shape):
    """Layer by layer, the oracle takes the device's own stored inputs (BF16
    activations and gradients), so each convolution kernel — forward,
    backward-data, backward-weights — is checked in isolation: only FP32
    accumulation order (and a rare last-bit BF16 flip) separates the two.
    (1, 48, 80) leaves partial 16x8 tiles on every level."""
    n, h, w = shape
    params, feats, tg = _problem(7 + w, n, h, w)
    denoiser.set_params(params)
    fb = hx.DeviceBuffer(gpu_ctx, feats.nbytes)
    tb = hx.DeviceBuffer(gpu_ctx, tg.nbytes)
    fb.upload(feats)
    tb.upload(tg)
    denoiser.forward_backward(fb, tb, n, h, w)
    P = dr.split_params(params.astype(np.float64))
    grad = denoiser.gradients()
    act = {name: denoiser.read_tensor(name) for name, _, _ in hx.DENOISER_TENSORS[:-1]}
    gr = {name: denoiser.read_tensor(name, gradient=True) for name, _, _ in hx.DENOISER_TENSORS[1:]}
    y = denoiser.read_output()[..., 0:3]
    scale = 1.0 / (3.0 * n * h * w)
    off = 0
    for i, ((name, srcs, cout, relu), (ci, co)) in enumerate(zip(dr.LAYERS, dr.layer_shapes())):
        wb = dr.bf16(P[i][0])
        b = P[i][1].astype(np.float32).astype(np.float64)
        x = np.concatenate([act[s] for s in _src_names(i)], axis=3)
        out = dr.OUTPUT_OF[i]
        pre = dr.conv(x, wb, b)
        if relu:
            want = dr.bf16(np.maximum(pre, 0.0))
            assert _rel(act[out], want) < 2e-3, (name, "forward", _rel(act[out], want))
        else:
            pre = pre + act["x"][..., 0:3]
            assert _rel(y, pre) < 1e-5, (name, "forward", _rel(y, pre))
        g = gr["gy"][..., 0:3] if out == "y" else gr[out]
        dw, db = dr.conv_wgrad(x, g)
        nw = 9 * ci * co
        assert _rel(grad[off:off + nw], dw.ravel() * scale) < 1e-4, (name, "wgrad", _rel(grad[off:off + nw], dw.ravel() * scale))
        assert _rel(grad[off + nw:off + nw + co], db * scale) < 1e-4, (name, "bgrad")
        off += nw + co
        if i == 0:
            continue
        # backward-data into the source gradients that nothing modifies later
        dx = dr.conv_dgrad(g, wb)
        o = 0
        for s, c in dr.LAYERS[i][1]:
            part = dx[..., o:o + c]
            o += c
            if s.startswith("p"):
                want = dr.bf16(part)
            elif s in ("u3", "u2", "u1", "u0", "d0", "d0b", "a4", "a0"):
                want = dr.bf16(np.where(act[s] > 0, part, 0.0))
            else:
                continue
            assert _rel(gr[s], want) < 2e-3, (name, "dgrad", s, _rel(gr[s], want))
    fb.close()
    tb.close()


def test_l2_linear_loss_matches_oracle(gpu_ctx, denoiser):
    n, h, w = 1, 64, 64
    params, feats, tg = _problem(17, n, h, w)
    denoiser.set_params(params)
    denoiser.set_loss(hx.DN_LOSS_L2_LINEAR)
    fb = hx.DeviceBuffer(gpu_ctx, feats.nbytes)
    tb = hx.DeviceBuffer(gpu_ctx, tg.nbytes)
    fb.upload(feats)
    tb.upload(tg)
    try:
        loss = denoiser.forward_backward(fb, tb, n, h, w)
    finally:
        denoiser.set_loss(hx.DN_LOSS_L1_LOG)
    ref_loss, ref_grad, t = dr.loss_and_grad(params, feats, tg, rnd=True, loss="l2lin")
    assert abs(loss - ref_loss) <= 1e-3 * ref_loss, (loss, ref_loss)
    gy = denoiser.read_tensor("gy", gradient=True)[..., 0:3]
    y = denoiser.read_output()[..., 0:3].astype(np.float64)
    want = dr.bf16(2.0 * (np.expm1(y) - tg[..., 0:3]) * np.exp(y))
    assert _rel(gy, want) < 1e-2
    grad = denoiser.gradients()
    assert _rel(grad, ref_grad) < 3e-2, _rel(grad, ref_grad)
    fb.close()
    tb.close()


def test_adam_step_matches_oracle(gpu_ctx, denoiser):
    n, h, w = 1, 32, 32
    params, feats, tg = _problem(11, n, h, w)
    denoiser.set_params(params)
    fb = hx.DeviceBuffer(gpu_ctx, feats.nbytes)
    tb = hx.DeviceBuffer(gpu_ctx, tg.nbytes)
    fb.upload(feats)
    tb.upload(tg)
    denoiser.forward_backward(fb, tb, n, h, w)
    g = denoiser.gradients()
    denoiser.adam_step(1e-3)
    got = denoiser.get_params()
    m = np.zeros_like(params)
    v = np.zeros_like(params)
    want = dr.adam(params.copy(), m, v, g, 1, 1e-3)
    assert np.allclose(got, want, rtol=1e-5, atol=1e-7)
    fb.close()
    tb.close()


def test_training_reduces_loss(gpu_ctx, denoiser):
    """A fixed batch: 60 Adam steps cut the loss (the kernels train)."""
    n, h, w = 2, 64, 64
    params, feats, tg = _problem(5, n, h, w)
    tg[..., 0:3] = np.expm1(np.log1p(feats[..., 0:3]) * 0.5)  # a learnable mapping
    denoiser.set_params(params)
    fb = hx.DeviceBuffer(gpu_ctx, feats.nbytes)
    tb = hx.DeviceBuffer(gpu_ctx, tg.nbytes)
    fb.upload(feats)
    tb.upload(tg)
    first = denoiser.train_step(fb, tb, n, h, w, 1e-3)
    for _ in range(59):
        last = denoiser.train_step(fb, tb, n, h, w, 1e-3)
    assert last < 0.5 * first, (first, last)
    fb.close()
    tb.close()


def test_trained_denoiser_beats_plain_accumulation(gpu_ctx):
    """Train on tracer-made pairs (1-spp features -> 512-spp targets of
    seeded scene variants), then on held-out variants compare the relative
    RMSE of the denoised 1-spp image and of the plain 1-spp image against the
    512-spp image."""
    from helios_gb300 import denoise_train as T
    W = H = 64
    train_seeds = list(range(100, 124))
    eval_seeds = [900, 901, 902, 903]
    kw = dict(quads=4000, level=3, env=(256, 128), mask_size=64)
    data = T.render_pairs(gpu_ctx, train_seeds + eval_seeds, W, H, 1, 512, scene_kw=kw)
    dn = hx.Denoiser(gpu_ctx)
    dn.set_params(dr.init_params(0))
    hist = T.train(dn, data, 600, batch=8, lr=2e-3, lr_final=3e-4, seed=1, count=len(train_seeds))
    plain, den, _, _ = T.evaluate(gpu_ctx, dn, data, len(train_seeds), len(eval_seeds))
    print("loss %.4f -> %.4f; held-out rel RMSE plain 1 spp %.3f, denoised %.3f" % (hist[0][1], hist[-1][1], plain,
                                                                                   den))
    assert hist[-1][1] < hist[0][1]
    assert den < 0.6 * plain, (plain, den)
    dn.close()
    data.close()



@pytest.mark.parametrize("W,H", [(96, 64), (90, 61)])
def test_accumulated_aovs_are_the_mean_of_per_sample_aovs(gpu_ctx, W, H):
    """AOV accumulation: the features' albedo / depth / normal after N frames
    equal the mean of the N per-sample primary-hit AOVs (same jitter); the
    90 x 61 frame has right and bottom remainders of the 8 x 4 tile order the
    paths are traced in."""
    from tests.helpers import small_icosphere_scene
    hs = small_icosphere_scene(level=3, quads=2000, pool=4, mask=64, env=(128, 64))
    sc = hx.Scene(gpu_ctx, hs)
    N = 4
    f = hx.frame_desc(hs.camera(), W, H)
    pol = hx.policy_reference()
    a = hx.PathIntegrator(gpu_ctx, sc, W, H, max_ray_bounces=4, policy=pol)
    a.set_aov_accumulation(True)
    a.render(f, 2)
    a.render(f, N - 2)  # two wavefronts: the running mean carries across calls
    buf = hx.DeviceBuffer(gpu_ctx, W * H * 48)
    a.features(f, buf)
    got = buf.download((H, W, 12))
    b = hx.PathIntegrator(gpu_ctx, sc, W, H, max_ray_bounces=4, policy=pol)
    acc = np.zeros((H, W, 12))
    for k in range(N):
        b.features(f, buf, frame_index=k)
        acc += buf.download((H, W, 12))
    acc /= N
    for lo, hi in ((4, 8), (8, 11)):
        assert np.allclose(got[..., lo:hi], acc[..., lo:hi], atol=1e-5), (lo, np.abs(got[..., lo:hi] - acc[..., lo:hi]).max())
    assert np.allclose(got[..., 0:3], a.read_accumulation()[..., 0:3])
    a.close()
    b.close()
    buf.close()
    sc.close()
