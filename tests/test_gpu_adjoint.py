"""Differentiable form on the GPU: forward parity, gradients against the
FP64 oracle adjoint and against central finite differences (eps 1e-3)."""
import numpy as np
import pytest

from aloha_gb300 import abi
from aloha_gb300 import scenes as S
from tests import scenes_for_tests as T

pytestmark = pytest.mark.gpu


def setup(make, descs, vox, tf, **params):
    ctx = make()
    ctx.set_bricks(descs, vox)
    ctx.set_transfer_function(tf)
    ctx.set_ranks(1)
    ctx.set_params(**params)
    return ctx


def rel_err(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))


def density_scene(n=64, seed=5, bricks=1):
    vol = S.blob_field((n, n, n), 12, (n / 16.0, n / 6.0), seed=seed)
    if bricks == 1:
        descs = S.single_brick((n, n, n))
    else:
        from aloha_gb300 import volfile as V
        descs = V.chopsuey_split((n, n, n), bricks)
    return vol, descs, S.extract_bricks(vol, descs)


@pytest.mark.parametrize("k", [1, 7, 32])
def test_forward_is_the_render(gpu_ctx_factory, oracle, k):
    vol, descs, vox = density_scene(48, bricks=8)
    tf = S.ramp_tf()
    W, H = 72, 64
    ctx = setup(gpu_ctx_factory, descs, vox, tf)
    cam = T.cameras((48, 48, 48), 1, W, H, seed=3)[0]
    ctx.set_camera(0, *cam)
    ctx.resize(0, W, H)
    img = np.zeros((H, W, 4), np.float32)
    ctx.forward(0, img, k)
    samples = ctx.stats().samples
    ref = oracle.render(descs, vox, tf, oracle.make_camera(*cam), W, H, oracle.make_params(), n_ranks=1,
                        want=("final", "fb"))
    np.testing.assert_array_equal(img, ref["final"])
    assert samples == ref["samples"]
    np.testing.assert_array_equal(ctx.render(0, width=W, height=H), ref["fb"])


@pytest.mark.parametrize("bricks,k", [(1, 32), (8, 32), (8, 5)])
def test_backward_matches_fp64_oracle(gpu_ctx_factory, oracle, bricks, k):
    n = 48
    vol, descs, vox = density_scene(n, bricks=bricks)
    tf = S.ramp_tf()
    W, H = 80, 80
    ctx = setup(gpu_ctx_factory, descs, vox, tf)
    rng = np.random.default_rng(bricks + k)
    dtf = np.zeros((tf.shape[0], 4), np.float32)
    dden = np.zeros((n, n, n), np.float32)
    ref_tf = np.zeros((tf.shape[0], 4))
    ref_den = np.zeros((n, n, n))
    for v, cam in enumerate(T.cameras((n, n, n), 2, W, H, seed=7)):
        ctx.set_camera(v, *cam)
        ctx.resize(v, W, H)
        img = np.zeros((H, W, 4), np.float32)
        ctx.forward(v, img, k)
        dl = rng.uniform(-1, 1, (H, W, 4)).astype(np.float32)
        ctx.backward(v, dl, dtf, dden, (0, 0, 0), (n, n, n))
        r = oracle.adjoint(descs, vox, tf, oracle.make_camera(*cam), W, H, dl, (0, 0, 0), (n, n, n))
        ref_tf += r["dtf"]
        ref_den += r["ddensity"]
    assert rel_err(dtf, ref_tf) < 5e-4
    assert rel_err(dden, ref_den) < 5e-4
    assert np.count_nonzero(dden) > 1000


@pytest.mark.parametrize("bricks", [1, 8])
def test_density_only_backward(gpu_ctx_factory, oracle, bricks):
    """Without a transfer-function gradient the backward skips empty
    macrocells; its density gradient must still match the FP64 oracle and the
    full backward's (up to the order of the atomic adds)."""
    n = 48
    vol, descs, vox = density_scene(n, seed=9, bricks=bricks)
    tf = S.ramp_tf()
    W, H = 80, 72
    ctx = setup(gpu_ctx_factory, descs, vox, tf)
    rng = np.random.default_rng(31 + bricks)
    full_tf = np.zeros((tf.shape[0], 4), np.float32)
    full_den = np.zeros((n, n, n), np.float32)
    only_den = np.zeros((n, n, n), np.float32)
    ref_den = np.zeros((n, n, n))
    for v, cam in enumerate(T.cameras((n, n, n), 2, W, H, seed=17)):
        ctx.set_camera(v, *cam)
        ctx.resize(v, W, H)
        ctx.forward(v, np.zeros((H, W, 4), np.float32), 32)
        dl = rng.uniform(-1, 1, (H, W, 4)).astype(np.float32)
        ctx.backward(v, dl, full_tf, full_den, (0, 0, 0), (n, n, n))
        ctx.backward(v, dl, None, only_den, (0, 0, 0), (n, n, n))
        ref_den += oracle.adjoint(descs, vox, tf, oracle.make_camera(*cam), W, H, dl, (0, 0, 0), (n, n, n))["ddensity"]
    assert np.count_nonzero(only_den) > 1000
    assert rel_err(only_den, ref_den) < 5e-4
    np.testing.assert_allclose(only_den, full_den, rtol=1e-4, atol=1e-6 * float(np.abs(full_den).max()))


@pytest.mark.parametrize("kw", [dict(jitter_mode=abi.JITTER_CONST, jitter_value=0.37), dict(dt=0.3),
                                dict(jitter_mode=abi.JITTER_HASH, dt=0.375)])
def test_inexact_step_sequences(gpu_ctx_factory, oracle, kw):
    """Jittered first samples and step sizes that are not powers of two make
    the t sequence inexact on most bricks, so the training forward and the
    density-only replay step their skipped runs sample by sample; the dt 0.375
    case mixes both.  Forward, checkpoints (through the gradients) and both
    backward forms must still match the oracle."""
    n = 48
    vol, descs, vox = density_scene(n, seed=11, bricks=8)
    tf = S.ramp_tf()
    W, H = 72, 64
    ctx = setup(gpu_ctx_factory, descs, vox, tf, **kw)
    params = oracle.make_params(**kw)
    rng = np.random.default_rng(41)
    dtf = np.zeros((tf.shape[0], 4), np.float32)
    dden = np.zeros((n, n, n), np.float32)
    only_den = np.zeros((n, n, n), np.float32)
    ref_tf = np.zeros((tf.shape[0], 4))
    ref_den = np.zeros((n, n, n))
    for v, cam in enumerate(T.cameras((n, n, n), 2, W, H, seed=43)):
        ctx.set_camera(v, *cam)
        ctx.resize(v, W, H)
        img = np.zeros((H, W, 4), np.float32)
        ctx.forward(v, img, 7)
        ref = oracle.render(descs, vox, tf, oracle.make_camera(*cam), W, H, params, n_ranks=1, want=("final",))
        np.testing.assert_array_equal(img, ref["final"])
        assert ctx.stats().samples == ref["samples"]
        dl = rng.uniform(-1, 1, (H, W, 4)).astype(np.float32)
        ctx.backward(v, dl, dtf, dden, (0, 0, 0), (n, n, n))
        ctx.backward(v, dl, None, only_den, (0, 0, 0), (n, n, n))
        r = oracle.adjoint(descs, vox, tf, oracle.make_camera(*cam), W, H, dl, (0, 0, 0), (n, n, n), params)
        ref_tf += r["dtf"]
        ref_den += r["ddensity"]
    assert rel_err(dtf, ref_tf) < 5e-4
    assert rel_err(dden, ref_den) < 5e-4
    assert rel_err(only_den, ref_den) < 5e-4
    assert np.count_nonzero(dden) > 1000


def _loss(ctx, views, W, H, weights):
    total = 0.0
    for v in views:
        img = np.zeros((H, W, 4), np.float32)
        ctx.forward(v, img, 32)
        total += float((img.astype(np.float64) * weights[v]).sum())
    return total


@pytest.mark.parametrize("et", [0.99, 2.0])
def test_central_differences(gpu_ctx_factory, et):
    """dL/dtf and dL/ddensity against (L(x+eps) - L(x-eps)) / 2eps, eps = 1e-3, 64 entries."""
    n = 32
    vol, descs, vox = density_scene(n)
    tf = S.ramp_tf()
    W = H = 64
    ctx = setup(gpu_ctx_factory, descs, vox, tf, et_alpha=et)
    views = [0, 1]
    for v, cam in zip(views, T.cameras((n, n, n), 2, W, H, seed=11)):
        ctx.set_camera(v, *cam)
        ctx.resize(v, W, H)
    rng = np.random.default_rng(17)
    weights = {v: rng.uniform(0.5, 1.5, (H, W, 4)) for v in views}
    dtf = np.zeros((tf.shape[0], 4), np.float32)
    dden = np.zeros((n, n, n), np.float32)
    for v in views:
        img = np.zeros((H, W, 4), np.float32)
        ctx.forward(v, img, 32)
        ctx.backward(v, weights[v].astype(np.float32), dtf, dden, (0, 0, 0), (n, n, n))
    eps = 1e-3
    errs = []
    def candidates(g, k=128):
        # the k entries of largest |gradient| (finite differences of tiny
        # gradients are dominated by fp32 rounding of the loss)
        flat = np.argsort(-np.abs(g).ravel())[:k]
        flat = flat[np.abs(g.ravel()[flat]) > 0]
        return [np.unravel_index(i, g.shape) for i in flat]

    big_tf, big_den = candidates(dtf), candidates(dden)
    picks = [("tf", tuple(int(v) for v in big_tf[i])) for i in rng.choice(len(big_tf), 32, replace=False)]
    picks += [("den", tuple(int(v) for v in big_den[i])) for i in rng.choice(len(big_den), 32, replace=False)]
    for kind, idx in picks:
        if kind == "tf":
            f = []
            for sgn in (1, -1):
                t2 = tf.copy()
                t2[idx] += sgn * eps
                ctx.set_transfer_function(t2)
                f.append(_loss(ctx, views, W, H, weights))
            ctx.set_transfer_function(tf)
            ad = dtf[idx]
        else:
            f = []
            for sgn in (1, -1):
                v2 = vox[0].copy()
                v2[idx] += sgn * eps
                ctx.update_brick(0, v2)
                f.append(_loss(ctx, views, W, H, weights))
            ctx.update_brick(0, vox[0])
            ad = dden[idx]
        fd = (f[0] - f[1]) / (2 * eps)
        errs.append(abs(fd - ad) / abs(ad))
    errs = np.array(errs)
    # piecewise-linear lookups, the |N.d| kink and (with ET) termination flips
    # make a few entries non-smooth at this eps
    assert np.median(errs) < 1e-2
    assert np.mean(errs < 5e-2) > 0.85


def test_autograd_function(gpu_ctx_factory):
    torch = pytest.importorskip("torch")
    from aloha_gb300.autograd import DifferentiableRenderer, render_views
    n, W = 32, 48
    vol = S.blob_field((n, n, n), 8, (2.0, 5.0), seed=21)
    r = DifferentiableRenderer((n, n, n), bricks=1, checkpoint_every=16)
    for v, cam in enumerate(T.cameras((n, n, n), 3, W, W, seed=23)):
        r.set_camera(v, cam, W, W)
    tf_t = torch.from_numpy(S.ramp_tf()).cuda().requires_grad_(True)
    target_tf = torch.from_numpy(S.seeded_tf(5)).cuda()
    den = torch.from_numpy(vol).cuda().requires_grad_(True)
    with torch.no_grad():
        target = render_views(r, target_tf, den, [0, 1, 2], (W, W))
    img = render_views(r, tf_t, den, [0, 1, 2], (W, W))
    loss = ((img - target) ** 2).sum()
    loss.backward()
    assert tf_t.grad is not None and torch.isfinite(tf_t.grad).all() and tf_t.grad.abs().sum() > 0
    assert den.grad is not None and torch.isfinite(den.grad).all() and den.grad.abs().sum() > 0
    # one gradient step on the transfer function lowers the loss
    with torch.no_grad():
        tf2 = (tf_t - 1e-3 * tf_t.grad / tf_t.grad.abs().max()).clamp(0, 1)
        loss2 = ((render_views(r, tf2, den, [0, 1, 2], (W, W)) - target) ** 2).sum()
    assert float(loss2) < float(loss.detach())
    r.close()


def test_backward_errors(gpu_ctx_factory):
    vol, descs, vox = density_scene(32, bricks=2)
    tf = S.ramp_tf()
    ctx = gpu_ctx_factory()
    ctx.set_bricks(descs, vox)
    ctx.set_transfer_function(tf)
    cam = T.cameras((32, 32, 32), 1, 16, 16)[0]
    ctx.set_camera(0, *cam)
    ctx.resize(0, 16, 16)
    img = np.zeros((16, 16, 4), np.float32)
    with pytest.raises(abi.AlohaError) as e:
        ctx.forward(0, img, 32)  # two virtual ranks
    assert e.value.code == abi.ERR_UNSUPPORTED
    ctx.set_ranks(1)
    dtf = np.zeros((256, 4), np.float32)
    dden = np.zeros((32, 32, 32), np.float32)
    with pytest.raises(abi.AlohaError) as e:
        ctx.backward(0, img, dtf, dden, (0, 0, 0), (32, 32, 32))  # no forward yet
    assert e.value.code == abi.ERR_NOT_READY
    ctx.forward(0, img, 32)
    with pytest.raises(abi.AlohaError) as e:
        ctx.backward(0, img, dtf, dden, (0, 0, 0), (16, 32, 32))  # grid does not cover the bricks
    assert e.value.code == abi.ERR_OUT_OF_RANGE
    # grids whose voxel count or row count is out of range are refused before
    # anything is allocated or launched
    for dims in ((1 << 21, 1 << 10, 1 << 10), (32, 1 << 16, 1 << 16), (2**31 - 1, 2**31 - 1, 2**31 - 1)):
        with pytest.raises(abi.AlohaError) as e:
            ctx.backward(0, img, dtf, dden, (0, 0, 0), dims)
        assert e.value.code == abi.ERR_OUT_OF_RANGE, dims
    with pytest.raises(abi.AlohaError) as e:  # grid_lo + grid_dims beyond int range
        ctx.backward(0, img, dtf, dden, (2**31 - 40, 0, 0), (64, 32, 32))
    assert e.value.code == abi.ERR_OUT_OF_RANGE
    ctx.set_camera(0, *cam)
    with pytest.raises(abi.AlohaError) as e:
        ctx.backward(0, img, dtf, dden, (0, 0, 0), (32, 32, 32))  # camera changed since the forward
    assert e.value.code == abi.ERR_NOT_READY


@pytest.mark.parametrize("bricks", [1, 8])
def test_gradient_buffer_is_clear_between_calls(gpu_ctx_factory, bricks):
    """The fold leaves the x-quad gradient buffer zero for the next call (no
    memset between calls): repeated density backwards agree, a larger grid
    around the bricks holds the same gradient with zeros outside, a smaller
    grid after it and calls after a failed one agree again."""
    n = 40
    vol, descs, vox = density_scene(n, seed=23, bricks=bricks)
    ctx = setup(gpu_ctx_factory, descs, vox, S.ramp_tf())
    W, H = 64, 56
    cam = T.cameras((n, n, n), 1, W, H, seed=5)[0]
    ctx.set_camera(0, *cam)
    ctx.resize(0, W, H)
    ctx.forward(0, np.zeros((H, W, 4), np.float32), 16)
    dl = np.random.default_rng(3).uniform(-1, 1, (H, W, 4)).astype(np.float32)

    def density(lo=(0, 0, 0), dims=(n, n, n)):
        g = np.zeros(dims[::-1], np.float32)
        ctx.backward(0, dl, None, g, lo, dims)
        return g

    first = density()
    assert np.count_nonzero(first) > 500
    tol = dict(rtol=1e-5, atol=1e-6 * float(np.abs(first).max()))
    np.testing.assert_allclose(density(), first, **tol)
    big = density((-3, -2, -1), (n + 7, n + 5, n + 2))
    np.testing.assert_allclose(big[1:1 + n, 2:2 + n, 3:3 + n], first, **tol)
    inner = np.zeros(big.shape, bool)
    inner[1:1 + n, 2:2 + n, 3:3 + n] = True
    assert not big[~inner].any()
    np.testing.assert_allclose(density(), first, **tol)
    with pytest.raises(abi.AlohaError):
        ctx.backward(0, dl, None, np.zeros((n, n, n), np.float32), (0, 0, 0), (n - 1, n, n))
    np.testing.assert_allclose(density(), first, **tol)


@pytest.mark.parametrize("bricks", [1, 8])
def test_tf_only_backward(gpu_ctx_factory, oracle, bricks):
    """Without a density gradient (dl_ddensity NULL) the backward skips the
    shading and stencil adjoints; its transfer-function gradient must match the
    FP64 oracle and the full backward's (up to the order of the atomic adds)."""
    n = 48
    vol, descs, vox = density_scene(n, seed=13, bricks=bricks)
    tf = S.ramp_tf()
    W, H = 80, 72
    ctx = setup(gpu_ctx_factory, descs, vox, tf)
    rng = np.random.default_rng(61 + bricks)
    full_tf = np.zeros((tf.shape[0], 4), np.float32)
    full_den = np.zeros((n, n, n), np.float32)
    only_tf = np.zeros((tf.shape[0], 4), np.float32)
    ref_tf = np.zeros((tf.shape[0], 4))
    for v, cam in enumerate(T.cameras((n, n, n), 2, W, H, seed=19)):
        ctx.set_camera(v, *cam)
        ctx.resize(v, W, H)
        ctx.forward(v, np.zeros((H, W, 4), np.float32), 32)
        dl = rng.uniform(-1, 1, (H, W, 4)).astype(np.float32)
        ctx.backward(v, dl, full_tf, full_den, (0, 0, 0), (n, n, n))
        ctx.backward(v, dl, only_tf, None, None, None)
        ref_tf += oracle.adjoint(descs, vox, tf, oracle.make_camera(*cam), W, H, dl, (0, 0, 0), (n, n, n))["dtf"]
    assert np.count_nonzero(only_tf) > 100
    assert rel_err(only_tf, ref_tf) < 5e-4
    np.testing.assert_allclose(only_tf, full_tf, rtol=1e-4, atol=1e-6 * float(np.abs(full_tf).max()))
    with pytest.raises(abi.AlohaError) as e:
        ctx.backward(0, dl, None, None, None, None)
    assert e.value.code == abi.ERR_NULL_POINTER


@pytest.mark.parametrize("where", ["host", "device"])
def test_backward_views_is_the_sum(gpu_ctx_factory, oracle, where):
    """aloha_backward_views over three views (of different sizes) equals the
    sum of three aloha_backward calls up to the order of the atomic adds, and
    the FP64 oracle's sum; it accumulates (+=) into what the buffers hold."""
    torch = pytest.importorskip("torch")
    n = 48
    vol, descs, vox = density_scene(n, seed=17, bricks=8)
    tf = S.ramp_tf()
    ctx = setup(gpu_ctx_factory, descs, vox, tf)
    rng = np.random.default_rng(71)
    sizes = [(80, 72), (64, 64), (96, 40)]
    views, dls = [0, 2, 1], []
    ref_tf = np.zeros((tf.shape[0], 4))
    ref_den = np.zeros((n, n, n))
    cams = T.cameras((n, n, n), 3, 80, 80, seed=43)
    for v in views:
        W, H = sizes[v]
        ctx.set_camera(v, *cams[v])
        ctx.resize(v, W, H)
        ctx.forward(v, np.zeros((H, W, 4), np.float32), 32)
        dl = rng.uniform(-1, 1, (H, W, 4)).astype(np.float32)
        dls.append(dl)
        r = oracle.adjoint(descs, vox, tf, oracle.make_camera(*cams[v]), W, H, dl, (0, 0, 0), (n, n, n))
        ref_tf += r["dtf"]
        ref_den += r["ddensity"]
    one_tf = np.zeros((tf.shape[0], 4), np.float32)
    one_den = np.zeros((n, n, n), np.float32)
    for v, dl in zip(views, dls):
        ctx.backward(v, dl, one_tf, one_den, (0, 0, 0), (n, n, n))
    start_tf = rng.uniform(-1, 1, (tf.shape[0], 4)).astype(np.float32)
    start_den = rng.uniform(-1, 1, (n, n, n)).astype(np.float32)
    if where == "host":
        many_tf, many_den, dl_in = start_tf.copy(), start_den.copy(), dls
    else:
        many_tf, many_den = torch.from_numpy(start_tf).cuda(), torch.from_numpy(start_den).cuda()
        dl_in = [torch.from_numpy(d).cuda() for d in dls]
    ctx.backward_views(views, dl_in, many_tf, many_den, (0, 0, 0), (n, n, n))
    if where == "device":
        torch.cuda.synchronize()
        many_tf, many_den = many_tf.cpu().numpy(), many_den.cpu().numpy()
    many_tf -= start_tf
    many_den -= start_den
    # both forms against the FP64 adjoint (three views of eight bricks)
    for got_tf, got_den in ((one_tf, one_den), (many_tf, many_den)):
        assert rel_err(got_tf, ref_tf) < 5e-4
        assert rel_err(got_den, ref_den) < 5e-4
    np.testing.assert_allclose(many_tf, one_tf, rtol=1e-4, atol=1e-5 * float(np.abs(one_tf).max()))
    np.testing.assert_allclose(many_den, one_den, rtol=1e-4, atol=1e-5 * float(np.abs(one_den).max()))
    # the transfer-function-only form, and the argument checks
    only_tf = np.zeros((tf.shape[0], 4), np.float32)
    ctx.backward_views(views, dls, only_tf, None, None, None)
    np.testing.assert_allclose(only_tf, one_tf, rtol=1e-4, atol=1e-5 * float(np.abs(one_tf).max()))
    for bad, code in [(([0, 0], dls[:2]), abi.ERR_INVALID_ARGUMENT), (([], []), abi.ERR_INVALID_ARGUMENT),
                      (([0, 5], dls[:2]), abi.ERR_OUT_OF_RANGE)]:
        with pytest.raises(abi.AlohaError) as e:
            ctx.backward_views(*bad, only_tf, None, None, None)
        assert e.value.code == code
    ctx.set_camera(2, *cams[2])  # view 2's checkpoints are stale now
    with pytest.raises(abi.AlohaError) as e:
        ctx.backward_views(views, dls, only_tf, None, None, None)
    assert e.value.code == abi.ERR_NOT_READY


@pytest.mark.parametrize("bricks", [1, 8])
def test_forward_views_equals_single_forwards(gpu_ctx_factory, oracle, bricks):
    """aloha_forward_views renders every view's image bit for bit as
    aloha_forward does (host and device images, different sizes, centre-out
    chunks across views), and leaves checkpoints the backward replays: the
    summed gradient of views forwarded together, and of views forwarded at two
    different checkpoint intervals, matches the FP64 oracle."""
    torch = pytest.importorskip("torch")
    n = 48
    vol, descs, vox = density_scene(n, seed=23, bricks=bricks)
    tf = S.ramp_tf()
    ctx = setup(gpu_ctx_factory, descs, vox, tf)
    sizes = {0: (64, 48), 3: (40, 40), 5: (96, 33), 7: (8, 8)}
    cams = T.cameras((n, n, n), 8, 64, 64, seed=61)
    ref_img = {}
    for v, (W, H) in sizes.items():
        ctx.set_camera(v, *cams[v])
        ctx.resize(v, W, H)
        ref = oracle.render(descs, vox, tf, oracle.make_camera(*cams[v]), W, H, oracle.make_params(), n_ranks=1,
                            want=("final",))
        ref_img[v] = ref["final"]
    views = [5, 0, 7, 3]
    imgs = [np.zeros((sizes[v][1], sizes[v][0], 4), np.float32) if i % 2 else
            torch.zeros((sizes[v][1], sizes[v][0], 4), device="cuda") for i, v in enumerate(views)]
    ctx.forward_views(views, imgs, 16)
    torch.cuda.synchronize()
    for v, img in zip(views, imgs):
        got = img.cpu().numpy() if hasattr(img, "cpu") else img
        np.testing.assert_array_equal(got, ref_img[v])
    rng = np.random.default_rng(3)
    dls = [rng.uniform(-1, 1, (sizes[v][1], sizes[v][0], 4)).astype(np.float32) for v in views]
    ref_tf = np.zeros((tf.shape[0], 4))
    ref_den = np.zeros((n, n, n))
    for v, dl in zip(views, dls):
        W, H = sizes[v]
        r = oracle.adjoint(descs, vox, tf, oracle.make_camera(*cams[v]), W, H, dl, (0, 0, 0), (n, n, n))
        ref_tf += r["dtf"]
        ref_den += r["ddensity"]
    for mixed in (False, True):
        if mixed:  # views 0 and 3 again, at another interval: two replay launches
            ctx.forward_views([0, 3], [np.zeros((sizes[v][1], sizes[v][0], 4), np.float32) for v in (0, 3)], 7)
        dtf = np.zeros((tf.shape[0], 4), np.float32)
        dden = np.zeros((n, n, n), np.float32)
        ctx.backward_views(views, dls, dtf, dden, (0, 0, 0), (n, n, n))
        assert rel_err(dtf, ref_tf) < 5e-4, mixed
        assert rel_err(dden, ref_den) < 5e-4, mixed
    with pytest.raises(abi.AlohaError) as e:
        ctx.forward_views([0, 0], [imgs[1], imgs[1]], 16)
    assert e.value.code == abi.ERR_INVALID_ARGUMENT


def test_many_chunk_training_forward(gpu_ctx_factory):
    """A training forward of many chunks per resident warp runs the instance
    with more CTAs per SM: two 1024x800 views forwarded together (51 200
    chunks) give the same images as each view forwarded alone (25 600 chunks,
    the other instance), and the same gradients afterwards."""
    torch = pytest.importorskip("torch")
    n = 32
    vol, descs, vox = density_scene(n, seed=29, bricks=8)
    tf = S.ramp_tf()
    ctx = setup(gpu_ctx_factory, descs, vox, tf)
    W, H = 1024, 800
    cams = T.cameras((n, n, n), 2, W, H, seed=67)
    for v in range(2):
        ctx.set_camera(v, *cams[v])
        ctx.resize(v, W, H)
    dev = "cuda"
    alone = [torch.zeros((H, W, 4), device=dev) for _ in range(2)]
    for v in range(2):
        ctx.forward(v, alone[v], 16)
    g = torch.Generator(device=dev).manual_seed(11)
    dls = [(torch.rand((H, W, 4), generator=g, device=dev) * 2 - 1).contiguous() for _ in range(2)]
    dtf1 = torch.zeros((256, 4), device=dev)
    dden1 = torch.zeros((n, n, n), device=dev)
    ctx.backward_views([0, 1], dls, dtf1, dden1, (0, 0, 0), (n, n, n))
    together = [torch.zeros((H, W, 4), device=dev) for _ in range(2)]
    ctx.forward_views([0, 1], together, 16)
    dtf2 = torch.zeros_like(dtf1)
    dden2 = torch.zeros_like(dden1)
    ctx.backward_views([0, 1], dls, dtf2, dden2, (0, 0, 0), (n, n, n))
    torch.cuda.synchronize()
    for v in range(2):
        assert float((alone[v][..., 3] > 0).float().mean()) > 0.05
        assert torch.equal(together[v], alone[v])
    for a, b in ((dtf2, dtf1), (dden2, dden1)):
        assert float(b.abs().max()) > 0
        torch.testing.assert_close(a, b, rtol=1e-4, atol=1e-5 * float(b.abs().max()))


def test_autograd_gradient_flags_and_uploads(gpu_ctx_factory):
    """The binding computes only the gradients autograd asks for, and uploads
    the bricks again only when the density tensor changed."""
    torch = pytest.importorskip("torch")
    from aloha_gb300.autograd import DifferentiableRenderer, render_views
    n, W = 32, 40
    vol = S.blob_field((n, n, n), 8, (2.0, 5.0), seed=27)
    r = DifferentiableRenderer((n, n, n), bricks=1, checkpoint_every=16)
    for v, cam in enumerate(T.cameras((n, n, n), 2, W, W, seed=29)):
        r.set_camera(v, cam, W, W)
    tf = torch.from_numpy(S.ramp_tf()).cuda()
    target = torch.rand((2, W, W, 4), device="cuda")
    den = torch.from_numpy(vol).cuda()
    # both gradients: the reference for the transfer-function gradient below
    tf_a = tf.clone().requires_grad_(True)
    den_a = den.clone().requires_grad_(True)
    ((render_views(r, tf_a, den_a, [0, 1], (W, W)) - target) ** 2).sum().backward()
    uploads = r.brick_uploads
    # transfer function only: no density gradient, and the same density
    # tensor is not uploaded again
    tf_b = tf.clone().requires_grad_(True)
    ((render_views(r, tf_b, den_a.detach(), [0, 1], (W, W)) - target) ** 2).sum().backward()
    assert r.brick_uploads == uploads + 1  # detach() is a new tensor object
    uploads = r.brick_uploads
    tf_c = tf.clone().requires_grad_(True)
    den_c = den.clone()  # does not require grad
    ((render_views(r, tf_c, den_c, [0, 1], (W, W)) - target) ** 2).sum().backward()
    assert r.brick_uploads == uploads + 1
    ((render_views(r, tf.clone().requires_grad_(True), den_c, [0, 1], (W, W)) - target) ** 2).sum().backward()
    assert r.brick_uploads == uploads + 1  # unchanged density: no upload
    den_c.mul_(1.0)  # in place: version bump, uploaded again
    render_views(r, tf, den_c, [0, 1], (W, W))
    assert r.brick_uploads == uploads + 2
    torch.testing.assert_close(tf_c.grad, tf_a.grad, rtol=1e-4, atol=1e-6 * float(tf_a.grad.abs().max()))
    torch.testing.assert_close(tf_b.grad, tf_a.grad, rtol=1e-4, atol=1e-6 * float(tf_a.grad.abs().max()))
    # density only
    den_d = den.clone().requires_grad_(True)
    ((render_views(r, tf, den_d, [0, 1], (W, W)) - target) ** 2).sum().backward()
    torch.testing.assert_close(den_d.grad, den_a.grad, rtol=1e-4, atol=1e-6 * float(den_a.grad.abs().max()))
    r.close()


@pytest.mark.parametrize("case", [
    dict(dims=(36, 32, 40), dt=0.1, k=64),        # long segments of short steps
    dict(dims=(36, 32, 40), dt=4.0, k=1),         # a checkpoint before every long step
    dict(dims=(36, 32, 40), et_alpha=0.05),       # rays end early
    dict(dims=(36, 32, 40), n_tf=1),              # one transfer-function entry
    dict(dims=(36, 32, 40), n_tf=2048),           # the largest transfer function
    dict(dims=(48, 48, 1)),                       # one voxel thick
    dict(dims=(3, 40, 2)),                        # thinner than the apron
])
def test_training_edge_cases(gpu_ctx_factory, oracle, case):
    """Extremes of the step, checkpoint interval, early termination,
    transfer-function size and volume shape for the differentiable form: the
    forward image equals the oracle's and both gradients are within 5e-4 of
    the FP64 adjoint."""
    from aloha_gb300 import volfile as V
    dims = case["dims"]
    rng = np.random.default_rng(sum(dims) + 7)
    vol = (S.blob_field(dims, 6, (1.0, 6.0), seed=int(rng.integers(1 << 20))) * np.float32(1.2)).astype(np.float32)
    descs = V.chopsuey_split(dims, 2)
    vox = S.extract_bricks(vol, descs)
    n_tf = case.get("n_tf", 256)
    tf = S.seeded_tf(int(rng.integers(1 << 20)), n=max(n_tf, 2))[:n_tf].copy() if n_tf > 1 else \
        np.array([[0.8, 0.4, 0.2, 0.3]], np.float32)
    params = {k: case[k] for k in ("dt", "et_alpha") if k in case}
    ctx = setup(gpu_ctx_factory, descs, vox, tf, **params)
    op = oracle.make_params(**params)
    W, H = 48, 40
    cams = S.orbit_cameras(dims, 2, W, H, seed=9, distance=1.5)
    nx, ny, nz = dims
    for v, cam in enumerate(cams):
        ctx.set_camera(v, *cam)
        ctx.resize(v, W, H)
    imgs = [np.zeros((H, W, 4), np.float32) for _ in cams]
    ctx.forward_views([0, 1], imgs, case.get("k", 32))
    dls = [rng.uniform(-1, 1, (H, W, 4)).astype(np.float32) for _ in cams]
    dtf = np.zeros((n_tf, 4), np.float32)
    dden = np.zeros((nz, ny, nx), np.float32)
    ctx.backward_views([0, 1], dls, dtf, dden, (0, 0, 0), (nx, ny, nz))
    ref_tf = np.zeros((n_tf, 4))
    ref_den = np.zeros((nz, ny, nx))
    for cam, img, dl in zip(cams, imgs, dls):
        ref = oracle.render(descs, vox, tf, oracle.make_camera(*cam), W, H, op, n_ranks=1, want=("final",))
        np.testing.assert_array_equal(img, ref["final"])
        r = oracle.adjoint(descs, vox, tf, oracle.make_camera(*cam), W, H, dl, (0, 0, 0), (nx, ny, nz), op)
        ref_tf += r["dtf"]
        ref_den += r["ddensity"]
    if np.linalg.norm(ref_tf) > 0:
        assert rel_err(dtf, ref_tf) < 5e-4, case
    if np.linalg.norm(ref_den) > 0:
        assert rel_err(dden, ref_den) < 5e-4, case
