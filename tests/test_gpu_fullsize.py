"""The configured workloads at their full sizes, checked against the oracle.

* Sort-last (512^3 fp32, 64 blobs, chopSuey 2x2x2 = 8 virtual ranks, 1024^2,
  the bench's volume and camera seeds 2001 / 2002): four whole frames
  bit-exact, sample counts included.
* Batched (the same field in uneven 3x2x2 bricks = 12 ranks, 64 views at
  1024^2 + 32 at 512^2 in one graph-captured persistent launch): four views
  read from the batch's own frame buffers (two of each size), bit-exact.
* Large (1024^3 fp32 in 4x4x4 chopSuey bricks = 64 ranks, 2048^2): two views
  under both work divisions, 8 spread rows of each checked bit-exact.
* Differentiable (128^3 single brick, 16 views at 256^2, L2 loss against
  targets from a second seeded transfer function, a checkpoint every 32
  samples): the transfer-function and density gradients within 1e-3 of the
  FP64 oracle adjoint, and central differences (eps 1e-3) on 64 uniformly
  random transfer-function entries and 64 uniformly random voxels, with
  early termination on and off.
* A near-opaque transfer function (alpha up to 1, and a band of alpha exactly
  1) with early termination off: the closed-form backward's division by the
  remaining transmittance against the FP64 adjoint.

The oracle runs on the host cores (OpenMP): a whole 1024^2 frame of the
sort-last workload takes about a second.  Up to ~30 GB of device memory and
~9 GB of host memory (the 1024^3 bricks for the oracle).
"""
import numpy as np
import pytest

from aloha_gb300 import abi
from aloha_gb300 import scenes as S
from aloha_gb300 import volfile as V

pytestmark = pytest.mark.gpu


def _field(torch, n, n_blobs, sigma, seed):
    """The bench's seeded blob field, built on the GPU, and its host copy."""
    vol = S.blob_field((n, n, n), n_blobs, sigma, seed=seed, device=torch.device("cuda", 0))
    return vol, vol.cpu().numpy()


def _assert_same(got, want, what):
    got = np.asarray(got).view(np.uint32)
    bad = int((got != want).sum())
    assert bad == 0, f"{what}: {bad} pixels differ from the oracle"


def test_sort_last_whole_frames_bit_exact(gpu_ctx_factory, oracle):
    torch = pytest.importorskip("torch")
    n, W = 512, 1024
    vol, vol_np = _field(torch, n, 64, (n / 16.0, n / 6.4), 2001)
    descs = V.chopsuey_split((n, n, n), 8)
    ctx = gpu_ctx_factory()
    ctx.set_bricks(descs, [V.brick_voxels(vol, d) for d in descs])
    del vol
    vox = [V.brick_voxels(vol_np, d) for d in descs]
    del vol_np
    tf = S.ramp_tf()
    ctx.set_transfer_function(tf)
    ctx.set_params()
    cams = S.orbit_cameras((n, n, n), 4, W, W, seed=2002)  # the first four of the workload's 256
    for i, cam in enumerate(cams):
        ctx.set_camera(0, *cam)
        ctx.resize(0, W, W)
        fb = ctx.render(0, width=W, height=W)
        samples = ctx.stats().samples
        ref = oracle.render(descs, vox, tf, oracle.make_camera(*cam), W, W, oracle.make_params(), n_ranks=8)
        _assert_same(fb, ref["fb"], f"camera {i}")
        assert samples == ref["samples"], f"camera {i}: {samples} samples vs {ref['samples']}"
        assert samples > 10**8


def test_batched_uneven_views_bit_exact(gpu_ctx_factory, oracle):
    torch = pytest.importorskip("torch")
    n = 512
    vol, vol_np = _field(torch, n, 64, (n / 16.0, n / 6.4), 2001)
    descs = S.grid_split((n, n, n), ([200, 380], [256], [300]))
    ctx = gpu_ctx_factory()
    ctx.set_bricks(descs, [V.brick_voxels(vol, d) for d in descs])
    del vol
    vox = [V.brick_voxels(vol_np, d) for d in descs]
    del vol_np
    tf = S.ramp_tf()
    ctx.set_transfer_function(tf)
    ctx.set_ranks(len(descs))
    ctx.set_params()
    sizes = [1024] * 64 + [512] * 32
    cams = [S.orbit_cameras((n, n, n), 1, w, w, seed=3002 + i)[0] for i, w in enumerate(sizes)]
    fbs = []
    for v, (w, cam) in enumerate(zip(sizes, cams)):
        ctx.set_camera(v, *cam)
        ctx.resize(v, w, w)
        fbs.append(torch.full((w, w), -1, dtype=torch.int32, device="cuda"))
    b = ctx.batch(list(range(len(sizes))), fbs)
    b.launch_graph()
    torch.cuda.synchronize()
    for v in (0, 37, 64, 95):
        w = sizes[v]
        ref = oracle.render(descs, vox, tf, oracle.make_camera(*cams[v]), w, w, oracle.make_params(),
                            n_ranks=len(descs))
        _assert_same(fbs[v].cpu().numpy(), ref["fb"], f"batch view {v} ({w}^2)")
    b.close()


def test_large_rows_bit_exact_both_splits(gpu_ctx_factory, oracle):
    torch = pytest.importorskip("torch")
    n, W = 1024, 2048
    dims = (n, n, n)
    vol, vol_np = _field(torch, n, 64, (n / 16.0, n / 6.4), 5001)
    descs = V.chopsuey_split(dims, 64)
    ctx = gpu_ctx_factory()
    ctx.set_bricks(descs, [V.brick_voxels(vol, d) for d in descs])
    del vol
    torch.cuda.empty_cache()
    vox = [V.brick_voxels(vol_np, d) for d in descs]
    del vol_np
    tf = S.ramp_tf()
    ctx.set_transfer_function(tf)
    ctx.set_ranks(64)
    ctx.set_params()
    rows = (3, 300, 611, 1000, 1024, 1337, 1702, 2044)
    for i, cam in enumerate(S.orbit_cameras(dims, 2, W, W, seed=5004)):
        ctx.set_camera(0, *cam)
        ctx.resize(0, W, W)
        frames = []
        for split in (abi.SPLIT_PIXELS, abi.SPLIT_RANKS):
            ctx.set_render_split(split)
            frames.append(ctx.render(0, width=W, height=W))
        c = oracle.make_camera(*cam)
        sched = oracle.schedule(descs, 64, list(c.org))
        for y in rows:
            ref = oracle.render(descs, vox, tf, c, W, W, oracle.make_params(), n_ranks=64, rows=(y, y + 1),
                                sched=sched)
            for name, fb in zip(("pixel split", "rank split"), frames):
                _assert_same(fb[y], ref["fb"][y], f"view {i} row {y} ({name})")
        assert int((frames[0] != 0).sum()) > W * W // 10


# ---------------------------------------------------------------- adjoint

def _rel(a, b):
    return float(np.linalg.norm(np.ravel(a - b)) / max(np.linalg.norm(np.ravel(b)), 1e-30))


def _c4_setup(torch, gpu_ctx_factory, et_alpha):
    n, W = 128, 256
    vol = S.blob_field((n, n, n), 16, (4.0, 12.0), seed=4001, device=torch.device("cuda", 0))
    vol_np = vol.cpu().numpy()
    descs = S.single_brick((n, n, n))
    vox = [V.brick_voxels(vol_np, d) for d in descs]
    cams = S.orbit_cameras((n, n, n), 16, W, W, seed=4002)
    ctx = gpu_ctx_factory()
    ctx.set_bricks(descs, vox)
    ctx.set_ranks(1)
    ctx.set_params(et_alpha=et_alpha)
    for v, cam in enumerate(cams):
        ctx.set_camera(v, *cam)
        ctx.resize(v, W, W)
    return ctx, descs, vox, cams


class _C4Loss:
    """L2 loss of the 16 views against targets of a second seeded transfer
    function, evaluated through the differentiable forward (K = 32)."""

    def __init__(self, torch, ctx, tf, K=32):
        self.torch, self.ctx, self.K = torch, ctx, K
        self.imgs = torch.empty((16, 256, 256, 4), dtype=torch.float32, device="cuda")
        self.target = self.images(S.seeded_tf(77))[0].double()
        self.tf = tf

    def images(self, table):
        self.ctx.set_transfer_function(table)
        samples = 0
        for v in range(16):
            self.ctx.forward(v, self.imgs[v], self.K)
            samples += self.ctx.stats().samples
        self.torch.cuda.synchronize()
        return self.imgs.clone(), samples

    def __call__(self, table):
        img, samples = self.images(table)
        return float(((img.double() - self.target) ** 2).sum()), img, samples

    def gradients(self):
        torch = self.torch
        img, _ = self.images(self.tf)
        grad = (2.0 * (img.double() - self.target)).float().contiguous()
        dtf = torch.zeros((256, 4), dtype=torch.float32, device="cuda")
        dden = torch.zeros((128, 128, 128), dtype=torch.float32, device="cuda")
        for v in range(16):
            self.ctx.backward(v, grad[v], dtf, dden, (0, 0, 0), (128, 128, 128))
        torch.cuda.synchronize()
        return grad, dtf.cpu().numpy(), dden.cpu().numpy()


def test_differentiable_configuration_fp64(gpu_ctx_factory, oracle):
    """128^3, 16 x 256^2, L2 loss against targets of a second seeded transfer
    function, K = 32, early termination at 0.99: the summed gradients of all
    16 views within relative 1e-3 (2-norm) of the oracle's FP64 adjoint,
    evaluated on the same fp32 inputs."""
    torch = pytest.importorskip("torch")
    ctx, descs, vox, cams = _c4_setup(torch, gpu_ctx_factory, 0.99)
    tf = S.ramp_tf()
    grad, dtf, dden = _C4Loss(torch, ctx, tf).gradients()
    grad_np = grad.cpu().numpy().astype(np.float64)
    ref_tf = np.zeros((256, 4))
    ref_den = np.zeros((128, 128, 128))
    for v, cam in enumerate(cams):
        r = oracle.adjoint(descs, vox, tf, oracle.make_camera(*cam), 256, 256, grad_np[v], (0, 0, 0), (128, 128, 128))
        ref_tf += r["dtf"]
        ref_den += r["ddensity"]
    # the configured bound; measured: about 3e-4 for the density gradient
    assert _rel(dtf, ref_tf) < 1e-3
    assert _rel(dden, ref_den) < 1e-3
    assert np.count_nonzero(dden) > 10**5


@pytest.mark.parametrize("et_alpha", [2.0, 0.99])
def test_differentiable_configuration_central_differences(gpu_ctx_factory, et_alpha):
    """Central differences, eps = 1e-3, on 64 uniformly random transfer-function
    entries and 64 uniformly random voxels of the differentiable configuration.
    Tolerance and exclusions, fixed here before any number is seen:
    * the loss is the float64 sum of the fp32 images' squared errors, so a
      difference quotient carries the images' rounding: for each entry the
      noise bound is 8 * sqrt(m) * 2^-24 * max|dL/dimage| / (2 eps), with m the
      number of image values that differ between the two perturbed renders;
    * early termination is held fixed by the adjoint (a discontinuity).  With
      it on (alpha 0.99, the configuration), an entry whose two perturbed
      renders take different numbers of samples has flipped some ray's
      termination and is excluded; with 10^6 rays nearly every alpha entry
      does, so the alpha entries are checked with termination off (alpha 2);
    * an entry where the loss is not smooth at this eps is excluded: the
      one-sided quotients (L(x+eps) - L(x)) / eps and (L(x) - L(x-eps)) / eps
      differ by more than 5% of the larger plus twice the noise bound (a
      piecewise-linear lookup crossing a texel centre, the |N.d| kink of the
      shading); at most a quarter of the entries of each kind may be excluded
      so;
    * every other entry must satisfy |fd - ad| <= 1e-2 |ad| + noise bound, and
      at least 16 transfer-function entries and 32 voxels must be checked.
    """
    torch = pytest.importorskip("torch")
    ctx, descs, vox, cams = _c4_setup(torch, gpu_ctx_factory, et_alpha)
    tf = S.ramp_tf()
    loss = _C4Loss(torch, ctx, tf)
    grad, dtf, dden = loss.gradients()
    eps = 1e-3
    gmax = float(grad.abs().max())
    n = 128
    rng = np.random.default_rng(4003)
    tf_idx = [tuple(int(i) for i in np.unravel_index(k, (256, 4))) for k in rng.choice(256 * 4, 64, replace=False)]
    den_idx = [tuple(int(i) for i in np.unravel_index(k, (n, n, n))) for k in rng.choice(n ** 3, 64, replace=False)]
    L0, _, _ = loss(tf)
    for kind, picks, ad_all in (("tf", tf_idx, dtf), ("density", den_idx, dden)):
        kinks, flips, checked, failed = 0, 0, 0, []
        for idx in picks:
            res = []
            for sgn in (1.0, -1.0):
                table = tf
                if kind == "tf":
                    table = tf.copy()
                    table[idx] += np.float32(sgn * eps)
                else:
                    v2 = vox[0].copy()
                    v2[idx] += np.float32(sgn * eps)
                    ctx.update_brick(0, v2)
                res.append(loss(table))
            if kind == "density":
                ctx.update_brick(0, vox[0])
            (Lp, ip, sp), (Lm, im, sm) = res
            if sp != sm:
                flips += 1
                continue
            m = int((ip != im).sum())
            noise = 8.0 * np.sqrt(m) * 2.0 ** -24 * gmax / (2 * eps)
            fd = (Lp - Lm) / (2 * eps)
            dp, dm = (Lp - L0) / eps, (L0 - Lm) / eps
            if abs(dp - dm) > 0.05 * max(abs(dp), abs(dm)) + 2 * noise:
                kinks += 1
                continue
            checked += 1
            ad = float(ad_all[idx])
            if abs(fd - ad) > 1e-2 * abs(ad) + noise:
                failed.append((idx, ad, fd, noise))
        assert kinks <= len(picks) // 4, f"{kind}: {kinks} of {len(picks)} entries not smooth at eps"
        assert checked >= (16 if kind == "tf" else 32), f"{kind}: only {checked} checked ({flips} termination flips)"
        assert not failed, f"{kind}: {failed[:5]}"


@pytest.mark.parametrize("tf_kind,et_alpha", [("ramp_to_1", 2.0), ("band_of_1", 2.0), ("step_to_1", 2.0),
                                              ("step_to_1", 0.99)])
def test_near_opaque_backward_matches_fp64(gpu_ctx_factory, oracle, tf_kind, et_alpha):
    """Alpha up to 1 with early termination off: rays run on far past the
    point where 1 - a vanishes, so the closed-form backward's division by the
    remaining transmittance is exercised where it is smallest.  A step to
    alpha 1 makes most rays opaque at their first visible sample, where the
    adjoint of the accumulated alpha is the rest of the ray's composite (and,
    with early termination, g_alpha)."""
    n, W = 48, 80
    vol = S.blob_field((n, n, n), 12, (n / 16.0, n / 6.0), seed=71)
    descs = V.chopsuey_split((n, n, n), 8)
    vox = S.extract_bricks(vol, descs)
    if tf_kind == "ramp_to_1":
        tf = S.ramp_tf(alpha_lo=0.1, alpha_max=1.0)
    elif tf_kind == "band_of_1":
        tf = S.ramp_tf(alpha_lo=0.1, alpha_max=0.5)
        tf[160:, 3] = 1.0  # a band of fully opaque entries
    else:
        tf = S.ramp_tf()
        tf[:, 3] = np.where(np.arange(256) < 60, 0.0, 1.0)  # transparent, then opaque
    ctx = gpu_ctx_factory()
    ctx.set_bricks(descs, vox)
    ctx.set_transfer_function(tf)
    ctx.set_ranks(1)
    ctx.set_params(et_alpha=et_alpha)
    params = oracle.make_params(et_alpha=et_alpha)
    rng = np.random.default_rng(73)
    dtf = np.zeros((256, 4), np.float32)
    dden = np.zeros((n, n, n), np.float32)
    ref_tf = np.zeros((256, 4))
    ref_den = np.zeros((n, n, n))
    opaque = 0
    for v, cam in enumerate(S.orbit_cameras((n, n, n), 2, W, W, seed=75)):
        ctx.set_camera(v, *cam)
        ctx.resize(v, W, W)
        img = np.zeros((W, W, 4), np.float32)
        ctx.forward(v, img, 16)
        opaque += int((img[..., 3] > 1.0 - 1e-6).sum())
        dl = rng.uniform(-1, 1, (W, W, 4)).astype(np.float32)
        ctx.backward(v, dl, dtf, dden, (0, 0, 0), (n, n, n))
        r = oracle.adjoint(descs, vox, tf, oracle.make_camera(*cam), W, W, dl, (0, 0, 0), (n, n, n), params)
        ref_tf += r["dtf"]
        ref_den += r["ddensity"]
    assert opaque > 200  # the case under test: rays that become opaque
    assert _rel(dtf, ref_tf) < 5e-4
    assert _rel(dden, ref_den) < 5e-4
