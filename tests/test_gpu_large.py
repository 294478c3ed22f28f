"""The batched and the large configurations at full size.

Batched: a 512^3 fp32 blob field in uneven 3x2x2 bricks (12 virtual ranks),
64 views at 1024^2 and 32 at 512^2 in one graph-captured persistent launch.
Large: a 1024^3 fp32 blob field in 4x4x4 chopSuey bricks (64 virtual ranks),
2048^2 frames, forward plus adjoint for the transfer function and the density
with a checkpoint every 64 samples.

The oracle cannot render these in seconds, so these checks use properties
that hold at any size: a batch equals the same views rendered one by one, the
two work divisions of a frame agree bit for bit, the differentiable forward
quantises to the render, and the adjoint is linear in dL/dimage with a
density part independent of whether the transfer-function gradient is taken.
About 65 GB of device memory at most.
"""
import numpy as np
import pytest

from aloha_gb300 import abi
from aloha_gb300 import scenes as S
from aloha_gb300 import volfile as V

pytestmark = pytest.mark.gpu

N, W, K = 1024, 2048, 64


def _rel(a, b):
    return float((a - b).double().norm() / max(float(b.double().norm()), 1e-30))


def test_512cube_uneven_bricks_96_views_batched(gpu_ctx_factory):
    torch = pytest.importorskip("torch")
    dev = torch.device("cuda", 0)
    n = 512
    vol = S.blob_field((n, n, n), 64, (n / 16.0, n / 6.4), seed=2001, device=dev)
    descs = S.grid_split((n, n, n), ([200, 380], [256], [300]))
    assert len(descs) == 12
    ctx = gpu_ctx_factory()
    ctx.set_bricks(descs, [V.brick_voxels(vol, d) for d in descs])
    del vol
    ctx.set_transfer_function(S.ramp_tf())
    ctx.set_ranks(12)
    ctx.set_params()
    sizes = [1024] * 64 + [512] * 32
    singles, samples = [], 0
    for v, w in enumerate(sizes):
        ctx.set_camera(v, *S.orbit_cameras((n, n, n), 1, w, w, seed=3002 + v)[0])
        ctx.resize(v, w, w)
        fb = torch.zeros((w, w), dtype=torch.int32, device=dev)
        ctx.render(v, fb)
        torch.cuda.synchronize()
        samples += ctx.stats().samples
        singles.append(fb)
    fbs = [torch.full_like(f, -1) for f in singles]
    b = ctx.batch(list(range(len(sizes))), fbs)
    b.autotune(reps=1)
    for f in fbs:
        f.fill_(-1)
    b.launch_graph()
    torch.cuda.synchronize()
    assert ctx.stats().samples == samples
    for got, want in zip(fbs, singles):
        assert torch.equal(got, want)
    b.close()
    ctx.close()


def test_1024cube_64_bricks_2048px(gpu_ctx_factory):
    torch = pytest.importorskip("torch")
    dev = torch.device("cuda", 0)
    dims = (N, N, N)
    vol = S.blob_field(dims, 64, (N / 16.0, N / 6.4), seed=5001, device=dev)
    descs = V.chopsuey_split(dims, 64)
    assert len(descs) == 64
    ctx = gpu_ctx_factory()
    ctx.set_bricks(descs, [V.brick_voxels(vol, d) for d in descs])
    del vol
    torch.cuda.empty_cache()
    ctx.set_transfer_function(S.ramp_tf())
    ctx.set_ranks(64)
    ctx.set_params()
    cam = S.orbit_cameras(dims, 1, W, W, seed=5002)[0]
    ctx.set_camera(0, *cam)
    ctx.resize(0, W, W)

    # 64 virtual ranks: the pixel split and the rank split give the same frame
    frames, samples = [], []
    for split in (abi.SPLIT_PIXELS, abi.SPLIT_RANKS):
        ctx.set_render_split(split)
        fb = torch.zeros((W, W), dtype=torch.int32, device=dev)
        ctx.render(0, fb)
        torch.cuda.synchronize()
        frames.append(fb)
        samples.append(ctx.stats().samples)
    assert torch.equal(frames[0], frames[1])
    assert samples[0] == samples[1] > 10**9
    assert float((frames[0] != 0).float().mean()) > 0.1
    del frames

    # one virtual rank: the differentiable forward quantises to the render
    ctx.set_ranks(1)
    ctx.set_render_split(abi.SPLIT_AUTO)
    fb1 = torch.zeros((W, W), dtype=torch.int32, device=dev)
    ctx.render(0, fb1)
    img = torch.empty((W, W, 4), dtype=torch.float32, device=dev)
    ctx.forward(0, img, K)
    torch.cuda.synchronize()
    q = (img.clamp(0.0, 1.0) * 255.0 + 0.5).to(torch.int64)
    packed = q[..., 0] | (q[..., 1] << 8) | (q[..., 2] << 16) | (q[..., 3] << 24)
    packed = torch.where(packed >= 2**31, packed - 2**32, packed).to(torch.int32)  # as the int32 view of RGBA8
    assert torch.equal(packed, fb1)
    del fb1, q, packed

    # the adjoint is linear in dL/dimage; its density part does not depend on
    # whether the transfer-function gradient is taken
    g = torch.Generator(device=dev).manual_seed(5003)
    dl = (torch.rand((W, W, 4), generator=g, device=dev) * 2.0 - 1.0).contiguous()
    lo, gd = (0, 0, 0), (N, N, N)
    dtf1 = torch.zeros((256, 4), dtype=torch.float32, device=dev)
    dden1 = torch.zeros(dims, dtype=torch.float32, device=dev)
    ctx.backward(0, dl, dtf1, dden1, lo, gd)
    dtf2 = torch.zeros_like(dtf1)
    dden2 = torch.zeros_like(dden1)
    ctx.backward(0, (2.0 * dl).contiguous(), dtf2, dden2, lo, gd)
    torch.cuda.synchronize()
    assert float(dtf1.abs().sum()) > 0 and int((dden1 != 0).sum()) > 10**6
    assert _rel(dtf2, 2.0 * dtf1) < 1e-5
    assert _rel(dden2, 2.0 * dden1) < 1e-5
    del dden2
    dden3 = torch.zeros_like(dden1)
    ctx.backward(0, dl, None, dden3, lo, gd)
    torch.cuda.synchronize()
    assert _rel(dden3, dden1) < 1e-5
    assert bool(torch.isfinite(dden1).all()) and bool(torch.isfinite(dtf1).all())
    ctx.close()
