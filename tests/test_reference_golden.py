"""Frames of the reference's own raygen (tests/golden/reference_frames.npz,
made by tests/golden/make_reference_golden.py from deviceCode.cpp compiled
unchanged) against the oracle (CPU, on every machine) and against the GPU
path through the C ABI.

Tolerance: the configured workloads' 1/255 per RGBA8 channel.  The reference
build rounds differently from the restatement (separate multiply and add in
generateRay, a plain trilinear per texture tap), so a few pixels sit one
level apart; the share of bit-identical pixels, the depth (relative 1e-5)
and the sample counts (early termination flips by a rounding at most in one
sample in a million) are bounded as well.
"""
import numpy as np
import pytest

from aloha_gb300 import abi
from tests.golden.make_reference_golden import load, scenes


def channels(fb):
    fb = np.asarray(fb, dtype=np.uint32)
    return np.stack([(fb >> (8 * c)) & 255 for c in range(4)], -1).astype(np.int32)


def pack(img):
    q = (np.clip(img, 0.0, 1.0) * np.float32(255.0) + np.float32(0.5)).astype(np.uint32)
    return q[..., 0] | (q[..., 1] << 8) | (q[..., 2] << 16) | (q[..., 3] << 24)


def check(gold, name, rank_images, rank_depth, samples):
    ref_fb = gold[name + "_fb"]
    mine = pack(rank_images)
    diff = np.abs(channels(ref_fb) - channels(mine))
    assert diff.max() <= 1, f"{name}: RGBA8 differs by {diff.max()}"
    assert (ref_fb == mine).mean() >= 0.999, name
    if name + "_depth" in gold:
        np.testing.assert_allclose(rank_depth, gold[name + "_depth"], rtol=1e-5, atol=0.0, err_msg=name)
    total = int(gold[name + "_samples"].sum(dtype=np.uint64))
    assert abs(int(samples) - total) <= max(4, total // 1_000_000), name


def test_oracle_matches_reference_frames(oracle):
    gold = load()
    for name, descs, vox, tf, cam, W, H, n_ranks in scenes():
        np.testing.assert_array_equal(oracle.partition_kd(descs, n_ranks)[0], gold[name + "_brick_rank"])
        r = oracle.render(descs, vox, tf, oracle.make_camera(*cam), W, H, oracle.make_params(crosshair=1),
                          n_ranks=n_ranks, order_mode=oracle.ORDER_REFERENCE_KD, want=("rank_images", "rank_depth"))
        check(gold, name, r["rank_images"], r["rank_depth"], r["samples"])


@pytest.mark.gpu
def test_gpu_matches_reference_frames(gpu_ctx_factory):
    gold = load()
    for name, descs, vox, tf, cam, W, H, n_ranks in scenes():
        ctx = gpu_ctx_factory()
        ctx.set_bricks(descs, vox)
        ctx.set_transfer_function(tf)
        ctx.set_ranks(n_ranks)
        ctx.set_params(crosshair=1, order_mode=abi.ORDER_REFERENCE_KD)
        ctx.set_camera(0, *cam)
        ctx.resize(0, W, H)
        imgs = np.zeros((n_ranks, H, W, 4), np.float32)
        depth = np.zeros((n_ranks, H, W), np.float32)
        ctx.render_partials(0, imgs, depth)
        check(gold, name, imgs, depth, ctx.stats().samples)
        ctx.close()
