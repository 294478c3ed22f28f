"""Golden vectors (tests/golden/golden.npz, made by tests/golden/make_golden.py):
the oracle must reproduce them on every machine, and so must the GPU path."""
import numpy as np
import pytest

from aloha_gb300 import scenes as S
from tests import scenes_for_tests as T
from tests.golden.make_golden import cases, load


def test_oracle_reproduces_golden_vectors():
    gold = load()
    now = cases()
    assert set(gold) == set(now)
    for k in gold:
        np.testing.assert_array_equal(now[k], gold[k], err_msg=k)


@pytest.mark.gpu
def test_gpu_reproduces_golden_vectors(gpu_ctx_factory):
    from aloha_gb300 import abi
    gold = load()
    # plain
    vol, descs, vox, tf = T.c1_scene()
    ctx = gpu_ctx_factory()
    ctx.set_bricks(descs, vox)
    ctx.set_transfer_function(tf)
    ctx.set_params()
    ctx.set_camera(0, *S.axis_camera((64, 64, 64), 96, 96))
    ctx.resize(0, 96, 96)
    np.testing.assert_array_equal(ctx.render(0, width=96, height=96), gold["plain_fb"])
    assert ctx.stats().samples == int(gold["plain_samples"].sum())
    # ranks
    vol, descs, vox, tf = T.chopsuey_scene(32, 8)
    ctx = gpu_ctx_factory()
    ctx.set_bricks(descs, vox)
    ctx.set_transfer_function(tf)
    cam = T.cameras((32, 32, 32), 1, 64, 48, seed=5)[0]
    ctx.set_camera(0, *cam)
    ctx.resize(0, 64, 48)
    for name, mode in (("ranks_fp32", abi.COMPOSITE_FP32), ("ranks_ubyte", abi.COMPOSITE_UBYTE)):
        ctx.set_params(composite_mode=mode)
        np.testing.assert_array_equal(ctx.render(0, width=64, height=48), gold[name + "_fb"])
        assert ctx.composite_order(0) == gold[name + "_order"].tolist()
    imgs = np.zeros((8, 48, 64, 4), np.float32)
    ctx.render_partials(0, imgs)
    np.testing.assert_array_equal(imgs, gold["ranks_fp32_rank_images"])
    # uneven bricks, crosshair, spp 2
    vol, descs, vox, tf = T.uneven_scene(48)
    ctx = gpu_ctx_factory()
    ctx.set_bricks(descs, vox)
    ctx.set_transfer_function(tf)
    ctx.set_params(crosshair=1, spp=2)
    ctx.set_camera(0, *T.cameras((48, 48, 48), 1, 56, 56, seed=6)[0])
    ctx.resize(0, 56, 56)
    np.testing.assert_array_equal(ctx.render(0, width=56, height=56), gold["uneven_fb"])
