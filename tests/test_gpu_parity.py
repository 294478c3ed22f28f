"""GPU parity: the CUDA path through the C ABI against the CPU oracle.

The CUDA kernels and the oracle share one fp32 evaluation order (explicit
fused multiply-adds, no contraction), so frames, per-rank float images,
depths and sample counts must be bit-identical.
"""
import numpy as np
import pytest

from aloha_gb300 import abi
from aloha_gb300 import scenes as S
from aloha_gb300 import volfile as V
from tests import scenes_for_tests as T

pytestmark = pytest.mark.gpu


# both work divisions of a frame: every parity test below that renders
# several virtual ranks runs under each
SPLITS = [abi.SPLIT_PIXELS, abi.SPLIT_RANKS]


def setup_ctx(make, descs, vox, tf, n_ranks=None, **params):
    ctx = make()
    ctx.set_bricks(descs, vox)
    ctx.set_transfer_function(tf)
    if n_ranks is not None:
        ctx.set_ranks(n_ranks)
    ctx.set_params(**params)
    return ctx


def oracle_frame(O, descs, vox, tf, cam, W, H, n_ranks=1, order_mode=0, want=("fb",), **params):
    return O.render(descs, vox, tf, O.make_camera(*cam), W, H, O.make_params(**params), n_ranks=n_ranks,
                    order_mode=order_mode, want=want)


def gpu_frame(ctx, cam, W, H, view=0):
    ctx.set_camera(view, *cam)
    ctx.resize(view, W, H)
    fb = ctx.render(view, width=W, height=H)
    return fb, ctx.stats().samples


def assert_same_fb(a, b):
    if not np.array_equal(a, b):
        diff = np.argwhere(a != b)
        y, x = diff[0]
        raise AssertionError(f"{len(diff)} pixels differ; first at ({x},{y}): {a[y, x]:08x} vs {b[y, x]:08x}")


@pytest.mark.parametrize("split", SPLITS)
def test_rank_assignment_changes(gpu_ctx_factory, oracle, split):
    """The visibility orders are cached per brick set and rank assignment;
    every change of either (partitionKD, an explicit assignment, back again)
    must rebuild them.  The same views render after each change."""
    vol, descs, vox, tf = T.chopsuey_scene(48, 8)
    W, H = 64, 56
    cams = T.cameras((48, 48, 48), 3, W, H, seed=27)
    ctx = setup_ctx(gpu_ctx_factory, descs, vox, tf, n_ranks=8)
    ctx.set_render_split(split)
    assignment = [0, 2, 1, 0, 2, 1, 1, 0]  # 3 virtual ranks of uneven brick sets
    for step in ("kd8", "explicit3", "kd4"):
        if step == "explicit3":
            ctx.set_rank_assignment(assignment, 3)
        elif step == "kd4":
            ctx.set_ranks(4)
        for cam in cams:
            fb, samples = gpu_frame(ctx, cam, W, H)
            if step == "kd8":
                ref = oracle_frame(oracle, descs, vox, tf, cam, W, H, n_ranks=8)
            elif step == "explicit3":
                ref = oracle.render(descs, vox, tf, oracle.make_camera(*cam), W, H, oracle.make_params(), n_ranks=3,
                                    brick_rank=assignment)
            else:
                ref = oracle_frame(oracle, descs, vox, tf, cam, W, H, n_ranks=4)
            assert_same_fb(fb, ref["fb"])
            assert samples == ref["samples"]


def test_plain_c1_bit_exact(gpu_ctx_factory, oracle):
    vol, descs, vox, tf = T.c1_scene()
    cam = S.axis_camera((64, 64, 64), 512, 512)
    ctx = setup_ctx(gpu_ctx_factory, descs, vox, tf)
    fb, samples = gpu_frame(ctx, cam, 512, 512)
    ref = oracle_frame(oracle, descs, vox, tf, cam, 512, 512)
    assert_same_fb(fb, ref["fb"])
    assert samples == ref["samples"]
    assert (fb != 0).mean() > 0.1


@pytest.mark.parametrize("split", SPLITS)
def test_partials_depth_bit_exact(gpu_ctx_factory, oracle, split):
    vol, descs, vox, tf = T.chopsuey_scene(48, 8)
    W, H = 72, 56
    ctx = setup_ctx(gpu_ctx_factory, descs, vox, tf, n_ranks=8)
    ctx.set_render_split(split)
    for cam in T.cameras((48, 48, 48), 3, W, H, seed=21):
        ctx.set_camera(0, *cam)
        ctx.resize(0, W, H)
        imgs = np.zeros((8, H, W, 4), np.float32)
        depth = np.zeros((8, H, W), np.float32)
        ctx.render_partials(0, imgs, depth)
        ref = oracle_frame(oracle, descs, vox, tf, cam, W, H, n_ranks=8, want=("rank_images", "rank_depth"))
        np.testing.assert_array_equal(imgs, ref["rank_images"])
        np.testing.assert_array_equal(depth, ref["rank_depth"])
        assert ctx.stats().samples == ref["samples"]


@pytest.mark.parametrize("mode", [abi.COMPOSITE_FP32, abi.COMPOSITE_UBYTE])
@pytest.mark.parametrize("n_ranks", [1, 2, 3, 8])
@pytest.mark.parametrize("split", SPLITS)
def test_virtual_ranks_bit_exact(gpu_ctx_factory, oracle, mode, n_ranks, split):
    vol, descs, vox, tf = T.chopsuey_scene(64, 8)
    W, H = 100, 76  # not a multiple of the ray tile
    ctx = setup_ctx(gpu_ctx_factory, descs, vox, tf, n_ranks=n_ranks, composite_mode=mode)
    ctx.set_render_split(split)
    for cam in T.cameras((64, 64, 64), 3, W, H, seed=n_ranks):
        fb, samples = gpu_frame(ctx, cam, W, H)
        ref = oracle_frame(oracle, descs, vox, tf, cam, W, H, n_ranks=n_ranks, composite_mode=mode)
        assert_same_fb(fb, ref["fb"])
        assert samples == ref["samples"]
        assert ctx.composite_order(0) == [int(r) for r in ref["rank_order"]]


@pytest.mark.parametrize("tile", [(8, 4), (8, 8), (16, 8), (32, 4)])
def test_render_tiles_bit_exact(gpu_ctx_factory, oracle, tile):
    vol, descs, vox, tf = T.chopsuey_scene(48, 8)
    W, H = 70, 42  # ragged against every tile shape
    ctx = setup_ctx(gpu_ctx_factory, descs, vox, tf, n_ranks=8)
    ctx.set_render_split(abi.SPLIT_PIXELS)  # chunk shapes apply to the pixel split
    ctx.set_render_tile(*tile)
    for cam in T.cameras((48, 48, 48), 2, W, H, seed=61):
        fb, samples = gpu_frame(ctx, cam, W, H)
        ref = oracle_frame(oracle, descs, vox, tf, cam, W, H, n_ranks=8)
        assert_same_fb(fb, ref["fb"])
        assert samples == ref["samples"]
    with pytest.raises(abi.AlohaError):
        ctx.set_render_tile(4, 4)
    with pytest.raises(abi.AlohaError):
        ctx.set_render_split(3)


@pytest.mark.parametrize("tile", [(8, 4), (8, 8), (16, 8), (32, 4)])
@pytest.mark.parametrize("jitter", [abi.JITTER_HASH, abi.JITTER_CONST])
def test_staged_stencil_loads_bit_exact(gpu_ctx_factory, oracle, tile, jitter):
    """The next sample's stencil rows staged in shared memory (cp.async) give
    the frames and sample counts of the direct loads: several ranks per pixel,
    empty-space skips between full samples (a staged sample dropped), the
    camera zoo's grazing and inside views, ragged frames, spp 2."""
    vol, descs, vox, tf = T.uneven_scene(48)
    W, H = 70, 42
    ctx = setup_ctx(gpu_ctx_factory, descs, vox, tf, n_ranks=4, jitter_mode=jitter, jitter_value=0.37, spp=2)
    ctx.set_render_split(abi.SPLIT_PIXELS)
    ctx.set_render_tile(*tile)
    ctx.set_render_staging(abi.STAGING_NEXT_SAMPLE)
    params = dict(jitter_mode=jitter, jitter_value=0.37, spp=2)
    cams = T.cameras((48, 48, 48), 2, W, H, seed=67) + _camera_zoo((48, 48, 48), W, H, seed=68)[::4]
    for cam in cams:
        fb, samples = gpu_frame(ctx, cam, W, H)
        ref = oracle_frame(oracle, descs, vox, tf, cam, W, H, n_ranks=4, **params)
        assert_same_fb(fb, ref["fb"])
        assert samples == ref["samples"]
    with pytest.raises(abi.AlohaError):
        ctx.set_render_staging(2)


@pytest.mark.parametrize("permille", [1000, 100])
@pytest.mark.parametrize("kw", [dict(), dict(jitter_mode=abi.JITTER_CONST, jitter_value=0.37),
                                dict(dt=0.3, spp=2), dict(dt=0.375, jitter_mode=abi.JITTER_NONE),
                                dict(et_alpha=2.0)])
def test_lane_groups_bit_exact(gpu_ctx_factory, oracle, permille, kw):
    """Costliest chunks rendered with 4 lanes per ray (all of them at 1000 per
    mille): frames and sample counts equal the oracle's -- inexact step
    sequences (dt 0.3, 0.375), a constant jitter, spp 2, no early termination,
    several ranks per pixel, the camera zoo's grazing and inside views, ragged
    frames."""
    vol, descs, vox, tf = T.uneven_scene(48)
    W, H = 70, 42
    ctx = setup_ctx(gpu_ctx_factory, descs, vox, tf, n_ranks=4, **kw)
    ctx.set_render_split(abi.SPLIT_PIXELS)
    ctx.set_chunk_order(abi.CHUNKS_PROBED)
    ctx.set_lane_groups(permille)
    cams = T.cameras((48, 48, 48), 2, W, H, seed=77) + _camera_zoo((48, 48, 48), W, H, seed=78)[::3]
    for cam in cams:
        fb, samples = gpu_frame(ctx, cam, W, H)
        ref = oracle_frame(oracle, descs, vox, tf, cam, W, H, n_ranks=4, **kw)
        assert_same_fb(fb, ref["fb"])
        assert samples == ref["samples"]
    with pytest.raises(abi.AlohaError):
        ctx.set_lane_groups(1001)


def test_staged_batch_equals_direct_batch(gpu_ctx_factory):
    torch = pytest.importorskip("torch")
    vol, descs, vox, tf = T.uneven_scene(64)
    ctx = setup_ctx(gpu_ctx_factory, descs, vox, tf, n_ranks=12)
    sizes = [(96, 96), (64, 48), (40, 72)]
    for v, (W, H) in enumerate(sizes):
        ctx.set_camera(v, *S.orbit_cameras((64, 64, 64), len(sizes), W, H, seed=71)[v])
        ctx.resize(v, W, H)
    singles = [ctx.render(v, width=W, height=H) for v, (W, H) in enumerate(sizes)]
    fbs = [torch.zeros((H, W), dtype=torch.int32, device="cuda") for (W, H) in sizes]
    b = ctx.batch(list(range(len(sizes))), fbs)
    for cfg in [(8, 4), (16, 8)]:
        b.set_staging(abi.STAGING_NEXT_SAMPLE)
        b.set_config(*cfg)
        assert b.staging() == abi.STAGING_NEXT_SAMPLE
        for f in fbs:
            f.zero_()
        b.launch_graph()
        torch.cuda.synchronize()
        for f, s in zip(fbs, singles):
            assert_same_fb(f.cpu().numpy().view(np.uint32), s)
    # direct loads with the march loop written out two steps per trip
    b.set_staging(abi.STAGING_NONE)
    for cfg in [(8, 4), (8, 8), (16, 8), (32, 4)]:
        b.set_unroll(2)
        b.set_config(*cfg)
        assert b.unroll() == 2
        for f in fbs:
            f.zero_()
        b.launch_graph() if cfg[0] == 8 else b.launch()
        torch.cuda.synchronize()
        for f, s in zip(fbs, singles):
            assert_same_fb(f.cpu().numpy().view(np.uint32), s)
    with pytest.raises(abi.AlohaError):
        b.set_unroll(3)
    w, h, ms = b.autotune(reps=1)
    assert b.staging() in (abi.STAGING_NONE, abi.STAGING_NEXT_SAMPLE) and b.unroll() in (1, 2) and ms > 0
    b.close()


def _camera_zoo(dims, W, H, seed):
    """Cameras that stress the rank split's screen rectangles: near, inside,
    grazing, far with a narrow field of view, off-centre targets."""
    rng = np.random.default_rng(seed)
    ext = float(max(dims))
    ctr = np.asarray(dims, np.float64) * 0.5
    cams = []
    for dist, fov in [(0.3, 90.0), (0.55, 70.0), (0.75, 60.0), (1.0, 45.0), (2.0, 30.0), (8.0, 4.0), (60.0, 0.4)]:
        for _ in range(3):
            d = rng.normal(size=3)
            d /= np.linalg.norm(d)
            org = ctr + d * dist * ext
            target = ctr + rng.uniform(-0.4, 0.4, size=3) * ext
            up = rng.normal(size=3)
            cams.append(S.look_at_camera(org, target, up, fov, W, H))
    return cams


@pytest.mark.parametrize("chunks", [abi.CHUNKS_RING, abi.CHUNKS_PROBED])
@pytest.mark.parametrize("scene", ["chopsuey8", "uneven12"])
def test_rank_split_matches_pixel_split(gpu_ctx_factory, scene, chunks):
    """The rank split skips the ranks whose screen rectangle misses a chunk;
    over many awkward cameras its frames must equal the pixel split's."""
    if scene == "chopsuey8":
        vol, descs, vox, tf = T.chopsuey_scene(48, 8)
        R = 8
    else:
        vol, descs, vox, tf = T.uneven_scene(48)
        R = 12
    W, H = 61, 45
    params = [dict(), dict(heat_map=1, heat_map_scale=0.02), dict(crosshair=1, composite_mode=abi.COMPOSITE_UBYTE)]
    for kw in params:
        ctx = setup_ctx(gpu_ctx_factory, descs, vox, tf, n_ranks=R, **kw)
        ctx.set_chunk_order(chunks)
        for cam in _camera_zoo((48, 48, 48), W, H, seed=len(kw)):
            ctx.set_render_split(abi.SPLIT_PIXELS)
            want, n_want = gpu_frame(ctx, cam, W, H)
            ctx.set_render_split(abi.SPLIT_RANKS)
            got, n_got = gpu_frame(ctx, cam, W, H)
            assert_same_fb(got, want)
            assert n_got == n_want


@pytest.mark.parametrize("tile", [(8, 4), (16, 8)])
@pytest.mark.parametrize("chunks", [abi.CHUNKS_RING, abi.CHUNKS_PROBED])
def test_chunk_order_bit_exact(gpu_ctx_factory, oracle, tile, chunks):
    """The probed (most expensive first) chunk order renders the same frames
    and sample counts as the ring order, on ragged frames."""
    vol, descs, vox, tf = T.chopsuey_scene(48, 8)
    ctx = setup_ctx(gpu_ctx_factory, descs, vox, tf, n_ranks=8)
    ctx.set_render_split(abi.SPLIT_PIXELS)
    ctx.set_render_tile(*tile)
    ctx.set_chunk_order(chunks)
    for (W, H), seed in [((70, 42), 5), ((129, 65), 6)]:
        cam = T.cameras((48, 48, 48), 1, W, H, seed=seed)[0]
        fb, samples = gpu_frame(ctx, cam, W, H)
        ref = oracle_frame(oracle, descs, vox, tf, cam, W, H, n_ranks=8)
        assert_same_fb(fb, ref["fb"])
        assert samples == ref["samples"]
    with pytest.raises(abi.AlohaError):
        ctx.set_chunk_order(3)


@pytest.mark.parametrize("split,chunks", [(abi.SPLIT_PIXELS, abi.CHUNKS_RING), (abi.SPLIT_PIXELS, abi.CHUNKS_PROBED),
                                          (abi.SPLIT_RANKS, abi.CHUNKS_RING), (abi.SPLIT_RANKS, abi.CHUNKS_PROBED)])
def test_tiny_and_thin_frames(gpu_ctx_factory, oracle, split, chunks):
    """Frames of a few pixels or a single row / column: ring slots mostly off
    the chunk grid, one chunk, partial chunks."""
    vol, descs, vox, tf = T.chopsuey_scene(32, 8)
    ctx = setup_ctx(gpu_ctx_factory, descs, vox, tf, n_ranks=8)
    ctx.set_render_split(split)
    ctx.set_chunk_order(chunks)
    for (W, H), seed in [((1, 1), 1), ((2, 3), 2), ((9, 1), 3), ((1, 17), 4), ((13, 5), 5)]:
        cam = S.look_at_camera([16.0 + 40.0 * seed % 7, 50.0, -30.0], [16.0, 16.0, 16.0], [0, 1, 0], 20.0, W, H)
        fb, samples = gpu_frame(ctx, cam, W, H)
        ref = oracle_frame(oracle, descs, vox, tf, cam, W, H, n_ranks=8)
        assert_same_fb(fb, ref["fb"])
        assert samples == ref["samples"]


def test_rank_split_across_resizes(gpu_ctx_factory, oracle):
    """The per-chunk tickets of the rank split are reset by the kernel itself;
    frames of growing and shrinking size in a row must all stay exact."""
    vol, descs, vox, tf = T.chopsuey_scene(48, 8)
    ctx = setup_ctx(gpu_ctx_factory, descs, vox, tf, n_ranks=8)
    ctx.set_render_split(abi.SPLIT_RANKS)
    for (W, H), seed in [((40, 24), 1), ((130, 70), 2), ((40, 24), 3), ((33, 97), 4)]:
        cam = T.cameras((48, 48, 48), 1, W, H, seed=seed)[0]
        fb, samples = gpu_frame(ctx, cam, W, H)
        ref = oracle_frame(oracle, descs, vox, tf, cam, W, H, n_ranks=8)
        assert_same_fb(fb, ref["fb"])
        assert samples == ref["samples"]


def test_uneven_bricks_bit_exact(gpu_ctx_factory, oracle):
    vol, descs, vox, tf = T.uneven_scene(64)
    W, H = 96, 96
    ctx = setup_ctx(gpu_ctx_factory, descs, vox, tf, n_ranks=12)
    for cam in T.cameras((64, 64, 64), 4, W, H, seed=9):
        fb, samples = gpu_frame(ctx, cam, W, H)
        ref = oracle_frame(oracle, descs, vox, tf, cam, W, H, n_ranks=12)
        assert_same_fb(fb, ref["fb"])
        assert samples == ref["samples"]


def test_reference_kd_order_mode(gpu_ctx_factory, oracle):
    vol, descs, vox, tf = T.uneven_scene(48)
    W, H = 64, 64
    ctx = setup_ctx(gpu_ctx_factory, descs, vox, tf, n_ranks=12, order_mode=abi.ORDER_REFERENCE_KD)
    for cam in T.cameras((48, 48, 48), 3, W, H, seed=4):
        fb, _ = gpu_frame(ctx, cam, W, H)
        ref = oracle_frame(oracle, descs, vox, tf, cam, W, H, n_ranks=12, order_mode=oracle.ORDER_REFERENCE_KD)
        assert_same_fb(fb, ref["fb"])


@pytest.mark.parametrize("kw", [
    dict(crosshair=1),
    dict(spp=3),
    dict(heat_map=1, heat_map_scale=0.01),
    dict(island_id=1, num_islands=3),
    dict(jitter_mode=abi.JITTER_NONE),
    dict(jitter_mode=abi.JITTER_CONST, jitter_value=0.37),
    dict(jitter_mode=abi.JITTER_HASH),
    dict(dt=2.0),
    dict(dt=0.25, et_alpha=0.5),
    dict(dt=0.375),
    dict(dt=0.3),
    dict(accum_id=0, crosshair=1, spp=2, composite_mode=abi.COMPOSITE_UBYTE),
])
@pytest.mark.parametrize("split", SPLITS)
def test_output_stage_options(gpu_ctx_factory, oracle, kw, split):
    vol, descs, vox, tf = T.chopsuey_scene(48, 4)
    W, H = 80, 64
    cam = T.cameras((48, 48, 48), 1, W, H, seed=13)[0]
    ctx = setup_ctx(gpu_ctx_factory, descs, vox, tf, n_ranks=4, **kw)
    ctx.set_render_split(split)
    fb, samples = gpu_frame(ctx, cam, W, H)
    ref = oracle_frame(oracle, descs, vox, tf, cam, W, H, n_ranks=4, **kw)
    assert_same_fb(fb, ref["fb"])
    assert samples == ref["samples"]


@pytest.mark.parametrize("split", SPLITS)
def test_progressive_accumulation(gpu_ctx_factory, oracle, split):
    vol, descs, vox, tf = T.chopsuey_scene(48, 2)
    W, H = 64, 48
    cam = T.cameras((48, 48, 48), 1, W, H, seed=17)[0]
    ctx = setup_ctx(gpu_ctx_factory, descs, vox, tf, n_ranks=2)
    ctx.set_render_split(split)
    ctx.set_camera(0, *cam)
    ctx.resize(0, W, H)
    acc = np.zeros((2, W * H, 4), np.float32)
    for k in range(3):
        ctx.set_params(accum_id=k, accumulate=1)
        fb = ctx.render(0, width=W, height=H)
        ref = oracle.render(descs, vox, tf, oracle.make_camera(*cam), W, H,
                            oracle.make_params(accum_id=k, accumulate=1), n_ranks=2, accum=acc)
        assert_same_fb(fb, ref["fb"])


@pytest.mark.parametrize("split,chunks", [(abi.SPLIT_PIXELS, abi.CHUNKS_RING), (abi.SPLIT_PIXELS, abi.CHUNKS_PROBED),
                                          (abi.SPLIT_RANKS, abi.CHUNKS_AUTO)])
def test_pathological_cameras(gpu_ctx_factory, oracle, split, chunks):
    vol, descs, vox, tf = T.chopsuey_scene(32, 8)
    W, H = 40, 40
    ctx = setup_ctx(gpu_ctx_factory, descs, vox, tf, n_ranks=8)
    ctx.set_render_split(split)
    ctx.set_chunk_order(chunks)
    cams = [
        S.look_at_camera([16.0, 16.0, 16.0], [40.0, 17.0, 15.0], [0, 1, 0], 60.0, W, H),  # inside, on a face
        S.look_at_camera([16.3, 5.0, 9.0], [16.3, 5.0, -30.0], [0, 1, 0], 30.0, W, H),   # axis-aligned rays
        S.look_at_camera([-50.0, 16.0, 16.0], [100.0, 16.0, 16.0], [0, 0, 1], 5.0, W, H),  # along x through faces
        S.look_at_camera([1e4, 2e3, -3e3], [16.0, 16.0, 16.0], [0, 1, 0], 0.5, W, H),  # far away
        S.look_at_camera([32.0, 32.0, 32.0], [0.0, 0.0, 0.0], [0, 1, 0], 90.0, W, H),   # on a corner
    ]
    for cam in cams:
        fb, samples = gpu_frame(ctx, cam, W, H)
        ref = oracle_frame(oracle, descs, vox, tf, cam, W, H, n_ranks=8)
        assert_same_fb(fb, ref["fb"])
        assert samples == ref["samples"]


@pytest.mark.parametrize("mode", [abi.COMPOSITE_FP32, abi.COMPOSITE_UBYTE])
def test_partials_then_composite_equals_fused(gpu_ctx_factory, mode):
    torch = pytest.importorskip("torch")
    vol, descs, vox, tf = T.chopsuey_scene(64, 8)
    W, H = 128, 96
    cam = T.cameras((64, 64, 64), 1, W, H, seed=23)[0]
    ctx = setup_ctx(gpu_ctx_factory, descs, vox, tf, n_ranks=8, composite_mode=mode)
    fused, _ = gpu_frame(ctx, cam, W, H)
    imgs = torch.zeros((8, H, W, 4), dtype=torch.float32, device="cuda")
    ctx.render_partials(0, imgs)
    out = torch.zeros((H, W), dtype=torch.int32, device="cuda")
    abi.composite_over(imgs, ctx.composite_order(0), W, H, mode, fb=out)
    torch.cuda.synchronize()
    assert_same_fb(out.cpu().numpy().view(np.uint32), fused)
    if mode == abi.COMPOSITE_UBYTE:
        # the same blend from externally quantised RGBA8 rank images
        q = (imgs.clamp(0, 1) * 255 + 0.5).to(torch.int32)
        packed = (q[..., 0] | (q[..., 1] << 8) | (q[..., 2] << 16) | (q[..., 3] << 24)).contiguous()
        out8 = abi.composite_over_rgba8(packed.cpu().numpy().view(np.uint32), ctx.composite_order(0), W, H)
        assert_same_fb(out8, fused)


def test_batch_equals_single_renders(gpu_ctx_factory):
    torch = pytest.importorskip("torch")
    vol, descs, vox, tf = T.uneven_scene(64)
    ctx = setup_ctx(gpu_ctx_factory, descs, vox, tf, n_ranks=12)
    sizes = [(96, 96), (64, 48), (96, 96), (40, 72), (64, 64)]
    singles = []
    for v, (W, H) in enumerate(sizes):
        cam = S.orbit_cameras((64, 64, 64), len(sizes), W, H, seed=31)[v]
        ctx.set_camera(v, *cam)
        ctx.resize(v, W, H)
        singles.append(ctx.render(v, width=W, height=H))
    fbs =[torch.zeros((H, W), dtype=torch.int32, device="cuda") for (W, H) in sizes]
    b = ctx.batch(list(range(len(sizes))), fbs)
    for cfg in [(16, 8), (8, 8), (32, 4)]:
        for f in fbs:
            f.zero_()
        b.set_config(*cfg)
        b.launch()
        torch.cuda.synchronize()
        for f, s in zip(fbs, singles):
            assert_same_fb(f.cpu().numpy().view(np.uint32), s)
    for f in fbs:
        f.zero_()
    b.launch_graph()
    b.launch_graph()
    torch.cuda.synchronize()
    for f, s in zip(fbs, singles):
        assert_same_fb(f.cpu().numpy().view(np.uint32), s)
    w, h, ms = b.autotune(reps=1)
    assert (w, h) in [(8, 4), (8, 8), (16, 8), (32, 4)] and ms > 0
    # a camera change is picked up by the next (graph) launch
    new_cam = S.orbit_cameras((64, 64, 64), 1, 96, 96, seed=99)[0]
    ctx.set_camera(0, *new_cam)
    b.launch_graph()
    torch.cuda.synchronize()
    assert_same_fb(fbs[0].cpu().numpy().view(np.uint32), ctx.render(0, width=96, height=96))
    b.close()
    # host frame buffers through the convenience entry point
    host = [np.zeros((H, W), np.uint32) for (W, H) in sizes]
    ctx.render_batch(list(range(len(sizes))), host)
    assert_same_fb(host[1], singles[1])


def test_frame_buffer_kinds(gpu_ctx_factory):
    """Device, page-locked host (written by the kernel directly) and pageable
    host frame buffers receive the same frame."""
    torch = pytest.importorskip("torch")
    vol, descs, vox, tf = T.chopsuey_scene(48, 8)
    W, H = 77, 53
    ctx = setup_ctx(gpu_ctx_factory, descs, vox, tf, n_ranks=8)
    for split in (abi.SPLIT_PIXELS, abi.SPLIT_RANKS):
        ctx.set_render_split(split)
        for cam in T.cameras((48, 48, 48), 2, W, H, seed=41):
            ctx.set_camera(0, *cam)
            ctx.resize(0, W, H)
            dev = torch.zeros((H, W), dtype=torch.int32, device="cuda")
            ctx.render(0, dev)
            torch.cuda.synchronize()
            pinned = torch.full((H, W), -1, dtype=torch.int32).pin_memory()
            ctx.render(0, pinned)
            pageable = np.full((H, W), 7, np.uint32)
            ctx.render(0, pageable)
            want = dev.cpu().numpy().view(np.uint32)
            assert_same_fb(pinned.numpy().view(np.uint32), want)
            assert_same_fb(pageable, want)


def test_device_tensors_as_inputs(gpu_ctx_factory, oracle):
    torch = pytest.importorskip("torch")
    vol, descs, vox, tf = T.chopsuey_scene(32, 2)
    dvox = [torch.from_numpy(v).cuda() for v in vox]
    dtf = torch.from_numpy(tf).cuda()
    ctx = setup_ctx(gpu_ctx_factory, descs, dvox, dtf, n_ranks=2)
    cam = T.cameras((32, 32, 32), 1, 48, 48, seed=2)[0]
    ctx.set_camera(0, *cam)
    ctx.resize(0, 48, 48)
    out = torch.zeros((48, 48), dtype=torch.int32, device="cuda")
    ctx.render(0, out)
    torch.cuda.synchronize()
    ref = oracle_frame(oracle, descs, vox, tf, cam, 48, 48, n_ranks=2)
    assert_same_fb(out.cpu().numpy().view(np.uint32), ref["fb"])


def test_error_paths(gpu_ctx_factory):
    vol, descs, vox, tf = T.chopsuey_scene(32, 2)
    ctx = gpu_ctx_factory()
    with pytest.raises(abi.AlohaError) as e:
        ctx.render(0, width=8, height=8)
    assert e.value.code in (abi.ERR_NOT_READY, abi.ERR_OUT_OF_RANGE)
    ctx.set_bricks(descs, vox)
    cam = T.cameras((32, 32, 32), 1, 16, 16)[0]
    ctx.set_camera(0, *cam)
    ctx.resize(0, 16, 16)
    with pytest.raises(abi.AlohaError) as e:
        ctx.render(0, width=16, height=16)  # no transfer function yet
    assert e.value.code == abi.ERR_NOT_READY
    ctx.set_transfer_function(tf)
    ok = ctx.render(0, width=16, height=16)
    with pytest.raises(abi.AlohaError) as e:
        ctx.set_camera(0, [float("nan"), 0, 0], cam[1], cam[2], cam[3])
    assert e.value.code == abi.ERR_INVALID_ARGUMENT
    with pytest.raises(abi.AlohaError) as e:
        ctx.set_ranks(5)
    assert e.value.code == abi.ERR_INVALID_ARGUMENT
    with pytest.raises(abi.AlohaError) as e:
        ctx.set_params(dt=0.0)
    assert e.value.code == abi.ERR_INVALID_ARGUMENT
    with pytest.raises(abi.AlohaError) as e:
        ctx.set_params(accum_id=3)
        ctx.render(0, width=16, height=16)  # no accumulation buffer exists
    assert e.value.code == abi.ERR_NOT_READY
    ctx.set_params()
    # a lost virtual rank: the render fails instead of returning a partial image
    ctx.drop_brick(1)
    with pytest.raises(abi.AlohaError) as e:
        ctx.render(0, width=16, height=16)
    assert e.value.code == abi.ERR_MISSING_BRICK
    ctx.update_brick(1, vox[1])
    np.testing.assert_array_equal(ctx.render(0, width=16, height=16), ok)
    bad = vox[0].copy()
    bad[3, 3, 3] = np.inf
    with pytest.raises(abi.AlohaError) as e:
        ctx.update_brick(0, bad)
    assert e.value.code == abi.ERR_INVALID_ARGUMENT
    with pytest.raises(abi.AlohaError) as e:
        ctx.set_rank_assignment([0, -1], 2)
    assert e.value.code == abi.ERR_MISSING_BRICK


def _band_tf(lo, hi, n=256, alpha=0.5):
    x = (np.arange(n) + 0.5) / n
    tf = S.ramp_tf(n).copy()
    tf[:, 3] = np.where((x >= lo) & (x <= hi), alpha, 0.0)
    return np.ascontiguousarray(tf, np.float32)


def test_empty_space_skipping_is_exact(gpu_ctx_factory, oracle):
    """Samples in macrocells whose transfer-function alpha is 0 are skipped on
    the GPU; frames and sample counts must not change."""
    vol, descs, vox, tf = T.chopsuey_scene(64, 8)
    W, H = 96, 80
    ctx = setup_ctx(gpu_ctx_factory, descs, vox, tf, n_ranks=8)
    cams = T.cameras((64, 64, 64), 2, W, H, seed=51)
    tfs = [_band_tf(0.5, 0.53), _band_tf(0.0, 0.01), _band_tf(0.99, 1.0), np.zeros((256, 4), np.float32),
           _band_tf(0.0, 1.0, alpha=0.05), _band_tf(0.3, 0.3001, n=64), tf]
    for t in tfs:
        ctx.set_transfer_function(t)  # masks are rebuilt before the next render
        for cam in cams:
            fb, samples = gpu_frame(ctx, cam, W, H)
            ref = oracle_frame(oracle, descs, vox, t, cam, W, H, n_ranks=8)
            assert_same_fb(fb, ref["fb"])
            assert samples == ref["samples"]
    # a brick update rebuilds its value ranges too
    bumped = vox[3] + np.float32(0.4)
    ctx.update_brick(3, bumped)
    vox2 = list(vox)
    vox2[3] = bumped
    for cam in cams:
        fb, samples = gpu_frame(ctx, cam, W, H)
        ref = oracle_frame(oracle, descs, vox2, tf, cam, W, H, n_ranks=8)
        assert_same_fb(fb, ref["fb"])
        assert samples == ref["samples"]


def test_full_size_rows_bit_exact(gpu_ctx_factory, oracle):
    """512^3 fp32, 2x2x2 chopSuey bricks, 1024^2: whole frame on the GPU, a
    spread of rows on the CPU oracle."""
    n, W, H = 512, 1024, 1024
    vol = S.blob_field((n, n, n), 64, (32.0, 80.0), seed=2001)
    descs = oracle.chopsuey_split((n, n, n), 8)
    vox = S.extract_bricks(vol, descs)
    tf = S.ramp_tf()
    ctx = setup_ctx(gpu_ctx_factory, descs, vox, tf, n_ranks=8)
    cams = S.orbit_cameras((n, n, n), 2, W, H, seed=2002)
    for cam in cams:
        fb, samples = gpu_frame(ctx, cam, W, H)
        for y0 in (101, 400, 512, 777):
            ref = oracle.render(descs, vox, tf, oracle.make_camera(*cam), W, H, oracle.make_params(), n_ranks=8,
                                rows=(y0, y0 + 2))
            assert_same_fb(fb[y0:y0 + 2], ref["fb"][y0:y0 + 2])
        assert samples > 1e7


def test_bricks_that_partitionkd_cannot_split(gpu_ctx_factory, oracle):
    """Two bricks separated only along y, in a volume whose longest axis is x:
    partitionKD's midplane split on x leaves both on one side, forever in the
    reference.  Uploading them still works (one rank per brick, brick i on
    rank i), aloha_set_ranks(2) refuses, and the frame equals the oracle's
    with that explicit assignment."""
    dims = (64, 24, 20)
    vol = S.blob_field(dims, 6, (2.0, 6.0), seed=5)
    descs = S.grid_split(dims, ([], [12], []))
    vox = S.extract_bricks(vol, descs)
    tf = S.ramp_tf()
    with pytest.raises(ValueError):
        oracle.partition_kd(descs, 2)
    ctx = gpu_ctx_factory()
    ctx.set_bricks(descs, vox)
    ctx.set_transfer_function(tf)
    W, H = 64, 48
    cam = S.look_at_camera([32.0, 80.0, -60.0], [32.0, 12.0, 10.0], [0, 1, 0], 40.0, W, H)
    identity = np.arange(2, dtype=np.int32)
    fb, samples = gpu_frame(ctx, cam, W, H)
    ref = oracle.render(descs, vox, tf, oracle.make_camera(*cam), W, H, oracle.make_params(), n_ranks=2,
                        brick_rank=identity)
    assert_same_fb(fb, ref["fb"])
    assert samples == ref["samples"]
    with pytest.raises(abi.AlohaError) as e:
        ctx.set_ranks(2)
    assert e.value.code == abi.ERR_INVALID_ARGUMENT
    ctx.set_ranks(1)  # one rank always partitions
    fb1, _ = gpu_frame(ctx, cam, W, H)
    assert_same_fb(fb1, oracle_frame(oracle, descs, vox, tf, cam, W, H, n_ranks=1)["fb"])


def test_two_contexts_are_independent(gpu_ctx_factory, oracle):
    """Two contexts on one GPU with different scenes, rank counts, transfer
    functions and parameters, driven on two CUDA streams at once: renders,
    a batch and the training forward of one overlap with the other's work,
    and every result equals the oracle's for its own context."""
    torch = pytest.importorskip("torch")
    _, da, va, tfa = T.chopsuey_scene(48, 8, seed=3)
    _, db, vb, _ = T.uneven_scene(56, seed=4)
    tfb = S.seeded_tf(19, n=200)
    A, B = gpu_ctx_factory(), gpu_ctx_factory()
    A.set_bricks(da, va)
    A.set_transfer_function(tfa)
    A.set_ranks(8)
    B.set_bricks(db, vb)
    B.set_transfer_function(tfb)
    B.set_ranks(3)
    pb = dict(dt=0.3, composite_mode=abi.COMPOSITE_UBYTE, jitter_mode=abi.JITTER_CONST, jitter_value=0.25)
    A.set_params()
    B.set_params(**pb)
    sa, sb = torch.cuda.Stream(), torch.cuda.Stream()
    W, H = 96, 80
    cams_a = S.orbit_cameras((48, 48, 48), 4, W, H, seed=5)
    cams_b = S.orbit_cameras((56, 56, 56), 4, W, H, seed=6)
    for v in range(4):
        A.set_camera(v, *cams_a[v])
        A.resize(v, W, H)
        B.set_camera(v, *cams_b[v])
        B.resize(v, W, H)
    fa = [torch.zeros((H, W), dtype=torch.int32, device="cuda") for _ in range(4)]
    fb = [torch.zeros((H, W), dtype=torch.int32, device="cuda") for _ in range(4)]
    batch_b = B.batch([0, 1, 2, 3], fb)
    torch.cuda.synchronize()
    for v in range(4):  # A's plain renders on sa overlap B's batch on sb
        A.render(v, fa[v], sa)
    batch_b.launch_graph(sb)
    torch.cuda.synchronize()
    for v in range(4):
        ra = oracle.render(da, va, tfa, oracle.make_camera(*cams_a[v]), W, H, oracle.make_params(), n_ranks=8)
        rb = oracle.render(db, vb, tfb, oracle.make_camera(*cams_b[v]), W, H, oracle.make_params(**pb), n_ranks=3)
        assert_same_fb(fa[v].cpu().numpy().view(np.uint32), ra["fb"])
        assert_same_fb(fb[v].cpu().numpy().view(np.uint32), rb["fb"])
    batch_b.close()
    # A's training forward on sa while B renders on sb
    A.set_ranks(1)
    imgs = [torch.zeros((H, W, 4), device="cuda") for _ in range(4)]
    A.forward_views([0, 1, 2, 3], imgs, 16, sa)
    for v in range(4):
        B.render(v, fb[v], sb)
    torch.cuda.synchronize()
    for v in range(4):
        ra = oracle.render(da, va, tfa, oracle.make_camera(*cams_a[v]), W, H, oracle.make_params(), n_ranks=1,
                           want=("final",))
        np.testing.assert_array_equal(imgs[v].cpu().numpy(), ra["final"])
        rb = oracle.render(db, vb, tfb, oracle.make_camera(*cams_b[v]), W, H, oracle.make_params(**pb), n_ranks=3)
        assert_same_fb(fb[v].cpu().numpy().view(np.uint32), rb["fb"])


@pytest.mark.parametrize("case", [
    dict(dims=(40, 36, 44), dt=0.05),                      # many samples per ray
    dict(dims=(40, 36, 44), dt=8.0),                       # steps longer than a macrocell
    dict(dims=(40, 36, 44), et_alpha=0.01),                # rays end after almost nothing
    dict(dims=(40, 36, 44), n_tf=1),                       # one transfer-function entry
    dict(dims=(40, 36, 44), n_tf=2048),                    # the largest transfer function
    dict(dims=(64, 64, 1)),                                # one voxel thick
    dict(dims=(3, 50, 2)),                                 # thinner than the apron
    dict(dims=(2, 2, 2)),                                  # two voxels a side
    dict(dims=(40, 36, 44), size=(1, 1)),                  # a single pixel
    dict(dims=(40, 36, 44), size=(1000, 3)),               # a wide strip
])
def test_edge_cases_bit_exact(gpu_ctx_factory, oracle, case):
    """Extremes of the step, early termination, transfer-function size, volume
    and frame shapes: the frame and sample count still equal the oracle's."""
    dims = case["dims"]
    rng = np.random.default_rng(sum(dims))
    vol = S.blob_field(dims, 6, (1.0, 6.0), seed=int(rng.integers(1 << 20)))
    vol = (vol * np.float32(1.2)).astype(np.float32)
    descs = V.chopsuey_split(dims, 2)
    vox = S.extract_bricks(vol, descs)
    n_tf = case.get("n_tf", 256)
    tf = S.seeded_tf(int(rng.integers(1 << 20)), n=max(n_tf, 2))[:n_tf].copy() if n_tf > 1 else \
        np.array([[0.8, 0.4, 0.2, 0.3]], np.float32)
    params = {k: case[k] for k in ("dt", "et_alpha") if k in case}
    W, H = case.get("size", (64, 48))
    ctx = setup_ctx(gpu_ctx_factory, descs, vox, tf, n_ranks=2, **params)
    for seed in (1, 2):
        cam = S.orbit_cameras(dims, 1, W, H, seed=seed, distance=1.5)[0]
        fb, samples = gpu_frame(ctx, cam, W, H)
        ref = oracle_frame(oracle, descs, vox, tf, cam, W, H, n_ranks=2, **params)
        assert_same_fb(fb, ref["fb"])
        assert samples == ref["samples"], (case, seed)
