"""Seeded random sweep of the render's configuration space against the oracle.

Each case draws, from its own seed, every choice the hand-written parity tests
make one at a time:
- a volume of odd, non-cubic dimensions, with values up to 1.4 so that the
  transfer function's border fade is hit;
- chopSuey or uneven grid bricks, with 1 to all ranks by partitionKD or a
  random explicit brick -> rank assignment;
- a transfer function of 2 to 1024 entries, some with zero-alpha bands so
  that empty-space skipping engages;
- a camera outside, near or inside the volume, with a random field of view
  and an image of 1 to 96 pixels a side;
- the step (powers of two and inexact steps), early termination (including
  off), jitter, spp, crosshair, composite mode and heat map;
- the work division: pixel or rank split, chunk order, chunk shape, stencil
  staging and lane groups.

Frames and sample counts must be bit-identical to the oracle, as everywhere.
Two more sweeps draw the batched launch (1 to 10 views of random sizes, every
chunk shape, CTA count and staging, plain or graph launch; each view's frame
bit-identical to the oracle's) and the differentiable form (random
single-rank scenes and checkpoint intervals; the training forward's float
image bit-identical, both gradients within 5e-4 of the FP64 adjoint), the
multi-view training calls (one forward launch over many views, a summed
backward), the standalone composites, and one context driven through random
call sequences.
"""
import numpy as np
import pytest

from aloha_gb300 import abi
from aloha_gb300 import scenes as S
from aloha_gb300 import volfile as V

pytestmark = pytest.mark.gpu

N_CASES = 48


def _volume(rng, dims):
    n_blobs = int(rng.integers(2, 12))
    lo = float(rng.uniform(1.0, 4.0))
    vol = S.blob_field(dims, n_blobs, (lo, lo + float(rng.uniform(1.0, 8.0))), seed=int(rng.integers(1 << 30)))
    return (vol * np.float32(rng.uniform(0.5, 1.4))).astype(np.float32)


def _bricks(rng, dims):
    if rng.random() < 0.5:
        return V.chopsuey_split(dims, int(rng.integers(1, 13)))
    cuts = []
    for d in dims:
        k = int(rng.integers(0, 3)) if d >= 8 else 0
        c = sorted(set(int(x) for x in rng.integers(2, d - 1, size=k))) if k else []
        cuts.append([x for i, x in enumerate(c) if i == 0 or x - c[i - 1] >= 2])
    return V.grid_split(dims, cuts)


def _tf(rng):
    n = int(rng.choice([2, 5, 64, 256, 1024]))
    tf = S.seeded_tf(int(rng.integers(1 << 30)), n=max(n, 2)).copy()
    if n >= 5 and rng.random() < 0.5:  # a zero-alpha band inside the table
        a = int(rng.integers(0, n - 1))
        b = int(rng.integers(a + 1, n + 1))
        tf[a:b, 3] = 0.0
    if rng.random() < 0.2:
        tf[:, 3] = np.minimum(1.0, tf[:, 3] * 3.0)  # near opaque
    return np.ascontiguousarray(tf, dtype=np.float32)


def _camera(rng, dims, W, H):
    c = np.asarray(dims, dtype=np.float64) * 0.5
    ext = float(max(dims))
    k = float(rng.choice([0.15, 0.6, 1.2, 2.5]))  # 0.15: inside the volume
    az, el = float(rng.uniform(0, 2 * np.pi)), float(rng.uniform(-1.3, 1.3))
    d = np.array([np.cos(el) * np.sin(az), np.sin(el), np.cos(el) * np.cos(az)])
    target = c + rng.uniform(-0.2, 0.2, 3) * ext
    if k < 0.5:
        fov = float(rng.uniform(40.0, 110.0))
    else:  # the volume fills a good part of the view
        fov = float(np.clip(np.degrees(2 * np.arctan(0.8 / k)) * rng.uniform(0.5, 1.5), 5.0, 120.0))
    return S.look_at_camera(c + k * ext * d, target, (0.0, 1.0, 0.0), fov, W, H)


def _case(seed):
    rng = np.random.default_rng(1000 + seed)
    dims = tuple(int(x) for x in rng.integers(9, 73, size=3))
    vol = _volume(rng, dims)
    descs = _bricks(rng, dims)
    vox = S.extract_bricks(vol, descs)
    nb = len(descs)
    n_ranks = int(rng.integers(1, nb + 1))
    brick_rank = None
    if n_ranks > 1 and rng.random() < 0.4:  # explicit assignment, every rank used
        brick_rank = np.concatenate([np.arange(n_ranks), rng.integers(0, n_ranks, nb - n_ranks)])
        rng.shuffle(brick_rank)
        brick_rank = brick_rank.astype(np.int32)
    W, H = (int(x) for x in rng.choice([1, 7, 33, 48, 64, 80, 96], p=[.05, .1, .15, .15, .2, .15, .2], size=2))
    params = dict(dt=float(rng.choice([0.5, 1.0, 0.25, 0.3, 0.375, 2.0])),
                  et_alpha=float(rng.choice([0.99, 0.5, 2.0])),
                  jitter_mode=int(rng.choice([abi.JITTER_NONE, abi.JITTER_CONST, abi.JITTER_HASH])),
                  jitter_value=float(rng.uniform(0.0, 1.0)),
                  spp=int(rng.choice([1, 1, 2])),
                  crosshair=int(rng.random() < 0.2),
                  composite_mode=int(rng.choice([abi.COMPOSITE_FP32, abi.COMPOSITE_UBYTE])),
                  heat_map=int(rng.random() < 0.15), heat_map_scale=float(rng.choice([1e-3, 0.05])))
    work = dict(split=int(rng.choice([abi.SPLIT_AUTO, abi.SPLIT_PIXELS, abi.SPLIT_RANKS])),
                chunks=int(rng.choice([abi.CHUNKS_AUTO, abi.CHUNKS_RING, abi.CHUNKS_PROBED])),
                tile=[(8, 4), (8, 8), (16, 8), (32, 4)][int(rng.integers(0, 4))],
                staging=int(rng.choice([abi.STAGING_NONE, abi.STAGING_NONE, abi.STAGING_NEXT_SAMPLE])),
                lane_groups=int(rng.choice([0, 0, 150, 1000])))
    if work["split"] == abi.SPLIT_RANKS and not 2 <= n_ranks <= 64:
        work["split"] = abi.SPLIT_PIXELS
    cam = _camera(rng, dims, W, H)
    return dict(dims=dims, descs=descs, vox=vox, tf=_tf(rng), n_ranks=n_ranks, brick_rank=brick_rank, W=W, H=H,
                params=params, work=work, cam=cam)


@pytest.mark.parametrize("seed", range(N_CASES))
def test_random_configuration_bit_exact(gpu_ctx_factory, oracle, seed):
    c = _case(seed)
    ctx = gpu_ctx_factory()
    ctx.set_bricks(c["descs"], c["vox"])
    ctx.set_transfer_function(c["tf"])
    if c["brick_rank"] is None:
        try:
            oracle.partition_kd(c["descs"], c["n_ranks"])
        except ValueError:
            # a brick set on which partitionKD's split makes no progress (the
            # reference loops forever there): refused on both sides, then an
            # explicit assignment
            with pytest.raises(abi.AlohaError):
                ctx.set_ranks(c["n_ranks"])
            c["brick_rank"] = (np.arange(len(c["descs"])) % c["n_ranks"]).astype(np.int32)
    if c["brick_rank"] is None:
        ctx.set_ranks(c["n_ranks"])
    else:
        ctx.set_rank_assignment(c["brick_rank"], c["n_ranks"])
    ctx.set_params(**c["params"])
    w = c["work"]
    ctx.set_render_split(w["split"])
    ctx.set_chunk_order(w["chunks"])
    ctx.set_render_tile(*w["tile"])
    ctx.set_render_staging(w["staging"])
    ctx.set_lane_groups(w["lane_groups"])
    W, H = c["W"], c["H"]
    ctx.set_camera(0, *c["cam"])
    ctx.resize(0, W, H)
    fb = ctx.render(0, width=W, height=H)
    samples = ctx.stats().samples
    ref = oracle.render(c["descs"], c["vox"], c["tf"], oracle.make_camera(*c["cam"]), W, H,
                        oracle.make_params(**c["params"]), n_ranks=c["n_ranks"], brick_rank=c["brick_rank"],
                        want=("fb",))
    where = f"case {seed}: dims {c['dims']}, {len(c['descs'])} bricks, {c['n_ranks']} ranks, {W}x{H}, {w}, " \
            f"{c['params']}"
    if not np.array_equal(fb, ref["fb"]):
        diff = np.argwhere(fb != ref["fb"])
        y, x = diff[0]
        raise AssertionError(f"{where}: {len(diff)} pixels differ; first at ({x},{y}): "
                             f"{fb[y, x]:08x} vs {ref['fb'][y, x]:08x}")
    assert samples == ref["samples"], where


def _partitioned(oracle, ctx, descs, n_ranks, rng):
    """Ranks by partitionKD where it can split the bricks, else a random
    assignment that uses every rank; returns the oracle's brick_rank."""
    try:
        oracle.partition_kd(descs, n_ranks)
        ctx.set_ranks(n_ranks)
        return None
    except ValueError:
        nb = len(descs)
        br = np.concatenate([np.arange(n_ranks), rng.integers(0, n_ranks, nb - n_ranks)]).astype(np.int32)
        rng.shuffle(br)
        ctx.set_rank_assignment(br, n_ranks)
        return br


@pytest.mark.parametrize("seed", range(16))
def test_random_batch_bit_exact(gpu_ctx_factory, oracle, seed):
    """One persistent launch (plain or graph-captured) over 1 to 10 views of
    random sizes and cameras, at a random chunk shape, CTA count and staging:
    every view's frame equals the oracle's."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(5000 + seed)
    dims = tuple(int(x) for x in rng.integers(9, 65, size=3))
    vol = _volume(rng, dims)
    descs = _bricks(rng, dims)
    vox = S.extract_bricks(vol, descs)
    tf = _tf(rng)
    ctx = gpu_ctx_factory()
    ctx.set_bricks(descs, vox)
    ctx.set_transfer_function(tf)
    n_ranks = int(rng.integers(1, len(descs) + 1))
    brick_rank = _partitioned(oracle, ctx, descs, n_ranks, rng)
    params = dict(dt=float(rng.choice([0.5, 1.0, 0.3, 0.375])), et_alpha=float(rng.choice([0.99, 0.6, 2.0])),
                  jitter_mode=int(rng.choice([abi.JITTER_NONE, abi.JITTER_CONST, abi.JITTER_HASH])),
                  jitter_value=float(rng.uniform()), spp=int(rng.choice([1, 2])),
                  composite_mode=int(rng.choice([abi.COMPOSITE_FP32, abi.COMPOSITE_UBYTE])),
                  crosshair=int(rng.random() < 0.2))
    ctx.set_params(**params)
    n_views = int(rng.integers(1, 11))
    views = [int(v) for v in rng.permutation(16)[:n_views]]
    sizes, cams = [], []
    for v in views:
        W, H = (int(x) for x in rng.choice([1, 9, 40, 64, 96], p=[.05, .15, .3, .25, .25], size=2))
        cam = _camera(rng, dims, W, H)
        ctx.set_camera(v, *cam)
        ctx.resize(v, W, H)
        sizes.append((W, H))
        cams.append(cam)
    fbs = [torch.full((H, W), -1, dtype=torch.int32, device="cuda") for (W, H) in sizes]
    b = ctx.batch(views, fbs)
    tile = [(8, 4), (8, 8), (16, 8), (32, 4)][int(rng.integers(0, 4))]
    b.set_config(*tile, int(rng.choice([0, 3, 5, 7])))
    b.set_staging(int(rng.choice([abi.STAGING_NONE, abi.STAGING_NEXT_SAMPLE])))
    b.set_unroll(int(rng.choice([1, 2])))
    if rng.random() < 0.5:
        b.launch()
    else:
        b.launch_graph()
        b.launch_graph()
    torch.cuda.synchronize()
    for f, (W, H), cam in zip(fbs, sizes, cams):
        ref = oracle.render(descs, vox, tf, oracle.make_camera(*cam), W, H, oracle.make_params(**params),
                            n_ranks=n_ranks, brick_rank=brick_rank, want=("fb",))
        got = f.cpu().numpy().view(np.uint32)
        assert np.array_equal(got, ref["fb"]), \
            f"seed {seed}: view {W}x{H}, {np.count_nonzero(got != ref['fb'])} pixels differ, tile {tile}"
    b.close()


@pytest.mark.parametrize("seed", range(24))
def test_random_differentiable_case(gpu_ctx_factory, oracle, seed):
    """The differentiable form on random single-rank scenes: the training
    forward's float image is bit-identical to the oracle's, and the gradients
    of a random dL/dRGBA are within 5e-4 (relative 2-norm) of the FP64
    adjoint, for a random checkpoint interval."""
    rng = np.random.default_rng(9000 + seed)
    dims = tuple(int(x) for x in rng.integers(9, 49, size=3))
    vol = _volume(rng, dims)
    descs = _bricks(rng, dims)
    vox = S.extract_bricks(vol, descs)
    tf = _tf(rng)
    params = dict(dt=float(rng.choice([0.5, 1.0, 0.3, 0.375])), et_alpha=float(rng.choice([0.99, 0.8, 2.0])),
                  jitter_mode=int(rng.choice([abi.JITTER_NONE, abi.JITTER_CONST, abi.JITTER_HASH])),
                  jitter_value=float(rng.uniform()))
    ctx = gpu_ctx_factory()
    ctx.set_bricks(descs, vox)
    ctx.set_transfer_function(tf)
    ctx.set_ranks(1)
    ctx.set_params(**params)
    W, H = (int(x) for x in rng.choice([7, 33, 64], size=2))
    cam = _camera(rng, dims, W, H)
    ctx.set_camera(0, *cam)
    ctx.resize(0, W, H)
    k = int(rng.choice([1, 5, 16, 32, 64]))
    img = np.zeros((H, W, 4), np.float32)
    ctx.forward(0, img, k)
    op = oracle.make_params(**params)
    ref = oracle.render(descs, vox, tf, oracle.make_camera(*cam), W, H, op, n_ranks=1, want=("final",))
    np.testing.assert_array_equal(img, ref["final"])
    dl = rng.uniform(-1, 1, (H, W, 4)).astype(np.float32)
    nx, ny, nz = dims
    dtf = np.zeros((tf.shape[0], 4), np.float32)
    dden = np.zeros((nz, ny, nx), np.float32)
    ctx.backward(0, dl, dtf, dden, (0, 0, 0), (nx, ny, nz))
    r = oracle.adjoint(descs, vox, tf, oracle.make_camera(*cam), W, H, dl, (0, 0, 0), (nx, ny, nz), op)

    def rel(a, b):
        return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))
    where = f"seed {seed}: dims {dims}, {len(descs)} bricks, {W}x{H}, K {k}, {params}, n_tf {tf.shape[0]}"
    if np.linalg.norm(r["dtf"]) > 0:
        assert rel(dtf, r["dtf"]) < 5e-4, where
    if np.linalg.norm(r["ddensity"]) > 0:
        assert rel(dden, r["ddensity"]) < 5e-4, where


@pytest.mark.parametrize("seed", range(12))
def test_random_call_sequences(gpu_ctx_factory, oracle, seed):
    """One context driven through a seeded random sequence of 14 calls:
    cameras, resizes, transfer functions (of other sizes too), brick updates
    and drops, rank changes, render parameters and the work division.  After
    each call the frame of a random view that has a camera and a size must
    equal the oracle's for the state the calls built (a dropped brick must
    make renders fail until its data is back).  This checks what the context
    caches (view schedules, split planes, chunk orders, macrocell tables)
    against every kind of change."""
    rng = np.random.default_rng(7000 + seed)
    dims = tuple(int(x) for x in rng.integers(12, 57, size=3))
    vol = _volume(rng, dims)
    descs = _bricks(rng, dims)
    nb = len(descs)
    vox = [np.ascontiguousarray(v) for v in S.extract_bricks(vol, descs)]
    tf = _tf(rng)
    ctx = gpu_ctx_factory()
    ctx.set_bricks(descs, vox)
    ctx.set_transfer_function(tf)
    st = dict(n_ranks=nb, brick_rank=None, params={}, views={}, dropped=set())
    try:
        oracle.partition_kd(descs, nb)
    except ValueError:
        st["brick_rank"] = np.arange(nb, dtype=np.int32)  # the upload's fallback numbering

    def set_camera(v):
        W, H = (int(x) for x in rng.choice([9, 33, 64, 80], size=2))
        cam = _camera(rng, dims, W, H)
        ctx.set_camera(v, *cam)
        old = st["views"].get(v, {})
        st["views"][v] = dict(old, cam=cam)
        if "size" not in old:
            ctx.resize(v, W, H)
            st["views"][v]["size"] = (W, H)

    ops = ["camera", "resize", "tf", "update", "drop", "ranks", "assign", "params", "work"]
    for step in range(14):
        op = "camera" if not st["views"] else str(rng.choice(ops))
        if op == "camera":
            set_camera(int(rng.integers(0, 4)))
        elif op == "resize":
            v = int(rng.choice(list(st["views"])))
            W, H = (int(x) for x in rng.choice([1, 9, 33, 64, 80], size=2))
            ctx.resize(v, W, H)
            st["views"][v]["size"] = (W, H)
        elif op == "tf":
            tf = _tf(rng)
            ctx.set_transfer_function(tf)
        elif op == "update":
            b = int(rng.integers(0, nb))
            vox[b] = np.ascontiguousarray((vox[b] * np.float32(rng.uniform(0.3, 1.5))).astype(np.float32))
            ctx.update_brick(b, vox[b])
            st["dropped"].discard(b)
        elif op == "drop":
            b = int(rng.integers(0, nb))
            ctx.drop_brick(b)
            st["dropped"].add(b)
        elif op in ("ranks", "assign"):
            n = int(rng.integers(1, nb + 1))
            if op == "ranks":
                try:
                    oracle.partition_kd(descs, n)
                except ValueError:
                    with pytest.raises(abi.AlohaError):
                        ctx.set_ranks(n)
                    continue
                ctx.set_ranks(n)
                st["n_ranks"], st["brick_rank"] = n, None
            else:
                br = np.concatenate([np.arange(n), rng.integers(0, n, nb - n)]).astype(np.int32)
                rng.shuffle(br)
                ctx.set_rank_assignment(br, n)
                st["n_ranks"], st["brick_rank"] = n, br
        elif op == "params":
            st["params"] = dict(dt=float(rng.choice([0.5, 1.0, 0.3])), et_alpha=float(rng.choice([0.99, 0.7, 2.0])),
                                jitter_mode=int(rng.choice([abi.JITTER_NONE, abi.JITTER_CONST, abi.JITTER_HASH])),
                                jitter_value=float(rng.uniform()),
                                composite_mode=int(rng.choice([abi.COMPOSITE_FP32, abi.COMPOSITE_UBYTE])))
            ctx.set_params(**st["params"])
        elif op == "work":
            split = int(rng.choice([abi.SPLIT_AUTO, abi.SPLIT_PIXELS, abi.SPLIT_RANKS]))
            ctx.set_render_split(split)
            ctx.set_chunk_order(int(rng.choice([abi.CHUNKS_AUTO, abi.CHUNKS_RING, abi.CHUNKS_PROBED])))
            ctx.set_render_tile(*[(8, 4), (8, 8), (16, 8), (32, 4)][int(rng.integers(0, 4))])
        v = int(rng.choice(list(st["views"])))
        W, H = st["views"][v]["size"]
        cam = st["views"][v]["cam"]
        where = f"seed {seed} step {step} ({op}): view {v} {W}x{H}, {st['n_ranks']} ranks, {nb} bricks"
        if st["dropped"]:
            with pytest.raises(abi.AlohaError) as e:
                ctx.render(v, width=W, height=H)
            assert e.value.code == abi.ERR_MISSING_BRICK, where
            continue
        fb = ctx.render(v, width=W, height=H)
        samples = ctx.stats().samples
        ref = oracle.render(descs, vox, tf, oracle.make_camera(*cam), W, H, oracle.make_params(**st["params"]),
                            n_ranks=st["n_ranks"], brick_rank=st["brick_rank"], want=("fb",))
        assert np.array_equal(fb, ref["fb"]), f"{where}: {np.count_nonzero(fb != ref['fb'])} pixels differ"
        assert samples == ref["samples"], where


@pytest.mark.parametrize("seed", range(12))
def test_random_multi_view_training(gpu_ctx_factory, oracle, seed):
    """aloha_forward_views over 2 to 12 views of random sizes (1 to 96 pixels a
    side) in one launch: every image bit-identical to the oracle's; then
    aloha_backward_views over them, some re-forwarded at a second checkpoint
    interval, with a random choice of gradients: the sums within 5e-4 of the
    FP64 adjoints' sum."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(11000 + seed)
    dims = tuple(int(x) for x in rng.integers(9, 41, size=3))
    vol = _volume(rng, dims)
    descs = _bricks(rng, dims)
    vox = S.extract_bricks(vol, descs)
    tf = _tf(rng)
    params = dict(dt=float(rng.choice([0.5, 1.0, 0.375])), et_alpha=float(rng.choice([0.99, 2.0])),
                  jitter_mode=int(rng.choice([abi.JITTER_NONE, abi.JITTER_HASH])))
    ctx = gpu_ctx_factory()
    ctx.set_bricks(descs, vox)
    ctx.set_transfer_function(tf)
    ctx.set_ranks(1)
    ctx.set_params(**params)
    op = oracle.make_params(**params)
    n_views = int(rng.integers(2, 13))
    views = [int(v) for v in rng.permutation(32)[:n_views]]
    sizes, cams = {}, {}
    for v in views:
        W, H = (int(x) for x in rng.choice([1, 5, 24, 40, 96], p=[.1, .15, .25, .3, .2], size=2))
        sizes[v] = (W, H)
        cams[v] = _camera(rng, dims, W, H)
        ctx.set_camera(v, *cams[v])
        ctx.resize(v, W, H)
    k = int(rng.choice([1, 7, 32]))
    imgs = [np.zeros((sizes[v][1], sizes[v][0], 4), np.float32) if rng.random() < 0.5 else
            torch.zeros((sizes[v][1], sizes[v][0], 4), device="cuda") for v in views]
    ctx.forward_views(views, imgs, k)
    torch.cuda.synchronize()
    for v, img in zip(views, imgs):
        W, H = sizes[v]
        ref = oracle.render(descs, vox, tf, oracle.make_camera(*cams[v]), W, H, op, n_ranks=1, want=("final",))
        got = img.cpu().numpy() if hasattr(img, "cpu") else img
        np.testing.assert_array_equal(got, ref["final"], err_msg=f"seed {seed} view {v} {W}x{H}")
    again = [v for v in views if rng.random() < 0.3]
    if again:
        ctx.forward_views(again, [np.zeros((sizes[v][1], sizes[v][0], 4), np.float32) for v in again],
                          int(rng.choice([3, 16, 64])))
    nx, ny, nz = dims
    dls = [rng.uniform(-1, 1, (sizes[v][1], sizes[v][0], 4)).astype(np.float32) for v in views]
    want_tf, want_den = [(True, True), (True, False), (False, True)][int(rng.integers(0, 3))]
    dtf = np.zeros((tf.shape[0], 4), np.float32) if want_tf else None
    dden = np.zeros((nz, ny, nx), np.float32) if want_den else None
    ctx.backward_views(views, dls, dtf, dden, (0, 0, 0) if want_den else None, (nx, ny, nz) if want_den else None)
    ref_tf = np.zeros((tf.shape[0], 4))
    ref_den = np.zeros((nz, ny, nx))
    for v, dl in zip(views, dls):
        W, H = sizes[v]
        r = oracle.adjoint(descs, vox, tf, oracle.make_camera(*cams[v]), W, H, dl, (0, 0, 0), (nx, ny, nz), op)
        ref_tf += r["dtf"]
        ref_den += r["ddensity"]

    def rel(a, b):
        return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))
    where = f"seed {seed}: {n_views} views, k {k}, re-forwarded {again}, gradients tf {want_tf} density {want_den}"
    if want_tf and np.linalg.norm(ref_tf) > 0:
        assert rel(dtf, ref_tf) < 5e-4, where
    if want_den and np.linalg.norm(ref_den) > 0:
        assert rel(dden, ref_den) < 5e-4, where


@pytest.mark.parametrize("seed", range(16))
def test_random_standalone_composites(oracle, seed):
    """The IceT stand-ins on their own: 1 to 64 random rank images (values
    partly outside [0, 1], so the quantisation clamps), a random order, both
    blend modes, through aloha_composite_over (device and host images),
    aloha_composite_over_noalloc and, for RGBA8 rank images,
    aloha_composite_over_rgba8; every frame equals the oracle's blend."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(13000 + seed)
    n = int(rng.choice([1, 2, 5, 12, 33, 64]))
    W, H = (int(x) for x in rng.choice([1, 7, 40, 96], size=2))
    imgs = rng.uniform(-0.1, 1.1, (n, H, W, 4)).astype(np.float32)
    imgs[..., :3] *= np.clip(imgs[..., 3:4], 0, 1)  # mostly premultiplied
    order = rng.permutation(n).astype(np.int32)
    L = abi.lib()
    stream = torch.cuda.current_stream()
    dev_imgs = torch.from_numpy(imgs).cuda()
    for mode in (abi.COMPOSITE_FP32, abi.COMPOSITE_UBYTE):
        want = oracle.composite_over(imgs, order, mode)
        host_out = abi.composite_over(imgs, order, W, H, mode)
        dev_out = torch.zeros((H, W), dtype=torch.int32, device="cuda")
        abi.composite_over(dev_imgs, order, W, H, mode, fb=dev_out, stream=stream)
        na_out = torch.full((H, W), -1, dtype=torch.int32, device="cuda")
        assert L.aloha_composite_over_noalloc(dev_imgs.data_ptr(), order.ctypes.data, n, W, H, mode,
                                              na_out.data_ptr(), stream.cuda_stream) == abi.OK
        torch.cuda.synchronize()
        np.testing.assert_array_equal(host_out, want, err_msg=f"seed {seed} mode {mode} host")
        np.testing.assert_array_equal(dev_out.cpu().numpy().view(np.uint32), want, err_msg=f"seed {seed} device")
        np.testing.assert_array_equal(na_out.cpu().numpy().view(np.uint32), want, err_msg=f"seed {seed} noalloc")
    packed = rng.integers(0, 2**32, (n, H, W), dtype=np.uint64).astype(np.uint32)
    np.testing.assert_array_equal(abi.composite_over_rgba8(packed, order, W, H),
                                  oracle.composite_over_rgba8(packed, order), err_msg=f"seed {seed} rgba8")
