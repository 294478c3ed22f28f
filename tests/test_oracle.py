"""CPU tests of the oracle: closed forms, layout, ordering, known answers.

The reference ships no tests, golden images or fixtures, so the oracle is
pinned by closed-form cases derived from the reference's own arithmetic
(deviceCode.cpp:245-298, waikikiRenderer.cpp:150-316, chopSuey.cpp:245-323)
and by the golden vectors under tests/golden/ (generated by
tests/golden/make_golden.py).
"""
import math

import numpy as np
import pytest

from aloha_gb300 import scenes as S
from tests import scenes_for_tests as T


def _adjacent_violations(O, descs, order, cam):
    """Pairs of face-adjacent bricks rendered back-to-front for this camera."""
    pos = {b: i for i, b in enumerate(order)}
    B = O.space_boxes(descs)
    bad = 0
    for i in range(len(B)):
        for j in range(len(B)):
            if i == j:
                continue
            for a in range(3):
                o1, o2 = [k for k in range(3) if k != a]
                touch = B[i, 3 + a] == B[j, a]
                ov1 = min(B[i, 3 + o1], B[j, 3 + o1]) > max(B[i, o1], B[j, o1])
                ov2 = min(B[i, 3 + o2], B[j, 3 + o2]) > max(B[i, o2], B[j, o2])
                if touch and ov1 and ov2:
                    if cam[a] < B[i, 3 + a] and pos[i] > pos[j]:
                        bad += 1
                    if cam[a] > B[i, 3 + a] and pos[j] > pos[i]:
                        bad += 1
    return bad


# ------------------------------------------------------------- primitives

def test_first_sample_t_lattice(oracle):
    rng = np.random.default_rng(0)
    for _ in range(2000):
        lower = np.float32(rng.uniform(0, 2000))
        dt = np.float32(rng.choice([0.25, 0.5, 1.0, 2.0]))
        ils = np.float32(rng.uniform(0, 1))
        t = np.float32(oracle.first_sample_t(lower, dt, ils))
        assert t >= lower
        assert t - dt < lower + 1e-3
        k = (t / dt) - ils
        assert abs(k - round(k)) < 2e-3


def test_tf_lookup_texel_centres_and_border(oracle):
    rng = np.random.default_rng(1)
    tf = rng.uniform(0, 1, (256, 4)).astype(np.float32)
    for i in (0, 1, 100, 254, 255):
        v = (i + 0.5) / 256.0
        np.testing.assert_array_equal(oracle.tf_lookup(tf, v), tf[i])
    # border colour 0: at v = 1 the lookup is half the last entry, at v = 0 half the first
    np.testing.assert_allclose(oracle.tf_lookup(tf, 1.0), 0.5 * tf[255], rtol=1e-6)
    np.testing.assert_allclose(oracle.tf_lookup(tf, 0.0), 0.5 * tf[0], rtol=1e-6)
    assert np.all(oracle.tf_lookup(tf, -0.01) == 0)
    assert np.all(oracle.tf_lookup(tf, 1.01) == 0)
    assert np.all(oracle.tf_lookup(tf, 5.0) == 0)


def test_stencil_linear_ramp_is_exact(oracle):
    n = 16
    z, y, x = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
    a, b, c = 0.5, -0.25, 0.125
    vol = (a * x + b * y + c * z).astype(np.float32)
    rng = np.random.default_rng(2)
    for _ in range(300):
        u = rng.uniform(1.0, n - 2.0, 3).astype(np.float32)
        val, gx, gy, gz = oracle.stencil(vol, u)
        assert val == pytest.approx(a * u[0] + b * u[1] + c * u[2], abs=2e-5)
        assert gx == pytest.approx(a, abs=1e-5)
        assert gy == pytest.approx(b, abs=1e-5)
        assert gz == pytest.approx(c, abs=1e-5)


def test_stencil_clamps_at_the_edge(oracle):
    vol = np.arange(4 * 4 * 4, dtype=np.float32).reshape(4, 4, 4)
    # far outside: every tap clamps to the corner voxel, gradient 0
    for u in ([-5, -5, -5], [50, 50, 50]):
        val, gx, gy, gz = oracle.stencil(vol, u)
        corner = vol[0, 0, 0] if u[0] < 0 else vol[3, 3, 3]
        assert val == corner and gx == 0 and gy == 0 and gz == 0


def test_jitter_hash_range(oracle):
    vals = np.array([oracle.jitter_hash(p, a, d) for p in range(200) for a in range(3) for d in range(3)])
    assert vals.min() >= 0.0 and vals.max() < 1.0
    assert 0.4 < vals.mean() < 0.6


# ---------------------------------------------------------- closed forms

def _single_brick(vol):
    descs = S.single_brick(vol.shape[::-1])
    return descs, S.extract_bricks(vol, descs)


def test_empty_transfer_function_gives_zero(oracle):
    vol, descs, vox, _ = T.c1_scene()
    tf = np.zeros((256, 4), np.float32)
    cam = oracle.make_camera(*S.axis_camera((64, 64, 64), 64, 64))
    r = oracle.render(descs, vox, tf, cam, 64, 64, want=("fb", "pixel_samples"))
    assert np.all(r["fb"] == 0)
    assert r["samples"] > 0  # no early termination: every sample is taken


def test_constant_density_closed_form(oracle):
    """Constant field, constant TF: alpha after n samples is 1-(1-a)^n, rgb = 0.1 c alpha."""
    n = 16
    vol = np.full((n, n, n), 0.5, np.float32)
    descs, vox = _single_brick(vol)
    a, col = float(np.float32(0.05)), np.array([0.8, 0.4, 0.2], np.float32)
    tf = np.tile(np.concatenate([col, [a]]).astype(np.float32), (256, 1))
    W = H = 16
    cam = oracle.make_camera(*S.axis_camera((n, n, n), W, H, distance=2.0))
    p = oracle.make_params(dt=0.5, et_alpha=2.0, jitter_mode=oracle.JITTER_NONE)  # no early termination
    r = oracle.render(descs, vox, tf, cam, W, H, p, precision="f64", want=("final", "pixel_samples"))
    fin, ns = r["final"].reshape(-1, 4), r["pixel_samples"].reshape(-1)
    for px in range(W * H):
        k = int(ns[px])
        alpha = 1 - (1 - a) ** k
        assert fin[px, 3] == pytest.approx(alpha, abs=1e-9)
        # gradient is exactly 0 -> shade = 0.1 (deviceCode.cpp:294)
        np.testing.assert_allclose(fin[px, :3], 0.1 * col * alpha, rtol=1e-6, atol=1e-9)
    assert ns.max() > 0


def test_early_termination_stops_at_threshold(oracle):
    n = 32
    vol = np.full((n, n, n), 0.9, np.float32)
    descs, vox = _single_brick(vol)
    a = 0.3
    tf = np.tile(np.array([1, 1, 1, a], np.float32), (256, 1))
    cam = oracle.make_camera(*S.axis_camera((n, n, n), 8, 8))
    p = oracle.make_params(jitter_mode=oracle.JITTER_NONE)
    r = oracle.render(descs, vox, tf, cam, 8, 8, p, want=("final", "pixel_samples"))
    k_et = math.ceil(math.log(0.01) / math.log(1 - a))  # first k with 1-(1-a)^k >= .99
    ns = r["pixel_samples"].reshape(-1)
    assert ns.max() == k_et
    assert np.all(r["final"].reshape(-1, 4)[ns == k_et, 3] >= 0.99)


def test_fp64_rerender_error_is_small(oracle):
    vol, descs, vox, tf = T.c1_scene()
    cam = oracle.make_camera(*S.axis_camera((64, 64, 64), 128, 128))
    r32 = oracle.render(descs, vox, tf, cam, 128, 128, want=("final",))
    r64 = oracle.render(descs, vox, tf, cam, 128, 128, precision="f64", want=("final",))
    err = np.abs(r32["final"] - r64["final"])
    assert np.median(err) < 1e-6
    assert np.mean(err) < 1e-4
    assert err.max() < 0.02  # bounded by one early-termination flip: (1-.99)*max alpha*colour


# ------------------------------------------------------------------ layout

def test_chopsuey_power_of_two_split(oracle):
    d = oracle.chopsuey_split((512, 512, 512), 8)
    assert len(d) == 8
    cells = set()
    for b in d:
        for a in range(3):
            assert b["cell_hi"][a] - b["cell_lo"][a] == 256
            assert b["voxel_lo"][a] == b["cell_lo"][a]
            assert b["voxel_hi"][a] == min(b["cell_hi"][a] + 1, 512)  # one-sided ghost (chopSuey.cpp:303,311)
            assert b["space_lo"][a] == b["cell_lo"][a] and b["space_hi"][a] == b["cell_hi"][a]
        cells.add(tuple(b["cell_lo"]))
    assert len(cells) == 8
    # brick 0 is the low corner; bricks 0-3 are x-lo, 4-7 x-hi
    assert d[0]["cell_lo"] == [0, 0, 0]
    assert all(b["cell_lo"][0] == 0 for b in d[:4]) and all(b["cell_lo"][0] == 256 for b in d[4:])


def test_chopsuey_n1_still_splits(oracle):
    # doSplit() runs unconditionally (chopSuey.cpp:260): -n 1 gives two bricks
    assert len(oracle.chopsuey_split((64, 64, 64), 1)) == 2


def test_chopsuey_odd_sizes_cover_volume(oracle):
    dims = (67, 45, 30)
    d = oracle.chopsuey_split(dims, 7)
    assert len(d) >= 7
    covered = np.zeros(dims[::-1], np.int32)
    for b in d:
        lo, hi = b["cell_lo"], b["cell_hi"]
        covered[lo[2]:hi[2], lo[1]:hi[1], lo[0]:hi[0]] += 1
    assert np.all(covered == 1)


def test_grid_split_matches_chopsuey_ghost_rule():
    d = S.grid_split((512, 512, 512), ([200, 380], [256], [300]))
    assert len(d) == 12
    ext = sorted({b["cell_hi"][0] - b["cell_lo"][0] for b in d})
    assert ext == [132, 180, 200]
    for b in d:
        for a in range(3):
            assert b["voxel_hi"][a] == min(b["cell_hi"][a] + 1, 512)


# ---------------------------------------------------------------- ordering

def test_partition_kd_one_brick_per_rank(oracle):
    d = oracle.chopsuey_split((512, 512, 512), 8)
    cr, kd = oracle.partition_kd(d, 8)
    assert sorted(cr.tolist()) == list(range(8))


def test_partition_kd_groups(oracle):
    d = oracle.chopsuey_split((512, 512, 512), 8)
    cr, kd = oracle.partition_kd(d, 2)
    assert sorted(np.bincount(cr).tolist()) == [4, 4]
    # the two ranks are separated by the x = 256 plane
    xs = {r: {b["cell_lo"][0] for k, b in enumerate(d) if cr[k] == r} for r in range(2)}
    assert xs[0] != xs[1] and all(len(v) == 1 for v in xs.values())


def test_partition_kd_rejects_more_ranks_than_bricks(oracle):
    d = oracle.chopsuey_split((64, 64, 64), 2)
    with pytest.raises(ValueError):
        oracle.partition_kd(d, 4)


def test_reference_order_from_plus_z(oracle):
    d = oracle.chopsuey_split((512, 512, 512), 8)
    cr, kd = oracle.partition_kd(d, 8)
    assert oracle.composite_order_kd(kd, [256, 256, 2000], 8) == [7, 6, 5, 4, 3, 2, 1, 0]


def test_face_order_equals_kd_order_for_power_of_two_bricks(oracle):
    d = oracle.chopsuey_split((512, 512, 512), 8)
    cr, kd = oracle.partition_kd(d, 8)
    rng = np.random.default_rng(5)
    for _ in range(300):
        cam = rng.uniform(-600, 1100, 3)
        assert list(oracle.schedule(d, 8, cam)[0]) == oracle.composite_order_kd(kd, cam, 8)


def test_face_order_is_valid_for_uneven_bricks(oracle):
    """The reference's midplane test mis-orders uneven bricks; the face order never does."""
    d = S.grid_split((512, 512, 512), ([200, 380], [256], [300]))
    cr, kd = oracle.partition_kd(d, 12)
    r2b = {int(cr[k]): k for k in range(12)}
    rng = np.random.default_rng(6)
    kd_bad = 0
    for _ in range(300):
        cam = rng.uniform(-600, 1100, 3)
        faces = [r2b[r] for r in oracle.schedule(d, 12, cam)[0]]
        assert _adjacent_violations(oracle, d, faces, cam) == 0
        kd_bad += _adjacent_violations(oracle, d, [r2b[r] for r in oracle.composite_order_kd(kd, cam, 12)], cam) > 0
    assert kd_bad > 0  # documents the reference's mis-ordering for uneven bricks


# ------------------------------------------------------------- composites

def test_ubyte_and_fp32_agree_for_one_rank(oracle):
    vol, descs, vox, tf = T.c1_scene()
    cam = oracle.make_camera(*S.axis_camera((64, 64, 64), 64, 64))
    a = oracle.render(descs, vox, tf, cam, 64, 64, oracle.make_params(composite_mode=oracle.COMPOSITE_FP32))
    b = oracle.render(descs, vox, tf, cam, 64, 64, oracle.make_params(composite_mode=oracle.COMPOSITE_UBYTE))
    np.testing.assert_array_equal(a["fb"], b["fb"])


def test_rank_images_compose_to_final(oracle):
    vol, descs, vox, tf = T.chopsuey_scene(32, 8)
    cam = oracle.make_camera(*T.cameras((32, 32, 32), 1, 48, 48)[0])
    r = oracle.render(descs, vox, tf, cam, 48, 48, n_ranks=8, want=("final", "rank_images"))
    comp = np.zeros((48, 48, 4), np.float32)
    for k in r["rank_order"]:
        img = r["rank_images"][k]
        comp = np.float32(1) * comp + (np.float32(1) - comp[..., 3:4]) * img
    np.testing.assert_allclose(comp, r["final"], atol=2e-7)


def test_crosshair_inverts_row_and_column(oracle):
    vol, descs, vox, tf = T.c1_scene()
    cam = oracle.make_camera(*S.axis_camera((64, 64, 64), 32, 32))
    a = oracle.render(descs, vox, tf, cam, 32, 32, oracle.make_params(crosshair=0), want=("final",))["final"]
    b = oracle.render(descs, vox, tf, cam, 32, 32, oracle.make_params(crosshair=1), want=("final",))["final"]
    np.testing.assert_allclose(b[16, :, :], 1 - a[16, :, :], atol=1e-7)
    np.testing.assert_allclose(b[:, 16, :], 1 - a[:, 16, :], atol=1e-7)
    np.testing.assert_array_equal(np.delete(np.delete(a, 16, 0), 16, 1), np.delete(np.delete(b, 16, 0), 16, 1))


def test_progressive_accumulation_averages_frames(oracle):
    vol, descs, vox, tf = T.c1_scene()
    cam = oracle.make_camera(*S.axis_camera((64, 64, 64), 24, 24))
    acc = np.zeros((1, 24 * 24, 4), np.float32)
    frames = []
    for k in range(3):
        p = oracle.make_params(accum_id=k, accumulate=1)
        frames.append(oracle.render(descs, vox, tf, cam, 24, 24, p, want=("final",), accum=acc)["final"])
        single = oracle.render(descs, vox, tf, cam, 24, 24, oracle.make_params(accum_id=k), want=("final",))
        if k == 0:
            np.testing.assert_array_equal(frames[0], single["final"])
    np.testing.assert_allclose(acc.reshape(24, 24, 4) / 3.0, frames[-1], rtol=1e-6, atol=1e-7)


def test_islands_partition_the_image(oracle):
    vol, descs, vox, tf = T.c1_scene()
    cam = oracle.make_camera(*S.axis_camera((64, 64, 64), 48, 40))
    full = oracle.render(descs, vox, tf, cam, 48, 40, want=("final",))["final"]
    parts = [oracle.render(descs, vox, tf, cam, 48, 40, oracle.make_params(island_id=i, num_islands=3),
                           want=("final",))["final"] for i in range(3)]
    np.testing.assert_array_equal(sum(parts), full)
    assert all(np.any(p != 0) for p in parts)
