"""The C++ drop-in (include/aloha_renderer.hpp) driven like the reference's
viewer drives maui::Renderer: a .vol file, colour map, resize and camera
events, render(fb) into host memory; checked against the oracle."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from aloha_gb300 import volfile as V
from tests import scenes_for_tests as T

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def render_vol(tmp_path_factory):
    from aloha_gb300 import abi
    abi.lib()
    out = str(tmp_path_factory.mktemp("cpp") / "render_vol")
    cxx = shutil.which("g++") or "g++"
    lib_dir = os.path.join(ROOT, "aloha_gb300")
    subprocess.run([cxx, "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", "render_vol.cpp"), "-o", out, "-L", lib_dir, "-laloha_gb300",
                    f"-Wl,-rpath,{lib_dir}"], check=True)
    return out


@pytest.mark.parametrize("n_ranks", [0, 2])
def test_cpp_renderer_matches_oracle(render_vol, oracle, tmp_path, n_ranks):
    vol, descs, vox, tf = T.chopsuey_scene(48, 8)
    vpath, tpath, opath = (str(tmp_path / f) for f in ("s.vol", "tf.f32", "fb.u32"))
    V.write_vol(vpath, (48, 48, 48), descs, vox)
    tf.astype(np.float32).tofile(tpath)
    W, H = 80, 64
    cam = T.cameras((48, 48, 48), 1, W, H, seed=41)[0]
    args = [render_vol, vpath, tpath, str(tf.shape[0]), opath, str(W), str(H), str(n_ranks)]
    args += [repr(float(v)) for c in cam for v in c]
    subprocess.run(args, check=True)
    fb = np.fromfile(opath, dtype=np.uint32).reshape(H, W)
    ranks = n_ranks or 8
    ref = oracle.render(descs, vox, tf, oracle.make_camera(*cam), W, H, oracle.make_params(), n_ranks=ranks)
    np.testing.assert_array_equal(fb, ref["fb"])


def test_raw_volume_through_chopsuey_and_cpp_renderer(render_vol, oracle, tmp_path):
    """A raw uint8 volume -> the chopSuey tool -> .vol -> the C++ renderer:
    the frame equals the in-memory path (the same volume normalised and split
    in Python, rendered through the C ABI) and the oracle."""
    from aloha_gb300 import abi
    from aloha_gb300 import chopsuey
    from aloha_gb300 import scenes as S
    raw = S.plain_c1_volume(seed=3)[:, :, :60]  # 60 x 64 x 64, x fastest
    raw = np.ascontiguousarray(raw)
    dims = (raw.shape[2], raw.shape[1], raw.shape[0])
    raw_path, vpath, tpath, opath = (str(tmp_path / f) for f in ("in.raw", "s.vol", "tf.f32", "fb.u32"))
    raw.tofile(raw_path)
    assert chopsuey.main([raw_path, "-dims", *map(str, dims), "-type", "uint8", "-n", "6", "-o", vpath]) == 0
    tf = S.ramp_tf()
    tf.astype(np.float32).tofile(tpath)
    W, H = 72, 64
    cam = T.cameras(dims, 1, W, H, seed=43)[0]
    args = [render_vol, vpath, tpath, str(tf.shape[0]), opath, str(W), str(H), "0"]
    args += [repr(float(v)) for c in cam for v in c]
    subprocess.run(args, check=True)
    fb = np.fromfile(opath, dtype=np.uint32).reshape(H, W)
    vol = V.normalize_raw(raw)
    descs = V.chopsuey_split(dims, 6)
    vox = [V.brick_voxels(vol, d) for d in descs]
    with abi.Context(0) as ctx:
        ctx.set_bricks(descs, vox)
        ctx.set_transfer_function(tf)
        ctx.set_params()
        ctx.set_camera(0, *cam)
        ctx.resize(0, W, H)
        np.testing.assert_array_equal(ctx.render(0, width=W, height=H), fb)
    ref = oracle.render(descs, vox, tf, oracle.make_camera(*cam), W, H, oracle.make_params(), n_ranks=len(descs))
    np.testing.assert_array_equal(fb, ref["fb"])


def test_cpp_training_views_match_oracle(oracle, tmp_path):
    """tests/cpp/train_views.cpp: one aloha_forward_views launch over three
    views and one aloha_backward_views call, from C++ with host buffers; the
    images equal the oracle's and the gradients its FP64 adjoint's sum."""
    from aloha_gb300 import abi
    abi.lib()
    exe = str(tmp_path / "train_views")
    cxx = shutil.which("g++") or "g++"
    lib_dir = os.path.join(ROOT, "aloha_gb300")
    subprocess.run([cxx, "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", "train_views.cpp"), "-o", exe, "-L", lib_dir, "-laloha_gb300",
                    f"-Wl,-rpath,{lib_dir}"], check=True)
    n = 40
    vol, descs, vox, tf = T.chopsuey_scene(n, 4)
    W, H, k, nv = 48, 40, 16, 3
    cams = T.cameras((n, n, n), nv, W, H, seed=47)
    rng = np.random.default_rng(5)
    dl = rng.uniform(-1, 1, (nv, H, W, 4)).astype(np.float32)
    paths = {f: str(tmp_path / f) for f in ("s.vol", "tf.f32", "cams.f32", "dl.f32", "img.f32", "dtf.f32",
                                             "dden.f32")}
    V.write_vol(paths["s.vol"], (n, n, n), descs, vox)
    tf.astype(np.float32).tofile(paths["tf.f32"])
    np.asarray([[x for c in cam for x in c] for cam in cams], np.float32).tofile(paths["cams.f32"])
    dl.tofile(paths["dl.f32"])
    subprocess.run([exe, paths["s.vol"], paths["tf.f32"], str(tf.shape[0]), str(k), str(W), str(H), str(nv),
                    paths["cams.f32"], paths["dl.f32"], paths["img.f32"], paths["dtf.f32"], paths["dden.f32"],
                    str(n), str(n), str(n)], check=True)
    img = np.fromfile(paths["img.f32"], np.float32).reshape(nv, H, W, 4)
    dtf = np.fromfile(paths["dtf.f32"], np.float32).reshape(tf.shape[0], 4)
    dden = np.fromfile(paths["dden.f32"], np.float32).reshape(n, n, n)
    ref_tf = np.zeros((tf.shape[0], 4))
    ref_den = np.zeros((n, n, n))
    for v, cam in enumerate(cams):
        ref = oracle.render(descs, vox, tf, oracle.make_camera(*cam), W, H, oracle.make_params(), n_ranks=1,
                            want=("final",))
        np.testing.assert_array_equal(img[v], ref["final"])
        r = oracle.adjoint(descs, vox, tf, oracle.make_camera(*cam), W, H, dl[v], (0, 0, 0), (n, n, n))
        ref_tf += r["dtf"]
        ref_den += r["ddensity"]
    for got, want in ((dtf, ref_tf), (dden, ref_den)):
        assert np.linalg.norm(got - want) / np.linalg.norm(want) < 5e-4
