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
