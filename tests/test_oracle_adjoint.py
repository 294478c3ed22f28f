"""The oracle's FP64 adjoint, the reference every GPU gradient test compares
with, checked on its own against central differences of the oracle's FP64
render (CPU only): the 12 largest transfer-function and density gradient
entries of a weighted-sum loss, eps 1e-4, step 0.5 (exact in float, so the
float sample set the adjoint follows is the FP64 render's), no jitter, no
early termination.  Agreement is to about 1e-7 relative; the bound is 1e-5."""
import numpy as np

from aloha_gb300 import scenes as S
from oracle import oracle as O


def test_fp64_adjoint_matches_central_differences():
    n = 20
    vol = S.blob_field((n, n, n), 5, (2.0, 5.0), seed=3)
    descs = S.single_brick((n, n, n))
    vox = S.extract_bricks(vol, descs)
    tf = S.ramp_tf(64)
    W = H = 20
    cam = O.make_camera(*S.orbit_cameras((n, n, n), 1, W, H, seed=4)[0])
    params = O.make_params(et_alpha=2.0, jitter_mode=O.JITTER_NONE)
    wts = np.random.default_rng(1).uniform(0.5, 1.5, (H, W, 4))

    def loss(tf_, vox_):
        r = O.render(descs, vox_, tf_, cam, W, H, params, precision="f64", want=("final",))
        return float((np.asarray(r["final"], np.float64) * wts).sum())

    g = O.adjoint(descs, vox, tf, cam, W, H, wts, (0, 0, 0), (n, n, n), params)
    eps = 1e-4
    errs = []
    for flat in np.argsort(-np.abs(g["dtf"]).ravel())[:12]:
        i, ch = divmod(int(flat), 4)
        tp, tm = tf.copy(), tf.copy()
        tp[i, ch] += eps
        tm[i, ch] -= eps
        fd = (loss(tp, vox) - loss(tm, vox)) / (float(tp[i, ch]) - float(tm[i, ch]))
        errs.append(abs(fd - g["dtf"][i, ch]) / abs(g["dtf"][i, ch]))
    v0 = vox[0]
    for flat in np.argsort(-np.abs(g["ddensity"]).ravel())[:12]:
        z, y, x = np.unravel_index(int(flat), (n, n, n))
        vp, vm = v0.copy(), v0.copy()
        vp[z, y, x] += eps
        vm[z, y, x] -= eps
        fd = (loss(tf, [vp]) - loss(tf, [vm])) / (float(vp[z, y, x]) - float(vm[z, y, x]))
        errs.append(abs(fd - g["ddensity"][z, y, x]) / abs(g["ddensity"][z, y, x]))
    assert max(errs) < 1e-5, errs
