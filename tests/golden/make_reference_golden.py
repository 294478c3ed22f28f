"""Generates tests/golden/reference_frames.npz from the reference's own code.

The frames come from the reference raygen (deviceCode.cpp compiled unchanged,
oracle/_ref, driven by oracle/ref_harness.cpp): per virtual rank the RGBA8
frame that renderFrame writes (crosshair included, as the reference always
draws it), its depth buffer and per-pixel sample counts, plus the rank
assignment of the reference's partitionKD.  The scenes are rebuilt from
seeds by tests/scenes_for_tests.py, so only the outputs are stored.  The
fixtures let the oracle and the GPU path be checked against the reference
where its sources are absent (the GPU host).  Run from the repository root
where the reference sources are present:

    python tests/golden/make_reference_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

PATH = os.path.join(HERE, "reference_frames.npz")


def scenes():
    """(name, descs, voxels, tf, camera tuple, W, H, n_ranks) of every fixture."""
    from aloha_gb300 import scenes as S
    from tests import scenes_for_tests as T

    out = []
    vol, descs, vox, tf = T.c1_scene()
    out.append(("c1", descs, vox, tf, S.axis_camera(vol.shape[::-1], 512, 512), 512, 512, 1))
    vol, descs, vox, tf = T.chopsuey_scene(64, 8)
    for i, cam in enumerate(T.cameras((64, 64, 64), 2, 128, 96, seed=21)):
        out.append((f"sortlast{i}", descs, vox, tf, cam, 128, 96, 8))
    vol, descs, vox, tf = T.uneven_scene(64)
    for i, cam in enumerate(T.cameras((64, 64, 64), 2, 96, 80, seed=22)):
        out.append((f"uneven{i}_r12", descs, vox, tf, cam, 96, 80, 12))
        out.append((f"uneven{i}_r3", descs, vox, tf, cam, 96, 80, 3))
    return out


def load():
    return dict(np.load(PATH))


def main():
    from oracle import oracle as O
    from oracle import reference as R

    data = {}
    for name, descs, vox, tf, cam, W, H, n_ranks in scenes():
        r = R.render_ranks(descs, vox, tf, O.make_camera(*cam), W, H, n_ranks=n_ranks)
        data[name + "_fb"] = r["fb"]
        if name != "c1":  # depth is pinned on the small scenes; 1 MB of floats at 512^2
            data[name + "_depth"] = r["depth"]
        data[name + "_samples"] = r["samples"].astype(np.uint32)
        data[name + "_brick_rank"] = r["brick_rank"].astype(np.int32)
    np.savez_compressed(PATH, **data)
    print({k: v.shape for k, v in data.items()})


if __name__ == "__main__":
    main()
