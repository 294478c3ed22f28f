"""Generates the golden vectors in this folder from the CPU oracle.

The reference ships no golden images or fixtures, so these are regression
vectors of the oracle itself: they pin its outputs across compilers and
machines (the x86 container and the Arm GPU host must reproduce them bit for
bit) and give the GPU tests a fixed target.  Run from the repository root:

    python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)


def cases():
    from aloha_gb300 import scenes as S
    from oracle import oracle as O
    from tests import scenes_for_tests as T

    out = {}
    # plain single brick, 96x96, default parameters
    vol, descs, vox, tf = T.c1_scene()
    cam = S.axis_camera((64, 64, 64), 96, 96)
    r = O.render(descs, vox, tf, O.make_camera(*cam), 96, 96, O.make_params(), want=("fb", "pixel_samples"))
    out["plain_fb"] = r["fb"]
    out["plain_samples"] = r["pixel_samples"]
    # 8 chopSuey bricks as 8 virtual ranks, fp32 and ubyte composites, 64x48
    vol, descs, vox, tf = T.chopsuey_scene(32, 8)
    cam = T.cameras((32, 32, 32), 1, 64, 48, seed=5)[0]
    for name, mode in (("ranks_fp32", O.COMPOSITE_FP32), ("ranks_ubyte", O.COMPOSITE_UBYTE)):
        r = O.render(descs, vox, tf, O.make_camera(*cam), 64, 48, O.make_params(composite_mode=mode), n_ranks=8,
                     want=("fb", "rank_images"))
        out[name + "_fb"] = r["fb"]
        out[name + "_order"] = np.asarray(r["rank_order"], np.int32)
    out["ranks_fp32_rank_images"] = r["rank_images"]
    # uneven 3x2x2 bricks, crosshair and spp 2
    vol, descs, vox, tf = T.uneven_scene(48)
    cam = T.cameras((48, 48, 48), 1, 56, 56, seed=6)[0]
    r = O.render(descs, vox, tf, O.make_camera(*cam), 56, 56, O.make_params(crosshair=1, spp=2), n_ranks=12)
    out["uneven_fb"] = r["fb"]
    # layouts and orders
    d = O.chopsuey_split((512, 512, 512), 8)
    out["chopsuey_512_8"] = np.array([b["cell_lo"] + b["cell_hi"] + b["voxel_lo"] + b["voxel_hi"] for b in d],
                                     np.int32)
    cr, kd = O.partition_kd(O.chopsuey_split((512, 512, 512), 8), 2)
    out["partition_512_8_r2"] = cr.astype(np.int32)
    return out


def load():
    return dict(np.load(os.path.join(HERE, "golden.npz")))


if __name__ == "__main__":
    data = cases()
    np.savez_compressed(os.path.join(HERE, "golden.npz"), **data)
    print({k: v.shape for k, v in data.items()})
