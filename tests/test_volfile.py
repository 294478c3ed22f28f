"""The product's chopSuey splitter and .vol reader/writer (CPU)."""
import os

import numpy as np
import pytest

from aloha_gb300 import volfile as V
from tests import scenes_for_tests as T


@pytest.mark.parametrize("dims,n", [((512, 512, 512), 8), ((64, 64, 64), 1), ((67, 45, 30), 7),
                                    ((1024, 1024, 1024), 64), ((100, 37, 250), 12), ((16, 16, 16), 5)])
def test_chopsuey_split_matches_oracle(oracle, dims, n):
    assert V.chopsuey_split(dims, n) == oracle.chopsuey_split(dims, n)


def test_chopsuey_rejects_impossible_counts():
    with pytest.raises(ValueError):
        V.chopsuey_split((2, 2, 2), 9)
    with pytest.raises(ValueError):
        V.chopsuey_split((0, 4, 4), 2)


def test_vol_round_trip(tmp_path):
    vol, descs, vox, tf = T.chopsuey_scene(32, 8)
    path = os.path.join(tmp_path, "scene.vol")
    V.write_vol(path, (32, 32, 32), descs, vox)
    header, d2, v2 = V.read_vol(path)
    assert header["n"] == 8 and header["cell_hi"] == [32, 32, 32]
    assert header["voxel_hi"] == [33, 33, 33]  # root voxel range dims+1 (chopSuey.cpp:251)
    for a, b, va, vb in zip(descs, d2, vox, v2):
        for k in ("cell_lo", "cell_hi", "voxel_lo", "voxel_hi", "space_lo", "space_hi"):
            assert a[k] == b[k]
        assert b["value_range"] == [float(np.float32(va.min())), float(np.float32(va.max()))]
        np.testing.assert_array_equal(va, vb)
    # a rank reads only its own bricks (waikikiRenderer.cpp:637-665)
    _, _, part = V.read_vol(path, bricks={2, 5})
    assert part[0] is None and part[2] is not None and part[5] is not None
    np.testing.assert_array_equal(part[5], vox[5])


def test_vol_header_layout_is_80_bytes_per_brick(tmp_path):
    vol, descs, vox, tf = T.chopsuey_scene(16, 2)
    path = os.path.join(tmp_path, "s.vol")
    V.write_vol(path, (16, 16, 16), descs, vox)
    expect = 8 + 72 + sum(80 + 4 * v.size for v in vox)
    assert os.path.getsize(path) == expect
