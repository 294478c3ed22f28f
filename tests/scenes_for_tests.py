"""Seeded test scenes shared by the oracle and GPU parity tests."""
from __future__ import annotations

import numpy as np

from aloha_gb300 import scenes as S


def c1_scene():
    """64^3 uint8 single brick, normalized /255 (the plain configuration)."""
    raw = S.plain_c1_volume(seed=1)
    vol = S.normalize_raw(raw)
    descs = S.single_brick(vol.shape[::-1])
    vox = S.extract_bricks(vol, descs)
    return vol, descs, vox, S.ramp_tf()


def blob_volume(n: int, n_blobs: int = 16, seed: int = 7):
    return S.blob_field((n, n, n), n_blobs, (n / 16.0, n / 6.0), seed)


def chopsuey_scene(n: int = 64, n_bricks: int = 8, seed: int = 7):
    from oracle import oracle as O
    vol = blob_volume(n, seed=seed)
    descs = O.chopsuey_split((n, n, n), n_bricks)
    vox = S.extract_bricks(vol, descs)
    return vol, descs, vox, S.ramp_tf()


def uneven_scene(n: int = 64, seed: int = 11):
    """3x2x2 uneven split (cuts scaled from 200,380 / 256 / 300 of 512)."""
    vol = blob_volume(n, seed=seed)
    cuts = ([n * 200 // 512, n * 380 // 512], [n // 2], [n * 300 // 512])
    descs = S.grid_split((n, n, n), cuts)
    vox = S.extract_bricks(vol, descs)
    return vol, descs, vox, S.ramp_tf()


def cameras(dims, n, W, H, seed=3, distance=2.0):
    return S.orbit_cameras(dims, n, W, H, seed=seed, distance=distance)
