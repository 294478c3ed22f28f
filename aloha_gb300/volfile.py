"""chopSuey brick layout and the .vol brick file format.

``chopsuey_split`` restates chopSuey's VolumeSplitter (chopSuey.cpp:245-323):
the domain with the largest space volume is split at the middle of its longest
cell axis until the requested count is reached (``-n 1`` still gives two
bricks, chopSuey.cpp:260); each brick's voxel range is its cell range plus a
one-sided upper ghost layer clamped to the volume, min(cell.hi + 1, dims).

``.vol`` layout (chopSuey.cpp:325-349, read at waikikiRenderer.cpp:597-665),
all little-endian:
    uint64 numBricks; box3i cellRange; box3i voxelRange; box3f spaceRange
    per brick: box3i cellRange; box3i voxelRange; box3f spaceRange;
               interval<float> valueRange; float voxels[voxelRange volume]
(box3i = 6 int32, box3f = 6 float32, x-fastest voxels).  The root voxel range
is written as [0, dims+1) exactly as chopSuey does (chopSuey.cpp:251).

Raw volumes (volume.h:37-98, FileMapping.cpp): a headerless x-fastest file of
dims x*y*z voxels of 1, 2 or 4 bytes (uint8, uint16, float32), mapped into
memory and read brick by brick; ``normalize_raw`` converts like Volume::get.
``chop_raw`` is the chopSuey tool's volume path (chopSuey.cpp:361-441):
raw file -> split -> .vol, one brick in memory at a time.
"""
from __future__ import annotations

import struct

import numpy as np

HEADER = struct.Struct("<Q6i6i6f")
BRICK = struct.Struct("<6i6i6f2f")


def _brick(cell_lo, cell_hi, dims):
    return {"cell_lo": list(cell_lo), "cell_hi": list(cell_hi), "voxel_lo": list(cell_lo),
            "voxel_hi": [min(cell_hi[a] + 1, int(dims[a])) for a in range(3)],
            "space_lo": [float(v) for v in cell_lo], "space_hi": [float(v) for v in cell_hi],
            "value_range": [0.0, 0.0]}


def chopsuey_split(dims, n: int) -> list[dict]:
    """Brick descriptors of chopSuey's middle-split partition of a `dims` (x,y,z) volume."""
    dims = [int(d) for d in dims]
    if any(d <= 0 for d in dims):
        raise ValueError("volume dimensions must be positive")
    if n > dims[0] * dims[1] * dims[2]:
        raise ValueError("more bricks than cells")
    domains = [([0, 0, 0], list(dims))]
    while True:
        # domain with the largest space volume (float product, first on ties)
        pick, best = 0, np.float32(0.0)
        for k, (lo, hi) in enumerate(domains):
            vol = np.float32(hi[0] - lo[0]) * np.float32(hi[1] - lo[1]) * np.float32(hi[2] - lo[2])
            if vol > best:
                pick, best = k, vol
        lo, hi = domains.pop(pick)
        size = [hi[a] - lo[a] for a in range(3)]
        axis = 0
        if size[1] > size[0] and size[1] >= size[2]:
            axis = 1
        elif size[2] > size[0] and size[2] >= size[1]:
            axis = 2
        plane = int(np.float32(lo[axis]) + np.float32(size[axis]) * np.float32(0.5))
        l_hi = list(hi)
        l_hi[axis] = plane
        r_lo = list(lo)
        r_lo[axis] = plane
        for a_lo, a_hi in ((lo, l_hi), (r_lo, hi)):
            if all(a_hi[a] - a_lo[a] > 0 for a in range(3)):
                domains.append((list(a_lo), list(a_hi)))
        if len(domains) >= n:
            break
    return [_brick(lo, hi, dims) for lo, hi in domains]


def grid_split(dims, cuts) -> list[dict]:
    """Axis-aligned grid of bricks at the given interior cuts, chopSuey's ghost rule."""
    edges = [[0] + sorted(int(c) for c in cuts[a]) + [int(dims[a])] for a in range(3)]
    out = []
    for z0, z1 in zip(edges[2][:-1], edges[2][1:]):
        for y0, y1 in zip(edges[1][:-1], edges[1][1:]):
            for x0, x1 in zip(edges[0][:-1], edges[0][1:]):
                out.append(_brick([x0, y0, z0], [x1, y1, z1], dims))
    return out


def brick_voxels(volume, desc):
    """The brick's voxel range of a (nz, ny, nx) volume (numpy or torch),
    contiguous; numpy float volumes become float32, other numpy types keep
    their type (a raw volume before normalisation)."""
    lo, hi = desc["voxel_lo"], desc["voxel_hi"]
    v = volume[lo[2]:hi[2], lo[1]:hi[1], lo[0]:hi[0]]
    if hasattr(v, "contiguous"):
        return v.contiguous()
    v = np.asarray(v)
    return np.ascontiguousarray(v, dtype=np.float32 if v.dtype.kind == "f" else v.dtype)


def write_vol(path: str, dims, descs, voxels) -> None:
    """Write bricks as chopSuey's saveVols does (value ranges recomputed)."""
    dims = [int(d) for d in dims]
    with open(path, "wb") as f:
        f.write(HEADER.pack(len(descs), 0, 0, 0, *dims, 0, 0, 0, *[d + 1 for d in dims],
                            0.0, 0.0, 0.0, *[float(d) for d in dims]))
        for d, v in zip(descs, voxels):
            v = np.ascontiguousarray(np.asarray(v, dtype=np.float32))
            n = [d["voxel_hi"][a] - d["voxel_lo"][a] for a in range(3)]
            if v.size != n[0] * n[1] * n[2]:
                raise ValueError("voxel array does not match the brick's voxel range")
            f.write(BRICK.pack(*d["cell_lo"], *d["cell_hi"], *d["voxel_lo"], *d["voxel_hi"],
                               *d["space_lo"], *d["space_hi"], float(v.min()), float(v.max())))
            f.write(v.tobytes())


def read_vol(path: str, bricks=None):
    """Read a .vol file -> (header dict, descs, voxel arrays).  `bricks` selects
    which bricks' voxels to load (others are skipped, as a rank does at
    waikikiRenderer.cpp:637-665); None loads all."""
    with open(path, "rb") as f:
        h = HEADER.unpack(f.read(HEADER.size))
        header = {"n": h[0], "cell_lo": list(h[1:4]), "cell_hi": list(h[4:7]), "voxel_lo": list(h[7:10]),
                  "voxel_hi": list(h[10:13]), "space_lo": list(h[13:16]), "space_hi": list(h[16:19])}
        descs, vox = [], []
        for i in range(h[0]):
            b = BRICK.unpack(f.read(BRICK.size))
            d = {"cell_lo": list(b[0:3]), "cell_hi": list(b[3:6]), "voxel_lo": list(b[6:9]),
                 "voxel_hi": list(b[9:12]), "space_lo": list(b[12:15]), "space_hi": list(b[15:18]),
                 "value_range": [b[18], b[19]]}
            n = [d["voxel_hi"][a] - d["voxel_lo"][a] for a in range(3)]
            count = n[0] * n[1] * n[2]
            descs.append(d)
            if bricks is None or i in bricks:
                vox.append(np.fromfile(f, dtype="<f4", count=count).reshape(n[2], n[1], n[0]))
            else:
                f.seek(4 * count, 1)
                vox.append(None)
    return header, descs, vox


RAW_TYPES = {"uint8": np.dtype("u1"), "uint16": np.dtype("<u2"), "float": np.dtype("<f4")}
BPC_TYPES = {1: "uint8", 2: "uint16", 4: "float"}


def normalize_raw(raw) -> np.ndarray:
    """Volume::get's conversion (volume.h:75-88): uint8 /255, uint16 /65535,
    float32 as is, each voxel converted to float and divided in float."""
    raw = np.asarray(raw)
    if raw.dtype == np.uint8:
        return raw.astype(np.float32) / np.float32(255.0)
    if raw.dtype == np.uint16:
        return raw.astype(np.float32) / np.float32(65535.0)
    return raw.astype(np.float32)


def read_raw(path: str, dims, type_name: str) -> np.ndarray:
    """Memory-maps a raw volume as a (z, y, x) array of its stored type; the
    file must hold at least dims x*y*z voxels."""
    if type_name not in RAW_TYPES:
        raise ValueError(f"unknown voxel type {type_name!r} (uint8, uint16 or float)")
    nx, ny, nz = (int(d) for d in dims)
    if min(nx, ny, nz) <= 0:
        raise ValueError("volume dimensions must be positive")
    dt = RAW_TYPES[type_name]
    import os
    need = nx * ny * nz * dt.itemsize
    have = os.path.getsize(path)
    if have < need:
        raise ValueError(f"{path}: {have} bytes, dims {nx}x{ny}x{nz} of {type_name} need {need}")
    return np.memmap(path, dtype=dt, mode="r", shape=(nz, ny, nx))


def chop_raw(raw_path: str, dims, type_name: str, n: int, out_path: str) -> list[dict]:
    """chopSuey's volume path: split the raw volume into `n` bricks (at least
    two, as the tool gives) and write them as a .vol file, each brick
    normalised like Volume::get with its value range.  Returns the bricks."""
    raw = read_raw(raw_path, dims, type_name)
    descs = chopsuey_split(dims, n)
    dims = [int(d) for d in dims]
    with open(out_path, "wb") as f:
        f.write(HEADER.pack(len(descs), 0, 0, 0, *dims, 0, 0, 0, *[d + 1 for d in dims],
                            0.0, 0.0, 0.0, *[float(d) for d in dims]))
        for d in descs:
            v = np.ascontiguousarray(normalize_raw(brick_voxels(raw, d)), dtype="<f4")
            d["value_range"] = [float(v.min()), float(v.max())]
            f.write(BRICK.pack(*d["cell_lo"], *d["cell_hi"], *d["voxel_lo"], *d["voxel_hi"],
                               *d["space_lo"], *d["space_hi"], *d["value_range"]))
            f.write(v.tobytes())
    return descs
