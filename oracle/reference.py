"""ctypes binding of the reference's own volume code, built on the CPU.

TEST INFRASTRUCTURE ONLY.  ``make -C oracle ref`` compiles, from the reference
sources where they lie (``ALOHA_REFERENCE_DIR``, default the reference
checkout): ``deviceCode.cpp`` unchanged against ``oracle/ref_shim/`` plus the
Partitioner of ``waikikiRenderer.cpp`` into ``oracle/_ref/libaloha_reference.so``
(driven by ``oracle/ref_harness.cpp``), and the whole ``chopSuey`` tool into
``oracle/_ref/chopSuey``.  Only tests (and the fixture script under
``tests/golden/``) use this module, to pin the restatement in
``aloha_oracle.hpp`` to the reference; where the reference sources are absent
``available()`` is False and those tests skip.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import threading

import numpy as np

from . import oracle as O

_HERE = os.path.dirname(os.path.abspath(__file__))
_REF_DIR = os.environ.get("ALOHA_REFERENCE_DIR", "/root/reference")
_LIB_PATH = os.path.join(_HERE, "_ref", "libaloha_reference.so")
CHOPSUEY = os.path.join(_HERE, "_ref", "chopSuey")
_LOCK = threading.Lock()
_LIB = None
_BUILT = False


def available() -> bool:
    """True when the reference sources this binding compiles are present."""
    return all(os.path.exists(os.path.join(_REF_DIR, f))
               for f in ("deviceCode.cpp", "deviceCode.h", "waikikiRenderer.cpp", "chopSuey.cpp", "FileMapping.cpp"))


def build() -> None:
    global _BUILT
    if _BUILT:
        return
    if not available():
        if os.path.exists(_LIB_PATH):  # built earlier on this machine
            _BUILT = True
            return
        raise RuntimeError("reference sources not found")
    subprocess.run(["make", "-s", "-C", _HERE, "ref", f"REF={_REF_DIR}"], check=True)
    _BUILT = True


def lib():
    global _LIB
    with _LOCK:
        if _LIB is None:
            build()
            L = ctypes.CDLL(_LIB_PATH)
            fp = ctypes.POINTER(ctypes.c_float)
            ip = ctypes.POINTER(ctypes.c_int)
            up = ctypes.POINTER(ctypes.c_uint32)
            L.ref_render_rank.argtypes = [ctypes.POINTER(O.BrickDesc), ctypes.POINTER(fp), ctypes.c_int, ip,
                                          ctypes.c_int, fp, ctypes.c_int, fp, ctypes.c_int, ctypes.c_int,
                                          ctypes.c_float, ctypes.c_float, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                          ctypes.c_float, fp, up, fp, up, ctypes.c_int]
            L.ref_render_rank_rows.argtypes = L.ref_render_rank.argtypes[:-1] + [ctypes.c_int, ctypes.c_int,
                                                                                  ctypes.c_int]
            L.ref_partition.argtypes = [fp, ctypes.c_int, ctypes.c_int, fp, ctypes.c_int, ip, ip]
            _LIB = L
    return _LIB


def _p(a: np.ndarray, ct):
    return a.ctypes.data_as(ctypes.POINTER(ct))


def partition(descs, n_ranks: int, points=()):
    """The reference's partitionKD (brick -> rank) and computeCompositeOrder
    for each reference point: (brick_rank, [order per point])."""
    boxes = O.space_boxes(descs)
    n = len(descs)
    pts = np.ascontiguousarray(np.asarray(points, dtype=np.float32).reshape(-1, 3))
    br = np.full(n, -1, dtype=np.int32)
    orders = np.zeros((max(len(pts), 1), n_ranks), dtype=np.int32)
    k = lib().ref_partition(_p(boxes, ctypes.c_float), n, int(n_ranks), _p(pts, ctypes.c_float), len(pts),
                            _p(br, ctypes.c_int), _p(orders, ctypes.c_int))
    if k < 0:
        raise RuntimeError("reference partition failed")
    return br, [list(map(int, orders[i, :k])) for i in range(len(pts))]


def render_ranks(descs, voxels, tf, camera, W: int, H: int, *, dt: float = 0.5, spp: int = 1, accum_id: int = 0,
                 jitter_mode: int = O.JITTER_HASH, jitter_value: float = 0.0, n_ranks: int = 1, brick_rank=None,
                 accum=None, threads: int = 0, rows=None) -> dict:
    """Every rank's frame through the reference raygen (renderFrame with its
    crosshair, accumulation and make_rgba), one rank at a time as each MPI
    rank would.  Bricks go to ranks by the reference's partitionKD unless
    `brick_rank` is given; a rank's bricks are its brick buffer in id order
    (the .vol load order) and are tested front to back during traversal.
    Returns fb [R,H,W] uint32, depth [R,H,W], samples [R,H,W], accum
    [R,H*W,4] (pass it back with accum_id + 1 for progressive frames).
    `rows` = (y0, y1) renders only those rows (the rest stay zero)."""
    cam = np.array(list(camera.org) + list(camera.dir_00) + list(camera.dir_du) + list(camera.dir_dv),
                   dtype=np.float32)
    if brick_rank is None:
        brick_rank, _ = partition(descs, n_ranks)
    brick_rank = np.asarray(brick_rank, dtype=np.int32)
    # front-to-back brick order of the whole volume, for the traversal test order
    boxes = O.space_boxes(descs)
    order = O.visibility_order(boxes, np.arange(len(descs)), len(descs), list(camera.org))
    md = O.max_depth(descs, list(camera.org))
    tf = np.ascontiguousarray(tf, dtype=np.float32)
    npx = W * H
    out = {"fb": np.zeros((n_ranks, H, W), np.uint32), "depth": np.zeros((n_ranks, H, W), np.float32),
           "samples": np.zeros((n_ranks, H, W), np.uint32)}
    acc = np.zeros((n_ranks, npx, 4), np.float32) if accum is None else np.ascontiguousarray(accum, np.float32)
    for r in range(n_ranks):
        mine = [b for b in range(len(descs)) if brick_rank[b] == r]
        local = {b: i for i, b in enumerate(mine)}
        test = np.array([local[b] for b in order if b in local], dtype=np.int32)
        arr = (O.BrickDesc * max(len(mine), 1))(*[O.dict_to_desc(descs[b]) for b in mine])
        vox = [np.ascontiguousarray(voxels[b], dtype=np.float32) for b in mine]
        vptr = (ctypes.POINTER(ctypes.c_float) * max(len(mine), 1))(*[_p(v, ctypes.c_float) for v in vox])
        fb = np.zeros(npx, np.uint32)
        depth = np.zeros(npx, np.float32)
        smp = np.zeros(npx, np.uint32)
        a = np.ascontiguousarray(acc[r])
        y0, y1 = (0, H) if rows is None else (int(rows[0]), int(rows[1]))
        rc = lib().ref_render_rank_rows(arr, vptr, len(mine), _p(test, ctypes.c_int), len(test),
                                        _p(tf, ctypes.c_float), tf.shape[0], _p(cam, ctypes.c_float), W, H, dt, md,
                                        spp, accum_id, jitter_mode, jitter_value, _p(a, ctypes.c_float),
                                        _p(fb, ctypes.c_uint32), _p(depth, ctypes.c_float), _p(smp, ctypes.c_uint32),
                                        y0, y1, threads)
        if rc != 0:
            raise RuntimeError(f"reference render failed ({rc})")
        acc[r] = a
        out["fb"][r] = fb.reshape(H, W)
        out["depth"][r] = depth.reshape(H, W)
        out["samples"][r] = smp.reshape(H, W)
    out["accum"] = acc
    out["brick_rank"] = brick_rank
    return out


class BandRenderer:
    """Row bands of frames of one scene through the reference raygen, one rank
    after another as each MPI rank would, then the ordered RGBA8 blend of the
    rank images (the IceT step) in the order of the reference's
    computeCompositeOrder.  The per-rank buffers are allocated once, so that
    repeated calls time the raygen and the blend (the timed CPU arm of the
    benchmark)."""

    def __init__(self, descs, voxels, tf, W: int, H: int, n_ranks: int, *, dt: float = 0.5,
                 jitter_mode: int = O.JITTER_HASH, threads: int = 0):
        self.descs, self.W, self.H, self.n_ranks = descs, int(W), int(H), int(n_ranks)
        self.dt, self.jitter_mode, self.threads = float(dt), int(jitter_mode), int(threads)
        self.tf = np.ascontiguousarray(tf, dtype=np.float32)
        self.brick_rank, _ = partition(descs, n_ranks)
        self.boxes = O.space_boxes(descs)
        npx = self.W * self.H
        self.ranks = []
        for r in range(self.n_ranks):
            mine = [b for b in range(len(descs)) if self.brick_rank[b] == r]
            vox = [np.ascontiguousarray(voxels[b], dtype=np.float32) for b in mine]
            self.ranks.append({
                "mine": mine, "local": {b: i for i, b in enumerate(mine)}, "vox": vox,
                "arr": (O.BrickDesc * max(len(mine), 1))(*[O.dict_to_desc(descs[b]) for b in mine]),
                "vptr": (ctypes.POINTER(ctypes.c_float) * max(len(mine), 1))(*[_p(v, ctypes.c_float) for v in vox]),
                "fb": np.zeros(npx, np.uint32), "depth": np.zeros(npx, np.float32),
                "samples": np.zeros(npx, np.uint32), "accum": np.zeros((npx, 4), np.float32)})

    def render(self, camera, rows) -> tuple[np.ndarray, int]:
        """Rows [y0, y1) of the composited RGBA8 frame and the samples taken."""
        y0, y1 = int(rows[0]), int(rows[1])
        org = list(camera.org)
        cam = np.array(org + list(camera.dir_00) + list(camera.dir_du) + list(camera.dir_dv), dtype=np.float32)
        order = O.visibility_order(self.boxes, np.arange(len(self.descs)), len(self.descs), org)
        md = O.max_depth(self.descs, org)
        samples = 0
        for rk in self.ranks:
            test = np.array([rk["local"][b] for b in order if b in rk["local"]], dtype=np.int32)
            rc = lib().ref_render_rank_rows(rk["arr"], rk["vptr"], len(rk["mine"]), _p(test, ctypes.c_int),
                                            len(test), _p(self.tf, ctypes.c_float), self.tf.shape[0],
                                            _p(cam, ctypes.c_float), self.W, self.H, self.dt, md, 1, 0,
                                            self.jitter_mode, 0.0, _p(rk["accum"], ctypes.c_float),
                                            _p(rk["fb"], ctypes.c_uint32), _p(rk["depth"], ctypes.c_float),
                                            _p(rk["samples"], ctypes.c_uint32), y0, y1, self.threads)
            if rc != 0:
                raise RuntimeError(f"reference render failed ({rc})")
            samples += int(rk["samples"][y0 * self.W:y1 * self.W].sum(dtype=np.uint64))
        _, orders = partition(self.descs, self.n_ranks, [org])
        acc = np.zeros(((y1 - y0) * self.W, 4), np.float32)
        for r in orders[0]:  # front to back, premultiplied "over" of the RGBA8 rank images
            q = self.ranks[r]["fb"][y0 * self.W:y1 * self.W]
            c = np.stack([(q >> (8 * k)) & 255 for k in range(4)], axis=1).astype(np.float32) / 255.0
            acc += (1.0 - acc[:, 3:4]) * c
        q8 = np.clip(np.rint(acc * 255.0), 0, 255).astype(np.uint32)
        fb = q8[:, 0] | (q8[:, 1] << 8) | (q8[:, 2] << 16) | (q8[:, 3] << 24)
        return fb.reshape(y1 - y0, self.W), samples


def loadable() -> bool:
    """True when the reference build can be used here: its sources are
    present (it is built on first use), or it is already built for this
    machine."""
    if available():
        return True
    if not os.path.exists(_LIB_PATH):
        return False
    try:
        ctypes.CDLL(_LIB_PATH)
    except OSError:
        return False
    return True


def chopsuey(raw_path: str, dims, type_name: str, n: int, out_path: str) -> None:
    """Runs the reference chopSuey tool: raw volume -> .vol with n bricks."""
    build()
    subprocess.run([CHOPSUEY, raw_path, "-dims", *[str(int(d)) for d in dims], "-type", type_name, "-n", str(int(n)),
                    "-o", out_path], check=True, stdout=subprocess.DEVNULL)
