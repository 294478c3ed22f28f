"""ctypes binding of the CPU oracle (``liboracle.so``).

TEST INFRASTRUCTURE ONLY.  The oracle is what results are compared against: ``tests/``,
``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline arm may load it;
the product package ``aloha_gb300`` never imports it.

The oracle restates the reference's volume path (``deviceCode.cpp``,
``waikikiRenderer.cpp``, ``chopSuey.cpp``); see ``aloha_oracle.hpp`` for the
per-function citations and the fixed fp32 evaluation order.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "liboracle.so")
_LOCK = threading.Lock()
_LIB = None

JITTER_NONE, JITTER_CONST, JITTER_HASH = 0, 1, 2
COMPOSITE_FP32, COMPOSITE_UBYTE = 0, 1
ORDER_FACES, ORDER_REFERENCE_KD = 0, 1

c_int_p = ctypes.POINTER(ctypes.c_int)
c_float_p = ctypes.POINTER(ctypes.c_float)
c_double_p = ctypes.POINTER(ctypes.c_double)
c_u32_p = ctypes.POINTER(ctypes.c_uint32)
c_u64_p = ctypes.POINTER(ctypes.c_uint64)


class BrickDesc(ctypes.Structure):
    _fields_ = [("cell_lo", ctypes.c_int32 * 3), ("cell_hi", ctypes.c_int32 * 3),
                ("voxel_lo", ctypes.c_int32 * 3), ("voxel_hi", ctypes.c_int32 * 3),
                ("space_lo", ctypes.c_float * 3), ("space_hi", ctypes.c_float * 3),
                ("value_lo", ctypes.c_float), ("value_hi", ctypes.c_float)]


class Camera(ctypes.Structure):
    _fields_ = [("org", ctypes.c_float * 3), ("dir_00", ctypes.c_float * 3),
                ("dir_du", ctypes.c_float * 3), ("dir_dv", ctypes.c_float * 3)]


class Params(ctypes.Structure):
    _fields_ = [("dt", ctypes.c_float), ("et_alpha", ctypes.c_float),
                ("jitter_mode", ctypes.c_int32), ("jitter_value", ctypes.c_float),
                ("crosshair", ctypes.c_int32), ("spp", ctypes.c_int32),
                ("accum_id", ctypes.c_int32), ("accumulate", ctypes.c_int32),
                ("heat_map", ctypes.c_int32), ("heat_map_scale", ctypes.c_float),
                ("composite_mode", ctypes.c_int32), ("island_id", ctypes.c_int32),
                ("num_islands", ctypes.c_int32)]


class Scene(ctypes.Structure):
    _fields_ = [("descs", ctypes.POINTER(BrickDesc)), ("voxels", ctypes.POINTER(c_float_p)),
                ("n_bricks", ctypes.c_int), ("tf", c_float_p), ("n_tf", ctypes.c_int)]


class Schedule(ctypes.Structure):
    _fields_ = [("n_ranks", ctypes.c_int), ("rank_order", c_int_p),
                ("rank_start", c_int_p), ("rank_bricks", c_int_p)]


class Outputs32(ctypes.Structure):
    _fields_ = [("fb", c_u32_p), ("final_rgba", c_float_p), ("rank_images", c_float_p),
                ("rank_depth", c_float_p), ("accum", c_float_p), ("pixel_samples", c_u32_p),
                ("samples", c_u64_p)]


class Outputs64(ctypes.Structure):
    _fields_ = [("fb", c_u32_p), ("final_rgba", c_double_p), ("rank_images", c_double_p),
                ("rank_depth", c_float_p), ("accum", c_double_p), ("pixel_samples", c_u32_p),
                ("samples", c_u64_p)]


def build(force: bool = False) -> str:
    """Compile liboracle.so from the C++ restatement with the committed Makefile."""
    src = [os.path.join(_HERE, f) for f in ("aloha_oracle.cpp", "aloha_oracle.hpp", "Makefile")]
    if force or not os.path.exists(_LIB_PATH) or \
            os.path.getmtime(_LIB_PATH) < max(os.path.getmtime(s) for s in src):
        subprocess.run(["make", "-s", "-B", "-C", _HERE, "liboracle.so"], check=True)
    return _LIB_PATH


def lib():
    global _LIB
    with _LOCK:
        if _LIB is None:
            build()
            L = ctypes.CDLL(_LIB_PATH)
            L.ora_render_f32.argtypes = [ctypes.POINTER(Scene), ctypes.POINTER(Schedule), ctypes.POINTER(Camera),
                                         ctypes.c_int, ctypes.c_int, ctypes.POINTER(Params), ctypes.c_float,
                                         ctypes.POINTER(Outputs32), ctypes.c_int, ctypes.c_int, ctypes.c_int]
            L.ora_render_f64.argtypes = [ctypes.POINTER(Scene), ctypes.POINTER(Schedule), ctypes.POINTER(Camera),
                                         ctypes.c_int, ctypes.c_int, ctypes.POINTER(Params), ctypes.c_float,
                                         ctypes.POINTER(Outputs64), ctypes.c_int, ctypes.c_int, ctypes.c_int]
            L.ora_chopsuey_split.argtypes = [c_int_p, ctypes.c_int, ctypes.POINTER(BrickDesc), ctypes.c_int]
            L.ora_partition_kd.argtypes = [c_float_p, ctypes.c_int, ctypes.c_int, c_int_p, c_int_p, ctypes.c_int]
            L.ora_composite_order_kd.argtypes = [c_int_p, ctypes.c_int, c_float_p, c_int_p, ctypes.c_int]
            L.ora_visibility_order.argtypes = [c_float_p, c_int_p, ctypes.c_int, ctypes.c_int, c_float_p, c_int_p]
            L.ora_max_depth.argtypes = [c_float_p, c_float_p, c_float_p]
            L.ora_max_depth.restype = ctypes.c_float
            L.ora_jitter_hash.argtypes = [ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32]
            L.ora_jitter_hash.restype = ctypes.c_float
            L.ora_first_sample_t.argtypes = [ctypes.c_float, ctypes.c_float, ctypes.c_float]
            L.ora_first_sample_t.restype = ctypes.c_float
            L.ora_tf_lookup.argtypes = [c_float_p, ctypes.c_int, ctypes.c_float, c_float_p]
            L.ora_stencil.argtypes = [c_float_p, c_int_p, c_float_p, c_float_p]
            _LIB = L
    return _LIB


def _ptr(a: np.ndarray, ctype):
    return a.ctypes.data_as(ctypes.POINTER(ctype))


# ----------------------------------------------------------------- layout

def chopsuey_split(dims, n: int) -> list[dict]:
    """Brick descriptors of chopSuey's VolumeSplitter for a volume of `dims` (x,y,z)."""
    d = np.asarray(dims, dtype=np.int32)
    out = (BrickDesc * 4096)()
    k = lib().ora_chopsuey_split(_ptr(d, ctypes.c_int), int(n), out, 4096)
    if k < 0:
        raise ValueError("chopSuey split failed")
    return [desc_to_dict(out[i]) for i in range(k)]


def desc_to_dict(d: BrickDesc) -> dict:
    return {"cell_lo": list(d.cell_lo), "cell_hi": list(d.cell_hi),
            "voxel_lo": list(d.voxel_lo), "voxel_hi": list(d.voxel_hi),
            "space_lo": list(d.space_lo), "space_hi": list(d.space_hi),
            "value_range": [d.value_lo, d.value_hi]}


def dict_to_desc(d: dict) -> BrickDesc:
    b = BrickDesc()
    for k in ("cell_lo", "cell_hi", "voxel_lo", "voxel_hi", "space_lo", "space_hi"):
        getattr(b, k)[:] = list(d[k])
    vr = d.get("value_range", (0.0, 0.0))
    b.value_lo, b.value_hi = float(vr[0]), float(vr[1])
    return b


def space_boxes(descs) -> np.ndarray:
    return np.array([list(d["space_lo"]) + list(d["space_hi"]) for d in descs], dtype=np.float32)


# --------------------------------------------------------------- ordering

def partition_kd(descs, n_ranks: int):
    """partitionKD over the bricks' space ranges -> (brick_rank, kd nodes)."""
    boxes = space_boxes(descs)
    n = len(descs)
    cr = np.zeros(n, dtype=np.int32)
    kd = np.zeros((4 * n + 8, 4), dtype=np.int32)
    k = lib().ora_partition_kd(_ptr(boxes, ctypes.c_float), n, int(n_ranks), _ptr(cr, ctypes.c_int),
                               _ptr(kd, ctypes.c_int), kd.shape[0])
    if k < 0:
        raise ValueError("partitionKD failed")
    return cr, kd[:k].copy()


def composite_over(images: np.ndarray, order, mode: int = COMPOSITE_FP32) -> np.ndarray:
    """The ordered composite (IceT stand-in) of float rank images [n][H][W][4]
    front to back in `order`: RGBA8 frame [H][W]."""
    images = np.ascontiguousarray(images, dtype=np.float32)
    n, H, W = images.shape[:3]
    o = np.ascontiguousarray(order, dtype=np.int32)
    fb = np.zeros((H, W), np.uint32)
    L = lib()
    L.ora_composite_over.argtypes = [c_float_p, c_int_p, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                     ctypes.POINTER(ctypes.c_uint32)]
    L.ora_composite_over(_ptr(images, ctypes.c_float), _ptr(o, ctypes.c_int), o.size, H * W, int(mode),
                         _ptr(fb, ctypes.c_uint32))
    return fb


def composite_over_rgba8(images: np.ndarray, order) -> np.ndarray:
    """The same for RGBA8 rank images [n][H][W] (packed uint32)."""
    images = np.ascontiguousarray(images, dtype=np.uint32)
    n, H, W = images.shape
    o = np.ascontiguousarray(order, dtype=np.int32)
    fb = np.zeros((H, W), np.uint32)
    L = lib()
    L.ora_composite_over_rgba8.argtypes = [ctypes.POINTER(ctypes.c_uint32), c_int_p, ctypes.c_int, ctypes.c_int,
                                           ctypes.POINTER(ctypes.c_uint32)]
    L.ora_composite_over_rgba8(_ptr(images, ctypes.c_uint32), _ptr(o, ctypes.c_int), o.size, H * W,
                               _ptr(fb, ctypes.c_uint32))
    return fb


def composite_order_kd(kd: np.ndarray, ref, n_ranks: int) -> list[int]:
    r = np.asarray(ref, dtype=np.float32)
    kd = np.ascontiguousarray(kd, dtype=np.int32)
    o = np.zeros(max(n_ranks, 1) + len(kd), dtype=np.int32)
    k = lib().ora_composite_order_kd(_ptr(kd, ctypes.c_int), kd.shape[0], _ptr(r, ctypes.c_float),
                                     _ptr(o, ctypes.c_int), o.shape[0])
    return [int(v) for v in o[:k]]


def visibility_order(boxes: np.ndarray, item_of_box, n_items: int, cam) -> list[int]:
    boxes = np.ascontiguousarray(boxes, dtype=np.float32)
    iob = np.ascontiguousarray(item_of_box, dtype=np.int32)
    c = np.asarray(cam, dtype=np.float32)
    o = np.zeros(max(n_items, 1), dtype=np.int32)
    k = lib().ora_visibility_order(_ptr(boxes, ctypes.c_float), _ptr(iob, ctypes.c_int), boxes.shape[0],
                                   int(n_items), _ptr(c, ctypes.c_float), _ptr(o, ctypes.c_int))
    return [int(v) for v in o[:k]]


def schedule(descs, n_ranks: int, cam_org, order_mode: int = ORDER_FACES, brick_rank=None):
    """Virtual-rank schedule for one camera: (rank_order, rank_start, rank_bricks, brick_rank)."""
    n = len(descs)
    kd = None
    if brick_rank is None:
        brick_rank, kd = partition_kd(descs, n_ranks)
    brick_rank = np.asarray(brick_rank, dtype=np.int32)
    boxes = space_boxes(descs)
    if order_mode == ORDER_REFERENCE_KD:
        if kd is None:
            raise ValueError("reference KD order needs partitionKD's tree")
        rank_order = composite_order_kd(kd, cam_org, n_ranks)
    else:
        rank_order = visibility_order(boxes, brick_rank, n_ranks, cam_org)
    brick_order = visibility_order(boxes, np.arange(n), n, cam_org)
    rank_start = [0]
    rank_bricks = []
    for r in range(n_ranks):
        rank_bricks += [b for b in brick_order if brick_rank[b] == r]
        rank_start.append(len(rank_bricks))
    return (np.asarray(rank_order, np.int32), np.asarray(rank_start, np.int32),
            np.asarray(rank_bricks, np.int32), brick_rank)


def max_depth(descs, org) -> float:
    boxes = space_boxes(descs)
    lo = boxes[:, :3].min(axis=0).astype(np.float32)
    hi = boxes[:, 3:].max(axis=0).astype(np.float32)
    o = np.asarray(org, dtype=np.float32)
    return float(lib().ora_max_depth(_ptr(lo, ctypes.c_float), _ptr(hi, ctypes.c_float), _ptr(o, ctypes.c_float)))


# ----------------------------------------------------------------- render

def make_params(**kw) -> Params:
    p = Params()
    defaults = dict(dt=0.5, et_alpha=0.99, jitter_mode=JITTER_HASH, jitter_value=0.0, crosshair=0, spp=1,
                    accum_id=0, accumulate=0, heat_map=0, heat_map_scale=1e-5, composite_mode=COMPOSITE_FP32,
                    island_id=0, num_islands=1)
    defaults.update(kw)
    for k, v in defaults.items():
        setattr(p, k, v)
    return p


def make_camera(org, dir_00, dir_du, dir_dv) -> Camera:
    c = Camera()
    c.org[:] = [float(v) for v in org]
    c.dir_00[:] = [float(v) for v in dir_00]
    c.dir_du[:] = [float(v) for v in dir_du]
    c.dir_dv[:] = [float(v) for v in dir_dv]
    return c


def render(descs, voxels, tf: np.ndarray, camera, W: int, H: int, params: Params | None = None, *,
           n_ranks: int = 1, order_mode: int = ORDER_FACES, brick_rank=None, precision: str = "f32",
           want=("fb",), accum: np.ndarray | None = None, rows=None, threads: int = 0, sched=None) -> dict:
    """Render one view on the CPU.

    descs: brick descriptors (dicts); voxels: one float32 array per brick, shape
    (nz, ny, nx) of its voxel range; tf: (n, 4) float32 RGBA table; camera:
    oracle Camera (org, dir_00, dir_du, dir_dv).
    """
    params = params or make_params()
    dt = np.float64 if precision == "f64" else np.float32
    ctype = ctypes.c_double if precision == "f64" else ctypes.c_float
    nb = len(descs)
    if sched is None:
        sched = schedule(descs, n_ranks, list(camera.org), order_mode, brick_rank)
    rank_order, rank_start, rank_bricks, _ = sched
    n_ranks = len(rank_start) - 1
    desc_arr = (BrickDesc * nb)(*[dict_to_desc(d) for d in descs])
    vox = [np.ascontiguousarray(v, dtype=np.float32) for v in voxels]
    for d, v in zip(descs, vox):
        n = [d["voxel_hi"][a] - d["voxel_lo"][a] for a in range(3)]
        if v.size != n[0] * n[1] * n[2]:
            raise ValueError("voxel array does not match the brick's voxel range")
    vptr = (c_float_p * nb)(*[_ptr(v, ctypes.c_float) for v in vox])
    tf = np.ascontiguousarray(tf, dtype=np.float32)
    sc = Scene(desc_arr, vptr, nb, _ptr(tf, ctypes.c_float), tf.shape[0])
    sch = Schedule(n_ranks, _ptr(rank_order, ctypes.c_int), _ptr(rank_start, ctypes.c_int),
                   _ptr(rank_bricks, ctypes.c_int) if rank_bricks.size else c_int_p())
    md = max_depth(descs, list(camera.org))
    res = {}
    npx = W * H
    fb = np.zeros(npx, dtype=np.uint32) if "fb" in want else None
    final = np.zeros((npx, 4), dtype=dt) if "final" in want else None
    rimg = np.zeros((n_ranks, npx, 4), dtype=dt) if "rank_images" in want else None
    rdepth = np.zeros((n_ranks, npx), dtype=np.float32) if "rank_depth" in want else None
    psamp = np.zeros(npx, dtype=np.uint32) if "pixel_samples" in want else None
    if accum is not None:
        if accum.dtype != dt or accum.shape != (n_ranks, npx, 4):
            raise ValueError("accum buffer must be (n_ranks, W*H, 4) of the render precision")
    samples = np.zeros(1, dtype=np.uint64)
    O = Outputs64 if precision == "f64" else Outputs32

    def P(a, ct):
        return _ptr(a, ct) if a is not None else ctypes.POINTER(ct)()

    out = O(P(fb, ctypes.c_uint32), P(final, ctype), P(rimg, ctype), P(rdepth, ctypes.c_float),
            P(accum, ctype), P(psamp, ctypes.c_uint32), _ptr(samples, ctypes.c_uint64))
    r0, r1 = (0, H) if rows is None else rows
    fn = lib().ora_render_f64 if precision == "f64" else lib().ora_render_f32
    rc = fn(ctypes.byref(sc), ctypes.byref(sch), ctypes.byref(camera), W, H, ctypes.byref(params), md,
            ctypes.byref(out), r0, r1, threads)
    if rc != 0:
        raise RuntimeError(f"oracle render failed ({rc})")
    res["samples"] = int(samples[0])
    res["rank_order"] = rank_order
    res["max_depth"] = md
    if fb is not None:
        res["fb"] = fb.reshape(H, W)
    if final is not None:
        res["final"] = final.reshape(H, W, 4)
    if rimg is not None:
        res["rank_images"] = rimg.reshape(n_ranks, H, W, 4)
    if rdepth is not None:
        res["rank_depth"] = rdepth.reshape(n_ranks, H, W)
    if psamp is not None:
        res["pixel_samples"] = psamp.reshape(H, W)
    return res


def adjoint(descs, voxels, tf: np.ndarray, camera, W: int, H: int, dl_drgba: np.ndarray,
            grid_lo, grid_dims, params: Params | None = None, threads: int = 0, sched=None) -> dict:
    """FP64 adjoint of the single-rank render: dL/dtf (n,4) and dL/ddensity on
    the grid (dims z,y,x) for dL/dRGBA (H,W,4) of the frame before quantisation."""
    params = params or make_params()
    L = lib()
    if not getattr(L, "_adj_ready", False):
        L.ora_adjoint_f64.argtypes = [ctypes.POINTER(Scene), ctypes.POINTER(Schedule), ctypes.POINTER(Camera),
                                      ctypes.c_int, ctypes.c_int, ctypes.POINTER(Params), c_double_p, c_double_p,
                                      c_double_p, c_int_p, c_int_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, c_u64_p]
        L._adj_ready = True
    nb = len(descs)
    if sched is None:
        sched = schedule(descs, 1, list(camera.org))
    rank_order, rank_start, rank_bricks, _ = sched
    desc_arr = (BrickDesc * nb)(*[dict_to_desc(d) for d in descs])
    vox = [np.ascontiguousarray(v, dtype=np.float32) for v in voxels]
    vptr = (c_float_p * nb)(*[_ptr(v, ctypes.c_float) for v in vox])
    tf = np.ascontiguousarray(tf, dtype=np.float32)
    sc = Scene(desc_arr, vptr, nb, _ptr(tf, ctypes.c_float), tf.shape[0])
    sch = Schedule(1, _ptr(rank_order, ctypes.c_int), _ptr(rank_start, ctypes.c_int), _ptr(rank_bricks, ctypes.c_int))
    dl = np.ascontiguousarray(dl_drgba, dtype=np.float64).reshape(H, W, 4)
    dtf = np.zeros((tf.shape[0], 4), np.float64)
    gd = [int(v) for v in grid_dims]
    dgrid = np.zeros((gd[2], gd[1], gd[0]), np.float64)
    glo = np.asarray(grid_lo, dtype=np.int32)
    gdim = np.asarray(gd, dtype=np.int32)
    samples = np.zeros(1, np.uint64)
    rc = L.ora_adjoint_f64(ctypes.byref(sc), ctypes.byref(sch), ctypes.byref(camera), W, H, ctypes.byref(params),
                           _ptr(dl, ctypes.c_double), _ptr(dtf, ctypes.c_double), _ptr(dgrid, ctypes.c_double),
                           _ptr(glo, ctypes.c_int), _ptr(gdim, ctypes.c_int), 0, H, threads,
                           _ptr(samples, ctypes.c_uint64))
    if rc != 0:
        raise RuntimeError("oracle adjoint failed (single rank and spp 1 only)")
    return {"dtf": dtf, "ddensity": dgrid, "samples": int(samples[0])}


def jitter_hash(pixel: int, accum_id: int, draw: int) -> float:
    return float(lib().ora_jitter_hash(pixel, accum_id, draw))


def first_sample_t(lower: float, dt: float, ils: float) -> float:
    return float(lib().ora_first_sample_t(lower, dt, ils))


def tf_lookup(tf: np.ndarray, v: float) -> np.ndarray:
    tf = np.ascontiguousarray(tf, dtype=np.float32)
    out = np.zeros(4, dtype=np.float32)
    lib().ora_tf_lookup(_ptr(tf, ctypes.c_float), tf.shape[0], v, _ptr(out, ctypes.c_float))
    return out


def stencil(voxels: np.ndarray, u) -> np.ndarray:
    """(value, gx, gy, gz) of the seven-tap stencil at voxel coordinate u of a (nz,ny,nx) brick."""
    v = np.ascontiguousarray(voxels, dtype=np.float32)
    n = np.array([v.shape[2], v.shape[1], v.shape[0]], dtype=np.int32)
    uu = np.asarray(u, dtype=np.float32)
    out = np.zeros(4, dtype=np.float32)
    lib().ora_stencil(_ptr(v, ctypes.c_float), _ptr(n, ctypes.c_int), _ptr(uu, ctypes.c_float),
                      _ptr(out, ctypes.c_float))
    return out
