"""ctypes binding of libaloha_gb300.so (the C ABI declared in include/aloha.h).

The library is required: every entry point raises if it was not built, there
is no CPU fallback.  Arrays may be numpy (host) or torch tensors (host or
CUDA); the library detects device pointers itself.
"""
from __future__ import annotations

import ctypes
import os
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libaloha_gb300.so")
_LOCK = threading.Lock()
_LIB = None

OK = 0
ERR_INVALID_ARGUMENT, ERR_NULL_POINTER, ERR_OUT_OF_RANGE, ERR_NOT_READY = 1, 2, 3, 4
ERR_OUT_OF_MEMORY, ERR_CUDA, ERR_TIMEOUT, ERR_MISSING_BRICK, ERR_UNSUPPORTED = 5, 6, 7, 8, 9
JITTER_NONE, JITTER_CONST, JITTER_HASH = 0, 1, 2
COMPOSITE_FP32, COMPOSITE_UBYTE = 0, 1
ORDER_FACES, ORDER_REFERENCE_KD = 0, 1
SPLIT_AUTO, SPLIT_PIXELS, SPLIT_RANKS = 0, 1, 2
CHUNKS_AUTO, CHUNKS_RING, CHUNKS_PROBED = 0, 1, 2
STAGING_NONE, STAGING_NEXT_SAMPLE = 0, 1

# Every exported symbol of include/aloha.h (checked by the CPU test suite).
EXPORTS = [
    "aloha_abi_version", "aloha_status_string", "aloha_create", "aloha_destroy", "aloha_last_error",
    "aloha_default_render_params", "aloha_set_render_params", "aloha_set_bricks", "aloha_update_brick",
    "aloha_drop_brick", "aloha_set_transfer_function", "aloha_set_ranks", "aloha_set_rank_assignment",
    "aloha_set_camera", "aloha_resize", "aloha_get_composite_order", "aloha_render", "aloha_render_partials",
    "aloha_composite_over", "aloha_composite_over_rgba8", "aloha_get_stats", "aloha_batch_create",
    "aloha_batch_set_config", "aloha_batch_get_config", "aloha_batch_launch", "aloha_batch_launch_graph",
    "aloha_batch_autotune", "aloha_batch_destroy", "aloha_render_batch", "aloha_forward", "aloha_backward",
    "aloha_composite_over_noalloc", "aloha_set_render_tile", "aloha_set_render_split", "aloha_set_chunk_order",
    "aloha_set_render_staging", "aloha_batch_set_staging", "aloha_batch_get_staging", "aloha_set_lane_groups",
    "aloha_backward_views", "aloha_forward_views", "aloha_batch_set_unroll", "aloha_batch_get_unroll",
]


class AlohaError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"[{code}] {msg}")
        self.code = code


class BrickDesc(ctypes.Structure):
    _fields_ = [("cell_lo", ctypes.c_int32 * 3), ("cell_hi", ctypes.c_int32 * 3),
                ("voxel_lo", ctypes.c_int32 * 3), ("voxel_hi", ctypes.c_int32 * 3),
                ("space_lo", ctypes.c_float * 3), ("space_hi", ctypes.c_float * 3),
                ("value_range", ctypes.c_float * 2)]


class RenderParams(ctypes.Structure):
    _fields_ = [("dt", ctypes.c_float), ("et_alpha", ctypes.c_float), ("jitter_mode", ctypes.c_int32),
                ("jitter_value", ctypes.c_float), ("crosshair", ctypes.c_int32), ("spp", ctypes.c_int32),
                ("accum_id", ctypes.c_int32), ("accumulate", ctypes.c_int32), ("heat_map", ctypes.c_int32),
                ("heat_map_scale", ctypes.c_float), ("composite_mode", ctypes.c_int32),
                ("island_id", ctypes.c_int32), ("num_islands", ctypes.c_int32), ("order_mode", ctypes.c_int32)]


class Stats(ctypes.Structure):
    _fields_ = [("samples", ctypes.c_uint64), ("n_bricks", ctypes.c_int32), ("n_ranks", ctypes.c_int32),
                ("brick_bytes", ctypes.c_uint64)]


P = ctypes.c_void_p
I = ctypes.c_int
F3 = ctypes.POINTER(ctypes.c_float)

_SIGS = {
    "aloha_abi_version": ([], I),
    "aloha_status_string": ([I], ctypes.c_char_p),
    "aloha_create": ([I, ctypes.POINTER(P)], I),
    "aloha_destroy": ([P], I),
    "aloha_last_error": ([P], ctypes.c_char_p),
    "aloha_default_render_params": ([ctypes.POINTER(RenderParams)], I),
    "aloha_set_render_params": ([P, ctypes.POINTER(RenderParams)], I),
    "aloha_set_bricks": ([P, ctypes.POINTER(BrickDesc), ctypes.POINTER(P), I], I),
    "aloha_update_brick": ([P, I, P], I),
    "aloha_drop_brick": ([P, I], I),
    "aloha_set_transfer_function": ([P, P, I], I),
    "aloha_set_ranks": ([P, I], I),
    "aloha_set_rank_assignment": ([P, P, I, I], I),
    "aloha_set_camera": ([P, I, F3, F3, F3, F3], I),
    "aloha_resize": ([P, I, I, I], I),
    "aloha_get_composite_order": ([P, I, P, I, ctypes.POINTER(I)], I),
    "aloha_render": ([P, I, P, P], I),
    "aloha_render_partials": ([P, I, P, P, P], I),
    "aloha_composite_over": ([P, P, I, I, I, I, P, P], I),
    "aloha_composite_over_rgba8": ([P, P, I, I, I, P, P], I),
    "aloha_get_stats": ([P, ctypes.POINTER(Stats)], I),
    "aloha_batch_create": ([P, P, I, ctypes.POINTER(P), ctypes.POINTER(P)], I),
    "aloha_batch_set_config": ([P, I, I, I], I),
    "aloha_batch_get_config": ([P, ctypes.POINTER(I), ctypes.POINTER(I), ctypes.POINTER(I)], I),
    "aloha_batch_launch": ([P, P], I),
    "aloha_batch_launch_graph": ([P, P], I),
    "aloha_batch_autotune": ([P, P, I, ctypes.POINTER(I), ctypes.POINTER(I), ctypes.POINTER(ctypes.c_float)], I),
    "aloha_batch_destroy": ([P], I),
    "aloha_render_batch": ([P, P, I, ctypes.POINTER(P), P], I),
    "aloha_forward": ([P, I, P, I, P], I),
    "aloha_backward": ([P, I, P, P, P, P, P, P], I),
    "aloha_backward_views": ([P, I, P, P, P, P, P, P, P], I),
    "aloha_forward_views": ([P, I, P, P, I, P], I),
    "aloha_batch_set_unroll": ([P, I], I),
    "aloha_batch_get_unroll": ([P, ctypes.POINTER(I)], I),
    "aloha_composite_over_noalloc": ([P, P, I, I, I, I, P, P], I),
    "aloha_set_render_tile": ([P, I, I], I),
    "aloha_set_render_split": ([P, I], I),
    "aloha_set_chunk_order": ([P, I], I),
    "aloha_set_render_staging": ([P, I], I),
    "aloha_set_lane_groups": ([P, I], I),
    "aloha_batch_set_staging": ([P, I], I),
    "aloha_batch_get_staging": ([P, ctypes.POINTER(I)], I),
}


def lib():
    """Load libaloha_gb300.so; raises if it has not been built."""
    global _LIB
    with _LOCK:
        if _LIB is None:
            if not os.path.exists(LIB_PATH):
                raise RuntimeError(f"{LIB_PATH} is missing: build it with "
                                   "`python -c 'import __graft_entry__ as g; g.build()'` (no CPU fallback exists)")
            L = ctypes.CDLL(LIB_PATH)
            for name, (args, res) in _SIGS.items():
                fn = getattr(L, name)
                fn.argtypes = args
                fn.restype = res
            _LIB = L
    return _LIB


def _addr(x) -> int:
    """Raw address of a numpy array or torch tensor (must stay alive)."""
    if x is None:
        return 0
    if isinstance(x, np.ndarray):
        if not x.flags["C_CONTIGUOUS"]:
            raise ValueError("array must be C-contiguous")
        return x.ctypes.data
    if hasattr(x, "data_ptr"):
        if not x.is_contiguous():
            raise ValueError("tensor must be contiguous")
        return x.data_ptr()
    raise TypeError(f"unsupported buffer type {type(x)}")


def _stream(stream) -> int:
    if stream is None:
        return 0
    if isinstance(stream, int):
        return stream
    return int(getattr(stream, "cuda_stream", 0))


_F3 = ctypes.c_float * 3


def _f3(v):
    try:
        return _F3(*v)  # Python floats and ints convert directly
    except TypeError:
        return _F3(*[float(t) for t in v])


def make_desc(d: dict) -> BrickDesc:
    b = BrickDesc()
    for k in ("cell_lo", "cell_hi", "voxel_lo", "voxel_hi", "space_lo", "space_hi"):
        getattr(b, k)[:] = list(d[k])
    b.value_range[:] = list(d.get("value_range", (0.0, 0.0)))
    return b


class Context:
    """One renderer on one GPU (the C ABI's aloha_ctx)."""

    def __init__(self, device: int = 0):
        self._lib = lib()
        h = P()
        rc = self._lib.aloha_create(device, ctypes.byref(h))
        if rc != OK:
            raise AlohaError(rc, f"aloha_create failed: {self._lib.aloha_status_string(rc).decode()}")
        self.h = h
        self._keep = {}

    def close(self):
        if getattr(self, "h", None):
            self._lib.aloha_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _check(self, rc: int):
        if rc != OK:
            msg = self._lib.aloha_last_error(self.h).decode()
            raise AlohaError(rc, f"{self._lib.aloha_status_string(rc).decode()}: {msg}")

    # ---- scene
    def set_bricks(self, descs, voxels):
        n = len(descs)
        arr = (BrickDesc * n)(*[make_desc(d) for d in descs])
        ptrs = (P * n)(*[_addr(v) for v in voxels])
        self._check(self._lib.aloha_set_bricks(self.h, arr, ptrs, n))
        self.n_bricks = n

    def update_brick(self, brick: int, voxels):
        self._check(self._lib.aloha_update_brick(self.h, brick, _addr(voxels)))

    def drop_brick(self, brick: int):
        self._check(self._lib.aloha_drop_brick(self.h, brick))

    def set_transfer_function(self, tf):
        n = int(tf.shape[0])
        self._check(self._lib.aloha_set_transfer_function(self.h, _addr(tf), n))

    def set_ranks(self, n_ranks: int):
        self._check(self._lib.aloha_set_ranks(self.h, int(n_ranks)))

    def set_rank_assignment(self, brick_rank, n_ranks: int):
        br = np.ascontiguousarray(brick_rank, dtype=np.int32)
        self._check(self._lib.aloha_set_rank_assignment(self.h, _addr(br), br.size, int(n_ranks)))

    def set_camera(self, view: int, org, dir_00, dir_du, dir_dv):
        self._check(self._lib.aloha_set_camera(self.h, view, _f3(org), _f3(dir_00), _f3(dir_du), _f3(dir_dv)))

    def resize(self, view: int, width: int, height: int):
        self._check(self._lib.aloha_resize(self.h, view, int(width), int(height)))

    def default_params(self) -> RenderParams:
        p = RenderParams()
        self._lib.aloha_default_render_params(ctypes.byref(p))
        return p

    def set_params(self, params: RenderParams | None = None, **kw):
        p = params or self.default_params()
        for k, v in kw.items():
            setattr(p, k, v)
        self._check(self._lib.aloha_set_render_params(self.h, ctypes.byref(p)))
        self.params = p

    def composite_order(self, view: int) -> list[int]:
        buf = np.zeros(65536, dtype=np.int32)
        n = I()
        self._check(self._lib.aloha_get_composite_order(self.h, view, _addr(buf), buf.size, ctypes.byref(n)))
        return [int(v) for v in buf[:n.value]]

    # ---- render
    def set_render_tile(self, tile_w: int, tile_h: int):
        self._check(self._lib.aloha_set_render_tile(self.h, int(tile_w), int(tile_h)))

    def set_chunk_order(self, mode: int):
        """CHUNKS_AUTO, CHUNKS_RING (centre-out) or CHUNKS_PROBED (most expensive
        first by a coarse probe); frames are bit-identical."""
        self._check(self._lib.aloha_set_chunk_order(self.h, int(mode)))

    def set_render_staging(self, mode: int):
        """STAGING_NONE or STAGING_NEXT_SAMPLE (the next sample's stencil rows
        copied into shared memory with cp.async); frames are bit-identical."""
        self._check(self._lib.aloha_set_render_staging(self.h, int(mode)))

    def set_lane_groups(self, permille: int):
        """Share (per mille) of a cost-ordered frame's costliest 8x4 chunks rendered
        with 4 lanes per ray; frames are bit-identical; 0 is off."""
        self._check(self._lib.aloha_set_lane_groups(self.h, int(permille)))

    def set_render_split(self, mode: int):
        """SPLIT_AUTO, SPLIT_PIXELS (one thread per pixel over all ranks) or
        SPLIT_RANKS ((chunk, rank) work items); frames are bit-identical."""
        self._check(self._lib.aloha_set_render_split(self.h, int(mode)))

    def render(self, view: int, fb=None, stream=None, width: int | None = None, height: int | None = None):
        """Render into `fb` (uint32 W*H, numpy or torch); allocates a numpy buffer if None."""
        if fb is None:
            if width is None or height is None:
                raise ValueError("pass fb or width/height")
            fb = np.zeros((height, width), dtype=np.uint32)
        self._check(self._lib.aloha_render(self.h, view, _addr(fb), _stream(stream)))
        return fb

    def render_partials(self, view: int, rank_images, rank_depth=None, stream=None):
        self._check(self._lib.aloha_render_partials(self.h, view, _addr(rank_images), _addr(rank_depth),
                                                    _stream(stream)))
        return rank_images

    def render_batch(self, views, fbs, stream=None):
        n = len(views)
        v = np.ascontiguousarray(views, dtype=np.int32)
        ptrs = (P * n)(*[_addr(f) for f in fbs])
        self._check(self._lib.aloha_render_batch(self.h, _addr(v), n, ptrs, _stream(stream)))

    def forward(self, view: int, rgba, checkpoint_every: int = 32, stream=None):
        """Differentiable render of `view` into float RGBA (H, W, 4); keeps checkpoints for backward()."""
        self._check(self._lib.aloha_forward(self.h, view, _addr(rgba), int(checkpoint_every), _stream(stream)))
        return rgba

    def forward_views(self, views, rgba, checkpoint_every: int = 32, stream=None):
        """forward() of several views in one launch: rgba[i] (H, W, 4) receives views[i]'s image."""
        n = len(views)
        if len(rgba) != n:
            raise ValueError("one image per view")
        v = np.ascontiguousarray(views, dtype=np.int32)
        ptrs = (P * n)(*[_addr(r) for r in rgba])
        self._check(self._lib.aloha_forward_views(self.h, n, _addr(v), ptrs, int(checkpoint_every), _stream(stream)))
        return rgba

    def backward(self, view: int, dl_drgba, dl_dtf, dl_ddensity, grid_lo, grid_dims, stream=None):
        """Accumulate dL/dtf and dL/ddensity (on the grid at grid_lo, dims x,y,z) for dL/dRGBA.
        dl_dtf may be None: density gradient only (the replay then skips empty space).
        dl_ddensity may be None: transfer-function gradient only (grid_lo, grid_dims ignored)."""
        lo = None if grid_lo is None else np.ascontiguousarray(grid_lo, dtype=np.int32)
        dims = None if grid_dims is None else np.ascontiguousarray(grid_dims, dtype=np.int32)
        self._check(self._lib.aloha_backward(self.h, view, _addr(dl_drgba), _addr(dl_dtf), _addr(dl_ddensity),
                                             _addr(lo), _addr(dims), _stream(stream)))

    def backward_views(self, views, dl_drgba, dl_dtf, dl_ddensity, grid_lo, grid_dims, stream=None):
        """backward() of several views, summed: dl_drgba[i] belongs to views[i].  One
        accumulation buffer and one fold for all of them."""
        n = len(views)
        if len(dl_drgba) != n:
            raise ValueError("one dL/dRGBA per view")
        v = np.ascontiguousarray(views, dtype=np.int32)
        ptrs = (P * n)(*[_addr(g) for g in dl_drgba])
        lo = None if grid_lo is None else np.ascontiguousarray(grid_lo, dtype=np.int32)
        dims = None if grid_dims is None else np.ascontiguousarray(grid_dims, dtype=np.int32)
        self._check(self._lib.aloha_backward_views(self.h, n, _addr(v), ptrs, _addr(dl_dtf), _addr(dl_ddensity),
                                                   _addr(lo), _addr(dims), _stream(stream)))

    def stats(self) -> Stats:
        s = Stats()
        self._check(self._lib.aloha_get_stats(self.h, ctypes.byref(s)))
        return s

    def batch(self, views, fbs) -> "Batch":
        return Batch(self, views, fbs)


class Batch:
    """A fixed list of (view, device frame buffer) items rendered by one persistent launch."""

    def __init__(self, ctx: Context, views, fbs):
        self.ctx = ctx
        self._views = np.ascontiguousarray(views, dtype=np.int32)
        self._fbs = list(fbs)
        n = len(self._fbs)
        ptrs = (P * n)(*[_addr(f) for f in self._fbs])
        h = P()
        ctx._check(ctx._lib.aloha_batch_create(ctx.h, _addr(self._views), n, ptrs, ctypes.byref(h)))
        self.h = h

    def set_config(self, tile_w: int, tile_h: int, ctas_per_sm: int = 0):
        self.ctx._check(self.ctx._lib.aloha_batch_set_config(self.h, tile_w, tile_h, ctas_per_sm))

    def config(self):
        w, h, c = I(), I(), I()
        self.ctx._check(self.ctx._lib.aloha_batch_get_config(self.h, ctypes.byref(w), ctypes.byref(h),
                                                             ctypes.byref(c)))
        return w.value, h.value, c.value

    def set_staging(self, stage: int):
        self.ctx._check(self.ctx._lib.aloha_batch_set_staging(self.h, int(stage)))

    def staging(self) -> int:
        s = I()
        self.ctx._check(self.ctx._lib.aloha_batch_get_staging(self.h, ctypes.byref(s)))
        return s.value

    def set_unroll(self, steps: int):
        """March steps per loop trip: 1 or 2 (direct loads only)."""
        self.ctx._check(self.ctx._lib.aloha_batch_set_unroll(self.h, int(steps)))

    def unroll(self) -> int:
        s = I()
        self.ctx._check(self.ctx._lib.aloha_batch_get_unroll(self.h, ctypes.byref(s)))
        return s.value

    def launch(self, stream=None):
        self.ctx._check(self.ctx._lib.aloha_batch_launch(self.h, _stream(stream)))

    def launch_graph(self, stream=None):
        self.ctx._check(self.ctx._lib.aloha_batch_launch_graph(self.h, _stream(stream)))

    def autotune(self, stream=None, reps: int = 2):
        w, h, ms = I(), I(), ctypes.c_float()
        self.ctx._check(self.ctx._lib.aloha_batch_autotune(self.h, _stream(stream), reps, ctypes.byref(w),
                                                           ctypes.byref(h), ctypes.byref(ms)))
        return w.value, h.value, ms.value

    def close(self):
        if getattr(self, "h", None):
            self.ctx._lib.aloha_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def composite_over(rank_images, order, width: int, height: int, mode: int = COMPOSITE_FP32, fb=None, stream=None):
    """IceT stand-in: ordered over of float rank images [n][H][W][4] -> RGBA8."""
    L = lib()
    o = np.ascontiguousarray(order, dtype=np.int32)
    if fb is None:
        fb = np.zeros((height, width), dtype=np.uint32)
    rc = L.aloha_composite_over(_addr(rank_images), _addr(o), o.size, width, height, mode, _addr(fb),
                                _stream(stream))
    if rc != OK:
        raise AlohaError(rc, L.aloha_status_string(rc).decode())
    return fb


def composite_over_rgba8(rank_fbs, order, width: int, height: int, fb=None, stream=None):
    L = lib()
    o = np.ascontiguousarray(order, dtype=np.int32)
    if fb is None:
        fb = np.zeros((height, width), dtype=np.uint32)
    rc = L.aloha_composite_over_rgba8(_addr(rank_fbs), _addr(o), o.size, width, height, _addr(fb), _stream(stream))
    if rc != OK:
        raise AlohaError(rc, L.aloha_status_string(rc).decode())
    return fb
