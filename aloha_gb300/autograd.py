"""torch.autograd binding of the differentiable march.

``render_views(renderer, tf, density, views)`` returns float RGBA images
(views, H, W, 4) that are differentiable with respect to the transfer-function
table ``tf`` (n, 4) and the density volume ``density`` (nz, ny, nx), both CUDA
float32 tensors.  The forward stores the march state every K samples; the
backward replays each K-sample segment from its checkpoint in parallel (see
csrc/adjoint.cu) and accumulates the gradients.  All views of one call go
through one training-forward launch (aloha_forward_views) and one summed
backward (aloha_backward_views).
"""
from __future__ import annotations

import weakref

import torch

from . import abi
from . import volfile


class DensityTracker:
    """Whether a density tensor still holds what was last uploaded: the same
    tensor object (held by a weak reference, so a new tensor that reuses a
    freed block at the same address never passes) at the same autograd
    version counter (bumped by every in-place update)."""

    def __init__(self):
        self._ref = None
        self._version = None

    def current(self, t: torch.Tensor) -> bool:
        ref = self._ref() if self._ref is not None else None
        return ref is t and t._version == self._version

    def record(self, t: torch.Tensor):
        self._ref = weakref.ref(t)
        self._version = t._version

    def invalidate(self):
        self._ref = None


class DifferentiableRenderer:
    """A context holding one volume split into bricks (one virtual rank)."""

    def __init__(self, dims, bricks: int | list = 1, checkpoint_every: int = 32, device: int = 0, **params):
        self.dims = [int(d) for d in dims]
        if isinstance(bricks, int):
            self.descs = volfile.grid_split(self.dims, ([], [], [])) if bricks == 1 else \
                volfile.chopsuey_split(self.dims, bricks)
        else:
            self.descs = list(bricks)
        self.k = int(checkpoint_every)
        self.ctx = abi.Context(device)
        self._uploaded = False
        self._params = params
        self._density = DensityTracker()
        self.brick_uploads = 0  # bricks copied to the context so far

    def invalidate(self):
        """Forget the uploaded density: the next render uploads it again.  Needed
        only after writes that bypass the tensor's version counter (through
        ``tensor.data`` or another tensor sharing its storage)."""
        self._density.invalidate()

    def _upload(self, tf: torch.Tensor, density: torch.Tensor):
        if not self._density.current(density):
            # the bricks (padding, macrocell tables) are rebuilt only when the
            # density may have changed: another tensor object, or an in-place
            # update of this one (which bumps its version counter)
            vox = [volfile.brick_voxels(density.detach(), d) for d in self.descs]
            if not self._uploaded:
                self.ctx.set_bricks(self.descs, vox)
                self.ctx.set_ranks(1)
                self.ctx.set_params(**self._params)
                self._uploaded = True
            else:
                for i, v in enumerate(vox):
                    self.ctx.update_brick(i, v)
            self.brick_uploads += len(vox)
            self._density.record(density)
        self.ctx.set_transfer_function(tf.detach().contiguous())

    def set_camera(self, view: int, cam, width: int, height: int):
        self.ctx.set_camera(view, *cam)
        self.ctx.resize(view, width, height)

    def close(self):
        self.ctx.close()


class _Render(torch.autograd.Function):
    @staticmethod
    def forward(ctx, tf, density, renderer: DifferentiableRenderer, views, size):
        if not (tf.is_cuda and density.is_cuda):
            raise ValueError("tf and density must be CUDA tensors")
        if tf.dtype != torch.float32 or density.dtype != torch.float32:
            raise ValueError("tf and density must be float32")
        W, H = size
        renderer._upload(tf, density)
        stream = torch.cuda.current_stream()
        out = torch.empty((len(views), H, W, 4), dtype=torch.float32, device=density.device)
        # all views in one launch (a view listed twice is rendered once and copied)
        first = {}
        for i, v in enumerate(views):
            first.setdefault(v, i)
        renderer.ctx.forward_views(list(first), [out[i] for i in first.values()], renderer.k, stream)
        for i, v in enumerate(views):
            if first[v] != i:
                out[i].copy_(out[first[v]])
        ctx.renderer, ctx.views = renderer, list(views)
        ctx.tf_shape, ctx.density_shape = tf.shape, density.shape
        return out

    @staticmethod
    def backward(ctx, grad):
        r: DifferentiableRenderer = ctx.renderer
        want_tf, want_density = ctx.needs_input_grad[0], ctx.needs_input_grad[1]
        if not (want_tf or want_density):
            return None, None, None, None, None
        grad = grad.contiguous().float()
        # without a transfer-function gradient the backward skips empty space;
        # without a density gradient it skips the shading and stencil adjoints
        dtf = torch.zeros(ctx.tf_shape, dtype=torch.float32, device=grad.device) if want_tf else None
        dden = torch.zeros(ctx.density_shape, dtype=torch.float32, device=grad.device) if want_density else None
        stream = torch.cuda.current_stream()
        nz, ny, nx = ctx.density_shape
        lo, dims = ((0, 0, 0), (nx, ny, nz)) if want_density else (None, None)
        # all views in one call: one accumulation buffer, cleared and folded once.
        # A view listed twice rendered the same image twice from its last
        # checkpoints, so its output gradients are summed first.
        per_view: dict[int, torch.Tensor] = {}
        for i, v in enumerate(ctx.views):
            per_view[v] = grad[i] if v not in per_view else per_view[v] + grad[i]
        r.ctx.backward_views(list(per_view), list(per_view.values()), dtf, dden, lo, dims, stream)
        return dtf, dden, None, None, None


def render_views(renderer: DifferentiableRenderer, tf: torch.Tensor, density: torch.Tensor, views, size):
    """Differentiable render of `views` (each set with renderer.set_camera at `size` = (W, H))."""
    return _Render.apply(tf, density, renderer, list(views), tuple(size))
