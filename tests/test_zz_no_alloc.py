"""aloha_composite_over_noalloc: the ordered composite for callers that cannot
allocate device memory during the call.  Its output must equal
aloha_composite_over's (bit for bit, like every composite test here) on two
calls in a row, which share the library's fixed staging array.

Kept in its own file, collected last, and independent of the other tests'
state: it builds its own images and runs alone in a fresh process as well as
after the rest of the suite.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _images(torch, n_ranks, H, W, seed):
    g = torch.Generator(device="cuda").manual_seed(seed)
    imgs = torch.rand((n_ranks, H, W, 4), generator=g, device="cuda", dtype=torch.float32)
    imgs[..., :3] *= imgs[..., 3:4]  # premultiplied colour
    return imgs.contiguous()


@pytest.mark.parametrize("mode", [0, 1])
def test_noalloc_composite_matches_allocating_composite(mode):
    torch = pytest.importorskip("torch")
    from aloha_gb300 import abi
    L = abi.lib()
    stream = torch.cuda.current_stream()
    calls = [(8, 96, 128, 1), (3, 40, 56, 2)]  # two calls in a row, different sizes and orders
    for n_ranks, H, W, seed in calls:
        imgs = _images(torch, n_ranks, H, W, seed)
        order = np.random.default_rng(seed).permutation(n_ranks).astype(np.int32)
        want = torch.zeros((H, W), dtype=torch.int32, device="cuda")
        got = torch.full((H, W), -1, dtype=torch.int32, device="cuda")
        rc = L.aloha_composite_over(imgs.data_ptr(), order.ctypes.data, n_ranks, W, H, mode, want.data_ptr(),
                                    stream.cuda_stream)
        assert rc == abi.OK
        rc = L.aloha_composite_over_noalloc(imgs.data_ptr(), order.ctypes.data, n_ranks, W, H, mode,
                                            got.data_ptr(), stream.cuda_stream)
        assert rc == abi.OK
        torch.cuda.synchronize()
        assert torch.equal(got, want)


def test_noalloc_composite_reads_the_order_once():
    """A page-locked order buffer overwritten with out-of-range indices right
    after the call returns must not reach the kernel: the call works on its own
    snapshot of the order."""
    torch = pytest.importorskip("torch")
    from aloha_gb300 import abi
    L = abi.lib()
    stream = torch.cuda.current_stream()
    n_ranks, H, W = 6, 64, 80
    imgs = _images(torch, n_ranks, H, W, 5)
    order_np = np.random.default_rng(5).permutation(n_ranks).astype(np.int32)
    pinned = torch.from_numpy(order_np.copy()).pin_memory()
    want = torch.zeros((H, W), dtype=torch.int32, device="cuda")
    got = torch.full((H, W), -1, dtype=torch.int32, device="cuda")
    assert L.aloha_composite_over(imgs.data_ptr(), order_np.ctypes.data, n_ranks, W, H, 0, want.data_ptr(),
                                  stream.cuda_stream) == abi.OK
    assert L.aloha_composite_over_noalloc(imgs.data_ptr(), pinned.data_ptr(), n_ranks, W, H, 0, got.data_ptr(),
                                          stream.cuda_stream) == abi.OK
    pinned.fill_(1 << 20)  # out of range for every rank image
    torch.cuda.synchronize()
    assert torch.equal(got, want)


def test_noalloc_composite_rejects_what_it_cannot_serve():
    torch = pytest.importorskip("torch")
    from aloha_gb300 import abi
    L = abi.lib()
    imgs = _images(torch, 2, 8, 8, 3)
    fb = torch.zeros((8, 8), dtype=torch.int32, device="cuda")
    order = np.array([1, 0], np.int32)
    big = np.arange(4097, dtype=np.int32)
    assert L.aloha_composite_over_noalloc(imgs.data_ptr(), big.ctypes.data, 4097, 8, 8, 0, fb.data_ptr(),
                                          None) == abi.ERR_OUT_OF_RANGE
    host_fb = np.zeros((8, 8), np.uint32)
    assert L.aloha_composite_over_noalloc(imgs.data_ptr(), order.ctypes.data, 2, 8, 8, 0, host_fb.ctypes.data,
                                          None) == abi.ERR_INVALID_ARGUMENT
    bad = np.array([0, 2], np.int32)
    assert L.aloha_composite_over_noalloc(imgs.data_ptr(), bad.ctypes.data, 2, 8, 8, 0, fb.data_ptr(),
                                          None) == abi.ERR_OUT_OF_RANGE
    assert L.aloha_composite_over_noalloc(None, order.ctypes.data, 2, 8, 8, 0, fb.data_ptr(),
                                          None) == abi.ERR_NULL_POINTER


def test_noalloc_composite_refuses_stream_capture():
    """Its order copy is from pageable memory, which a capture cannot record:
    on a capturing stream the call returns ALOHA_ERR_UNSUPPORTED without
    touching the stream, and the caller's capture still ends and replays."""
    torch = pytest.importorskip("torch")
    from aloha_gb300 import abi
    L = abi.lib()
    n_ranks, H, W = 4, 32, 48
    imgs = _images(torch, n_ranks, H, W, 9)
    order = np.arange(n_ranks, dtype=np.int32)
    fb = torch.zeros((H, W), dtype=torch.int32, device="cuda")
    x = torch.zeros(16, device="cuda")
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    side = torch.cuda.Stream()
    with torch.cuda.graph(g, stream=side, capture_error_mode="relaxed"):
        rc = L.aloha_composite_over_noalloc(imgs.data_ptr(), order.ctypes.data, n_ranks, W, H, 0, fb.data_ptr(),
                                            torch.cuda.current_stream().cuda_stream)
        x.add_(1.0)
    assert rc == abi.ERR_UNSUPPORTED
    g.replay()
    torch.cuda.synchronize()
    assert float(x.sum()) == 16.0
    assert int(fb.abs().sum()) == 0  # nothing was composited during the capture
