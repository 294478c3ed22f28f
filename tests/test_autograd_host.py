"""Host logic of the torch binding (no GPU): when the differentiable
renderer must upload the density again."""
import pytest

torch = pytest.importorskip("torch")

from aloha_gb300.autograd import DensityTracker  # noqa: E402


def test_tracker_follows_object_and_version():
    t = DensityTracker()
    a = torch.zeros(4, 4, 4)
    assert not t.current(a)
    t.record(a)
    assert t.current(a)
    a.add_(1.0)  # in-place update bumps the version counter
    assert not t.current(a)
    t.record(a)
    assert t.current(a)
    b = a.clone()  # same values, another tensor
    assert not t.current(b)
    t.invalidate()
    assert not t.current(a)


def test_tracker_never_matches_a_new_tensor_at_a_reused_address():
    t = DensityTracker()
    a = torch.zeros(1 << 16)
    t.record(a)
    del a
    # new tensors of the same size, possibly in the freed block: never current
    for _ in range(8):
        b = torch.zeros(1 << 16)
        assert not t.current(b)
        del b
