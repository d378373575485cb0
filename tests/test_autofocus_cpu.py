"""Host logic of the autofocus operator, with a stand-in processor (no GPU): the
resident trajectory is re-set only when the offsets change, so an autograd
forward/backward pair leaves the forward's kept per-chirp sums usable, and the
operator asks the processor to keep them."""
import pytest

torch = pytest.importorskip("torch")


class FakeProcessor:
    def __init__(self):
        self.calls = []

    def prepare(self, *args):
        self.calls.append(("prepare", args))

    def uploadGrid(self):
        self.calls.append(("uploadGrid",))

    def path(self):
        return "fp32_bulk"

    def numPixels(self):
        return 6

    def numChirps(self):
        return 4

    def keepChirpSums(self, keep=True):
        self.calls.append(("keepChirpSums", keep))

    def setChirpOffsetsDevice(self, offsets, stream=None):
        self.calls.append(("setChirpOffsetsDevice", None if offsets is None else offsets.clone()))


def _offset_calls(p):
    return [c for c in p.calls if c[0] == "setChirpOffsetsDevice"]


def test_offsets_are_set_only_when_they_change():
    from sarlabtdc import autofocus

    p = FakeProcessor()
    op = autofocus.FocusOperator(p)
    assert ("keepChirpSums", True) in p.calls
    a = torch.zeros((4, 3), dtype=torch.float64)
    b = a.clone()
    b[2, 1] = 1e-4
    op._set_offsets(None)           # the base trajectory is already resident
    assert _offset_calls(p) == []
    op._set_offsets(a)
    op._set_offsets(a.clone())      # equal values: nothing to do
    assert len(_offset_calls(p)) == 1
    op._set_offsets(b)
    op._set_offsets(b)
    assert len(_offset_calls(p)) == 2
    assert torch.equal(_offset_calls(p)[-1][1], b)
    op._set_offsets(None)
    assert _offset_calls(p)[-1][1] is None
    op._set_offsets(a)
    assert len(_offset_calls(p)) == 4
    a[0, 0] = 5.0                   # changed in place: the operator compares with its own copy
    op._set_offsets(a)
    assert len(_offset_calls(p)) == 5


def test_keep_sums_can_be_turned_off():
    from sarlabtdc import autofocus

    p = FakeProcessor()
    autofocus.FocusOperator(p, keep_sums=False)
    assert ("keepChirpSums", False) in p.calls


def test_operator_refuses_paths_without_an_adjoint():
    from sarlabtdc import autofocus

    p = FakeProcessor()
    p.path = lambda: "general"
    with pytest.raises(RuntimeError, match="FP32-bulk"):
        autofocus.FocusOperator(p)


def test_hat_basis_interpolates_between_control_points():
    import pytest
    import torch

    from sarlabtdc import autofocus

    B = autofocus.hat_basis(101, 11, "cpu")
    assert B.shape == (101, 11) and B.dtype == torch.float64
    assert torch.allclose(B.sum(1), torch.ones(101, dtype=torch.float64))
    # control point k sits on chirp 10 k; values between them are linear
    theta = torch.arange(11, dtype=torch.float64) ** 2
    v = B @ theta
    for k in range(11):
        assert float(v[10 * k]) == float(theta[k])
    assert abs(float(v[5]) - 0.5 * (theta[0] + theta[1])) < 1e-12
    with pytest.raises(ValueError):
        autofocus.hat_basis(10, 11, "cpu")
