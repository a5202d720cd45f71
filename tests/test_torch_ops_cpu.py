"""The registered PyTorch operators without a GPU: every C-ABI entry point
the Python API routes through has a ``torch.ops.gbofdft`` operator with a
schema and a fake (meta) implementation giving the output shapes and dtypes,
and there is no CPU kernel behind them (CPU tensors raise)."""
import pytest
import torch

from dftpy_gb300 import torch_ops


def test_every_operator_is_registered_with_a_schema():
    for name in torch_ops.OPS:
        op = getattr(torch.ops.gbofdft, name)
        assert str(op.default._schema).startswith("gbofdft::%s(" % name)
    # handles are plain ints, never symbolic
    assert "SymInt" not in str(torch.ops.gbofdft.eval.default._schema)
    assert "Tensor(a!) workspace" in str(torch.ops.gbofdft.optimize_tn.default._schema)


def test_fake_implementations_give_shapes_and_dtypes():
    x = torch.empty(4, 6, 10, device="meta", dtype=torch.float32)
    pot, en = torch.ops.gbofdft.eval(x, 0, 0, 3)
    assert pot.shape == x.shape and pot.dtype == torch.float32
    assert en.shape == (8,) and en.dtype == torch.float64
    X = torch.ops.gbofdft.fft_r2c(x.double(), 0)
    assert X.shape == (4, 6, 6) and X.dtype == torch.complex128
    y = torch.ops.gbofdft.fft_c2r(X, 0, 11)
    assert y.shape == (4, 6, 11) and y.dtype == torch.float64
    assert torch.ops.gbofdft.convolve(x, 0, 3, torch.empty(4, 6, 6, device="meta"), 1.0).shape == x.shape
    ws = torch.empty(16, device="meta", dtype=torch.float64)
    assert torch.ops.gbofdft.optimize_tn(x, 0, 0, 0, ws, 0, 0).shape == x.shape
    assert torch.ops.gbofdft.optimize_tn_split(x.double(), 0, 0, 0, 0, 0, ws, 0, ws.clone(), 0, 0).dtype == \
        torch.float64


def test_fake_tensor_mode_traces_the_evaluation():
    from torch._subclasses.fake_tensor import FakeTensorMode
    with FakeTensorMode():
        x = torch.empty(8, 8, 8, dtype=torch.float64)
        pot, en = torch.ops.gbofdft.eval(x, 0, 0, 2)
        assert pot.shape == (8, 8, 8) and en.shape == (8,)


@pytest.mark.parametrize("name,args", [("fft_r2c", (torch.zeros(4, 4, 4), 0)),
                                       ("eval", (torch.zeros(4, 4, 4), 0, 0, 3))])
def test_no_cpu_kernel(name, args):
    with pytest.raises(NotImplementedError):
        getattr(torch.ops.gbofdft, name)(*args)
