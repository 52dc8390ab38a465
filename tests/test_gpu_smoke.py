"""The package entry point's smoke run (one small step on cuda:0 checked against the oracle)."""
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("needs a CUDA device", allow_module_level=True)


def test_smoke_entry_point():
    import __graft_entry__

    __graft_entry__.smoke()
