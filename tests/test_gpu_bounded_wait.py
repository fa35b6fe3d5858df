"""Failure detection without a GPU fault: the stage kernel's waits on its TMA
copies are bounded, and a wait that runs out is reported as a status the host
reads (ENL_ERR_TIMEOUT) while the context stays usable.  The test makes the
wait run out on an mbarrier that nothing completes."""
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from enlightning_gb300 import _lib  # noqa: E402

ENL_OK, ENL_ERR_TIMEOUT = 0, 4


def test_wait_that_nothing_completes_returns_timeout():
    L = _lib.lib()
    L.enl_get_last_error()  # start from a clear error word
    assert L.enl_check_bounded_wait(1000, 1) == ENL_OK
    assert L.enl_check_bounded_wait(1000, 0) == ENL_ERR_TIMEOUT
    # the context is still usable afterwards
    x = torch.arange(8, device="cuda", dtype=torch.float32)
    assert float(x.sum().item()) == 28.0
    assert L.enl_check_bounded_wait(10, 1) == ENL_OK
    assert L.enl_get_last_error() == 0
