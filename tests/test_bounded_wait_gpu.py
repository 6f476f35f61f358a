"""The pipeline's waits are bounded: a wait on an mbarrier that nothing
arrives on gives up after its limit and raises the abort flag, and the
context keeps working afterwards.  No fault, no hang."""
import ctypes

import numpy as np
import pytest

from dasp_gb300 import _lib
from tests.wfs_cases import Case

pytestmark = pytest.mark.gpu


def test_bounded_wait_gives_up_and_context_stays_usable():
    to, ab = ctypes.c_int(-1), ctypes.c_int(-1)
    # about a quarter of a second at the maximum SM clock
    _lib.check(_lib.lib().shwfs_selftest_bounded_wait(500_000_000, ctypes.byref(to), ctypes.byref(ab)), "selftest")
    assert to.value == 1 and ab.value == 1
    c = Case(nsubx=8, p=8, N=16, sig=1e4)
    eng = c.engine()
    eng.set_form("fp16")
    eng.run(0)  # the tensor-core pipeline still runs and reports no timeout
    oc, _ = c.oracle_run(c.oracle("f64"))
    lit = c.lit()
    assert np.abs(c.cents.reshape(-1, 2)[lit] - oc.reshape(-1, 2)[lit]).max() < 1e-3
    eng.free()
