"""Failure detection on the GPU without a fault: a kernel's bounded mbarrier wait runs out on a
barrier that nothing completes, the kernel reports the timeout through the status word the host
reads after every call, and the context stays usable (a reconstruction right after it is still
bit-exact)."""
import ctypes as C

import numpy as np
import pytest

from recview_gb300 import abi
from tests.rvtest import fbp_case

pytestmark = pytest.mark.gpu


def test_bounded_wait_runs_out_and_reports(gpu):
    ms = C.c_double()
    assert gpu.RvTestBoundedWait(8, C.byref(ms)) == abi.RV_ERR_KERNEL_STATUS
    assert 0.0 < ms.value < 5000.0
    # the status was cleared: a second check reports its own timeout again, nothing stale
    assert gpu.RvTestBoundedWait(8, C.byref(ms)) == abi.RV_ERR_KERNEL_STATUS


def test_bounded_wait_arguments(gpu):
    ms = C.c_double()
    assert gpu.RvTestBoundedWait(7, C.byref(ms)) == abi.RV_ERR_BAD_ARGUMENT
    assert gpu.RvTestBoundedWait(17, C.byref(ms)) == abi.RV_ERR_BAD_ARGUMENT


def test_context_usable_after_timeout(gpu, oracle):
    ms = C.c_double()
    assert gpu.RvTestBoundedWait(8, C.byref(ms)) == abi.RV_ERR_KERNEL_STATUS
    ri = fbp_case(7, 200, 181, 99.6, 2, oracle=oracle)
    from tests.test_gpu_parity import _gpu_slice
    got = _gpu_slice(ri)
    assert np.array_equal(got, oracle.reconstruct(ri, threads=4))
