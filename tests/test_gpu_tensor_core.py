"""tcgen05 plumbing (tensor-memory allocation, swizzled shared-memory
descriptors, kind::tf32 MMA, commit to an mbarrier, tensor-memory load) on an
exact small product."""
import ctypes as C

import pytest

from conftest import load_package

pytestmark = pytest.mark.gpu


def test_tcgen05_tf32_product_exact():
    bsl = load_package()
    L = bsl.lib()
    L.bsl_selftest_tensor_core.argtypes = [C.POINTER(C.c_double)]
    err = C.c_double(-1.0)
    rc = L.bsl_selftest_tensor_core(C.byref(err))
    assert rc == 0, L.bsl_last_error().decode()
    assert err.value == 0.0
