"""Failure detection of the bounded device waits, exercised by host-side
injection only.

Every wait of the potential-block stream (bulk copies on an mbarrier ring) and
of the tensor-core kinetic (MMA and stage hand-overs) is bounded; a wait that
runs out records a time-out in a device status word, the kernel drains what it
has in flight and returns, and the C ABI turns the word into BSL_ERR_CUDA with
the stage named.  Here the host sets the word before the run
(bsl_debug_inject_timeout): the kernels then issue no copies or MMAs and skip
every wait, so nothing on the GPU waits or faults.  Checked: the run and the
host-state step return the error with the right message, and the same handle,
with the injection cleared, gives results bit-identical to a run that never
saw it.
"""
import os

import numpy as np
import pytest

from conftest import case_info, load_package

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ham():
    bsl = load_package()
    d, man, extra = case_info("seed1_n6_l3_odd")
    cwd = os.getcwd()
    os.chdir(d)
    try:
        h = bsl.Hamiltonian("hv_input.txt", man["calculator"], extra_input=extra, precision="mixed")
    finally:
        os.chdir(cwd)
    assert h.kinetic_engine() == "tensor"
    yield bsl, h
    h.close()


@pytest.mark.parametrize("mask,message", [(1, "potential-block stream"), (2, "tensor-core kinetic"),
                                          (3, "potential-block stream")])
def test_injected_timeout_is_reported_and_handle_recovers(ham, mask, message):
    bsl, h = ham
    a0, b0, _ = h.lanczos(24)
    h.inject_timeout(mask)
    try:
        with pytest.raises(bsl.BslError, match=message) as ei:
            h.lanczos(24)
        assert ei.value.code == bsl.ERR_CUDA
        vec = np.full(h.basis_size, 1.0 / np.sqrt(h.basis_size))
        rvec = np.zeros(h.basis_size)
        with pytest.raises(bsl.BslError, match=message):
            h.step_host(vec, rvec)
    finally:
        h.inject_timeout(0)
    a1, b1, _ = h.lanczos(24)
    assert np.array_equal(a0, a1) and np.array_equal(b0, b1)


def test_injection_rejects_unknown_bits(ham):
    bsl, h = ham
    with pytest.raises(bsl.BslError) as ei:
        h.inject_timeout(4)
    assert ei.value.code == bsl.ERR_INPUT
