"""bsl_lanczos_orthonormalize_static: the Lanczos step that allocates no device
memory.  Callers that cannot allocate (inside a CUDA graph capture, under a
pre-reserved memory pool, in loops that cannot take an allocation's device
synchronisation) run the recurrence on their own device buffers with it.

Checked through the C ABI against bsl_lanczos_step_host (the same loop body
with library-managed memory), two iterations in a row, at the FP64 tolerance
of the other parity tests.  The device buffers below belong to the test
(allocated with torch); the entry point itself allocates nothing.
"""
import ctypes as C
import os

import numpy as np
import pytest

from conftest import case_info, load_package

pytestmark = pytest.mark.gpu


def test_orthonormalize_static_matches_step_host():
    torch = pytest.importorskip("torch")
    bsl = load_package()
    L = bsl.lib()
    L.bsl_lanczos_orthonormalize_static.argtypes = [C.c_void_p, C.c_void_p, C.c_longlong, C.c_void_p, C.c_void_p]
    d, man, extra = case_info("seed1_n6_l3_odd")
    cwd = os.getcwd()
    os.chdir(d)
    try:
        h = bsl.Hamiltonian("hv_input.txt", man["calculator"], extra_input=extra, precision="fp64")
    finally:
        os.chdir(cwd)
    D = h.basis_size
    vec_a = np.full(D, 1.0 / np.sqrt(D))
    rvec_a = np.zeros(D)
    vec_b = vec_a.copy()
    rvec_b = rvec_a.copy()
    dev = torch.device("cuda", 0)
    dv = torch.empty(D, dtype=torch.float64, device=dev)
    dr = torch.empty(D, dtype=torch.float64, device=dev)
    dabb = torch.zeros(3, dtype=torch.float64, device=dev)
    for step in range(2):
        # library-managed path: r += H v, then the rest of the loop body
        a_ref, b_ref, b2_ref = h.step_host(vec_a, rvec_a)
        # caller-owned path: r += H v on the host, the rest on device buffers
        h.hv(vec_b, rvec_b)
        dv.copy_(torch.from_numpy(vec_b))
        dr.copy_(torch.from_numpy(rvec_b))
        rc = L.bsl_lanczos_orthonormalize_static(dv.data_ptr(), dr.data_ptr(), D, dabb.data_ptr(),
                                                 C.c_void_p(torch.cuda.current_stream().cuda_stream))
        assert rc == 0, L.bsl_last_error().decode()
        torch.cuda.synchronize()
        vec_b[:] = dv.cpu().numpy()
        rvec_b[:] = dr.cpu().numpy()
        abb = dabb.cpu().numpy()
        assert abs(abb[0] - a_ref) <= 1e-12 * max(1.0, abs(a_ref)), (step, abb[0], a_ref)
        assert abs(abb[1] - b_ref) <= 1e-12 * b_ref and abs(abb[2] - b2_ref) <= 1e-12 * b2_ref
        assert np.max(np.abs(vec_b - vec_a)) <= 1e-10 * np.max(np.abs(vec_a))
        assert np.max(np.abs(rvec_b - rvec_a)) <= 1e-10 * np.max(np.abs(rvec_a))
    # sizes beyond the static scratch are rejected with a clear error
    rc = L.bsl_lanczos_orthonormalize_static(dv.data_ptr(), dr.data_ptr(), 8388609, dabb.data_ptr(), None)
    assert rc == bsl.ERR_INPUT and b"static scratch capacity" in L.bsl_last_error()
    h.close()
