"""bsl_lanczos_orthonormalize_static: the Lanczos step that allocates no device
memory.  Applications that reserve all GPU memory up front in their own pool,
or loops that cannot take the synchronisation an allocation may imply, run the
recurrence on their own device buffers with it.

Checked through the C ABI against bsl_lanczos_step_host (the same loop body
with library-managed memory), two iterations in a row, at the FP64 tolerance
of the other parity tests; on a vector of many reduction blocks against numpy,
two calls in a row; and for its argument checks and breakdown report.  The
device buffers below belong to the test (allocated with torch); the entry point
itself allocates nothing.
"""
import ctypes as C
import os

import numpy as np
import pytest

from conftest import case_info, load_package

pytestmark = pytest.mark.gpu


def entry(bsl):
    L = bsl.lib()
    L.bsl_lanczos_orthonormalize_static.argtypes = [C.c_void_p, C.c_void_p, C.c_longlong, C.c_void_p, C.c_void_p]
    return L


def numpy_step(v, r):
    """The reference loop body (lanczosEigenValuesVectors.cpp:202-238) in numpy."""
    a = v @ r
    r = r - a * v
    b2 = r @ r
    b = np.sqrt(b2)
    return r / b, -b * v, a, b, b2


def test_orthonormalize_static_matches_step_host():
    torch = pytest.importorskip("torch")
    bsl = load_package()
    L = entry(bsl)
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


def test_orthonormalize_static_many_blocks_matches_numpy():
    """300,001 elements (147 reduction blocks, a ragged last one), two calls in
    a row, against the same loop body in numpy (FP64, 1e-12 relative)."""
    torch = pytest.importorskip("torch")
    bsl = load_package()
    L = entry(bsl)
    n = 300001
    rng = np.random.default_rng(11)
    v = rng.standard_normal(n)
    v /= np.linalg.norm(v)
    r = rng.standard_normal(n)
    dev = torch.device("cuda", 0)
    dv = torch.from_numpy(v).to(dev)
    dr = torch.from_numpy(r).to(dev)
    dabb = torch.zeros(3, dtype=torch.float64, device=dev)
    s = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    for step in range(2):
        v, r, a, b, b2 = numpy_step(v, r)
        rc = L.bsl_lanczos_orthonormalize_static(dv.data_ptr(), dr.data_ptr(), n, dabb.data_ptr(), s)
        assert rc == 0, L.bsl_last_error().decode()
        torch.cuda.synchronize()
        abb = dabb.cpu().numpy()
        assert abs(abb[0] - a) <= 1e-12 * max(1.0, abs(a)), (step, abb[0], a)
        assert abs(abb[1] - b) <= 1e-12 * b and abs(abb[2] - b2) <= 1e-12 * b2
        assert np.max(np.abs(dv.cpu().numpy() - v)) <= 1e-12 * np.max(np.abs(v))
        assert np.max(np.abs(dr.cpu().numpy() - r)) <= 1e-12 * np.max(np.abs(r))
        # the next call continues from r + "H v" = r + 0.5 v (any vector will do)
        r = r + 0.5 * v
        dr.add_(0.5 * dv)


def test_orthonormalize_static_rejects_overlap_and_reports_breakdown():
    torch = pytest.importorskip("torch")
    bsl = load_package()
    L = entry(bsl)
    dev = torch.device("cuda", 0)
    buf = torch.zeros(4096, dtype=torch.float64, device=dev)
    dabb = torch.zeros(3, dtype=torch.float64, device=dev)
    p = buf.data_ptr()
    # overlapping vector ranges and an overlapping result buffer are refused
    rc = L.bsl_lanczos_orthonormalize_static(p, p + 8 * 1000, 2048, dabb.data_ptr(), None)
    assert rc == bsl.ERR_INPUT and b"overlap" in L.bsl_last_error()
    rc = L.bsl_lanczos_orthonormalize_static(p, p + 8 * 2048, 2048, p + 8 * 100, None)
    assert rc == bsl.ERR_INPUT and b"overlap" in L.bsl_last_error()
    # r + H v = 3 v exactly: r - alpha v = 0, beta = 0 (a breakdown); the
    # vectors stay unscaled and d_abb[1] carries the zero
    n = 2048
    v = torch.zeros(n, dtype=torch.float64, device=dev)
    v[5] = 1.0
    r = 3.0 * v
    s = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    rc = L.bsl_lanczos_orthonormalize_static(v.data_ptr(), r.data_ptr(), n, dabb.data_ptr(), s)
    assert rc == 0, L.bsl_last_error().decode()
    torch.cuda.synchronize()
    abb = dabb.cpu().numpy()
    assert abb[0] == 3.0 and abb[1] == 0.0 and abb[2] == 0.0
    assert np.all(np.isfinite(v.cpu().numpy())) and v[5].item() == 1.0
    assert np.all(r.cpu().numpy() == 0.0)
