"""The FP64 Hellmann-Feynman oracle (oracle/bsl_oracle.cpp, hf_gradient),
pinned on the CPU.

For a fixed vector psi the Rayleigh quotient E = psi.H psi / psi.psi has
dE/dtheta = psi.(dH/dtheta) psi / psi.psi exactly, for any psi, so no
eigenvector is needed:

* centres of mass and Euler angles: the fixture holds E at +-1e-5 of 9 of
  the cage's rigid-body coordinates, computed by the compiled reference's own
  H v (tests/golden/make_golden.py, case hf_fd_seed1_n5_l3_odd: 5^3 grid, odd
  l <= 3, 6 theta x 10 phi, the generated cage seed 1); the oracle's site
  derivatives through its complex-step chain rule match these central
  differences;
* site and Alavi charges: the reference fixes them at compile time, so the
  central differences use the oracle's own potential (bit-identical to the
  reference's at the standard charges) with the charges moved.
"""
import os

import numpy as np
import pytest

from conftest import GOLDEN, OracleModel

CALC = "linRotCartSph_NoQuad_ContGrid_Alavi_SPCE"
CASE = os.path.join(GOLDEN, "hf_fd_seed1_n5_l3_odd")


@pytest.fixture(scope="module")
def model():
    cwd = os.getcwd()
    os.chdir(CASE)
    try:
        m = OracleModel(CALC, "hv_input.txt", threads=4)
    finally:
        os.chdir(cwd)
    yield m
    m.close()


def rayleigh(m, psi):
    return float(psi @ m.hv(psi) / (psi @ psi))


def test_rigid_body_derivatives_match_reference_differences(model):
    fx = np.load(os.path.join(CASE, "ref_rayleigh_fd.npz"))
    psi, e_pm, h, params = fx["psi"], fx["e_pm"], float(fx["step"]), fx["params"]
    # the unperturbed oracle H gives the reference's quotient (both sides of each difference bracket it)
    e0 = rayleigh(model, psi)
    assert np.all(np.abs(e_pm - e0) < 1e-3)
    dq, dr, da = model.hf_gradient(psi, 60)
    dcm, dea = model.rigid_body_gradient(dr)
    for (kind, m, k), (ep, em) in zip(params, e_pm):
        fd = (ep - em) / (2 * h)
        an = (dcm if kind == 0 else dea)[0, m, k]
        assert abs(an - fd) <= 2e-6 * max(abs(fd), 1e-2), (kind, m, k, an, fd)


def test_charge_derivatives_match_oracle_differences(model):
    fx = np.load(os.path.join(CASE, "ref_rayleigh_fd.npz"))
    psi = fx["psi"]
    dq, dr, da = model.hf_gradient(psi, 60)
    q0 = np.tile([-0.8476, 0.4238, 0.4238], 20)
    qa0 = np.array([0.4932, -0.9864])
    h = 1e-5
    try:
        for w in (0, 1, 8, 31, 59):
            e = []
            for s in (1.0, -1.0):
                q = q0.copy()
                q[w] += s * h
                model.set_charges(q_site=q)
                e.append(rayleigh(model, psi))
            fd = (e[0] - e[1]) / (2 * h)
            assert abs(dq[0, w] - fd) <= 1e-6 * max(abs(fd), 1e-1), (w, dq[0, w], fd)
        model.set_charges(q_site=q0)
        for k in (0, 1):
            e = []
            for s in (1.0, -1.0):
                qa = qa0.copy()
                qa[k] += s * h
                model.set_charges(q_alavi=qa)
                e.append(rayleigh(model, psi))
            fd = (e[0] - e[1]) / (2 * h)
            assert abs(da[0, k] - fd) <= 1e-6 * max(abs(fd), 1e-1), (k, da[0, k], fd)
    finally:
        model.set_charges(q_site=q0, q_alavi=qa0)
