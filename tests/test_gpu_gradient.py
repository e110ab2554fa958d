"""Hellmann-Feynman derivatives of the levels with respect to the cage
(site charges, rigid-body coordinates, Alavi H2 charges) against central
differences of the levels, and the torch.autograd wrapper."""
import os

import numpy as np
import pytest

from conftest import case_info, load_package

pytestmark = pytest.mark.gpu
NITER = 200
NLEV = 3


@pytest.fixture(scope="module")
def bsl():
    return load_package()


def setup_case(bsl):
    d, man, _ = case_info("seed1_n6_l3_odd")
    cwd = os.getcwd()
    os.chdir(d)  # the HvInputFile names its cage relative to its directory
    try:
        p = bsl.parse_hv_input("hv_input.txt")
    finally:
        os.chdir(cwd)
    cm, ea = bsl.read_cage_xyz(os.path.join(d, "cage_seed1.xyz"))
    q = bsl.cage_sites(cm, ea)[1]
    qa = np.array([0.4932, -0.9864])
    return d, p, cm, ea, q, qa


def levels(bsl, p, cm, ea, q, qa, grads=False):
    h = bsl.Hamiltonian.from_cage(p, cm, ea, q, qa)
    try:
        a, b, b2 = h.lanczos(NITER, start="normal", seed=1)
        ev, _ = bsl.good_eigenvalues(a, b, b2, -10.0, 10.0)
        ev = ev[:NLEV]
        if not grads:
            return ev, None
        rows = bsl.tm_eigenvectors(a, b, b2, ev)
        psi = h.ritz(NITER, rows, start="normal", seed=1)
        return ev, h.hf_gradient(psi, 3 * cm.shape[0])
    finally:
        h.close()


def test_cage_arrays_give_the_file_hamiltonian(bsl):
    d, p, cm, ea, q, qa = setup_case(bsl)
    cwd = os.getcwd()
    os.chdir(d)
    try:
        hf = bsl.Hamiltonian("hv_input.txt")
    finally:
        os.chdir(cwd)
    ha = bsl.Hamiltonian.from_cage(p, cm, ea)
    v = np.random.default_rng(4).standard_normal(hf.basis_size)
    uf, ua = np.zeros(hf.basis_size), np.zeros(hf.basis_size)
    hf.hv(v, uf)
    ha.hv(v, ua)
    assert np.array_equal(uf, ua)
    hf.close()
    ha.close()


def test_hf_gradient_matches_finite_differences(bsl):
    d, p, cm, ea, q, qa = setup_case(bsl)
    ev, (dq, dr, da) = levels(bsl, p, cm, ea, q, qa, grads=True)
    dcm, dea = bsl.rigid_body_gradient(cm, ea, dr)
    h = 1e-4

    def fd(mod):
        plus = levels(bsl, p, *mod(+h))[0]
        minus = levels(bsl, p, *mod(-h))[0]
        return (plus - minus) / (2 * h)

    def with_q(w):
        def mod(s):
            q2 = q.copy()
            q2[w] += s
            return cm, ea, q2, qa
        return mod

    def with_cm(m, k):
        def mod(s):
            c2 = cm.copy()
            c2[m, k] += s
            return c2, ea, q, qa
        return mod

    def with_ea(m, k):
        def mod(s):
            e2 = ea.copy()
            e2[m, k] += s
            return cm, e2, q, qa
        return mod

    def with_qa(k):
        def mod(s):
            a2 = qa.copy()
            a2[k] += s
            return cm, ea, q, a2
        return mod

    checks = [(with_q(0), dq[:, 0]), (with_q(7), dq[:, 7]), (with_cm(2, 0), dcm[:, 2, 0]),
              (with_cm(11, 2), dcm[:, 11, 2]), (with_ea(4, 1), dea[:, 4, 1]), (with_ea(15, 0), dea[:, 15, 0]),
              (with_qa(0), da[:, 0]), (with_qa(1), da[:, 1])]
    for mod, hf in checks:
        f = fd(mod)
        assert np.allclose(hf, f, rtol=2e-4, atol=2e-5), (hf, f)


def test_autograd_function(bsl):
    torch = pytest.importorskip("torch")
    d, p, cm, ea, q, qa = setup_case(bsl)
    Fn = bsl.cage_levels_function()
    tcm = torch.tensor(cm, dtype=torch.float64, requires_grad=True)
    tea = torch.tensor(ea, dtype=torch.float64, requires_grad=True)
    tq = torch.tensor(q, dtype=torch.float64, requires_grad=True)
    tqa = torch.tensor(qa, dtype=torch.float64, requires_grad=True)
    setup = {"params": p, "niter": NITER, "nlev": NLEV, "emin": -10.0, "emax": 10.0, "seed": 1}
    E = Fn.apply(tcm, tea, tq, tqa, setup)
    w = torch.tensor([1.0, -0.5, 0.25], dtype=torch.float64)
    (E * w).sum().backward()
    ev, (dq, dr, da) = levels(bsl, p, cm, ea, q, qa, grads=True)
    dcm, dea = bsl.rigid_body_gradient(cm, ea, dr)
    wn = w.numpy()
    assert np.allclose(E.detach().numpy(), ev, rtol=0, atol=1e-12)
    assert np.allclose(tq.grad.numpy(), wn @ dq, rtol=1e-10, atol=1e-12)
    assert np.allclose(tcm.grad.numpy(), np.einsum("n,nmk->mk", wn, dcm), rtol=1e-10, atol=1e-12)
    assert np.allclose(tea.grad.numpy(), np.einsum("n,nmk->mk", wn, dea), rtol=1e-10, atol=1e-12)
    assert np.allclose(tqa.grad.numpy(), wn @ da, rtol=1e-10, atol=1e-12)


def test_hf_gradient_tip4p(bsl):
    """The same derivatives with TIP4P water (4 sites per molecule, charge on M,
    Lennard-Jones on O): central differences on an M charge, an H charge, a
    centre and an angle."""
    d, p, cm, ea, q, qa = setup_case(bsl)
    T4 = bsl.POT_ALAVI_TIP4P
    q4 = bsl.cage_sites(cm, ea, potential=T4)[1]
    assert q4.shape == (80,) and abs(q4.sum()) < 1e-12

    def lev(cm_, ea_, q_, grads=False):
        h = bsl.Hamiltonian.from_cage(p, cm_, ea_, q_, qa, potential=T4)
        try:
            a, b, b2 = h.lanczos(NITER, start="normal", seed=1)
            ev, _ = bsl.good_eigenvalues(a, b, b2, -10.0, 10.0)
            ev = ev[:NLEV]
            if not grads:
                return ev, None
            rows = bsl.tm_eigenvectors(a, b, b2, ev)
            return ev, h.hf_gradient(h.ritz(NITER, rows, start="normal", seed=1), 80)
        finally:
            h.close()

    ev, (dq, dr, da) = lev(cm, ea, q4, grads=True)
    dcm, dea = bsl.rigid_body_gradient(cm, ea, dr, potential=T4)
    h = 1e-4
    for w in (3, 9):  # M site of molecule 0, H site of molecule 2
        qp, qm = q4.copy(), q4.copy()
        qp[w] += h
        qm[w] -= h
        f = (lev(cm, ea, qp)[0] - lev(cm, ea, qm)[0]) / (2 * h)
        assert np.allclose(dq[:, w], f, rtol=2e-4, atol=2e-5), (dq[:, w], f)
    cp, cq = cm.copy(), cm.copy()
    cp[6, 1] += h
    cq[6, 1] -= h
    f = (lev(cp, ea, q4)[0] - lev(cq, ea, q4)[0]) / (2 * h)
    assert np.allclose(dcm[:, 6, 1], f, rtol=2e-4, atol=2e-5), (dcm[:, 6, 1], f)
    ep, eq = ea.copy(), ea.copy()
    ep[9, 2] += h
    eq[9, 2] -= h
    f = (lev(cm, ep, q4)[0] - lev(cm, eq, q4)[0]) / (2 * h)
    assert np.allclose(dea[:, 9, 2], f, rtol=2e-4, atol=2e-5), (dea[:, 9, 2], f)


def test_hf_gradient_needs_continuous_grid(bsl):
    """The point-grid potentials are piecewise constant in the cage coordinates:
    the derivative entry point refuses them instead of returning zeros."""
    d, man, extra = case_info("point_cage11_n10_l2_odd")
    cwd = os.getcwd()
    os.chdir(d)
    try:
        h = bsl.Hamiltonian("hv_input.txt", man["calculator"], extra_input=extra)
    finally:
        os.chdir(cwd)
    psi = np.random.default_rng(0).standard_normal((1, h.basis_size))
    with pytest.raises(bsl.BslError) as e:
        h.hf_gradient(psi, 60)
    assert e.value.code == bsl.ERR_UNSUPPORTED
    h.close()
