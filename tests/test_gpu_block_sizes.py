"""Block sizes and grids the fixtures do not reach, on generated inputs (the
dodecahedral SPC/E cage, seed 1, continuous angular grid):

* the potential stream's large specialised block sizes: 21 functions (odd
  l <= 5, the benchmark's), 28 (even l <= 6), 25 (all l <= 4) and 36 (all
  l <= 5);
* a grid above the 64 points per axis of the mixed-precision kinetic kernels:
  the FP64 path runs there, the mixed path is refused with an error.

FP64 H v against the oracle <= 1e-10 relative; mixed H v against FP64 <= 2e-6;
the first 6 mixed alpha/beta against FP64 <= 1e-6 of max |alpha| (on bases
this small the recurrence amplifies the difference of the roundings
exponentially, so later coefficients are not comparable); after 400
iterations the 8 lowest converged FP64 levels each have a mixed level within
1e-3 cm^-1 (both engines where the grid allows the tensor cores).
"""
import os

import numpy as np
import pytest

from conftest import OracleModel, load_inputs, load_package, oracle_lancbis

pytestmark = pytest.mark.gpu
CALC = "linRotCartSph_NoQuad_ContGrid_Alavi_SPCE"
CM_TOL_MIXED = 1e-3 / 83.5935  # kJ/mol


def stable_levels(alpha, beta, drop=40, tol=1e-10, emax=30.0):
    """FP64 Ritz values below emax that the run without its last `drop`
    iterations already has to within tol (converged levels)."""
    b = np.concatenate([[0.0], beta])
    ev, _ = oracle_lancbis(alpha, b, b * b, -10.0, emax)
    n = len(alpha) - drop
    ev2, _ = oracle_lancbis(alpha[:n], b[:n + 1], (b * b)[:n + 1], -10.0, emax)
    return np.array([e for e in ev if np.min(np.abs(ev2 - e)) <= tol])


@pytest.fixture(scope="module")
def bsl():
    return load_package()


def rel(a, b):
    return np.max(np.abs(a - b)) / np.max(np.abs(b))


def write_case(tmp, n, l_max, sym, theta, phi):
    inp = load_inputs()
    cage = os.path.join(tmp, "cage.xyz")
    inp.write_cage_xyz(cage, inp.dodecahedral_cage(1))
    hv = os.path.join(tmp, "hv_input.txt")
    inp.write_hv_input(hv, inp.hv_fields(n, 0.08, l_max, theta, phi, cage, "generated", sym))
    return hv


def check_case(bsl, hv, engines, niter):
    h = bsl.Hamiltonian(hv, CALC, precision="fp64")
    m = OracleModel(CALC, hv)
    try:
        assert h.basis_size == m.D
        v = np.random.default_rng(7).standard_normal(h.basis_size)
        u = np.zeros(h.basis_size)
        h.hv(v, u)
        assert rel(u, m.hv(v)) <= 1e-10
        a, b, _ = h.lanczos(niter)
        scale = np.max(np.abs(a))
        low = None
        if niter >= 400:
            low = np.sort(stable_levels(a, b[1:]))[:8]
            assert len(low) == 8
        h.set_precision("mixed")
        for engine in engines:
            h.set_kinetic_engine(engine)
            um = np.zeros(h.basis_size)
            h.hv(v, um)
            assert rel(um, u) <= 2e-6, engine
            am, bm, bm2 = h.lanczos(niter)
            assert np.max(np.abs(am[:6] - a[:6])) <= 1e-6 * scale, engine
            assert np.max(np.abs(bm[1:7] - b[1:7])) <= 1e-6 * scale, engine
            if low is not None:
                evm, _ = bsl.good_eigenvalues(am, bm, bm2, -10.0, 40.0, unit_roundoff=bsl.MIXED_UNIT_ROUNDOFF,
                                               rel_noise=bsl.MIXED_REL_NOISE)
                dev = np.array([np.min(np.abs(evm - e)) for e in low])
                assert dev.max() <= CM_TOL_MIXED, (engine, dev.max() * 83.5935)
        return h
    finally:
        m.close()


@pytest.mark.parametrize("l_max,sym,nn", [(5, "Odd", 21), (6, "Even", 28), (4, "All", 25), (5, "All", 36)])
def test_large_blocks_match_oracle_and_fp64(bsl, tmp_path, l_max, sym, nn):
    hv = write_case(str(tmp_path), 8, l_max, sym, 8, 8)
    h = check_case(bsl, hv, ("simt", "tensor"), 400)
    assert h.nn == nn
    h.close()


def test_grid_above_64_runs_fp64_and_refuses_mixed(bsl, tmp_path):
    hv = write_case(str(tmp_path), 66, 1, "Odd", 2, 2)
    h = bsl.Hamiltonian(hv, CALC, precision="fp64")
    m = OracleModel(CALC, hv)
    try:
        assert h.basis_size == m.D and h.nn == 3
        v = np.random.default_rng(7).standard_normal(h.basis_size)
        u = np.zeros(h.basis_size)
        h.hv(v, u)
        assert rel(u, m.hv(v)) <= 1e-10
        a, b, _ = h.lanczos(5)
        ao, bo, _ = m.lanczos(5)
        assert np.max(np.abs(a - ao)) <= 1e-8 * np.max(np.abs(ao))
        assert np.max(np.abs(b - bo)) <= 1e-8 * np.max(np.abs(ao))
        h.set_precision("mixed")
        with pytest.raises(bsl.BslError, match="64 points"):
            h.hv(v, np.zeros(h.basis_size))
    finally:
        m.close()
        h.close()
