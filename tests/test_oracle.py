"""The oracle restatement pinned against the reference's own outputs.

ref_hv.npy / ref_alpha_beta.npz / ref_boundstates.txt were produced by the
unmodified reference (tests/golden/make_golden.py); stored_2013_runs.json is
copied from the reference's stored SmallBasisTest2 runs.
"""
import json
import os

import numpy as np
import pytest

from conftest import BLOCK_CASES, CASES, GOLDEN, OracleModel, case_info, oracle_lancbis, read_boundstates


@pytest.mark.parametrize("name", CASES + BLOCK_CASES + ["cpu_workload"])
def test_oracle_hv_matches_reference(name, in_case_dir):
    d, man, extra = in_case_dir(name)
    m = OracleModel(man["calculator"], "hv_input.txt", extra)
    assert m.D == man["basis_size"]
    v = np.random.default_rng(man["hv_seed"]).standard_normal(m.D)
    u = m.hv(v)
    if os.path.exists("ref_hv.npy"):
        ref = np.load("ref_hv.npy")
        err = np.max(np.abs(u - ref)) / np.max(np.abs(ref))
    else:
        s = np.load("ref_hv_sample.npz")
        ref = s["val"]
        err = np.max(np.abs(u[s["idx"]] - ref)) / np.max(np.abs(ref))
        assert abs(np.linalg.norm(u) - man["hv_norm"]) <= 1e-12 * man["hv_norm"]
    assert err <= 1e-12, err
    m.close()


@pytest.mark.parametrize("name", CASES + BLOCK_CASES)
def test_oracle_lanczos_matches_reference(name, in_case_dir):
    d, man, extra = in_case_dir(name)
    m = OracleModel(man["calculator"], "hv_input.txt", extra)
    ref = np.load("ref_alpha_beta.npz")
    niter = man["niter"]
    a, b, b2 = m.lanczos(niter)
    # the first iterations agree to rounding; later ones drift as any
    # Lanczos run without reorthogonalisation amplifies rounding differences
    k = 30
    assert np.max(np.abs(a[:k] - ref["alpha"][:k]) / np.abs(ref["alpha"][:k]).max()) <= 1e-12
    assert np.max(np.abs(b[1:k + 1] - ref["beta"][:k]) / ref["beta"][:k].max()) <= 1e-12
    ev, er = oracle_lancbis(a, b, b2)
    bs = read_boundstates("ref_boundstates.txt")
    stable = converged_levels(ref["alpha"], ref["beta"])
    for e in stable:
        assert np.min(np.abs(ev - e)) <= 1e-9, e
    m.close()


def converged_levels(alpha, beta, drop=40, tol=1e-10):
    """Good eigenvalues of T_m that are already present in T_{m-drop}."""
    b = np.concatenate([[0.0], beta])
    ev, _ = oracle_lancbis(alpha, b, b * b)
    n = len(alpha) - drop
    ev2, _ = oracle_lancbis(alpha[:n], b[:n + 1], (b * b)[:n + 1])
    return np.array([e for e in ev if np.min(np.abs(ev2 - e)) <= tol])


def test_oracle_tail_reproduces_stored_2013_run():
    """Reference alpha/beta (final tree) through the oracle tail reproduce the
    reference's own stored 2013-09-03 19:06 run on its converged levels."""
    stored = json.load(open(os.path.join(GOLDEN, "stored_2013_runs.json")))["SmallBasisTest2_2013-09-03_19_06_47"]
    ref = np.load(os.path.join(GOLDEN, "cage11_n10_l3_all", "ref_alpha_beta.npz"))
    assert len(ref["alpha"]) == stored["niter"]
    b = np.concatenate([[0.0], ref["beta"]])
    ev, er = oracle_lancbis(ref["alpha"], b, b * b)
    levels = np.array(stored["levels"])
    low = levels[levels[:, 0] < -3.0]
    assert len(low) >= 10
    for e, _ in low:
        assert np.min(np.abs(ev - e)) <= 1e-9, e
    # and the reference's boundstates.txt for the same run agrees entirely
    bs = read_boundstates(os.path.join(GOLDEN, "cage11_n10_l3_all", "ref_boundstates.txt"))
    assert len(bs) == len(ev)
    assert np.max(np.abs(bs[:, 0] - ev)) <= 1e-13


def test_oracle_point_grid_reproduces_stored_2013_run():
    """Point-grid Alavi SPC/E (linRotCartSph_NoQuad_Alavi_SPCE): the reference's
    alpha/beta (final tree) through the oracle tail reproduce the reference's
    own stored 2013-08-30 15:06 run (same inputs) on its converged levels, and
    the final tree's boundstates.txt agrees with the stored one there."""
    stored = json.load(open(os.path.join(GOLDEN, "stored_2013_runs.json")))["SmallBasisTest2_2013-08-30_15_06_49"]
    d = os.path.join(GOLDEN, "point_cage11_n10_l2_odd")
    ref = np.load(os.path.join(d, "ref_alpha_beta.npz"))
    assert len(ref["alpha"]) == stored["niter"]
    b = np.concatenate([[0.0], ref["beta"]])
    ev, er = oracle_lancbis(ref["alpha"], b, b * b)
    levels = np.array(stored["levels"])
    conv = levels[levels[:, 1] < 1e-8]
    assert len(conv) >= 10
    for e, _ in conv:
        assert np.min(np.abs(ev - e)) <= 5e-12, e
    bs = read_boundstates(os.path.join(d, "ref_boundstates.txt"))
    assert len(bs) == len(ev) == len(levels)
    assert np.max(np.abs(bs[:, 0] - ev)) <= 1e-13


def test_oracle_coulomb_is_orientation_independent():
    """The Coulomb calculator's V does not depend on the H2 orientation, so its
    V blocks are diagonal in (l, m) (orthonormal tesseral harmonics on the
    exact quadrature) and the origin point, where 1/|r| is infinite, carries
    the clipped value."""
    d, man, extra = case_info("coulomb_n9_l2_all")
    cwd = os.getcwd()
    os.chdir(d)
    try:
        m = OracleModel(man["calculator"], "hv_input.txt", extra)
        v1, v2 = m.vgrid()
        blocks = m.vblocks()
    finally:
        os.chdir(cwd)
    nn = m.nn
    b = blocks.reshape(-1, nn, nn)
    off = b - np.einsum("pi,ij->pij", np.einsum("pii->pi", b), np.eye(nn))
    assert np.max(np.abs(off)) <= 1e-12 * np.max(np.abs(b))
    assert np.min(v1) == -20.0 and np.array_equal(v1, v2)


def test_oracle_isoharmosc_analytic():
    """IsoHarmOsc levels = hbar w (n + 3/2) + B l(l+1) up to the DVR error."""
    d, man, extra = case_info("iso_n20_l2_all")
    bs = read_boundstates(os.path.join(d, "ref_boundstates.txt"))
    hbar, w, B = 0.0635077857002, 24.1, 0.709652722117881
    analytic = np.array(sorted({hbar * w * (n + 1.5) + B * l * (l + 1) for n in range(8) for l in range(3)}))
    for e in bs[:6, 0]:
        assert np.min(np.abs(analytic - e)) <= 5e-4, e
