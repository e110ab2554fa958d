"""GPU parity through the C ABI against the reference's own outputs and the oracle.

Tolerances
  FP64 path: Hv <= 1e-10 relative (max |du| / max |u|); eigenvalues <= 1e-6 cm^-1
  mixed path: Hv <= 2e-6 relative; converged levels <= 1e-3 cm^-1 of the FP64 run
"""
import os

import numpy as np
import pytest

from conftest import CASES, REF_ONLY_CASES, OracleModel, case_info, load_package, oracle_lancbis, read_boundstates

pytestmark = pytest.mark.gpu
KJ_TO_CM = 83.5935
CM_TOL_FP64 = 1e-6 / KJ_TO_CM
CM_TOL_MIXED = 1e-3 / KJ_TO_CM


@pytest.fixture(scope="module")
def bsl():
    return load_package()


def make(bsl, name, precision="fp64"):
    d, man, extra = case_info(name)
    cwd = os.getcwd()
    os.chdir(d)
    try:
        h = bsl.Hamiltonian("hv_input.txt", man["calculator"], extra_input=extra, precision=precision)
    finally:
        os.chdir(cwd)
    return h, d, man, extra


def rel(a, b):
    return np.max(np.abs(a - b)) / np.max(np.abs(b))


@pytest.mark.parametrize("name", CASES + REF_ONLY_CASES)
def test_hv_fp64_matches_reference(bsl, name):
    h, d, man, _ = make(bsl, name)
    assert h.basis_size == man["basis_size"]
    v = np.random.default_rng(man["hv_seed"]).standard_normal(h.basis_size)
    u = np.zeros(h.basis_size)
    h.hv(v, u)
    ref = np.load(os.path.join(d, "ref_hv.npy"))
    assert rel(u, ref) <= 1e-10
    # accumulation contract: uec += H vec
    u2 = np.ones(h.basis_size)
    h.hv(v, u2)
    assert rel(u2 - 1.0, ref) <= 1e-10
    h.close()


def test_hv_cpu_workload_fp64_and_mixed(bsl):
    h, d, man, _ = make(bsl, "cpu_workload")
    s = np.load(os.path.join(d, "ref_hv_sample.npz"))
    v = np.random.default_rng(man["hv_seed"]).standard_normal(h.basis_size)
    u = np.zeros(h.basis_size)
    h.hv(v, u)
    assert rel(u[s["idx"]], s["val"]) <= 1e-10
    assert abs(np.linalg.norm(u) - man["hv_norm"]) <= 1e-10 * man["hv_norm"]
    h.set_precision("mixed")
    for engine in ("simt", "tensor"):
        h.set_kinetic_engine(engine)
        um = np.zeros(h.basis_size)
        h.hv(v, um)
        assert rel(um, u) <= 2e-6, engine
    h.close()


@pytest.mark.parametrize("name", CASES + REF_ONLY_CASES)
def test_hv_mixed_engines_match_fp64(bsl, name):
    """Both kinetic engines of the mixed path against the FP64 path (2e-6 relative)."""
    h, d, man, _ = make(bsl, name)
    v = np.random.default_rng(man["hv_seed"]).standard_normal(h.basis_size)
    u = np.zeros(h.basis_size)
    h.hv(v, u)
    h.set_precision("mixed")
    assert h.kinetic_engine() == "tensor"  # the default engine where the grid allows it
    out = {}
    for engine in ("simt", "tensor"):
        h.set_kinetic_engine(engine)
        out[engine] = np.zeros(h.basis_size)
        h.hv(v, out[engine])
        assert rel(out[engine], u) <= 2e-6, (engine, rel(out[engine], u))
    assert rel(out["tensor"], out["simt"]) <= 2e-6
    h.close()


@pytest.mark.parametrize("name", ["cage11_n10_l3_all", "seed1_n6_l3_odd", "point_cage11_n10_l2_odd",
                                  "coulomb_n9_l2_all"])
def test_potential_grid_and_blocks_match_oracle(bsl, name):
    """V(x, y, z, theta, phi) and the V blocks against the oracle; for the point
    grid every value is a table lookup, so a nearest-point index that differed
    from the reference's would show as an O(1) error here."""
    h, d, man, extra = make(bsl, name)
    cwd = os.getcwd()
    os.chdir(d)
    try:
        m = OracleModel(man["calculator"], "hv_input.txt", extra)
    finally:
        os.chdir(cwd)
    g1, g2 = h.vgrid()
    o1, o2 = m.vgrid()
    assert rel(g1, o1) <= 1e-13 and rel(g2, o2) <= 1e-13
    blk = h.vblocks().reshape(-1, h.nn, h.nn)
    ob = m.vblocks().reshape(-1, m.nn, m.nn)
    keep = full_indices(h)
    ob = ob[:, keep][:, :, keep]
    assert np.max(np.abs(blk - ob)) <= 1e-12 * np.max(np.abs(ob))
    h.close()
    m.close()


def full_indices(h):
    lmax = h.params.l_max
    sym = h.params.symmetry
    out, n = [], 0
    for mm in range(-lmax, lmax + 1):
        for l in range(abs(mm), lmax + 1):
            if sym == 0 or (sym == 1 and l % 2 == 0) or (sym == 2 and l % 2 == 1):
                out.append(n)
            n += 1
    return np.array(out)


def stable_levels(alpha, beta, drop=40, tol=1e-10, emax=10.0):
    b = np.concatenate([[0.0], beta])
    ev, _ = oracle_lancbis(alpha, b, b * b, -10.0, emax)
    n = len(alpha) - drop
    ev2, _ = oracle_lancbis(alpha[:n], b[:n + 1], (b * b)[:n + 1], -10.0, emax)
    return np.array([e for e in ev if np.min(np.abs(ev2 - e)) <= tol])


@pytest.mark.parametrize("name", CASES + REF_ONLY_CASES + ["cpu_workload"])
def test_lanczos_fp64_eigenvalues_match_reference(bsl, name):
    h, d, man, _ = make(bsl, name)
    ref = np.load(os.path.join(d, "ref_alpha_beta.npz"))
    niter = man["niter"]
    a, b, b2 = h.lanczos(niter)
    k = 20
    assert np.max(np.abs(a[:k] - ref["alpha"][:k])) <= 1e-10 * np.max(np.abs(ref["alpha"][:k]))
    assert np.max(np.abs(b[1:k + 1] - ref["beta"][:k])) <= 1e-10 * np.max(ref["beta"][:k])
    ev, er = bsl.good_eigenvalues(a, b, b2)
    levels = stable_levels(ref["alpha"], ref["beta"])
    assert len(levels) >= 3
    for e in levels:
        assert np.min(np.abs(ev - e)) <= CM_TOL_FP64, (e, np.min(np.abs(ev - e)) * KJ_TO_CM)
    h.close()


@pytest.mark.parametrize("engine", ["simt", "tensor"])
def test_lanczos_mixed_levels_within_1e3_cm(bsl, engine):
    h, d, man, _ = make(bsl, "cpu_workload")
    niter = man["niter"]
    a, b, b2 = h.lanczos(niter, start="normal", seed=0)
    # bound levels: the lowest 20 converged levels below 30 kJ/mol
    stable = stable_levels(a, b[1:], emax=30.0)
    h.set_precision("mixed")
    h.set_kinetic_engine(engine)
    am, bm, bm2 = h.lanczos(niter, start="normal", seed=0)
    evm, _ = bsl.good_eigenvalues(am, bm, bm2, -10.0, 40.0, unit_roundoff=bsl.MIXED_UNIT_ROUNDOFF,
                                  rel_noise=bsl.MIXED_REL_NOISE)
    low = np.sort(stable)[:20]
    assert len(low) >= 8
    dev = np.array([np.min(np.abs(evm - e)) for e in low])
    assert dev.max() <= CM_TOL_MIXED, dev.max() * KJ_TO_CM
    h.close()


def test_isoharmosc_analytic_levels(bsl):
    h, d, man, _ = make(bsl, "iso_n20_l2_all")
    a, b, b2 = h.lanczos(man["niter"])
    ev, _ = bsl.good_eigenvalues(a, b, b2)
    hbar, w, B = 0.0635077857002, 24.1, 0.709652722117881
    analytic = np.array(sorted({hbar * w * (n + 1.5) + B * l * (l + 1) for n in range(8) for l in range(3)}))
    assert abs(ev[0] - 1.5 * hbar * w) <= 5e-4
    for e in ev[:6]:
        assert np.min(np.abs(analytic - e)) <= 5e-4
    h.close()


def test_step_host_matches_oracle_loop(bsl):
    h, d, man, extra = make(bsl, "seed1_n6_l3_odd")
    D = h.basis_size
    vec = np.full(D, 1.0 / np.sqrt(D))
    rvec = np.zeros(D)
    alphas = []
    for _ in range(5):
        a, b, b2 = h.step_host(vec, rvec)
        alphas.append(a)
    ref = np.load(os.path.join(d, "ref_alpha_beta.npz"))
    assert np.max(np.abs(np.array(alphas) - ref["alpha"][:5])) <= 1e-10 * np.max(np.abs(ref["alpha"][:5]))
    h.close()


def test_step_host_pinned_buffers_match_pageable(bsl):
    """Page-locked vec/rvec are written by the step's last pass directly; the
    results are bit-identical to the copy path of ordinary host memory."""
    torch = pytest.importorskip("torch")
    h, d, man, extra = make(bsl, "seed1_n6_l3_odd")
    D = h.basis_size
    out = []
    for pinned in (False, True):
        if pinned:
            vec = torch.empty(D, dtype=torch.float64, pin_memory=True).numpy()
            rvec = torch.empty(D, dtype=torch.float64, pin_memory=True).numpy()
        else:
            vec, rvec = np.empty(D), np.empty(D)
        vec[:] = 1.0 / np.sqrt(D)
        rvec[:] = 0.0
        ab = [h.step_host(vec, rvec) for _ in range(4)]
        out.append((np.array(ab), vec.copy(), rvec.copy()))
    for x, y in zip(out[0], out[1]):
        assert np.array_equal(x, y)
    h.close()


def test_ritz_vectors_match_oracle(bsl):
    import ctypes as C
    from conftest import load_oracle, ptr
    h, d, man, extra = make(bsl, "seed1_n6_l3_odd")
    niter = 120
    a, b, b2 = h.lanczos(niter)
    ev, _ = bsl.good_eigenvalues(a, b, b2)
    ng = 2
    rows = bsl.tm_eigenvectors(a, b, b2, ev[:ng])
    R = h.ritz(niter, rows)
    cwd = os.getcwd()
    os.chdir(d)
    try:
        m = OracleModel(man["calculator"], "hv_input.txt", extra)
    finally:
        os.chdir(cwd)
    out = np.zeros(ng * m.D)
    load_oracle().orc_ritz(m.h, niter, ptr(np.ascontiguousarray(rows.reshape(-1))), ng, ptr(out), 8)
    out = out.reshape(ng, m.D)
    for n in range(ng):
        assert np.max(np.abs(R[n] - out[n])) <= 1e-6 * np.max(np.abs(out[n]))
        # Ritz vector is an eigenvector of H: ||H x - E x|| small
        x = R[n] / np.linalg.norm(R[n])
        u = np.zeros(h.basis_size)
        h.hv(x, u)
        keep = np.zeros(h.basis_size, bool)
        npts = h.basis_size // (h.params.l_max + 1) ** 2
        for s in full_indices(h):
            keep[s * npts:(s + 1) * npts] = True
        assert np.linalg.norm(u[keep] - ev[n] * x[keep]) <= 1e-4
    h.close()
    m.close()


def test_mixed_recurrence_tracks_fp64(bsl):
    """Mixed path (FP32 blocks and kinetic, double-float Lanczos buffers): the
    first 40 alpha/beta agree with the FP64 path to 1e-5 relative."""
    h, d, man, _ = make(bsl, "cpu_workload")
    a, b, _ = h.lanczos(40)
    h.set_precision("mixed")
    am, bm, _ = h.lanczos(40)
    scale = np.max(np.abs(a))
    assert np.max(np.abs(am - a)) <= 1e-5 * scale
    assert np.max(np.abs(bm[1:] - b[1:])) <= 1e-5 * scale
    h.close()


def test_ritz_vectors_mixed_are_eigenvectors(bsl):
    """Loop 2 on the double-float buffers: Ritz vectors of the mixed run are
    eigenvectors of H (residual <= 1e-4) and overlap the FP64 ones to 1e-6."""
    h, d, man, extra = make(bsl, "seed1_n6_l3_odd")
    niter = 120

    def ritz_pair(precision):
        h.set_precision(precision)
        a, b, b2 = h.lanczos(niter)
        mixed = precision == "mixed"
        ev, _ = bsl.good_eigenvalues(a, b, b2, unit_roundoff=bsl.MIXED_UNIT_ROUNDOFF if mixed else None,
                                     rel_noise=bsl.MIXED_REL_NOISE if mixed else None)
        rows = bsl.tm_eigenvectors(a, b, b2, ev[:1])
        x = h.ritz(niter, rows)[0]
        return ev[0], x / np.linalg.norm(x)

    e64, x64 = ritz_pair("fp64")
    em, xm = ritz_pair("mixed")
    assert abs(em - e64) <= CM_TOL_MIXED
    assert 1.0 - abs(float(x64 @ xm)) <= 1e-6
    h.set_precision("fp64")
    u = np.zeros(h.basis_size)
    h.hv(xm, u)
    keep = np.zeros(h.basis_size, bool)
    npts = h.basis_size // (h.params.l_max + 1) ** 2
    for s in full_indices(h):
        keep[s * npts:(s + 1) * npts] = True
    assert np.linalg.norm(u[keep] - em * xm[keep]) <= 1e-4
    h.close()


def test_lanczos_batch_matches_separate_runs(bsl):
    """Three problems (two grids and symmetry blocks, both precisions' default
    engines) in one batched call give bit-identical alpha/beta to separate runs."""
    names = ["seed1_n6_l3_odd", "seed0_n5_l4_even", "cpu_workload"]
    hs = [make(bsl, n)[0] for n in names]
    hs[2].set_precision("mixed")
    niter = 60
    sep = [h.lanczos(niter, start="normal", seed=3) for h in hs]
    bat = bsl.lanczos_batch(hs, niter, start="normal", seed=3)
    for (a, b, b2), (ab, bb, b2b) in zip(sep, bat):
        assert np.array_equal(a, ab) and np.array_equal(b, bb) and np.array_equal(b2, b2b)
    for h in hs:
        h.close()
