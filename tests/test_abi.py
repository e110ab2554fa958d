"""C ABI: the library loads and exports every entry point of include/bsl.h;
input parsing and error reporting; the host-side Cullum-Willoughby tail
against the oracle's restatement of the Fortran.  No GPU needed."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from conftest import GOLDEN, REPO, case_info, load_oracle, load_package, oracle_lancbis, ptr


@pytest.fixture(scope="module")
def bsl():
    pkg = load_package()
    if not os.path.exists(pkg.LIB_PATH):
        import importlib.util
        spec = importlib.util.spec_from_file_location("bsl_build", os.path.join(REPO, "boundstate-lanczos_gb300",
                                                                              "build.py"))
        b = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(b)
        b.build()
    return pkg


def header_functions():
    txt = open(os.path.join(REPO, "include", "bsl.h")).read()
    return sorted(set(re.findall(r"\b(bsl_[a-z0-9_]+)\s*\(", txt)))


def test_exports_every_declared_symbol(bsl):
    L = bsl.lib()
    names = header_functions()
    assert len(names) >= 20
    for n in names:
        assert hasattr(L, n), n


def test_parse_hv_input_fields(bsl, in_case_dir):
    in_case_dir("cpu_workload")
    p = bsl.parse_hv_input("hv_input.txt")
    assert (p.nx, p.ny, p.nz, p.l_max, p.theta_points, p.phi_points) == (15, 15, 15, 4, 12, 12)
    assert p.x_max == 0.08 and p.symmetry == bsl.SYM["Even"]
    assert p.geometry_filename == b"cage_seed0.xyz"
    assert p.ceiling_potential == 18.0 and p.rotational_constant == 0.709648713


def test_parse_errors(bsl, tmp_path, in_case_dir):
    with pytest.raises(bsl.BslError) as e:
        bsl.parse_hv_input(str(tmp_path / "missing.txt"))
    assert e.value.code == bsl.ERR_INPUT and "could not be opened" in str(e.value)
    d, _, _ = in_case_dir("cpu_workload")
    txt = open("hv_input.txt").read()
    bad = tmp_path / "trunc.txt"
    bad.write_text("\n".join(txt.split("\n")[:10]))
    with pytest.raises(bsl.BslError) as e:
        bsl.parse_hv_input(str(bad))
    assert "truncated" in str(e.value)
    sym = tmp_path / "sym.txt"
    sym.write_text(txt.replace("rotationalSymmetry(All/Even/Odd)= Even", "rotationalSymmetry(All/Even/Odd)= Both"))
    with pytest.raises(bsl.BslError) as e:
        bsl.parse_hv_input(str(sym))
    assert "Symmeterizer" in str(e.value)
    big = tmp_path / "big.txt"
    big.write_text(txt.replace("x_max(nm)= 0.08\n", "x_max(nm)= 0.5\n", 1))
    with pytest.raises(bsl.BslError) as e:
        bsl.parse_hv_input(str(big))
    assert "potential universe" in str(e.value)
    geo = tmp_path / "geo.txt"
    geo.write_text(txt.replace("cage_seed0.xyz", "no_such_cage.xyz"))
    with pytest.raises(bsl.BslError) as e:
        bsl.parse_hv_input(str(geo))
    assert "could not be opened" in str(e.value)
    with pytest.raises(bsl.BslError):
        bsl.hv_interface_setup("linRotCartSph_NoSuchCalculator")


def test_calculator_strings_and_coulomb_input(bsl, tmp_path):
    """Every NoQuad HvCalculator string of the reference registry
    (interface.cpp:90-246), with and without the _GB300 suffix, maps to its
    potential; the Coulomb potential file (argv[3]) is read in token order."""
    import ctypes as C
    L = bsl.lib()
    for name, pot in bsl.CALCULATORS.items():
        out = C.c_int(-1)
        assert L.bsl_calculator_potential(name.encode(), C.byref(out)) == bsl.OK, name
        assert out.value == pot, name
    for base, pot in (("linRotCartSph_NoQuad_Alavi_SPCE", bsl.POT_POINT_ALAVI_SPCE),
                      ("linRotCartSph_NoQuad_Alavi_TIP4P", bsl.POT_POINT_ALAVI_TIP4P),
                      ("linRotCartSph_NoQuad_Coulomb", bsl.POT_COULOMB)):
        assert bsl.CALCULATORS[base] == bsl.CALCULATORS[base + "_GB300"] == pot
    d, man, extra = case_info("coulomb_n9_l2_all")
    p = bsl.HvParams()
    assert L.bsl_parse_coulomb_input(os.path.join(d, extra).encode(), C.byref(p)) == bsl.OK
    assert (p.coulomb_centre_charge, p.coulomb_mol_charge, p.coulomb_ceiling) == (0.1, -0.1, -20.0)
    assert p.potential == bsl.POT_COULOMB
    bad = tmp_path / "c.txt"
    bad.write_text("#\n#\ncentreCharge= 1.0\n")
    assert L.bsl_parse_coulomb_input(str(bad).encode(), C.byref(p)) == bsl.ERR_INPUT


@pytest.mark.parametrize("name", ["cage11_n10_l3_all", "seed1_n6_l3_odd", "seed0_n5_l4_even", "iso_n20_l2_all",
                                  "cpu_workload", "tip4p_seed1_n6_l3_odd", "point_cage11_n10_l2_odd",
                                  "point_tip4p_seed1_n6_l3_odd", "coulomb_n9_l2_all"])
def test_tail_matches_oracle(bsl, name):
    d, man, _ = case_info(name)
    ref = np.load(os.path.join(d, "ref_alpha_beta.npz"))
    b = np.concatenate([[0.0], ref["beta"]])
    ev, er = bsl.good_eigenvalues(ref["alpha"], b, b * b)
    ev0, er0 = oracle_lancbis(ref["alpha"], b, b * b)
    assert len(ev) == len(ev0)
    assert np.array_equal(ev, ev0)
    assert np.allclose(er, er0, rtol=1e-12, atol=1e-300)


def test_tail_unit_roundoff(bsl):
    """bsl_good_eigenvalues_unit at the FP64 unit roundoff is the reference tail;
    a larger unit merges copies of a level that scatter (as under an inexact H v)."""
    d, man, _ = case_info("cpu_workload")
    ref = np.load(os.path.join(d, "ref_alpha_beta.npz"))
    a = ref["alpha"]
    b = np.concatenate([[0.0], ref["beta"]])
    ev, er = bsl.good_eigenvalues(a, b, b * b)
    eu, eru = bsl.good_eigenvalues(a, b, b * b, unit_roundoff=2.0 * 1.1102230246251565e-16)
    assert np.array_equal(ev, eu) and np.array_equal(er, eru)
    # two blocks: level 1.0 once, and level 2.0 as two copies 1e-9 apart joined by a
    # tiny coupling; the FP64 tolerance sees two simple eigenvalues, a unit of 1e-12 one double
    rng = np.random.default_rng(5)
    m = 60
    diag = np.concatenate([[1.0, 2.0, 2.0 + 1e-9], 5.0 + rng.random(m - 3)])
    off = np.concatenate([[0.0], [1e-3, 1e-13], 0.5 + 0.1 * rng.random(m - 3)])
    e64, _ = bsl.good_eigenvalues(diag, off, off * off, 0.0, 3.0)
    e12, _ = bsl.good_eigenvalues(diag, off, off * off, 0.0, 3.0, unit_roundoff=1e-12)
    near2 = lambda e: int(np.sum(np.abs(e - 2.0) < 1e-6))
    assert near2(e12) <= near2(e64)


def test_tm_eigenvectors_match_oracle(bsl):
    d, man, _ = case_info("seed1_n6_l3_odd")
    ref = np.load(os.path.join(d, "ref_alpha_beta.npz"))
    a = ref["alpha"]
    b = np.concatenate([[0.0], ref["beta"]])
    ev, _ = bsl.good_eigenvalues(a, b, b * b)
    ng = min(4, len(ev))
    rows = bsl.tm_eigenvectors(a, b, b * b, ev[:ng])
    L = load_oracle()
    out = np.zeros(len(a) * ng)
    L.orc_trivec(len(a), ptr(a), ptr(b), ptr(b * b), ptr(np.ascontiguousarray(ev[:ng])), ng, ptr(out))
    assert np.allclose(rows.reshape(-1), out, rtol=0, atol=1e-14)
    # eigenvector property on the leading block: T y = E y
    for n in range(ng):
        y = rows[n]
        m = np.max(np.nonzero(np.abs(y) > 0)[0]) + 1
        T = np.diag(a[:m]) + np.diag(b[1:m], 1) + np.diag(b[1:m], -1)
        assert np.linalg.norm(T @ y[:m] - ev[n] * y[:m]) <= 1e-6 * max(1.0, abs(ev[n]))


def test_tail_breakdown_free_on_tiny_matrix(bsl):
    # 1x1 and 2x2 Lanczos matrices
    a = np.array([1.5, -0.5])
    b = np.array([0.0, 0.25, 0.1])
    ev, er = bsl.good_eigenvalues(a, b, b * b, -10, 10)
    w = np.linalg.eigvalsh(np.array([[1.5, 0.25], [0.25, -0.5]]))
    for e in ev:
        assert np.min(np.abs(w - e)) <= 1e-12


def _lanczos_limits(d):
    lines = open(os.path.join(d, "lanczos_input.txt")).read().split("\n")
    vals = {l.split("=")[0]: l.split("=")[1].strip() for l in lines if "=" in l}
    return float(vals["EigenvalueOpenLowerLimit(kJ/mol)"]), float(vals["EigenvalueClosedUpperLimit(kJ/mol)"])


@pytest.mark.parametrize("name", ["cage11_n10_l3_all", "seed1_n6_l3_odd", "seed0_n5_l4_even", "iso_n20_l2_all",
                                  "cpu_workload", "tip4p_seed1_n6_l3_odd", "point_cage11_n10_l2_odd",
                                  "point_tip4p_seed1_n6_l3_odd", "coulomb_n9_l2_all"])
def test_boundstates_file_matches_reference(bsl, name, tmp_path):
    """boundstates.txt written from the tail on the reference's alpha/beta has the
    reference's layout, states and eigenvalues (the stored alpha/beta are the
    reference's printed values, so the last digits can move: 1e-10 relative); the
    error column depends on the random start of the inverse iteration and is
    compared to a factor 10."""
    d, man, _ = case_info(name)
    ref = np.load(os.path.join(d, "ref_alpha_beta.npz"))
    b = np.concatenate([[0.0], ref["beta"]])
    emin, emax = _lanczos_limits(d)
    ev, er = bsl.good_eigenvalues(ref["alpha"], b, b * b, emin, emax)
    rlines = open(os.path.join(d, "ref_boundstates.txt")).read().split("\n")
    descr = rlines[1].split("simulation ", 1)[1]
    bsl.write_boundstates(str(tmp_path), descr, ev, er)
    mlines = open(os.path.join(tmp_path, "boundstates.txt")).read().split("\n")
    assert len(mlines) == len(rlines)
    assert mlines[:4] == rlines[:4]
    for m, r in zip(mlines[4:], rlines[4:]):
        mf, rf = m.split(), r.split()
        assert mf[:1] == rf[:1]
        if mf:
            assert len(mf[1]) == len(rf[1]) and float(mf[1]) == pytest.approx(float(rf[1]), rel=1e-10, abs=1e-12)
            em, erf = float(mf[2]), float(rf[2])
            assert (em < 1e-12 and erf < 1e-12) or abs(np.log10(max(em, 1e-300) / max(erf, 1e-300))) < 1.0
    zpe = open(os.path.join(tmp_path, "states_zpe.txt")).read().split("\n")
    assert zpe[3] == "Zero Point Energy = %.15e kJ/mol" % ev[0]
    assert float(zpe[-2].split()[1]) == pytest.approx(ev[-1] - ev[0], rel=1e-15)


def test_lv_and_ritz_file_layout(bsl, tmp_path):
    """lv and eigVecFile.txt follow the reference's layout (squared coefficients
    with running norms; one row per basis index)."""
    d, man, _ = case_info("seed1_n6_l3_odd")
    ref = np.load(os.path.join(d, "ref_alpha_beta.npz"))
    a = ref["alpha"]
    b = np.concatenate([[0.0], ref["beta"]])
    ev, _ = bsl.good_eigenvalues(a, b, b * b)
    rows = bsl.tm_eigenvectors(a, b, b * b, ev[:2])
    bsl.write_tm_vectors(str(tmp_path), "case", rows)
    lv = open(os.path.join(tmp_path, "lv")).read().split("\n")
    assert lv[0] == "" and lv[2] == "Number of Eigenvectors: 2"
    assert lv[3] == "Iteration | Coefficient Squared | Cumulative Norm "
    body = [l.split() for l in lv[4:] if l.strip()]
    assert len(body) == len(a)
    last = np.array([float(x) for x in body[-1][1:]])
    assert np.allclose(last[1::2], np.sum(rows ** 2, axis=1), rtol=1e-14)
    ritz = np.random.default_rng(1).standard_normal((2, 7))
    bsl.write_ritz_vectors(str(tmp_path), "case", ritz)
    ev_lines = open(os.path.join(tmp_path, "eigVecFile.txt")).read().split("\n")
    assert ev_lines[2] == "Number of Ritz vectors: 2"
    assert ev_lines[4] == "0 %.15e %.15e " % (ritz[0, 0], ritz[1, 0])
    assert len([l for l in ev_lines[4:] if l.strip()]) == 7


def test_rigid_body_chain_rule_matches_finite_differences(bsl):
    """bsl_rigid_body_gradient: d(g . sites)/d(centre, angles) against central
    differences of bsl_cage_sites (host only)."""
    cm, ea = bsl.read_cage_xyz(os.path.join(case_info("seed1_n6_l3_odd")[0], "cage_seed1.xyz"))
    rng = np.random.default_rng(2)
    g = rng.standard_normal((2, 3 * cm.shape[0], 3))
    dcm, dea = bsl.rigid_body_gradient(cm, ea, g)

    def f(c, e, n):
        return float(np.sum(g[n] * bsl.cage_sites(c, e)[0]))

    h = 1e-6
    for n in range(2):
        for m, k in [(0, 0), (3, 1), (7, 2), (19, 0)]:
            cp, cq = cm.copy(), cm.copy()
            cp[m, k] += h
            cq[m, k] -= h
            assert (f(cp, ea, n) - f(cq, ea, n)) / (2 * h) == pytest.approx(dcm[n, m, k], rel=1e-6, abs=1e-9)
            ep, eq = ea.copy(), ea.copy()
            ep[m, k] += h
            eq[m, k] -= h
            assert (f(cm, ep, n) - f(cm, eq, n)) / (2 * h) == pytest.approx(dea[n, m, k], rel=1e-6, abs=1e-9)


def test_cage_sites_charges(bsl):
    cm, ea = bsl.read_cage_xyz(os.path.join(case_info("seed1_n6_l3_odd")[0], "cage_seed1.xyz"))
    xyz, q = bsl.cage_sites(cm, ea)
    assert xyz.shape == (60, 3) and np.allclose(q[:3], [-0.8476, 0.4238, 0.4238])
    assert abs(q.sum()) < 1e-12
    # the O-H distance of SPC/E (1 A) in every molecule
    for m in range(20):
        assert np.linalg.norm(xyz[3 * m + 1] - xyz[3 * m]) == pytest.approx(0.1, rel=1e-8)
    qs = np.arange(60, dtype=float)
    assert np.array_equal(bsl.cage_sites(cm, ea, qs)[1], qs)


def test_null_handles_and_bad_arguments_return_status(bsl):
    """Every entry point given a null handle returns BSL_ERR_STATE ("null
    handle"); null buffers and bad sizes give BSL_ERR_INPUT; size queries give
    -1.  None of them touches the GPU or exits the process."""
    L = bsl.lib()
    state = {
        "bsl_hv_apply": lambda: L.bsl_hv_apply(None, None, None),
        "bsl_hv_apply_device": lambda: L.bsl_hv_apply_device(None, None, None, None),
        "bsl_lanczos_run": lambda: L.bsl_lanczos_run(None, 10, 0, 0, None, None, None),
        "bsl_lanczos_step_host": lambda: L.bsl_lanczos_step_host(None, None, None, None, None, None),
        "bsl_ritz_vectors": lambda: L.bsl_ritz_vectors(None, 10, None, 1, None),
        "bsl_ritz_vectors_start": lambda: L.bsl_ritz_vectors_start(None, 10, 0, 0, None, 1, None),
        "bsl_set_precision": lambda: L.bsl_set_precision(None, 0),
        "bsl_set_kinetic_engine": lambda: L.bsl_set_kinetic_engine(None, 0),
        "bsl_hf_gradient": lambda: L.bsl_hf_gradient(None, 1, None, None, None, None),
        "bsl_last_run_ms_per_iter": lambda: L.bsl_last_run_ms_per_iter(None, None),
        "bsl_copy_vgrid": lambda: L.bsl_copy_vgrid(None, None, None),
        "bsl_copy_vblocks": lambda: L.bsl_copy_vblocks(None, None),
    }
    for name, call in state.items():
        assert call() == bsl.ERR_STATE, name
        assert b"null handle" in L.bsl_last_error(), name
    inputs = {
        "bsl_hv_prep": lambda: L.bsl_hv_prep(None, None),
        "bsl_lanczos_run_batch": lambda: L.bsl_lanczos_run_batch(None, 0, 10, 0, 0, None, None, None),
        "bsl_good_eigenvalues": lambda: L.bsl_good_eigenvalues(0, None, None, None, -1.0, 1.0, None, None, None),
        "bsl_tm_eigenvectors": lambda: L.bsl_tm_eigenvectors(0, None, None, None, None, 0, None),
    }
    for name, call in inputs.items():
        assert call() == bsl.ERR_INPUT, name
    for name in ("bsl_basis_size", "bsl_packed_size", "bsl_packed_nn", "bsl_vgrid_size", "bsl_vblock_size",
                 "bsl_kinetic_engine", "bsl_launches_per_iteration"):
        assert getattr(L, name)(None) == -1, name
    assert L.bsl_stream(None) is None


def test_prep_without_a_gpu_fails_loudly(bsl, in_case_dir):
    """No CPU fallback: where no GPU is usable, preparing H returns
    BSL_ERR_CUDA with the CUDA runtime's text."""
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    in_case_dir("seed1_n6_l3_odd")
    with pytest.raises(bsl.BslError) as e:
        bsl.Hamiltonian("hv_input.txt")
    assert e.value.code == bsl.ERR_CUDA and "CUDA" in str(e.value)


def test_input_writers_round_trip_through_the_parser(bsl, tmp_path):
    """inputs.py writes HvInputFiles the C ABI parser reads back field by field
    (the benchmark's 54^3 workload and a point-grid universe)."""
    from conftest import load_inputs
    inp = load_inputs()
    cage = str(tmp_path / "cage.xyz")
    inp.write_cage_xyz(cage, inp.dodecahedral_cage(1))
    cfg = inp.CONFIG_METRIC
    path = str(tmp_path / "hv_input.txt")
    inp.write_hv_input(path, inp.hv_fields(cfg["n"], cfg["x_max"], cfg["l_max"], cfg["theta_points"],
                                           cfg["phi_points"], cage, "metric", cfg["sym"]))
    p = bsl.parse_hv_input(path)
    assert (p.nx, p.ny, p.nz, p.l_max) == (54, 54, 54, 5)
    assert (p.theta_points, p.phi_points) == (cfg["theta_points"], cfg["phi_points"])
    assert p.x_max == p.y_max == p.z_max == cfg["x_max"]
    assert (p.pnx, p.px_max) == (54, cfg["x_max"])
    assert p.symmetry == bsl.SYM[cfg["sym"]] and p.geometry_filename == cage.encode()
    assert p.total_mass == 2.01588 and p.rotational_constant == 0.709648713 and p.ceiling_potential == 18.0
    inp.write_hv_input(path, inp.hv_fields(6, 0.08, 3, 8, 7, cage, "point", "Odd", point_grid=(13, 0.1)))
    p = bsl.parse_hv_input(path)
    assert (p.nx, p.pnx, p.pny, p.pnz) == (6, 13, 13, 13) and p.px_max == p.pz_max == 0.1
    # the generated cage: one water at each vertex of the dodecahedron
    waters = inp.dodecahedral_cage(1)
    assert len(waters) == 20


def test_every_exported_c_symbol_is_declared(bsl):
    """The library's extern "C" exports are exactly the entry points that
    include/bsl.h declares (no undeclared C API); the three reference-signature
    functions of include/bsl_reference_shim.h are exported with C++ linkage,
    and nothing else (internal helpers have hidden visibility)."""
    import shutil
    import subprocess
    nm = shutil.which("nm")
    if nm is None:
        pytest.skip("nm not available")
    lib_path = os.path.join(REPO, "boundstate-lanczos_gb300", "libbsl_gb300.so")
    out = subprocess.run([nm, "-D", "--defined-only", lib_path], capture_output=True, text=True, check=True).stdout
    text = [ln.split()[-1] for ln in out.splitlines() if len(ln.split()) == 3 and ln.split()[1] == "T"]
    c_exports = {s for s in text if s.startswith("bsl_")}
    assert c_exports == set(header_functions())
    cpp = [s for s in text if s.startswith("_Z")]
    for name in ("bsl_reference_storage", "Hv_Prep_linRotCartSph_NoQuad_GB300", "Hv_linRotCartSph_NoQuad_GB300"):
        assert sum(name in s for s in cpp) == 1, name
    # internal helpers are built with hidden visibility: nothing else is exported
    assert len(cpp) == 3, cpp
    assert not [s for s in text if not s.startswith("bsl_") and not s.startswith("_Z")]
