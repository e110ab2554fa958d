"""The spherical-harmonic form of the potential blocks (bsl_gaunt.h, written
by boundstate-lanczos_gb300/gen_gaunt.py), checked on the CPU:

* the committed header is what the generator writes;
* the oracle's FP64 blocks of reference fixtures and of a generated case at
  the benchmark's angular grid (40 theta x 70 phi, odd l <= 5) are reproduced
  by the expansion to 1e-12 of their largest element: nn (nn + 1) / 2 block
  elements per point are the nc coefficients c_k(p) exactly (the identity holds
  node by node of the quadrature).
"""
import importlib.util
import os
import subprocess
import sys

import numpy as np
import pytest

from conftest import PKG_DIR, OracleModel, case_info, load_inputs

CALC = "linRotCartSph_NoQuad_ContGrid_Alavi_SPCE"


def generator():
    spec = importlib.util.spec_from_file_location("bsl_gen_gaunt", os.path.join(PKG_DIR, "gen_gaunt.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_header_is_generated():
    r = subprocess.run([sys.executable, os.path.join(PKG_DIR, "gen_gaunt.py"), "--check"])
    assert r.returncode == 0, "csrc/bsl_gaunt.h differs from gen_gaunt.py's output"


def check_blocks(m, lmax, sym):
    gen = generator()
    fun, pairs, lm, G = gen.expansion(lmax, sym)
    full = [(l, mm) for mm in range(-lmax, lmax + 1) for l in range(abs(mm), lmax + 1)]
    pos = [full.index(f) for f in fun]
    nn_full = (lmax + 1) ** 2
    vb = m.vblocks().reshape(-1, nn_full, nn_full)
    V = np.stack([vb[:, pos[a], pos[b]] for a, b in pairs], axis=1)  # [N, ntri]
    c, *_ = np.linalg.lstsq(G, V.T, rcond=None)
    resid = np.abs(V.T - G @ c).max()
    assert resid <= 1e-12 * np.abs(V).max(), resid
    return len(lm), len(pairs)


@pytest.mark.parametrize("name,lmax,sym", [("seed1_n6_l3_odd", 3, "Odd"), ("seed0_n5_l4_even", 4, "Even")])
def test_fixture_blocks_are_the_expansion(in_case_dir, name, lmax, sym):
    d, man, extra = in_case_dir(name)
    m = OracleModel(man["calculator"], "hv_input.txt", extra, threads=4)
    try:
        check_blocks(m, lmax, sym)
    finally:
        m.close()


def test_benchmark_angular_grid_blocks_are_the_expansion(tmp_path):
    inp = load_inputs()
    cage = os.path.join(str(tmp_path), "cage.xyz")
    inp.write_cage_xyz(cage, inp.dodecahedral_cage(1))
    hv = os.path.join(str(tmp_path), "hv.txt")
    inp.write_hv_input(hv, inp.hv_fields(5, 0.08, 5, 40, 35, cage, "gaunt", "Odd"))
    m = OracleModel(CALC, hv, threads=4)
    try:
        nc, ntri = check_blocks(m, 5, "Odd")
        assert (nc, ntri) == (66, 231)
    finally:
        m.close()
