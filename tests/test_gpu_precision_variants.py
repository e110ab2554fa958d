"""Precision variants of the mixed path (bsl_set_kinetic_slices,
bsl_set_potential_format) on reference fixtures: H v against the FP64 path
with 1-4 tensor-core kinetic slices, with BF16 potential blocks and with FP32
blocks instead of the default spherical-harmonic coefficients, the default
configuration unchanged by a round trip through the variants (the cached
iteration graph follows every switch), and the refusals."""
import os

import numpy as np
import pytest

from conftest import case_info, load_package

pytestmark = pytest.mark.gpu


def hamiltonian(bsl, name):
    d, man, extra = case_info(name)
    cwd = os.getcwd()
    os.chdir(d)
    try:
        return bsl.Hamiltonian("hv_input.txt", man["calculator"], extra_input=extra, precision="fp64")
    finally:
        os.chdir(cwd)


def rel(a, b):
    return np.max(np.abs(a - b)) / np.max(np.abs(b))


def test_kinetic_slices_and_bf16_blocks():
    bsl = load_package()
    h = hamiltonian(bsl, "seed0_n5_l4_even")  # 15 functions: both block formats
    try:
        v = np.random.default_rng(5).standard_normal(h.basis_size)
        u64 = np.zeros(h.basis_size)
        h.hv(v, u64)
        h.set_precision("mixed")
        default_format = h.potential_format()
        assert default_format == "gaunt" and 0 <= h.gaunt_residual() <= 1e-12
        a0, b0, _ = h.lanczos(40)
        err = {}
        for sl in (1, 2, 3, 4):
            h.set_kinetic_slices(sl)
            u = np.zeros(h.basis_size)
            h.hv(v, u)
            err[sl] = rel(u, u64)
            h.lanczos(24)  # the graph of every variant is captured and replayed
        # the kinetic error falls by ~2^-9 per slice until the FP32 blocks dominate
        assert err[1] <= 2e-2 and err[2] <= 1e-4 and err[3] <= 1e-6 and err[4] <= 1e-7, err
        assert err[1] > 10 * err[2] > 100 * err[3], err
        h.set_potential_format("bf16")
        ub = np.zeros(h.basis_size)
        h.hv(v, ub)
        eb = rel(ub, u64)
        assert 1e-5 < eb <= 1e-2, eb
        h.lanczos(24)
        h.set_potential_format("fp32")
        uf = np.zeros(h.basis_size)
        h.hv(v, uf)
        assert rel(uf, u64) <= 1e-7, rel(uf, u64)
        h.set_potential_format(default_format)
        a1, b1, _ = h.lanczos(40)
        assert np.array_equal(a0, a1) and np.array_equal(b0, b1)
        with pytest.raises(bsl.BslError):
            h.set_kinetic_slices(5)
    finally:
        h.close()


def test_bf16_blocks_need_a_specialised_block_size():
    bsl = load_package()
    h = hamiltonian(bsl, "seed1_n6_l3_odd")  # 10 functions
    try:
        with pytest.raises(bsl.BslError) as e:
            h.set_potential_format("bf16")
        assert e.value.code == bsl.ERR_UNSUPPORTED
    finally:
        h.close()
