"""Runs of every length on the graph-replayed fused iteration: a Lanczos run of
n iterations launches n // 32 replays of the 32-iteration graph and n % 32
direct iterations, each run starts with the block product of the start
vector, and the beta that the last iteration leaves pending is finished by a
closing kernel.  The kernels are deterministic, so the alpha/beta of an
n-iteration run must equal the first n of a longer run bit for bit, whatever
split of graph replays and direct launches n gives; and they follow the FP64
path (first 6 within 1e-6 of max |alpha|)."""
import os

import numpy as np
import pytest

from conftest import case_info, load_package

pytestmark = pytest.mark.gpu


def test_every_run_length_is_a_prefix_of_a_longer_run():
    bsl = load_package()
    d, man, extra = case_info("seed1_n6_l3_odd")
    cwd = os.getcwd()
    os.chdir(d)
    try:
        h = bsl.Hamiltonian("hv_input.txt", man["calculator"], extra_input=extra, precision="fp64")
    finally:
        os.chdir(cwd)
    try:
        a64, b64, _ = h.lanczos(72, start="normal", seed=5)
        h.set_precision("mixed")
        assert h.kinetic_engine() == "tensor"
        A, B, B2 = h.lanczos(72, start="normal", seed=5)
        scale = np.max(np.abs(a64))
        assert np.max(np.abs(A[:6] - a64[:6])) <= 1e-6 * scale
        assert np.max(np.abs(B[1:7] - b64[1:7])) <= 1e-6 * scale
        for n in (1, 2, 31, 32, 33, 40, 64, 65, 71):
            a, b, b2 = h.lanczos(n, start="normal", seed=5)
            assert np.array_equal(a, A[:n]), n
            assert np.array_equal(b, B[:n + 1]) and np.array_equal(b2, B2[:n + 1]), n
    finally:
        h.close()
