"""The launch-shape autotuner (bsl_autotune) on a single problem and on a
grouped batch: it returns shapes in range, the tuned runs agree with the
default ones (the shapes only split the same sums differently: the first 10
alpha/beta within 1e-12 of max |alpha|, all 40 within 1e-8), and a second call with the
same problem sizes takes the cached choice."""
import os
import time

import numpy as np
import pytest

from conftest import load_inputs, load_package

pytestmark = pytest.mark.gpu
CALC = "linRotCartSph_NoQuad_ContGrid_Alavi_SPCE"


def problem(bsl, tmp, k, n, lmax, sym):
    inp = load_inputs()
    cage = os.path.join(tmp, "cage.xyz")
    if not os.path.exists(cage):
        inp.write_cage_xyz(cage, inp.dodecahedral_cage(1))
    hv = os.path.join(tmp, "hv%d.txt" % k)
    inp.write_hv_input(hv, inp.hv_fields(n, 0.08, lmax, 8, 8, cage, "tune%d" % k, sym))
    return bsl.Hamiltonian(hv, CALC, precision="mixed")


def test_autotune_single_and_batch(tmp_path):
    bsl = load_package()
    h = problem(bsl, str(tmp_path), 0, 16, 5, "Odd")
    g = problem(bsl, str(tmp_path), 1, 12, 4, "Even")
    try:
        a0, b0, _ = h.lanczos(40, start="normal", seed=2)
        vs, up, ms = bsl.autotune([h], 64)
        assert 1 <= vs <= 3 and 1 <= up <= 3 and ms > 0
        a1, b1, _ = h.lanczos(40, start="normal", seed=2)
        scale = np.max(np.abs(a0))
        assert np.max(np.abs(a1[:10] - a0[:10])) <= 1e-12 * scale
        assert np.max(np.abs(b1[:11] - b0[:11])) <= 1e-12 * scale
        assert np.max(np.abs(a1 - a0)) <= 1e-8 * scale and np.max(np.abs(b1 - b0)) <= 1e-8 * scale
        t0 = time.perf_counter()
        assert bsl.autotune([h], 64) == (vs, up, ms)  # cached
        assert time.perf_counter() - t0 < 0.5
        vsb, upb, msb = bsl.autotune([h, g], 64)
        assert 1 <= vsb <= 3 and 1 <= upb <= 3 and msb > 0
        runs = bsl.lanczos_batch([h, g], 40, start="normal", seed=2)
        assert np.max(np.abs(runs[0][0][:10] - a0[:10])) <= 1e-12 * scale
    finally:
        h.close()
        g.close()
