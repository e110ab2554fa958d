"""The grids the benchmarks run on, checked against the oracle: edges of 27, 33
and 41 points (the batched small problems) and 54 points (the metric
problem), odd l <= 5 (21 functions, the benchmark's block), over +-0.4 A
with the generated SPC/E cage (seed 1).  The angular grid is cut to 8 theta x
16 phi so that the CPU oracle finishes in seconds at these sizes; the kernels
under test (tensor-core kinetic with its exact slicing at the largest class
sums, the potential-block stream at the full tile count, the FP64 path) do not
depend on the angular grid, which only enters the potential blocks.

Tolerances: FP64 H v against the oracle <= 1e-10 relative (max abs / max abs);
alpha_1 against the oracle's <= 1e-14 and the first 20 FP64 alpha/beta <= 2e-10
of max |alpha|;
mixed H v of both kinetic engines against FP64 <= 2e-6; the first 20 mixed
alpha/beta against FP64 <= 1e-6 of max |alpha|.
"""
import os

import numpy as np
import pytest

from conftest import OracleModel, load_inputs, load_package

pytestmark = pytest.mark.gpu
CALC = "linRotCartSph_NoQuad_ContGrid_Alavi_SPCE"


def rel(a, b):
    return np.max(np.abs(a - b)) / np.max(np.abs(b))


@pytest.mark.parametrize("n", [27, 33, 41, 54])
def test_metric_and_batch_grids_match_oracle(tmp_path, n):
    bsl = load_package()
    inp = load_inputs()
    cage = os.path.join(str(tmp_path), "cage.xyz")
    inp.write_cage_xyz(cage, inp.dodecahedral_cage(1))
    hv = os.path.join(str(tmp_path), "hv_input.txt")
    inp.write_hv_input(hv, inp.hv_fields(n, 0.08, 5, 8, 8, cage, "grid_edge_%d" % n, "Odd"))
    h = bsl.Hamiltonian(hv, CALC, precision="fp64")
    m = OracleModel(CALC, hv, threads=os.cpu_count() or 8)
    try:
        assert h.basis_size == m.D and h.nn == 21
        v = np.random.default_rng(n).standard_normal(h.basis_size)
        u = np.zeros(h.basis_size)
        h.hv(v, u)
        err64 = rel(u, m.hv(v))
        assert err64 <= 1e-10, err64
        a, b, _ = h.lanczos(20)
        ao, bo, _ = m.lanczos(20)
        scale = np.max(np.abs(ao))
        ea, eb = np.abs(a - ao) / scale, np.abs(b[1:] - bo[1:]) / scale
        # alpha_1 = v.Hv agrees to rounding (2e-16 measured at 54^3); from the
        # second iteration on, the recurrence amplifies the rounding differences
        # of the two FP64 summation orders (FMA-contracted on the GPU, the
        # reference's serial sums in the oracle) ~1e5-fold from the uniform start
        # (1.8e-11 at alpha_2, at most 1.1e-10 over the first 20 at 54^3, measured)
        assert ea[0] <= 1e-14, ea[0]
        assert ea.max() <= 2e-10 and eb.max() <= 2e-10, (ea, eb)
        h.set_precision("mixed")
        assert h.kinetic_engine() == "tensor"
        for engine in ("tensor", "simt"):
            h.set_kinetic_engine(engine)
            um = np.zeros(h.basis_size)
            h.hv(v, um)
            errm = rel(um, u)
            assert errm <= 2e-6, (engine, errm)
            am, bm, _ = h.lanczos(20)
            assert np.max(np.abs(am - a)) <= 1e-6 * scale, (engine, np.max(np.abs(am - a)) / scale)
            assert np.max(np.abs(bm - b)) <= 1e-6 * scale, (engine, np.max(np.abs(bm - b)) / scale)
    finally:
        m.close()
        h.close()
