"""Generate tests/golden/mixed_tail/cpu_workload_600.npz on a GB300.

The alpha/beta history of a 600-iteration Lanczos run of the cpu_workload
case (15^3, even l <= 4, 12 x 12 angular grid, normal start vector, seed 0)
on the mixed-precision path with the tensor-core kinetic, the spherical-
harmonic potential stream and the fused update, and the stable levels below
30 kJ/mol (at most 20) of the FP64 GPU run of the same case (good at 600
iterations and unchanged to 1e-10 kJ/mol without the last 40).  In this run the ground
level's four converged copies in T_600 scatter by 3.3e-8 kJ/mol, more than the
multiplicity window built on the unit roundoff alone (2.9e-9 kJ/mol), so the
tail without a noise floor discards the ground level as spurious.

    python tests/golden/make_mixed_tail_fixture.py [OUT.npz]      (needs the GPU)
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
from conftest import case_info, load_package  # noqa: E402


def stable_levels(bsl, a, b, b2, nlev=20, drop=40, tol=1e-10):
    ev, _ = bsl.good_eigenvalues(a, b, b2, -10.0, 30.0)
    n = len(a) - drop
    ev2, _ = bsl.good_eigenvalues(a[:n], b[:n + 1], b2[:n + 1], -10.0, 30.0)
    return np.sort(np.array([e for e in ev if np.min(np.abs(ev2 - e)) <= tol]))[:nlev]


def main():
    bsl = load_package()
    d, man, extra = case_info("cpu_workload")
    cwd = os.getcwd()
    os.chdir(d)
    try:
        h = bsl.Hamiltonian("hv_input.txt", man["calculator"], extra_input=extra, precision="fp64")
    finally:
        os.chdir(cwd)
    niter = 600
    a, b, b2 = h.lanczos(niter, start="normal", seed=0)
    ref = stable_levels(bsl, a, b, b2)
    h.set_precision("mixed")
    h.set_kinetic_engine("tensor")
    am, bm, bm2 = h.lanczos(niter, start="normal", seed=0)
    out = sys.argv[1] if len(sys.argv) > 1 else os.path.join(HERE, "mixed_tail", "cpu_workload_600.npz")
    os.makedirs(os.path.dirname(out), exist_ok=True)
    np.savez(out, alpha=am, beta=bm, beta2=bm2, fp64_levels=ref, potential_format=h.potential_format())
    h.close()
    print(out)


if __name__ == "__main__":
    main()
