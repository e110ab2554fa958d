"""The eigenvalue tail for runs of the mixed path (bsl_good_eigenvalues_noise).

With an inexact H v the converged copies of a level in T_m scatter by about
the relative H v error times max|T| (measured: 3.3e-8 kJ/mol for the ground
level of tests/golden/mixed_tail/cpu_workload_600.npz, a 600-iteration mixed
run on the GB300).  The multiplicity window built on a unit roundoff alone,
(m + 1000) u max|T|, is 2.9e-9 kJ/mol there: every copy looks simple, each has
a neighbour in T without its first row, and the ground level is discarded as
spurious.  The floor BSL_MIXED_REL_NOISE (1e-9 max|T|) widens only the
multiplicity window, so the copies count as one multiple eigenvalue, while a
level alone in that window keeps the spurious test in the unit-roundoff
window (a wider spurious test discards converged levels whose eigenvector has
a small first component: seen on an 8^3, 28-function basis).  The floor was
chosen on dumped runs of the GPU path (the metric problem at 10,000
iterations, cpu_workload at 600-2000 iterations with both kinetic engines, 16
batched problems at 3,000 iterations): every floor in [1e-10, 1e-8] recovered
all 400 compared levels, 3e-8 lost 1 and 1e-6 lost 20 (distinct
near-degenerate levels merged).
"""
import os

import numpy as np
import pytest

from conftest import load_package

KJ_TO_CM = 83.5935
FIX = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "mixed_tail", "cpu_workload_600.npz")


@pytest.fixture(scope="module")
def bsl():
    return load_package()


def found(levels, ref, tol_cm=1e-3):
    if not len(levels):
        return np.zeros(len(ref), bool)
    return np.array([np.min(np.abs(levels - e)) * KJ_TO_CM <= tol_cm for e in ref])


def test_zero_floor_is_the_unit_tail(bsl):
    r = np.load(FIX)
    a, b, b2 = r["alpha"], r["beta"], r["beta2"]
    for unit in (2.0 ** -52, bsl.MIXED_UNIT_ROUNDOFF):
        e0, r0 = bsl.good_eigenvalues(a, b, b2, -10.0, 40.0, unit_roundoff=unit)
        e1, r1 = bsl.good_eigenvalues(a, b, b2, -10.0, 40.0, unit_roundoff=unit, rel_noise=0.0)
        assert np.array_equal(e0, e1) and np.array_equal(r0, r1)


def test_noise_floor_keeps_the_ground_level(bsl):
    r = np.load(FIX)
    a, b, b2, ref = r["alpha"], r["beta"], r["beta2"], r["fp64_levels"]
    assert len(ref) >= 8
    unit_only, _ = bsl.good_eigenvalues(a, b, b2, -10.0, 40.0, unit_roundoff=bsl.MIXED_UNIT_ROUNDOFF)
    assert not found(unit_only, ref)[0]  # the failure the floor exists for
    levels, _ = bsl.good_eigenvalues(a, b, b2, -10.0, 40.0, unit_roundoff=bsl.MIXED_UNIT_ROUNDOFF,
                                     rel_noise=bsl.MIXED_REL_NOISE)
    assert found(levels, ref).all()
    # one entry per level: no two good levels closer than the floor's window
    window = bsl.MIXED_REL_NOISE * max(np.max(np.abs(a)), np.max(b[1:-1]))
    assert np.all(np.diff(np.sort(levels)) > window)


def noisy_lanczos(d, m, eps, seed):
    """Lanczos on diag(d) with a random error of relative size eps added to every H v."""
    rng = np.random.default_rng(seed)
    v = rng.standard_normal(len(d))
    v /= np.linalg.norm(v)
    vold, beta = np.zeros(len(d)), 0.0
    a, b = [], [0.0]
    scale = eps * np.max(np.abs(d)) / np.sqrt(len(d))
    for _ in range(m):
        w = d * v + scale * rng.standard_normal(len(d)) - beta * vold
        al = float(v @ w)
        w -= al * v
        beta = float(np.linalg.norm(w))
        a.append(al)
        b.append(beta)
        vold, v = v, w / beta
    b = np.array(b)
    return np.array(a), b, b * b


def test_noise_floor_on_a_noisy_recurrence(bsl):
    """A recurrence whose H v carries a 1e-9 relative error: with the floor each
    of the three isolated lowest levels is found once, for every start vector."""
    rng = np.random.default_rng(0)
    d = np.concatenate([[-3.7, -0.07, -0.045], np.sort(rng.uniform(0.4, 450.0, 2997))])
    for seed in range(4):
        a, b, b2 = noisy_lanczos(d, 600, 1e-9, seed)
        levels, _ = bsl.good_eigenvalues(a, b, b2, -10.0, 0.0, unit_roundoff=bsl.MIXED_UNIT_ROUNDOFF,
                                         rel_noise=bsl.MIXED_REL_NOISE)
        assert len(levels) == 3, (seed, levels)
        assert np.max(np.abs(np.sort(levels) - d[:3])) <= 1e-6
