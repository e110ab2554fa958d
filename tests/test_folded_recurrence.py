"""The Lanczos recurrence with folded scales, restated on the CPU in FP64.

The device loop never normalises or swaps vectors explicitly: it keeps two
buffers V, R with the logical v = sv V, r = sr R, forms R' = R + c H V
(c = sv/sr) and alpha = sv sr (V . R') in the potential stream, then
R_new = g (R' - alpha c V) with g = 2^e and beta^2 = (sr/g)^2 |R_new|^2 in the
update, and derives the next scales (`finish_update_pair` in
boundstate-lanczos_gb300/csrc/bsl_device.cuh): sv' = (sr/g)/beta, sr' = -beta sv,
the buffers swapping roles.  This checks that algebra against the reference's
plain loop (headLoop/LanczosCode/lanczosEigenValuesVectors.cpp:187-242:
u = H v; r += u; alpha = v.r; r -= alpha v; beta^2 = r.r; r /= beta;
v <- -beta v; swap) on a random symmetric matrix, and that the buffers keep a
norm near 1 over many iterations.
"""
import numpy as np


def plain_lanczos(H, v0, niter):
    v, r = v0.copy(), np.zeros_like(v0)
    alpha, beta = [], []
    for _ in range(niter):
        r += H @ v
        a = v @ r
        r -= a * v
        b = np.sqrt(r @ r)
        alpha.append(a)
        beta.append(b)
        r /= b
        v *= -b
        v, r = r, v
    return np.array(alpha), np.array(beta)


def folded_lanczos(H, v0, niter):
    V, R = v0.copy(), np.zeros_like(v0)
    sv, sr, e = 1.0, 1.0, 0
    alpha, beta, norms = [], [], []
    for _ in range(niter):
        c = sv / sr
        R = R + c * (H @ V)                # potential stream: R' = R + c H V
        a = sv * sr * (V @ R)              # alpha = sv sr (V . R')
        Rn = np.ldexp(R - a * c * V, e)    # update: R_new = g (R' - alpha c V)
        sr_g = np.ldexp(sr, -e)
        b = np.sqrt(sr_g * sr_g * (Rn @ Rn))
        alpha.append(a)
        beta.append(b)
        sv_n, sr_n = sr_g / b, -b * sv
        e = int(np.clip((np.frexp(sr_n)[1] - 1) - (np.frexp(b)[1] - 1), -60, 60))
        V, R = Rn, V                       # buffers swap roles
        sv, sr = sv_n, sr_n
        norms.append(np.linalg.norm(V))
    return np.array(alpha), np.array(beta), np.array(norms)


def test_folded_scales_reproduce_the_plain_recurrence():
    rng = np.random.default_rng(3)
    n = 400
    A = rng.standard_normal((n, n))
    H = (A + A.T) * 50.0 + np.diag(np.linspace(-200.0, 5000.0, n))  # spread like a kinetic spectrum
    v0 = np.full(n, 1.0 / np.sqrt(n))
    a, b = plain_lanczos(H, v0, 30)
    af, bf, norms = folded_lanczos(H, v0, 30)
    scale = np.abs(a).max()
    assert np.max(np.abs(af - a)) <= 1e-11 * scale
    assert np.max(np.abs(bf - b)) <= 1e-11 * scale
    # the power-of-two g keeps the stored buffers near unit norm from the
    # second update on (the first has g = 1 and leaves |V| = beta_1)
    assert abs(norms[0] - b[0]) <= 1e-9 * b[0]
    assert np.all((norms[1:] > 0.25) & (norms[1:] < 4.0))
