"""The exactness argument of the tensor-core kinetic, restated on the CPU.

The x/y and z kinetic kernels (boundstate-lanczos_gb300/csrc/bsl_kinetic_tc.cu)
cut T (host, `kinetic_smem_image`) and each plane of v (device, `slice4`) into
four 9-bit integer slices, multiply the slices on FP16 tensor cores with FP32
accumulation, keep the slice classes k + l <= 3 and accumulate the x and y
contractions of a plane pair in the same accumulator.  The FP32 accumulation
is exact when every class sum is an integer below 2^24.  This file restates
the slicing in numpy and checks: every slice is an integer in [-256, 256]
(exact in FP16); the worst case over all v of every class sum, x and y terms
together, stays below 2^24 for every grid the kernels accept (n <= 64); and the
recombined classes reproduce v T to ~2^-36 of max|v| max|T| per term.
"""
import numpy as np
import pytest


def sinc_dvr_t(n):
    """The sinc-DVR kinetic matrix up to its constant prefactor:
    (-1)^(i-i') {pi^2/3 on the diagonal, 2/(i-i')^2 off it}."""
    d = np.arange(n)[:, None] - np.arange(n)[None, :]
    off = 2.0 / np.where(d == 0, 1, d) ** 2
    return np.where(d == 0, np.pi ** 2 / 3, off) * np.where(d % 2 == 0, 1.0, -1.0)


def slice_t(T):
    """Host slicing: T = 2^(e - 8) (b0 + 2^-9 b1 + 2^-18 b2 + 2^-27 b3) + O(2^-37)."""
    e = np.frexp(np.abs(T).max())[1]
    r = np.ldexp(T, 8 - e)
    bs = []
    for _ in range(4):
        b = np.rint(r)
        bs.append(b)
        r = (r - b) * 512.0
    return bs, e


def slice_v(vh, vl):
    """Device slicing of one plane of double-float values (hi, lo): the plane
    is scaled so that max|y| is in [128, 256), then a0 = rint(yh),
    r = ((yh - a0) + yl) 512, a1 = rint(r), ... in FP32."""
    f32 = np.float32
    mx = np.abs(vh).max()
    e = int(np.floor(np.log2(mx))) + 1 if mx > 0 else 0
    sc = f32(2.0 ** (8 - e))
    yh, yl = (vh * sc).astype(f32), (vl * sc).astype(f32)
    a = [np.rint(yh)]
    r = ((yh - a[0]).astype(f32) + yl).astype(f32) * f32(512)
    for _ in range(3):
        ak = np.rint(r)
        a.append(ak)
        r = (r - ak).astype(f32) * f32(512)
    return a, e


@pytest.mark.parametrize("n", [5, 15, 27, 33, 41, 54, 64])
def test_class_sums_stay_below_2_24(n):
    bs, _ = slice_t(sinc_dvr_t(n))
    for b in bs:
        assert np.abs(b).max() <= 256 and np.all(b == np.rint(b))
    # worst case over v: every v slice at +-256 with the sign of the T slice
    worst = 0.0
    for c in range(4):
        rows = sum(256.0 * np.abs(bs[l]).sum(axis=1) for l in range(c + 1))  # pairs (k = c - l, l)
        worst = max(worst, 2.0 * rows.max())  # x and y contractions in one accumulator
    assert worst < 2.0 ** 24, (n, np.log2(worst))


@pytest.mark.parametrize("n", [27, 54])
def test_sliced_product_matches_fp64(n):
    rng = np.random.default_rng(n)
    T = sinc_dvr_t(n)
    bs, e_t = slice_t(T)
    x = np.linspace(-1.0, 1.0, n)
    v = np.exp(-6.0 * x ** 2)[None, :] * rng.standard_normal((64, 1)) + 1e-4 * rng.standard_normal((64, n))
    vh = v.astype(np.float32)
    vl = (v - vh).astype(np.float32)
    a, e_v = slice_v(vh, vl)
    for ak in a:
        assert np.abs(ak).max() <= 256
    classes = np.zeros((4, 64, n))
    for k in range(4):
        for l in range(4 - k):
            classes[k + l] += a[k] @ bs[l].T  # integers: exact in FP64 as in the FP32 accumulator
    assert np.abs(classes).max() < 2.0 ** 24
    res = sum(classes[c] * 2.0 ** (-9 * c) for c in range(4)) * 2.0 ** ((e_v - 8) + (e_t - 8))
    ref = (vh.astype(np.float64) + vl) @ T.T
    err = np.abs(res - ref).max() / (np.abs(v).max() * np.abs(T).max() * n)
    assert err < 2.0 ** -34, err
