"""The FP32 shortcuts that decide an FP64 quantity only where their error bound makes the answer certain,
restated in numpy (float32 arithmetic, each operation rounded as the kernels round it) and checked against
the FP64 answer on many random cases, including cases placed at the boundaries:
- the periodic image n = rint(d / box) of a guard-band pair (decide64_warp): the FP32 estimate is used only
  where it is certain, and there it equals the FP64 rint, which is then not near a half;
- the periodic image and the cell of a particle (k_assign): the FP32 estimate is used only away from the
  box and cell boundaries, and there it gives the cell whose FP64 local coordinate lies in [0, w).
"""
import numpy as np

f32 = np.float32


def _fma32(a, b, c):
    # float32 fma: the product of two float32 values is exact in float64; the sum is rounded once to float64
    # (at most one ulp of float64 away from the exact sum, far below the float32 ulp), then to float32
    return (a.astype(np.float64) * b.astype(np.float64) + c.astype(np.float64)).astype(f32)


def test_image_estimate_equals_the_fp64_rint():
    rng = np.random.default_rng(7)
    n = 400000
    box = rng.uniform(5.0, 400.0, n)
    # separations of close pairs in far images, and separations placed near a half box
    k = rng.integers(-2000, 2000, n).astype(np.float64)
    frac = np.where(rng.random(n) < 0.5, rng.uniform(-0.02, 0.02, n), rng.uniform(-0.5, 0.5, n))
    d = (k + frac) * box
    ib = 1.0 / box
    tf = d.astype(f32) * ib.astype(f32)  # d2f(d) * d2f(ib), one float32 product
    nf = np.rint(tf)
    certain = (np.abs(tf - nf) < f32(0.25)) & (np.abs(tf) < f32(1e5))
    t = d * ib
    n64 = np.rint(t)
    assert certain.mean() > 0.4
    assert np.array_equal(nf[certain].astype(np.float64), n64[certain])
    assert np.all(np.abs(t[certain] - n64[certain]) <= 0.5 - 1e-9)


def test_cell_estimate_equals_the_fp64_cell():
    rng = np.random.default_rng(11)
    m = 300000
    L = rng.uniform(20.0, 300.0, m)
    ncell = (np.floor(L / 1.15).astype(np.int64) // 2) * 2
    w = L / ncell
    shift = rng.random(m).astype(f32).astype(np.float64) * w
    # unwrapped positions: mostly in the box, some images away, some placed on cell and box boundaries
    img = np.where(rng.random(m) < 0.8, 0, rng.integers(-3, 4, m))
    x = rng.uniform(0.0, 1.0, m) * L + img * L
    on = rng.random(m) < 0.2
    cells = rng.integers(0, ncell)
    x[on] = (shift + cells * w)[on] + rng.uniform(-1e-5, 1e-5, on.sum())
    Lf, wf, shf = L.astype(f32), w.astype(f32), shift.astype(f32)
    inv_Lf, inv_wf = (1.0 / L).astype(f32), (1.0 / w).astype(f32)
    xf = x.astype(f32)  # the kernel truncates; either rounding lies within the same bound
    kf = np.floor(xf * inv_Lf)
    yg = _fma32(-kf, Lf, xf) - shf
    cg = np.floor(yg * inv_wf)
    lg = _fma32(-cg, wf, yg)
    mrg = f32(1e-6) * (np.abs(xf) + (np.abs(kf) + f32(3.0)) * Lf)
    easy = (yg >= mrg) & (yg < Lf - mrg) & (lg >= mrg) & (lg < wf - mrg) & (cg < ncell.astype(f32))
    assert easy[~on].mean() > 0.99 and easy[on].mean() < 0.5  # the boundary cases take the careful path
    y = np.where(kf == 0, x, x - kf.astype(np.float64) * L) - shift
    l64 = y - cg.astype(np.float64) * w
    lf = l64.astype(f32)
    assert np.all((y[easy] >= 0) & (y[easy] < L[easy]))
    assert np.all((lf[easy] >= 0) & (lf[easy] < wf[easy]))
    # the exact cell of y agrees with the FP32 estimate wherever the estimate was used
    assert np.array_equal(np.floor(y[easy] / w[easy]), cg[easy].astype(np.float64))
