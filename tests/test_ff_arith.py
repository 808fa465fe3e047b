"""The float-float Spline_Interp sum of the FP32D patch kernel, restated in
numpy float32 arithmetic (round to nearest, as the kernel's intrinsics).
Position sums: the 12 derivative terms are summed from a power of two `off`
at least twice a bound on their sum of |w v| (per-set maxima of the node
values times the weight-sum bounds h/4 and h^2/16), so every FastTwoSum step
is exact; off is then subtracted and the 4 value terms are added with
TwoSum.  Density and normal sums: all 16 terms from an offset whose bound
covers the value terms too (weight sum 1), off subtracted at the end.
Checks that each FastTwoSum is error-free on random spline data (values of
both signs, near-cancelling sums) and that the result matches the FP64 sum
to a few 1e-12 of sum |w v| (positions) or of the bound (the others): the
FP32 correction term is rounded on the scale of the offset, so the bound
costs accuracy against TwoSum alone (~1e-14), and the patch corrections of
the kernel agree with the FP64 kernel to a few 1e-12."""
import math

import numpy as np

F32 = np.float32


def split(v):
    h = F32(v)
    return h, F32(v - float(h))


def two_sum(a, b):
    s = F32(a + b)
    bb = F32(s - a)
    return s, F32(F32(a - F32(s - bb)) + F32(b - bb))


def two_prod_err(a, b):
    """fma(a, b, -a*b): exact in float64 for float32 inputs, exactly representable in float32."""
    p = F32(a * b)
    return p, F32(float(a) * float(b) - float(p))


def weights(s, t, hx, hy):
    cx = [1 + s * s * (-3 + 2 * s), s * s * (3 - 2 * s), hx * s * (1 + s * (-2 + s)), hx * s * s * (-1 + s)]
    cy = [1 + t * t * (-3 + 2 * t), t * t * (3 - 2 * t), hy * t * (1 + t * (-2 + t)), hy * t * t * (-1 + t)]
    ax, ay = (0, 0, 1, 1), (0, 1, 0, 1)
    w = np.zeros((4, 4))  # [node][slot u, u_th, u_ph, u_thph]
    for k in range(4):
        w[k] = [cx[ax[k]] * cy[ay[k]], cx[ax[k] + 2] * cy[ay[k]], cx[ax[k]] * cy[ay[k] + 2],
                cx[ax[k] + 2] * cy[ay[k] + 2]]
    return w


def ff_interp(w, v, bnd, hx, hy, full=False):
    """w, v: (4 nodes, 4 slots) FP64; bnd: max |v| per slot.  Returns the
    float-float sum as (s, c) and the number of inexact FastTwoSum steps.
    full: all 16 terms by FastTwoSum from the offset of the whole sum."""
    B = 1.01 * ((bnd[0] if full else 0.0) + hx / 4 * bnd[1] + hy / 4 * bnd[2] + hx * hy / 16 * bnd[3])
    off = F32(2.0 ** math.frexp(2 * B)[1])
    s, c, inexact = off, F32(0), 0
    for d in (1, 2, 3, 0):
        if d == 0 and not full:
            s = F32(s - off)  # exact: off/2 <= s <= 3 off/2
        for k in range(4):
            wh, wl = split(w[k, d])
            vh, vl = split(v[k, d])
            p, e = two_prod_err(wh, vh)
            t = F32(s + p)
            if d or full:
                err = F32(p - F32(t - s))
                inexact += float(s) + float(p) != float(t) + float(err)
            else:
                t, err = two_sum(s, p)
            s = t
            c = F32(c + F32(wh * vl))
            c = F32(c + F32(wl * vh))
            c = F32(c + F32(err + e))
    if full:
        inexact += float(s) - float(off) != float(F32(s - off))
        s = F32(s - off)
    return s, c, inexact


def test_fast_two_sum_exact_and_result_fp64_accurate():
    rng = np.random.default_rng(3)
    m, n = 50, 50
    hx, hy = 2 * math.pi / m, 2 * math.pi / n
    worst, total_inexact = 0.0, 0
    for trial in range(400):
        # node values of one set: values of either sign, derivatives up to 15x larger
        scale = 10.0 ** rng.uniform(-3, 1)
        v = np.zeros((4, 4))
        v[:, 0] = scale * rng.uniform(-1.5, 1.5, 4)
        v[:, 1:] = scale * rng.uniform(-15, 15, (4, 3))
        if trial % 4 == 0:  # near-cancelling interpolant: values about zero
            v[:, 0] -= v[:, 0].mean()
        bnd = np.abs(v).max(axis=0) * (1 + rng.uniform(0, 3))  # a cell-wide bound >= this stencil's
        w = weights(rng.uniform(), rng.uniform(), hx, hy)
        s, c, inexact = ff_interp(w, v, bnd, hx, hy)
        total_inexact += inexact
        exact = float(np.sum(w * v))
        got = float(s) + float(c)
        worst = max(worst, abs(got - exact) / (np.abs(w * v).sum()))
    assert total_inexact == 0
    assert worst < 5e-12, worst


def test_full_offset_fast_two_sum_exact():
    """All 16 terms from the offset of the whole sum (density and normal
    sets): every FastTwoSum and the final subtraction exact, the result
    within a few 1e-12 of the cell-wide bound of the FP64 sum."""
    rng = np.random.default_rng(5)
    m, n = 50, 50
    hx, hy = 2 * math.pi / m, 2 * math.pi / n
    worst, total_inexact = 0.0, 0
    for trial in range(400):
        scale = 10.0 ** rng.uniform(-3, 1)
        v = np.zeros((4, 4))
        v[:, 0] = scale * rng.uniform(-1.5, 1.5, 4)
        v[:, 1:] = scale * rng.uniform(-15, 15, (4, 3))
        if trial % 4 == 0:
            v[:, 0] -= v[:, 0].mean()
        bnd = np.abs(v).max(axis=0) * (1 + rng.uniform(0, 3))
        w = weights(rng.uniform(), rng.uniform(), hx, hy)
        s, c, inexact = ff_interp(w, v, bnd, hx, hy, full=True)
        total_inexact += inexact
        exact = float(np.sum(w * v))
        got = float(s) + float(c)
        B = bnd[0] + hx / 4 * bnd[1] + hy / 4 * bnd[2] + hx * hy / 16 * bnd[3]
        worst = max(worst, abs(got - exact) / B)
    assert total_inexact == 0
    assert worst < 1e-12, worst
