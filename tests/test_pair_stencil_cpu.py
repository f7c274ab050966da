"""CPU check of the float-pair stencil's arithmetic (wave_dev.cuh
pair_rhs_vals): the exact-sum form, emulated in IEEE float32 with exact
products, reproduces the FP64 residual -F(hi + lo) of the wave operator
(wave.py:67-122 inside the grid) to ~2^-46 of the largest stencil term,
including where F cancels to ~1e-9 of its terms.  The GPU parity tests
check the kernels themselves; this pins the algorithm."""
import numpy as np

from oracle import wave as W

F32 = np.float32


def _fma(a, b, c):
    # a * b is exact in float64 (48 significant bits); one rounding to
    # float32 after the add (double rounding is far below the bound here).
    return (a.astype(np.float64) * b.astype(np.float64) +
            c.astype(np.float64)).astype(F32)


def _two_sum_err(a, b, s):
    bb = (s - a).astype(F32)
    return ((a - (s - bb).astype(F32)).astype(F32) +
            (b - bb).astype(F32)).astype(F32)


def _split(x):
    h = F32(x)
    return h, F32(x - float(h))


def _pair_rhs(k, v0, v2, v1, vm, vp, w0, w2, w1, wm, wp):
    ah, al, ch, cl, bh, bl = (np.full_like(v0, x) for x in k)
    a = (v0 + v2).astype(F32)
    ea = _two_sum_err(v0, v2, a)
    b = (vm + vp).astype(F32)
    eb = _two_sum_err(vm, vp, b)
    p1 = (ah * a).astype(F32)
    e1 = _fma(ah, a, -p1)
    p2 = (ch * v1).astype(F32)
    e2 = _fma(ch, v1, -p2)
    p3 = (bh * b).astype(F32)
    e3 = _fma(bh, b, -p3)
    s = (p1 + p2).astype(F32)
    es = _two_sum_err(p1, p2, s)
    t = (s + p3).astype(F32)
    et = _two_sum_err(s, p3, t)
    c = (((es + et).astype(F32) + (e1 + e2).astype(F32)).astype(F32) +
         e3).astype(F32)
    for coef, val in ((al, a), (cl, v1), (bl, b), (ah, ea), (bh, eb),
                      (ah, (w0 + w2).astype(F32)), (ch, w1),
                      (bh, (wm + wp).astype(F32))):
        c = _fma(coef, val, c)
    return (-(t + c)).astype(F32)


def test_exact_sum_pair_stencil_bound():
    n = 160
    s = W.make_setup(n, n, "sine", seed=1, nmodes=16)
    ref = W.solve_march(s)
    hi = ref.astype(F32)
    lo = (ref - hi.astype(np.float64)).astype(F32)
    A = 1.0 / s.dt**2
    B = s.c**2 / s.dx**2
    k = _split(A) + _split(2 * B - 2 * A) + _split(-B)
    scale = 4.0 / s.dt**2 * np.abs(ref).max()  # largest stencil term
    for L, rel in ((lo, 1e-7), (np.zeros_like(lo), 1e-6)):
        u = hi.astype(np.float64) + L.astype(np.float64)
        fo = W.residual(s, u)[2:, 1:-1]
        got = _pair_rhs(k, hi[2:, 1:-1], hi[:-2, 1:-1], hi[1:-1, 1:-1],
                        hi[1:-1, :-2], hi[1:-1, 2:], L[2:, 1:-1],
                        L[:-2, 1:-1], L[1:-1, 1:-1], L[1:-1, :-2],
                        L[1:-1, 2:])
        err = np.abs(got.astype(np.float64) + fo).max()
        assert err <= 2.0**-46 * scale + rel * np.abs(fo).max(), err
