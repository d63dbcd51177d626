"""Derives the coefficients of LsExpG (ls_sweep_kernel.cuh): a rational
P5(x) / Q6(x) approximation of

    G(x) = (x - 1 + exp(-x)) / x^2,   x >= 0,

the exponential term from which the linear-source sweep rebuilds F1, F2 and
H (R. Ferrer and J. Rhodes, "A Linear Source Approximation Scheme for the
Method of Characteristics", Nucl. Sci. Eng. 182, 2016).

Form: P(0) = 1/2 (G(0) = 1/2), Q(0) = 1, and the leading coefficients of P
and Q equal, so that P/Q ~ 1/x like G for large x.  The remaining ten
coefficients minimise the maximum relative error on [0, 2000] by Lawson's
iteratively reweighted least squares on the linearised residual
P(x) - G(x) Q(x), with G from 40-digit arithmetic (mpmath).  Prints the
coefficients and the relative error of the FP32 evaluation.

    python openmoc_gb300/csrc/fit_ls_exponential.py
"""
import mpmath as mp
import numpy as np

mp.mp.dps = 40


def g_exact(x: float) -> float:
    x = mp.mpf(x)
    if x < mp.mpf("1e-3"):
        return float(sum((-x) ** k / mp.factorial(k + 2) for k in range(12)))
    return float((x - 1 + mp.e ** (-x)) / x ** 2)


def fit(xs, gx, w):
    cols = [xs ** k for k in range(1, 5)]          # p1..p4
    cols.append(xs ** 5 - gx * xs ** 6)            # p5 = q6
    cols += [-gx * xs ** j for j in range(1, 6)]   # q1..q5
    a = np.stack(cols, 1) * w[:, None]
    sol, *_ = np.linalg.lstsq(a, (gx - 0.5) * w, rcond=None)
    p = np.array([0.5] + list(sol[:4]) + [sol[4]])
    q = np.array([1.0] + list(sol[5:]) + [sol[4]])
    return p, q


def rational(p, q, x):
    return np.polyval(p[::-1], x) / np.polyval(q[::-1], x)


def main():
    xs = np.unique(np.concatenate([np.linspace(0, 4, 2000),
                                   np.geomspace(1e-6, 2000, 4000)]))
    gx = np.array([g_exact(x) if x > 0 else 0.5 for x in xs])
    p, q = fit(xs, gx, 1.0 / gx)
    lw = np.ones_like(xs)
    for _ in range(60):
        err = rational(p, q, xs) / gx - 1.0
        lw = lw * np.sqrt(np.abs(err) + 1e-18)
        lw /= lw.max()
        p, q = fit(xs, gx, np.sqrt(lw) / (gx * np.abs(np.polyval(q[::-1], xs))))
    print("max relative error (exact arithmetic): %.3e"
          % np.max(np.abs(rational(p, q, xs) / gx - 1.0)))
    for i, v in enumerate(p):
        print("  static constexpr float p%d = %.10ef;" % (i, v))
    for i, v in enumerate(q[1:], 1):
        print("  static constexpr float q%d = %.10ef;" % (i, v))
    # FP32 Horner evaluation, as the kernel does it
    xt = np.unique(np.concatenate([np.geomspace(1e-7, 5000, 20000),
                                   np.linspace(0, 20, 20001)[1:]])).astype(np.float32)
    pf, qf = p.astype(np.float32), q.astype(np.float32)
    num = np.full_like(xt, pf[5])
    for k in range(4, -1, -1):
        num = num * xt + pf[k]
    den = np.full_like(xt, qf[6])
    for k in range(5, -1, -1):
        den = den * xt + qf[k]
    ge = np.array([g_exact(float(x)) for x in xt])
    print("max relative error (FP32 evaluation): %.3e"
          % np.max(np.abs((num / den).astype(np.float64) / ge - 1.0)))


if __name__ == "__main__":
    main()
