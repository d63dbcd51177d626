"""Derives the coefficients of the linear source's two rational
approximations (R. Ferrer and J. Rhodes, "A Linear Source Approximation
Scheme for the Method of Characteristics", Nucl. Sci. Eng. 182, 2016):

* LsExpG (ls_sweep_kernel.cuh): G(x) = (x - 1 + exp(-x)) / x^2, x >= 0, from
  which the sweep rebuilds F1, F2 and H.  Form P5(x) / Q6(x), P(0) = 1/2
  (= G(0)), Q(0) = 1, leading coefficients equal so that P/Q ~ 1/x like G;
  the other ten coefficients minimise the maximum relative error on
  [0, 2000].
* ls_exp_g2 (linear_source.cu): G2(x) = 2/3 - (1 + 2/x)(1/x + 1/2 -
  (1 + 1/x)(1 - exp(-x))/x), used by the expansion constants.  Form
  x P5(x) / Q6(x), P(0) = -1/12 (the slope of G2 at 0, so small x keeps its
  relative accuracy), Q(0) = 1, p5 = q6 / 6 (G2 -> 1/6); the other ten
  coefficients minimise the maximum of |error| / max(|G2|, 1e-3) on
  [0, 3000] (G2 changes sign near x = 3.3).

Both by Lawson's iteratively reweighted least squares on the linearised
residual P - f Q, with f from 40-digit arithmetic (mpmath).  Prints the
coefficients and the errors of the FP32 evaluation.

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


def g2_exact(x: float) -> float:
    x = mp.mpf(x)
    if x < mp.mpf("0.5"):
        s, f = mp.mpf(0), mp.mpf(2)
        for m in range(1, 40):
            f *= m + 2
            s += (mp.mpf(m + 1) / f - 2 * mp.mpf(m + 2) / (f * (m + 3))) * (-x) ** m
        return float(s)
    f1 = (1 - mp.e ** (-x)) / x
    return float(mp.mpf(2) / 3 - (1 + 2 / x) * (1 / x + mp.mpf(1) / 2 - (1 + 1 / x) * f1))


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


def fit_g2(xs, gx, w):
    cols = [xs * xs ** k for k in range(1, 5)]          # p1..p4
    cols.append(xs * xs ** 5 / 6 - gx * xs ** 6)         # q6 (p5 = q6 / 6)
    cols += [-gx * xs ** j for j in range(1, 6)]         # q1..q5
    a = np.stack(cols, 1) * w[:, None]
    sol, *_ = np.linalg.lstsq(a, (gx + xs / 12.0) * w, rcond=None)
    p = np.array([-1.0 / 12.0] + list(sol[:4]) + [sol[4] / 6.0])
    q = np.array([1.0] + list(sol[5:]) + [sol[4]])
    return p, q


def main_g2():
    xs = np.unique(np.concatenate([np.linspace(0, 6, 3000),
                                   np.geomspace(1e-5, 3000, 4000)]))
    gx = np.array([g2_exact(x) for x in xs])
    den = np.maximum(np.abs(gx), 1e-3)
    ev = lambda p, q, x: x * rational(p, q, x)  # noqa: E731
    p, q = fit_g2(xs, gx, 1.0 / den)
    lw = np.ones_like(xs)
    for _ in range(100):
        err = (ev(p, q, xs) - gx) / den
        lw = lw * np.sqrt(np.abs(err) + 1e-20)
        lw /= lw.max()
        p, q = fit_g2(xs, gx, np.sqrt(lw) / (den * np.abs(np.polyval(q[::-1], xs))))
    print("G2: max |error| / max(|G2|, 1e-3) (exact arithmetic): %.3e"
          % np.max(np.abs(ev(p, q, xs) - gx) / den))
    print("  static constexpr float kG2P[6] = {%s};"
          % ", ".join("%.10ef" % v for v in p))
    print("  static constexpr float kG2Q[7] = {%s};"
          % ", ".join("%.10ef" % v for v in q))
    xt = np.unique(np.concatenate([np.geomspace(1e-7, 5000, 20000),
                                   np.linspace(0, 20, 20001)[1:]])).astype(np.float32)
    pf, qf = p.astype(np.float32), q.astype(np.float32)
    num = np.full_like(xt, pf[5])
    for k in range(4, -1, -1):
        num = num * xt + pf[k]
    den32 = np.full_like(xt, qf[6])
    for k in range(5, -1, -1):
        den32 = den32 * xt + qf[k]
    got = (xt * num / den32).astype(np.float64)
    ge = np.array([g2_exact(float(x)) for x in xt])
    big = np.abs(ge) > 1e-3
    print("G2 FP32: max abs error %.3e, max rel error where |G2| > 1e-3 %.3e, "
          "below x = 0.01 %.3e" % (np.max(np.abs(got - ge)),
                                   np.max(np.abs(got - ge)[big] / np.abs(ge[big])),
                                   np.max(np.abs(got - ge)[xt < 1e-2] /
                                          np.abs(ge[xt < 1e-2]))))


if __name__ == "__main__":
    main()
    main_g2()
