"""Coefficients of the polynomial in gbmath.cuh (tail_closed) that stands
for phi(q) = sum_{k>=3} q^(k-3) / k = (-ln(1 - q) - q - q^2/2) / q^3 on
0 <= q <= 0.3: the degree-8 Chebyshev interpolant of phi on that interval,
rewritten in powers of q.  Relative error below 3e-10 (FP64); run with
python to print the float literals."""
import numpy as np
from numpy.polynomial import chebyshev as C
from numpy.polynomial import polynomial as P

QMAX, DEG = 0.3, 8


def phi(q):
    q = np.asarray(q, dtype=np.float64)
    s = np.zeros_like(q)
    for k in range(3, 400):
        s += q ** (k - 3) / k
    return s


def coefficients():
    c = C.chebinterpolate(lambda t: phi((t + 1.0) * QMAX / 2.0), DEG)
    # t = 2 q / QMAX - 1: compose the Chebyshev series with that map
    mono_t = C.cheb2poly(c)
    out = np.zeros(DEG + 1)
    lin = np.array([-1.0, 2.0 / QMAX])
    powt = np.array([1.0])
    for k in range(DEG + 1):
        out[: len(powt)] += mono_t[k] * powt
        powt = P.polymul(powt, lin)
    return out


if __name__ == "__main__":
    a = coefficients()
    q = np.linspace(0.0, QMAX, 4001)
    err = np.abs(P.polyval(q, a.astype(np.float32).astype(np.float64)) / phi(q) - 1.0).max()
    print("// p(q) = sum a_k q^k, k = 0..%d; max relative error with FP32 coefficients %.1e" % (DEG, err))
    print("constexpr float kTailPoly[%d] = {%s};" % (DEG + 1, ", ".join("%.9ef" % v for v in a)))
