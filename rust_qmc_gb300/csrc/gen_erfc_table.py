"""Coefficients of the float-float erfc of the electron-gas Ewald sum
(qmc_heg_kernels.cuh, erfc_ff): Chebyshev interpolation of erfc on [0, 6]
at 64 first-kind nodes, computed with mpmath at 40 digits.  erfc(x) =
c_0 / 2 + sum_{k=1..42} c_k T_k(t), t = x / 3 - 1; |c_k| < 2e-18 for k > 42.
Prints the table as C++ initialisers (float-float pairs for k < 24, FP32
beyond).  Run: python gen_erfc_table.py"""
import mpmath as mp

N_NODES, DEG, FF_TERMS = 64, 42, 24


def coefficients():
    mp.mp.dps = 40
    xs = [mp.cos(mp.pi * (k + mp.mpf(1) / 2) / N_NODES) for k in range(N_NODES)]
    fx = [mp.erfc(3 * x + 3) for x in xs]
    c = []
    for j in range(DEG + 1):
        s = mp.fsum(fx[k] * mp.cos(mp.pi * j * (k + mp.mpf(1) / 2) / N_NODES) for k in range(N_NODES))
        c.append(2 * s / N_NODES)
    return c


def split(v):
    import numpy as np
    hi = np.float32(float(v))
    lo = np.float32(float(v - mp.mpf(float(hi))))
    return hi, lo


if __name__ == "__main__":
    import numpy as np
    c = coefficients()
    print("// float-float c_0 .. c_%d" % (FF_TERMS - 1))
    for k in range(FF_TERMS):
        hi, lo = split(c[k])
        print("    {%s, %s}," % (np.format_float_scientific(hi, unique=True) + "f",
                                 np.format_float_scientific(lo, unique=True) + "f"))
    print("// FP32 c_%d .. c_%d" % (FF_TERMS, DEG))
    print("    " + ", ".join(np.format_float_scientific(np.float32(float(c[k])), unique=True) + "f"
                             for k in range(FF_TERMS, DEG + 1)))
