"""Generate boys_table.inc: the Boys function F_m(T) on a grid, in FP64.

F_m(T) = int_0^1 t^(2m) exp(-T t^2) dt = gamma(m + 1/2, T) / (2 T^(m + 1/2)),
evaluated with mpmath at 40 significant digits and rounded once to double.
Grid T_g = g / 16 for g = 0..320 (T <= 20, the range of the series branch
of the reference's XGAMMAF), orders m = 0..22, plus exp(-T_g) in the last
column.  The device evaluates F_M(T) from the nearest grid point with a
seven-term Taylor expansion, F_M(T) = sum_k F_{M+k}(T_g) (T_g - T)^k / k!
(dF_m/dT = -F_{m+1}), and the lower orders by downward recursion.

Run:  python gen_boys_table.py > boys_table.inc
"""
import mpmath as mp

NGRID = 321      # T = 0, 1/16, ..., 20
STEP_INV = 16
NORD = 23        # m = 0..22 (highest order used 16, plus 6 Taylor terms)
NCOL = NORD + 1  # + exp(-T)


def boys(m, T):
    if T == 0:
        return mp.mpf(1) / (2 * m + 1)
    return mp.gammainc(m + mp.mpf(1) / 2, 0, T) / (2 * T ** (m + mp.mpf(1) / 2))


def main():
    mp.mp.dps = 40
    print("// generated by gen_boys_table.py: %d rows (T = g/%d) x %d columns "
          "(F_0..F_%d, exp(-T))" % (NGRID, STEP_INV, NCOL, NORD - 1))
    for g in range(NGRID):
        T = mp.mpf(g) / STEP_INV
        vals = [boys(m, T) for m in range(NORD)] + [mp.e ** (-T)]
        print(", ".join(repr(float(v)) for v in vals) + ",")


if __name__ == "__main__":
    main()
