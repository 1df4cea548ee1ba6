"""Generate nsem_pow_tables.h: the lookup tables of the double-double pow.

Run once when the table layout changes (needs mpmath, shipped with sympy):
    python nebulasem_gb300/csrc/gen_pow_tables.py > nebulasem_gb300/csrc/nsem_pow_tables.h

Tables (values from their mathematical definitions, 200-bit mpmath):
  LOG_R[i]      reduction factor r_i ~ 1/c_i on a 2^-9 grid, c_i the centre of
                bin i of width 1/128 starting at 0.703125, so that for m in the
                bin |m*r_i - 1| < 2^-7;
  LOG_NLR[i]    -log(r_i) as an unevaluated sum hi + lo;
  EXP2[j]       2^(j/64) as hi + lo, j = 0..63.
"""
import mpmath

mpmath.mp.prec = 200

BIN0 = mpmath.mpf("0.703125")
NBIN = 92  # covers [0.703125, 1.421875)


def dd(v):
    hi = float(v)
    lo = float(v - mpmath.mpf(hi))
    return hi, lo


def main():
    rows = []
    for i in range(NBIN):
        c = BIN0 + (mpmath.mpf(i) + mpmath.mpf("0.5")) / 128
        r = mpmath.nint((1 / c) * 512) / 512
        hi, lo = dd(-mpmath.log(r))
        rows.append((float(r), hi, lo))
    print("/* Generated by gen_pow_tables.py -- do not edit. */")
    print("#ifndef NSEM_POW_TABLES_H")
    print("#define NSEM_POW_TABLES_H")
    print(f"#define NSEM_LOG_NBIN {NBIN}")
    print("NSEM_TABLE double nsem_log_r[NSEM_LOG_NBIN] = {")
    for r, _, _ in rows:
        print(f"  {r!r},")
    print("};")
    print("NSEM_TABLE double nsem_log_nlr[NSEM_LOG_NBIN][2] = {")
    for _, hi, lo in rows:
        print(f"  {{{hi!r}, {lo!r}}},")
    print("};")
    print("NSEM_TABLE double nsem_exp2_64[64][2] = {")
    for j in range(64):
        hi, lo = dd(mpmath.power(2, mpmath.mpf(j) / 64))
        print(f"  {{{hi!r}, {lo!r}}},")
    print("};")
    ln2 = mpmath.log(2)
    # ln2 split so that n*hi is exact for |n| < 2^20
    hi = float(mpmath.floor(ln2 * 2**32) / 2**32)
    mid, lo = dd(ln2 - mpmath.mpf(hi))
    print(f"#define NSEM_LN2_HI {hi!r}")
    print(f"#define NSEM_LN2_MID {mid!r}")
    print(f"#define NSEM_LN2_LO {lo!r}")
    third_hi, third_lo = dd(mpmath.mpf(1) / 3)
    print(f"#define NSEM_THIRD_HI {third_hi!r}")
    print(f"#define NSEM_THIRD_LO {third_lo!r}")
    h6, l6 = dd(mpmath.mpf(1) / 6)
    h24, l24 = dd(mpmath.mpf(1) / 24)
    print(f"#define NSEM_SIXTH_HI {h6!r}")
    print(f"#define NSEM_SIXTH_LO {l6!r}")
    print(f"#define NSEM_24TH_HI {h24!r}")
    print(f"#define NSEM_24TH_LO {l24!r}")
    print(f"#define NSEM_INV_LN2_64 {float(64 / ln2)!r}")
    print("#endif")


if __name__ == "__main__":
    main()
