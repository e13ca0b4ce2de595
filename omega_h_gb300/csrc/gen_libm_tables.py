"""Writes ohg_libm_tables.inc: the tables of the correctly rounded log and exp
in ohg_libm.cuh, computed with mpmath at 200 bits and split into
double-double pairs (hi = the double nearest the value, lo = the double
nearest the rest).

    python omega_h_gb300/csrc/gen_libm_tables.py

log: for j = LOG_J0 .. LOG_J1, c_j = j / 256 covers [sqrt(1/2), sqrt(2)];
  inv_j = the double nearest 1 / c_j (1 exactly for j = 256) and
  L_j = log(1 / inv_j) as a double-double, so that
  log(f) = L_j + log(f * inv_j) exactly, with f * inv_j within 2^-8.5 of 1.
exp: T_j = 2^(j / 128) for j = 0 .. 127 as double-doubles.
sin, cos: sin(j/64) and cos(j/64) for j = 0 .. 51 as double-doubles.
Constants: ln 2 as HI + MID + LO with HI of 42 bits (k * HI exact for
|k| < 2^11) and ln 2 / 128 the same way with HI of 35 bits (exact for
|k| < 2^18); pi/2 the same way with HI of 33 bits (exact for |k| < 2^20);
pi and pi/2 as double-doubles.
"""
import os

import mpmath

mpmath.mp.prec = 200
HERE = os.path.dirname(os.path.abspath(__file__))


def dd(v):
    hi = float(v)
    lo = float(v - mpmath.mpf(hi))
    return hi, lo


def split_trailing_zeros(v, bits):
    """v as hi + lo with hi carrying at most `bits` significant bits."""
    hi = float(v)
    m, e = mpmath.frexp(mpmath.mpf(hi))
    scale = mpmath.mpf(2) ** (bits - e)
    hi = float(mpmath.floor(mpmath.mpf(hi) * scale + mpmath.mpf("0.5")) / scale)
    lo = float(v - mpmath.mpf(hi))
    return hi, lo


LOG_J0, LOG_J1 = 181, 362


def main():
    out = ["// Generated by gen_libm_tables.py (mpmath, 200 bits): do not edit.",
           f"#define OHG_LOG_J0 {LOG_J0}", f"#define OHG_LOG_J1 {LOG_J1}"]
    inv, lh, ll = [], [], []
    for j in range(LOG_J0, LOG_J1 + 1):
        c = mpmath.mpf(j) / 256
        iv = float(1 / c)
        Lh, Ll = dd(-mpmath.log(mpmath.mpf(iv)))
        inv.append(iv)
        lh.append(Lh)
        ll.append(Ll)
    th, tl = [], []
    for j in range(128):
        h, l = dd(mpmath.mpf(2) ** (mpmath.mpf(j) / 128))
        th.append(h)
        tl.append(l)
    ln2 = mpmath.log(2)

    def split3(v, bits):
        hi, _ = split_trailing_zeros(v, bits)
        mid = float(v - mpmath.mpf(hi))
        lo = float(v - mpmath.mpf(hi) - mpmath.mpf(mid))
        return hi, mid, lo

    ln2_3 = split3(ln2, 42)
    l128_3 = split3(ln2 / 128, 35)

    def arr(name, vals):
        # one copy in device memory (CUDA compiles) and one in host memory
        body = ",\n  ".join(", ".join(repr(v) for v in vals[i:i + 3]) for i in range(0, len(vals), 3))
        return ["#ifdef __CUDACC__",
                f"static __device__ const double ohg_libm_d_{name}[{len(vals)}] = {{\n  {body}}};",
                "#endif",
                f"static const double ohg_libm_h_{name}[{len(vals)}] = {{\n  {body}}};"]

    out += arr("log_inv", inv) + arr("log_hi", lh) + arr("log_lo", ll)
    out += arr("exp_hi", th) + arr("exp_lo", tl)
    # sin and cos of c_j = j/64, j = 0..51 (c_j up to pi/4 + 1/128)
    sh, sl, ch, cl = [], [], [], []
    for j in range(52):
        c = mpmath.mpf(j) / 64
        a, b = dd(mpmath.sin(c))
        sh.append(a)
        sl.append(b)
        a, b = dd(mpmath.cos(c))
        ch.append(a)
        cl.append(b)
    out += arr("sin_hi", sh) + arr("sin_lo", sl) + arr("cos_hi", ch) + arr("cos_lo", cl)
    out += [f"#define OHG_LN2_HI {ln2_3[0]!r}", f"#define OHG_LN2_MID {ln2_3[1]!r}",
            f"#define OHG_LN2_LO {ln2_3[2]!r}",
            f"#define OHG_LN2_128_HI {l128_3[0]!r}", f"#define OHG_LN2_128_MID {l128_3[1]!r}",
            f"#define OHG_LN2_128_LO {l128_3[2]!r}",
            f"#define OHG_INV_LN2_128 {float(128 / ln2)!r}"]
    pio2_3 = split3(mpmath.pi / 2, 33)
    pi_dd = dd(mpmath.pi)
    pio2_dd = dd(mpmath.pi / 2)
    out += [f"#define OHG_PIO2_HI {pio2_3[0]!r}", f"#define OHG_PIO2_MID {pio2_3[1]!r}",
            f"#define OHG_PIO2_LO {pio2_3[2]!r}", f"#define OHG_2_OVER_PI {float(2 / mpmath.pi)!r}",
            f"#define OHG_PI_DD_HI {pi_dd[0]!r}", f"#define OHG_PI_DD_LO {pi_dd[1]!r}",
            f"#define OHG_PIO2_DD_HI {pio2_dd[0]!r}", f"#define OHG_PIO2_DD_LO {pio2_dd[1]!r}"]
    with open(os.path.join(HERE, "ohg_libm_tables.inc"), "w") as f:
        f.write("\n".join(out) + "\n")


if __name__ == "__main__":
    main()
