"""Tables of sde_log.h (the table-driven logarithm of the FP64 inverse CDF),
computed with mpmath at 60 significant digits.

For j = 0..127 (the top 7 bits of the fraction of m in [1, 2)):
  k_j = round(256 / (1 + (j + 1/2) / 128)), so r = m k_j / 256 - 1 is small;
  L_j = log(256 / k_j), split into L_hi (a multiple of 2^-42) and L_lo.
ln 2 is split the same way, so e ln2_hi + L_hi[j] is exact for |e| <= 1022.

Run:  python gen_log_table.py   (prints the table block of sde_log.h)
"""
import mpmath

mpmath.mp.dps = 60


def split42(v):
    """v = hi + lo with hi a multiple of 2^-42 (as a float) and lo the
    remainder rounded to double."""
    hi = mpmath.nint(v * 2**42) / 2**42
    return float(hi), float(v - hi)


def hexs(x: float) -> str:
    return float.hex(x)


def main():
    ks, lhi, llo = [], [], []
    for j in range(128):
        c = 1 + (mpmath.mpf(j) + mpmath.mpf(1) / 2) / 128
        k = int(mpmath.nint(256 / c))
        L = mpmath.log(mpmath.mpf(256) / k)
        h, l = split42(L)
        ks.append(k / 256.0)
        lhi.append(h)
        llo.append(l)
    ln2_hi, ln2_lo = split42(mpmath.log(2))

    def block(name, vals):
        lines = [f"SDE_LOG_TAB double {name}[128] = {{"]
        for i in range(0, 128, 4):
            lines.append("    " + ", ".join(hexs(v) for v in vals[i:i + 4]) + ",")
        lines.append("};")
        return "\n".join(lines)

    print(f"#define SDE_LN2_HI {hexs(ln2_hi)}")
    print(f"#define SDE_LN2_LO {hexs(ln2_lo)}")
    print(block("sde_log_k", ks))
    print(block("sde_log_lhi", lhi))
    print(block("sde_log_llo", llo))


if __name__ == "__main__":
    main()
