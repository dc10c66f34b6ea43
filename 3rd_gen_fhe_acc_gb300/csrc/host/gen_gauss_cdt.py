"""Writes gauss_cdt.inc: the cumulative table used by the host key generator's
Gaussian sampler (fheacc_host.cpp).

The sampler reproduces the distribution of the reference's RNG_norm
(FHE_ACC_runtime/src/RNG.cpp:19-37): a normal variate with mean 0 and standard
deviation SIGMA, converted to int64 by truncation toward zero. The table holds,
for v = -K..K, floor(2^64 * P(V <= v)), computed with 80-digit arithmetic so
that every machine builds the same integer table. Run:
    python gen_gauss_cdt.py > gauss_cdt.inc
"""
import mpmath

SIGMA = mpmath.mpf("3.19")
K = 40


def main():
    mpmath.mp.dps = 80
    s2 = SIGMA * mpmath.sqrt(2)

    def p(v):
        k = abs(v)
        if k == 0:
            return mpmath.erf(1 / s2)
        return (mpmath.erf((k + 1) / s2) - mpmath.erf(k / s2)) / 2

    total = sum(p(v) for v in range(-K, K + 1))
    cum = mpmath.mpf(0)
    rows = []
    for v in range(-K, K + 1):
        cum += p(v) / total
        t = int(mpmath.floor(cum * mpmath.mpf(2) ** 64))
        rows.append(min(t, 2**64 - 1))
    rows[-1] = 2**64 - 1
    print("/* generated by gen_gauss_cdt.py: sigma = 3.19, support -%d..%d */" % (K, K))
    print("#define FHEACC_GAUSS_K %d" % K)
    print("static const uint64_t kGaussCdt[%d] = {" % (2 * K + 1))
    for i in range(0, len(rows), 3):
        print("    " + ", ".join("0x%016xULL" % r for r in rows[i:i + 3]) + ",")
    print("};")


if __name__ == "__main__":
    main()
