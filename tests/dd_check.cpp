// Host check of the double-float arithmetic (massivemds_gb300/csrc/dd.h) and the
// double-float normal-tail table (normal_dd.h: log Phi and phi / Phi) against
// long double references.
// Prints one line per check: name, max error, bound; exits 1 if a bound fails.
#include <cstdio>
#include <cstdlib>
#include <random>

#include "dd.h"
#include "normal_dd.h"

using namespace mdsx;

static int failures = 0;

static void report(const char* name, long double err, long double bound) {
    std::printf("%s %.3Le %.1Le\n", name, err, bound);
    if (!(err <= bound)) ++failures;
}

static long double ld(dd a) { return (long double)a.hi + (long double)a.lo; }

int main() {
    std::mt19937_64 rng(12345);
    std::uniform_real_distribution<double> uni(-4.0, 4.0);
    long double e_add = 0, e_mul = 0, e_sqr = 0, e_fma = 0, e_rsq = 0, e_rcp = 0, e_div = 0, e_split = 0;
    for (int t = 0; t < 200000; ++t) {
        const double x = uni(rng), y = uni(rng), w = uni(rng);
        const dd a = dd_from_double(x), b = dd_from_double(y), c = dd_from_double(w);
        const long double A = ld(a), B = ld(b), C = ld(c);
        e_split = std::max(e_split, std::fabs(A - (long double)x) / std::fabs((long double)x));
        if (std::fabs(A + B) > 1e-3L) e_add = std::max(e_add, std::fabs(ld(dd_add(a, b)) - (A + B)) / (std::fabs(A) + std::fabs(B)));
        e_mul = std::max(e_mul, std::fabs(ld(dd_mul(a, b)) - A * B) / std::fabs(A * B));
        e_sqr = std::max(e_sqr, std::fabs(ld(dd_sqr(a)) - A * A) / (A * A));
        const long double f = C + A * B;
        e_fma = std::max(e_fma, std::fabs(ld(dd_fma(a, b, c)) - f) / (std::fabs(C) + std::fabs(A * B)));
        const long double ax = std::fabs(A) + 1e-3L;
        const dd pa = dd_from_double((double)ax);
        e_rsq = std::max(e_rsq, std::fabs(ld(dd_rsqrt(pa)) * std::sqrt(ld(pa)) - 1.0L));
        e_rcp = std::max(e_rcp, std::fabs(ld(dd_rcp(a)) * A - 1.0L));
        if (std::fabs(A) > 1e-3L) e_div = std::max(e_div, std::fabs(ld(dd_div(b, a)) * A / B - 1.0L));
    }
    // accumulators: 20 000 products of mixed sign (a row's gradient sum) and
    // squares (the likelihood's sum), against long double, relative to sum |terms|
    long double e_dot = 0, e_sq = 0;
    for (int rep = 0; rep < 20; ++rep) {
        dd acc = dd_of(0.0f), sq = dd_of(0.0f);
        long double ref = 0, ref_abs = 0, ref_sq = 0;
        for (int t = 0; t < 20000; ++t) {
            const dd a = dd_from_double(uni(rng)), b = dd_from_double(uni(rng));
            dd_acc_fma(acc, a, b);
            dd_acc_sqr(sq, a);
            if (t % 32 == 31) {  // as the pair kernel: once per unit
                acc = dd_renorm(acc);
                sq = dd_renorm(sq);
            }
            ref += ld(a) * ld(b);
            ref_abs += std::fabs(ld(a) * ld(b));
            ref_sq += ld(a) * ld(a);
        }
        e_dot = std::max(e_dot, std::fabs((long double)dd_to_double(acc) - ref) / ref_abs);
        e_sq = std::max(e_sq, std::fabs((long double)dd_to_double(sq) - ref_sq) / ref_sq);
    }
    report("acc_fma_20000", e_dot, 1e-12L);
    report("acc_sqr_20000", e_sq, 1e-12L);
    report("split", e_split, 1e-14L);
    report("add", e_add, 2e-14L);
    report("mul", e_mul, 2e-14L);
    report("sqr", e_sqr, 2e-14L);
    report("fma", e_fma, 2e-14L);
    report("rsqrt", e_rsq, 1e-13L);
    report("rcp", e_rcp, 1e-13L);
    report("div", e_div, 1e-13L);

    static float tab[kNormalDDFloats];
    normal_dd_table(tab);
    const long double inv_sqrt_2pi = 0.398942280401432677939946059934381868L;
    long double e_l = 0, e_h = 0, e_h_rel = 0;
    std::uniform_real_distribution<double> zd(0.0, 9.0);
    for (int t = 0; t < 400000; ++t) {
        const double zz = t < 1000 ? t * (9.0 / 1000) : zd(rng);
        const dd z = dd_from_double(zz);
        const long double Z = ld(z);
        dd lc, ratio;
        normal_dd(z, tab, lc, ratio);
        const long double Q = 0.5L * std::erfc(Z / std::sqrt(2.0L));
        const long double PHI = inv_sqrt_2pi * std::exp(-0.5L * Z * Z);
        const long double L = std::log1p(-Q), H = PHI / (1.0L - Q);
        e_l = std::max(e_l, std::fabs(ld(lc) - L));
        e_h = std::max(e_h, std::fabs(ld(ratio) - H));
        if (Z < 8.0L) e_h_rel = std::max(e_h_rel, std::fabs(ld(ratio) - H) / H);
    }
    report("normal_logcdf_abs", e_l, 5e-14L);
    {
        static double tab64[kNormalF64Doubles];
        normal_f64_table(tab64);
        long double e_l64 = 0, e_h64 = 0;
        for (int t = 0; t < 400000; ++t) {
            const double zz = t < 1000 ? t * (9.0 / 1000) : zd(rng);
            const long double Z = zz;
            double lc, ratio;
            normal_f64(zz, tab64, lc, ratio);
            const long double Q = 0.5L * std::erfc(Z / std::sqrt(2.0L));
            const long double PHI = inv_sqrt_2pi * std::exp(-0.5L * Z * Z);
            e_l64 = std::max(e_l64, std::fabs((long double)lc - std::log1p(-Q)));
            e_h64 = std::max(e_h64, std::fabs((long double)ratio - PHI / (1.0L - Q)));
        }
        report("normal_f64_logcdf_abs", e_l64, 5e-16L);
        report("normal_f64_ratio_abs", e_h64, 5e-16L);
    }
    report("normal_ratio_abs", e_h, 5e-14L);
    report("normal_ratio_rel_z<8", e_h_rel, 5e-10L);
    return failures ? 1 : 0;
}
