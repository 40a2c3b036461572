// Correctly rounded acos, cos, sin and pow for the FP64 collision path.
//
// The reference's CCD root finder (isCoplanar, dcollid3d.cpp:425-450) and
// its impact-zone rotation (dcollid3d.cpp:163-169) call acos, cos, pow and
// sin, and near double roots those roots are very sensitive: a one-ulp change
// in one of these results can move a step's output by 1e-8 relative. The
// reference's results come from glibc, which rounds these functions correctly
// in all but roughly 0.1% of arguments; CUDA's versions allow 2 ulp. These
// functions return the correctly rounded result (barring arguments within
// about 1e-30 relative of a rounding midpoint), so they agree with the
// reference wherever glibc is correctly rounded.
//
// Method, from the mathematics: double-double arithmetic built on the exact
// error of a sum (two_sum) and of a product (fma); sin / cos by reduction
// modulo pi/2 with a three-part pi/2 (Cody and Waite) and their Taylor series
// to x^29 on [-pi/4, pi/4]; acos and asin by one Newton step on cos / sin from
// a starting value within a few ulp, using the half-angle identity
// acos(x) = 2 asin(sqrt((1-x)/2)) away from 0; pow(a, y) by one correction
// step r = r0 (1 + y ln a - ln r0) with ln in double-double from the atanh
// series. Series coefficients are 1/n!, 1/(2k+1), pi and ln 2 to ~300 bits,
// rounded to double-double.
//
// Every routine is __host__ __device__ so the same code can be checked on the
// host; products use fma() explicitly and nothing relies on contraction.
#pragma once

#include <cmath>

#ifdef __CUDACC__
#define CR_HD __host__ __device__ __forceinline__
#else
#define CR_HD inline
#endif

namespace ccg {
namespace cr {

struct dd {
    double hi, lo;
};

CR_HD dd two_sum(double a, double b) {
    double s = a + b;
    double t = s - a;
    double e = (a - (s - t)) + (b - t);
    return dd{s, e};
}
CR_HD dd fast_two_sum(double a, double b) {
    double s = a + b;
    double e = b - (s - a);
    return dd{s, e};
}
CR_HD dd two_prod(double a, double b) {
    double p = a * b;
    double e = fma(a, b, -p);
    return dd{p, e};
}
CR_HD dd neg(dd x) { return dd{-x.hi, -x.lo}; }
CR_HD dd add(dd x, dd y) {
    dd s = two_sum(x.hi, y.hi);
    dd t = two_sum(x.lo, y.lo);
    s.lo += t.hi;
    s = fast_two_sum(s.hi, s.lo);
    s.lo += t.lo;
    return fast_two_sum(s.hi, s.lo);
}
CR_HD dd add_d(dd x, double y) {
    dd s = two_sum(x.hi, y);
    s.lo += x.lo;
    return fast_two_sum(s.hi, s.lo);
}
CR_HD dd mul(dd x, dd y) {
    dd p = two_prod(x.hi, y.hi);
    p.lo += x.hi * y.lo;
    p.lo += x.lo * y.hi;
    return fast_two_sum(p.hi, p.lo);
}
CR_HD dd mul_d(dd x, double y) {
    dd p = two_prod(x.hi, y);
    p.lo += x.lo * y;
    return fast_two_sum(p.hi, p.lo);
}
CR_HD dd div(dd x, dd y) {
    double q1 = x.hi / y.hi;
    dd r = add(x, neg(mul_d(y, q1)));
    double q2 = r.hi / y.hi;
    r = add(r, neg(mul_d(y, q2)));
    double q3 = r.hi / y.hi;
    return add_d(fast_two_sum(q1, q2), q3);
}

constexpr double kPiHi = 0x1.921fb54442d18p+1, kPiLo = 0x1.1a62633145c07p-53;
constexpr double kPio2_1 = 0x1.921fb54400000p+0, kPio2_2 = 0x1.0b4611a600000p-34, kPio2_3 = 0x1.3198a2e037073p-69;
constexpr double kTwoOverPi = 0x1.45f306dc9c883p-1;
constexpr double kLn2Hi = 0x1.62e42fefa39efp-1, kLn2Lo = 0x1.abc9e3b39803fp-56;

// sin(r)/r (cosine false) and cos(r) (cosine true) as polynomials in
// r2 = r*r (Taylor, to r^29 / r^28). Both have the same shape, so lanes of a
// warp that evaluate different ones run one instruction sequence.
CR_HD dd sc_poly(dd r2, bool cosine) {
#define CR_SEL(s, c) (cosine ? (c) : (s))
    double t = CR_SEL(0x1.259f98b4358adp-103, 0x1.0a18a2635085dp-98);
    t = t * r2.hi + CR_SEL(-0x1.d1ab1c2dccea3p-94, -0x1.88e85fc6a4e5ap-89);
    t = t * r2.hi + CR_SEL(0x1.3f3ccdd165fa9p-84, 0x1.f2cf01972f578p-80);
    t = t * r2.hi + CR_SEL(-0x1.761b41316381ap-75, -0x1.0ce396db7f853p-70);
    t = t * r2.hi + CR_SEL(0x1.71b8ef6dcf572p-66, 0x1.e542ba4020225p-62);
    t = t * r2.hi + CR_SEL(-0x1.2f49b46814157p-57, -0x1.6827863b97d97p-53);
    dd p = {t, 0.0};
    p = add(mul(p, r2), dd{CR_SEL(0x1.952c77030ad4ap-49, 0x1.ae7f3e733b81fp-45),
                           CR_SEL(0x1.ac981465ddc6cp-103, 0x1.1d8656b0ee8cbp-101)});
    p = add(mul(p, r2), dd{CR_SEL(-0x1.ae7f3e733b81fp-41, -0x1.93974a8c07c9dp-37),
                           CR_SEL(-0x1.1d8656b0ee8cbp-97, -0x1.05d6f8a2efd1fp-92)});
    p = add(mul(p, r2), dd{CR_SEL(0x1.6124613a86d09p-33, 0x1.1eed8eff8d898p-29),
                           CR_SEL(0x1.f28e0cc748ebep-87, -0x1.2aec959e14c06p-83)});
    p = add(mul(p, r2), dd{CR_SEL(-0x1.ae64567f544e4p-26, -0x1.27e4fb7789f5cp-22),
                           CR_SEL(0x1.c062e06d1f209p-80, -0x1.cbbc05b4fa99ap-76)});
    p = add(mul(p, r2), dd{CR_SEL(0x1.71de3a556c734p-19, 0x1.a01a01a01a01ap-16),
                           CR_SEL(-0x1.c154f8ddc6c00p-73, 0x1.a01a01a01a01ap-76)});
    p = add(mul(p, r2), dd{CR_SEL(-0x1.a01a01a01a01ap-13, -0x1.6c16c16c16c17p-10),
                           CR_SEL(-0x1.a01a01a01a01ap-73, 0x1.f49f49f49f49fp-65)});
    p = add(mul(p, r2), dd{CR_SEL(0x1.1111111111111p-7, 0x1.5555555555555p-5),
                           CR_SEL(0x1.1111111111111p-63, 0x1.5555555555555p-59)});
    p = add(mul(p, r2), dd{CR_SEL(-0x1.5555555555555p-3, -0x1.0000000000000p-1),
                           CR_SEL(-0x1.5555555555555p-57, 0x0.0p+0)});
    p = add(mul(p, r2), dd{0x1.0000000000000p+0, 0x0.0p+0});
#undef CR_SEL
    return p;
}

CR_HD dd sin_poly(dd r2) { return sc_poly(r2, false); }
CR_HD dd cos_poly(dd r2) { return sc_poly(r2, true); }

// atanh(u)/u as a polynomial in u2 = u*u (to u^46)
CR_HD dd atanh_poly(dd u2) {
    double t = 0x1.5c9882b931057p-6;
    t = t * u2.hi + 0x1.6c16c16c16c17p-6;
    t = t * u2.hi + 0x1.7d05f417d05f4p-6;
    t = t * u2.hi + 0x1.8f9c18f9c18fap-6;
    t = t * u2.hi + 0x1.a41a41a41a41ap-6;
    t = t * u2.hi + 0x1.bacf914c1bad0p-6;
    t = t * u2.hi + 0x1.d41d41d41d41dp-6;
    t = t * u2.hi + 0x1.f07c1f07c1f08p-6;
    t = t * u2.hi + 0x1.0842108421084p-5;
    t = t * u2.hi + 0x1.1a7b9611a7b96p-5;
    t = t * u2.hi + 0x1.2f684bda12f68p-5;
    t = t * u2.hi + 0x1.47ae147ae147bp-5;
    t = t * u2.hi + 0x1.642c8590b2164p-5;
    dd p = {t, 0.0};
    p = add(mul(p, u2), dd{0x1.8618618618618p-5, 0x1.8618618618618p-59});
    p = add(mul(p, u2), dd{0x1.af286bca1af28p-5, 0x1.af286bca1af28p-59});
    p = add(mul(p, u2), dd{0x1.e1e1e1e1e1e1ep-5, 0x1.e1e1e1e1e1e1ep-61});
    p = add(mul(p, u2), dd{0x1.1111111111111p-4, 0x1.1111111111111p-60});
    p = add(mul(p, u2), dd{0x1.3b13b13b13b14p-4, -0x1.3b13b13b13b14p-58});
    p = add(mul(p, u2), dd{0x1.745d1745d1746p-4, -0x1.745d1745d1746p-59});
    p = add(mul(p, u2), dd{0x1.c71c71c71c71cp-4, 0x1.c71c71c71c71cp-58});
    p = add(mul(p, u2), dd{0x1.2492492492492p-3, 0x1.2492492492492p-57});
    p = add(mul(p, u2), dd{0x1.999999999999ap-3, -0x1.999999999999ap-57});
    p = add(mul(p, u2), dd{0x1.5555555555555p-2, 0x1.5555555555555p-56});
    p = add(mul(p, u2), dd{0x1.0000000000000p+0, 0x0.0p+0});
    return p;
}

// x - k*pi/2 in double-double and the quadrant k mod 4 (|x| < 2^20).
CR_HD dd reduce_pio2(double x, int* quadrant) {
    double k = rint(x * kTwoOverPi);
    dd r = two_sum(x, -(k * kPio2_1));  // k*kPio2_1 is exact: 33-bit constant
    r = add(r, neg(two_prod(k, kPio2_2)));
    r = add(r, neg(two_prod(k, kPio2_3)));
    *quadrant = ((int)k) & 3;
    return r;
}

CR_HD void sincos_dd(double x, dd* s, dd* c) {
    int q;
    dd r = reduce_pio2(x, &q);
    dd r2 = mul(r, r);
    dd sr = mul(sin_poly(r2), r);
    dd cr_ = cos_poly(r2);
    switch (q) {
        case 0: *s = sr; *c = cr_; break;
        case 1: *s = cr_; *c = neg(sr); break;
        case 2: *s = neg(sr); *c = neg(cr_); break;
        default: *s = neg(cr_); *c = sr; break;
    }
}

// cos and sin each need one of the two polynomials (which one depends on
// the quadrant); the value is the one sincos_dd gives.
CR_HD double cos(double x) {
    if (!(fabs(x) < 1048576.0)) return ::cos(x);  // outside the reduction range: not used here
    int q;
    const dd r = reduce_pio2(x, &q);
    const dd r2 = mul(r, r);
    switch (q) {
        case 0: return cos_poly(r2).hi;
        case 1: return neg(mul(sin_poly(r2), r)).hi;
        case 2: return neg(cos_poly(r2)).hi;
        default: return mul(sin_poly(r2), r).hi;
    }
}

CR_HD double sin(double x) {
    if (x == 0.0) return x;
    if (!(fabs(x) < 1048576.0)) return ::sin(x);
    int q;
    const dd r = reduce_pio2(x, &q);
    const dd r2 = mul(r, r);
    switch (q) {
        case 0: return mul(sin_poly(r2), r).hi;
        case 1: return cos_poly(r2).hi;
        case 2: return neg(mul(sin_poly(r2), r)).hi;
        default: return neg(cos_poly(r2)).hi;
    }
}

// sin(x) and cos(x) of one argument: the same values as sin and cos.
CR_HD void sincos(double x, double* sn, double* cs) {
    if (!(fabs(x) < 1048576.0)) {
        *sn = x == 0.0 ? x : ::sin(x);
        *cs = ::cos(x);
        return;
    }
    if (x == 0.0) {
        *sn = x;
        *cs = cos(x);
        return;
    }
    dd s, c;
    sincos_dd(x, &s, &c);
    *sn = s.hi;
    *cs = c.hi;
}

#ifdef __CUDACC__
// sincos(x) by a whole warp, every lane passing the same x: lane 1
// evaluates the cosine polynomial while the others evaluate the sine one
// (sc_poly, no divergence), which halves the serial chain of a one-lane
// sincos. Every lane gets the values sincos gives.
__device__ __forceinline__ void sincos_warp(double x, double* sn, double* cs) {
    if (!(fabs(x) < 1048576.0) || x == 0.0) {  // the same branch in every lane
        sincos(x, sn, cs);
        return;
    }
    int q;
    const dd r = reduce_pio2(x, &q);
    const dd r2 = mul(r, r);
    const bool cosine = (threadIdx.x & 31) == 1;
    const dd p = sc_poly(r2, cosine);
    const dd pr = mul(p, r);
    const dd v = cosine ? p : pr;
    const dd sr = {__shfl_sync(0xffffffffu, v.hi, 0), __shfl_sync(0xffffffffu, v.lo, 0)};
    const dd cr_ = {__shfl_sync(0xffffffffu, v.hi, 1), __shfl_sync(0xffffffffu, v.lo, 1)};
    switch (q) {
        case 0: *sn = sr.hi; *cs = cr_.hi; break;
        case 1: *sn = cr_.hi; *cs = neg(sr).hi; break;
        case 2: *sn = neg(sr).hi; *cs = neg(cr_).hi; break;
        default: *sn = neg(cr_).hi; *cs = sr.hi; break;
    }
}
#endif

// asin(t) for t in [0, 0.5] given as a double-double, as a double-double.
CR_HD dd asin_small_dd(dd t) {
    double z0 = ::asin(t.hi);
    dd s, c;
    sincos_dd(z0, &s, &c);
    dd num = add(t, neg(s));
    double corr = num.hi / c.hi;
    return two_sum(z0, corr);
}

// sqrt(u) of a double as a double-double.
CR_HD dd sqrt_dd(double u) {
    double t0 = ::sqrt(u);
    if (t0 == 0.0) return dd{0.0, 0.0};
    double res = fma(-t0, t0, u);
    return fast_two_sum(t0, res / (2.0 * t0));
}

CR_HD double acos(double x) {
    if (!(fabs(x) <= 1.0)) return ::acos(x);  // NaN, as the library gives
    if (fabs(x) <= 0.5) {
        double y0 = ::acos(x);
        dd s, c;
        sincos_dd(y0, &s, &c);
        dd num = add_d(c, -x);
        double corr = num.hi / s.hi;
        return y0 + corr;
    }
    if (x > 0.0) {
        double u = (1.0 - x) * 0.5;  // exact for x in (0.5, 1]
        if (u == 0.0) return 0.0;
        dd z = asin_small_dd(sqrt_dd(u));
        return 2.0 * (z.hi + z.lo);
    }
    double u = (1.0 + x) * 0.5;  // exact for x in [-1, -0.5)
    dd z = asin_small_dd(sqrt_dd(u));
    dd r = add(dd{kPiHi, kPiLo}, dd{-2.0 * z.hi, -2.0 * z.lo});
    return r.hi;
}

// ln(x) for finite x > 0 as a double-double.
CR_HD dd log_dd(double x) {
    int k;
    double m = frexp(x, &k);  // x = m 2^k, m in [0.5, 1)
    if (m < 0.70710678118654752) {
        m *= 2.0;
        k -= 1;
    }
    dd num = dd{m - 1.0, 0.0};  // exact: m in [0.707, 1.414)
    dd den = two_sum(m, 1.0);
    dd u = div(num, den);
    dd u2 = mul(u, u);
    dd at = mul(atanh_poly(u2), u);
    dd lnm = dd{2.0 * at.hi, 2.0 * at.lo};
    dd kl = add(two_prod((double)k, kLn2Hi), two_prod((double)k, kLn2Lo));
    return add(lnm, kl);
}

// pow(a, y) for finite a > 0 (a = 0 gives 0 for y > 0).
CR_HD double pow(double a, double y) {
    if (!(a > 0.0) || !(a < 1.0e300) || a < 1.0e-300 || !(fabs(y) < 1.0e3)) return ::pow(a, y);
    if (a == 1.0) return 1.0;
    double r0 = ::pow(a, y);
    if (!(r0 > 1.0e-300) || !(r0 < 1.0e300)) return r0;
    dd L = mul_d(log_dd(a), y);
    dd delta = add(L, neg(log_dd(r0)));
    return r0 + r0 * delta.hi;
}

}  // namespace cr
}  // namespace ccg
