// x^y for finite x > 0 and |y| <= 1 with a short chain of dependent FP64 operations, for the
// step control of the device-side adaptive Tsit5 drivers.  On GB300 each dependent FP64
// operation of a single thread costs tens of nanoseconds, and the control runs on the
// critical path of every step.
//
// Method: table-driven logarithm and exponential after P. T. P. Tang, "Table-driven
// implementation of the exponential function in IEEE floating-point arithmetic" (ACM TOMS 15,
// 1989) and "Table-driven implementation of the logarithm function" (ACM TOMS 16, 1990):
//   x = 2^e m, m in [1, 2);  c = 1/inv_c[i] near m (i: the top 7 bits of m's fraction);
//   log2 x = e + log2(1/inv_c[i]) + log2(1 + r),  r = m inv_c[i] - 1,  |r| < 2^-7;
//   z = y log2 x = k + j/256 + f,  |f| <= 1/512;
//   x^y = 2^k 2^(j/256) 2^f.
// log2(1 + r) and 2^f are Taylor polynomials of degree 7 and 6 (truncation below 2^-60),
// evaluated in Estrin form; e + log2(1/inv_c[i]) and y log2 x are carried as two doubles.
// The tables are computed on the host in long double (pow_build_tables).  The CPU test
// tests/native/pow_accuracy.cpp bounds the error against long double pow.
//
// The same code runs on the host (CPU test of the accuracy) and the device; on the device
// every product and sum is an explicit round-to-nearest intrinsic so that nothing is
// contracted differently from the host build.
#pragma once
#include <cstdint>
#include <cstring>

#ifdef __CUDACC__
#define FVM_HD __host__ __device__ __forceinline__
#else
#define FVM_HD inline
#endif

namespace fvm {

struct PowTables {
    double inv_c[128];  // RN(1 / (1 + (i + 1/2) / 128))
    double log_c[128];  // log2(1 / inv_c[i]), rounded
    double exp2j[256];  // 2^(j / 256), rounded
    double klog[8];     // Taylor coefficients of log2(1 + r): klog[n] = (-1)^(n+1) / (n ln 2), n = 1..7
    double kexp[7];     // Taylor coefficients of 2^f: kexp[n] = (ln 2)^n / n!, n = 1..6
};

FVM_HD double pow_mul(double a, double b) {
#ifdef __CUDA_ARCH__
    return __dmul_rn(a, b);
#else
    return a * b;
#endif
}
FVM_HD double pow_add(double a, double b) {
#ifdef __CUDA_ARCH__
    return __dadd_rn(a, b);
#else
    return a + b;
#endif
}
FVM_HD double pow_fma(double a, double b, double c) {
#ifdef __CUDA_ARCH__
    return __fma_rn(a, b, c);
#else
    return __builtin_fma(a, b, c);
#endif
}
FVM_HD int64_t pow_bits(double v) {
#ifdef __CUDA_ARCH__
    return __double_as_longlong(v);
#else
    int64_t b;
    std::memcpy(&b, &v, sizeof b);
    return b;
#endif
}
FVM_HD double pow_from_bits(int64_t b) {
#ifdef __CUDA_ARCH__
    return __longlong_as_double(b);
#else
    double v;
    std::memcpy(&v, &b, sizeof v);
    return v;
#endif
}

// The tables, from long double arithmetic (64-bit or 113-bit significands on the hosts here);
// host code.
inline void pow_build_tables(PowTables& T) {
    for (int i = 0; i < 128; ++i) {
        const long double c = 1.0L + (i + 0.5L) / 128.0L;
        const double inv = (double)(1.0L / c);
        T.inv_c[i] = inv;
        T.log_c[i] = (double)(-__builtin_log2l((long double)inv));
    }
    for (int j = 0; j < 256; ++j) T.exp2j[j] = (double)__builtin_exp2l(j / 256.0L);
    const long double ln2 = __builtin_logl(2.0L);
    T.klog[0] = 0.0;
    for (int n = 1; n < 8; ++n) T.klog[n] = (double)(((n & 1) ? 1.0L : -1.0L) / (n * ln2));
    long double pw = 1.0L, fact = 1.0L;
    T.kexp[0] = 1.0;
    for (int n = 1; n < 7; ++n) {
        pw *= ln2;
        fact *= n;
        T.kexp[n] = (double)(pw / fact);
    }
}

// x^y for finite x > 0 and |y log2 x| < 1000 (no checks: callers pass such values)
FVM_HD double pow_pos(double x, double y, const PowTables& T) {
    int64_t bits = pow_bits(x);
    int64_t ex = (bits >> 52) & 0x7ff;
    int64_t scale = 0;
    if (ex == 0) {  // subnormal: scale into the normal range
        bits = pow_bits(pow_mul(x, 18446744073709551616.0));  // 2^64
        ex = (bits >> 52) & 0x7ff;
        scale = 64;
    }
    const int64_t e = ex - 1023 - scale;
    const int i = (int)((bits >> 45) & 127);
    const double m = pow_from_bits((bits & 0x000fffffffffffffLL) | 0x3ff0000000000000LL);
    const double r = pow_fma(m, T.inv_c[i], -1.0);
    // log2(1 + r) = r (k1 + k2 r + k3 r^2 + ... + k7 r^6), Estrin
    const double r2 = pow_mul(r, r);
    const double a01 = pow_fma(T.klog[2], r, T.klog[1]);
    const double a23 = pow_fma(T.klog[4], r, T.klog[3]);
    const double a45 = pow_fma(T.klog[6], r, T.klog[5]);
    const double r4 = pow_mul(r2, r2);
    const double b0 = pow_fma(a23, r2, a01);
    const double b1 = pow_fma(T.klog[7], r2, a45);
    const double poly = pow_mul(r, pow_fma(b1, r4, b0));
    // log2 x = hi + lo + poly with hi + lo = e + log_c[i] exactly (Fast2Sum: |e| >= |log_c|
    // unless e = 0, when hi is log_c itself), so the rounding of a large e + log_c is not
    // amplified by y
    const double hi = pow_add((double)e, T.log_c[i]);
    const double lo = pow_add(pow_add((double)e, -hi), T.log_c[i]);
    const double tail = pow_add(lo, poly);
    // z = y log2 x as zh + zl
    const double zh = pow_mul(y, hi);
    const double zl = pow_fma(y, tail, pow_fma(y, hi, -zh));
    const double zn = pow_mul(zh, 256.0);
#ifdef __CUDA_ARCH__
    const double nn = rint(zn);
#else
    const double nn = __builtin_rint(zn);
#endif
    const int64_t n = (int64_t)nn;
    const double f = pow_add(pow_fma(nn, -0.00390625, zh), zl);  // zh - n / 256 is exact
    const int j = (int)(n & 255);
    const int64_t k = (n - j) / 256;
    // 2^f - 1 = f (e1 + e2 f + ... + e6 f^5), Estrin
    const double f2 = pow_mul(f, f);
    const double c01 = pow_fma(T.kexp[2], f, T.kexp[1]);
    const double c23 = pow_fma(T.kexp[4], f, T.kexp[3]);
    const double c45 = pow_fma(T.kexp[6], f, T.kexp[5]);
    const double f4 = pow_mul(f2, f2);
    const double d0 = pow_fma(c23, f2, c01);
    const double q = pow_mul(f, pow_fma(c45, f4, d0));
    const double v = pow_fma(T.exp2j[j], q, T.exp2j[j]);
    return pow_mul(v, pow_from_bits((k + 1023) << 52));
}

}  // namespace fvm
