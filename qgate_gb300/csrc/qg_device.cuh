// Device-side helpers: complex arithmetic on float2/double2 and index
// bit insertion.
#pragma once

#include <cuda_runtime.h>
#include "qg_internal.h"

namespace qg {

template <class R> struct CT;
template <> struct CT<float> { typedef float2 type; typedef float4 vec; };
template <> struct CT<double> { typedef double2 type; typedef double2 vec; };

template <class C> __device__ __forceinline__ C cmk(double re, double im) {
    C c;
    c.x = re;
    c.y = im;
    return c;
}
template <class C> __device__ __forceinline__ C cadd(C a, C b) {
    C c;
    c.x = a.x + b.x;
    c.y = a.y + b.y;
    return c;
}
template <class C> __device__ __forceinline__ C cmul(C a, C b) {
    C c;
    c.x = a.x * b.x - a.y * b.y;
    c.y = a.x * b.y + a.y * b.x;
    return c;
}
template <class C, class S> __device__ __forceinline__ C cscale(C a, S s) {
    C c;
    c.x = a.x * s;
    c.y = a.y * s;
    return c;
}
// m0 * a + m1 * b
template <class C> __device__ __forceinline__ C cdot2(C m0, C a, C m1, C b) {
    C c;
    c.x = m0.x * a.x - m0.y * a.y + m1.x * b.x - m1.y * b.y;
    c.y = m0.x * a.y + m0.y * a.x + m1.x * b.y + m1.y * b.x;
    return c;
}

// Matrix in the state's precision.
template <class R> struct MatR {
    typename CT<R>::type m00, m01, m10, m11;
};
template <class R> __device__ __forceinline__ MatR<R> to_matr(const double *v) {
    typedef typename CT<R>::type C;
    MatR<R> r;
    r.m00 = cmk<C>(v[0], v[1]);
    r.m01 = cmk<C>(v[2], v[3]);
    r.m10 = cmk<C>(v[4], v[5]);
    r.m11 = cmk<C>(v[6], v[7]);
    return r;
}
template <class R, class C> __device__ __forceinline__ void apply2(const MatR<R> &m, C &a, C &b) {
    C o0 = cdot2(m.m00, a, m.m01, b);
    C o1 = cdot2(m.m10, a, m.m11, b);
    a = o0;
    b = o1;
}

// ---- double-float arithmetic (complex128 register stages)
//
// An FP64 value carried as the unevaluated sum h + l of two FP32 values
// (|l| <= ulp(h) / 2): about 48 significant bits, with all arithmetic on the
// FP32 pipes, whose rate on GB300 is 64x the FP64 rate.  The error-free
// transformations are Knuth's two-sum and the FMA two-product (Dekker 1971;
// Shewchuk 1997); the explicit _rn intrinsics keep the compiler from
// contracting a rounded product into a later add.  Each operation's error is
// about 2^-48 of its operands' magnitude.
struct dfl {
    float h, l;
};
struct dfc {  // complex, 16 bytes like double2
    dfl x, y;
};

__device__ __forceinline__ dfl df_fast_two_sum(float a, float b) {  // |a| >= |b|
    const float s = __fadd_rn(a, b);
    return {s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ void df_two_sum(float a, float b, float &s, float &e) {
    s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}
// a * b as (product, error): product = fl(a.h b.h), error = the rest to FP32
// precision.
__device__ __forceinline__ void df_prod(dfl a, dfl b, float &p, float &e) {
    p = __fmul_rn(a.h, b.h);
    e = __fmaf_rn(a.h, b.h, -p);
    e = __fmaf_rn(a.h, b.l, e);
    e = __fmaf_rn(a.l, b.h, e);
}
__device__ __forceinline__ dfl df_neg(dfl a) { return {-a.h, -a.l}; }
// p0 + p1 (+ p2 + p3): products given as (p, e) pairs.
__device__ __forceinline__ dfl df_sum2(float p0, float e0, float p1, float e1) {
    float s, t;
    df_two_sum(p0, p1, s, t);
    return df_fast_two_sum(s, __fadd_rn(t, __fadd_rn(e0, e1)));
}
__device__ __forceinline__ dfl df_sum4(float p0, float e0, float p1, float e1, float p2, float e2,
                                       float p3, float e3) {
    float s, t1, t2, t3;
    df_two_sum(p0, p1, s, t1);
    df_two_sum(s, p2, s, t2);
    df_two_sum(s, p3, s, t3);
    const float err = __fadd_rn(__fadd_rn(__fadd_rn(t1, t2), __fadd_rn(t3, e0)),
                                __fadd_rn(__fadd_rn(e1, e2), e3));
    return df_fast_two_sum(s, err);
}
// FP64 -> double-float with integer work only (the FP64 pipe is scarce): h =
// the top 24 significant bits of v (truncated), l = the next 29 bits rounded
// to FP32, so |h + l - v| <= 2^-48 |v| for |v| >= 2^-74; smaller values keep
// only h (absolute error < 2^-97), values below 2^-126 read as zero.
__device__ __forceinline__ dfl df_from(double v) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(v);
    const unsigned hi32 = (unsigned)(b >> 32), lo32 = (unsigned)b;
    const int e = (int)((hi32 >> 20) & 0x7ffu);
    const unsigned sign = hi32 & 0x80000000u;
    if (e < 1023 - 126) return {__uint_as_float(sign), 0.f};
    const unsigned mh = ((hi32 & 0xfffffu) << 3) | (lo32 >> 29);
    const float h = __uint_as_float(sign | ((unsigned)(e - 1023 + 127) << 23) | mh);
    const unsigned r = lo32 & 0x1fffffffu;  // the rest: r * 2^(e - 1075)
    float l = 0.f;
    if (e >= 1075 - 126 && r) {
        l = __fmul_rn(__uint2float_rn(r), __uint_as_float((unsigned)(e - 1075 + 127) << 23));
        if (sign) l = -l;
    }
    return {h, l};
}
// FP32 -> FP64 by widening the bits (exact; zero and FP32 subnormals read as 0).
__device__ __forceinline__ double f32_widen(float f) {
    const unsigned u = __float_as_uint(f);
    const unsigned e = (u >> 23) & 0xffu;
    if (e == 0) return 0.;
    return __hiloint2double((int)((u & 0x80000000u) | ((e - 127u + 1023u) << 20) |
                                  ((u & 0x7fffffu) >> 3)),
                            (int)(u << 29));
}
// double-float -> FP64: one FP64 add.
__device__ __forceinline__ double df_to(dfl a) { return f32_widen(a.h) + f32_widen(a.l); }

// a * b
__device__ __forceinline__ dfc cmul(dfc a, dfc b) {
    float p0, e0, p1, e1, p2, e2, p3, e3;
    df_prod(a.x, b.x, p0, e0);
    df_prod(df_neg(a.y), b.y, p1, e1);
    df_prod(a.x, b.y, p2, e2);
    df_prod(a.y, b.x, p3, e3);
    return {df_sum2(p0, e0, p1, e1), df_sum2(p2, e2, p3, e3)};
}
// m0 * a + m1 * b
__device__ __forceinline__ dfc cdot2(dfc m0, dfc a, dfc m1, dfc b) {
    float p0, e0, p1, e1, p2, e2, p3, e3;
    dfc c;
    df_prod(m0.x, a.x, p0, e0);
    df_prod(df_neg(m0.y), a.y, p1, e1);
    df_prod(m1.x, b.x, p2, e2);
    df_prod(df_neg(m1.y), b.y, p3, e3);
    c.x = df_sum4(p0, e0, p1, e1, p2, e2, p3, e3);
    df_prod(m0.x, a.y, p0, e0);
    df_prod(m0.y, a.x, p1, e1);
    df_prod(m1.x, b.y, p2, e2);
    df_prod(m1.y, b.x, p3, e3);
    c.y = df_sum4(p0, e0, p1, e1, p2, e2, p3, e3);
    return c;
}

// Register arithmetic of the fused stages: complex64 as is; complex128 in
// double-float, converted from the staged tile on the first register load
// and back on the last store, with matrix entries packed on the host as
// (h, l) FP32 pairs in the 8-byte slots of the op's FP64 entries.
template <class C> struct Mat2C {
    C m00, m01, m10, m11;
};
template <class C> __device__ __forceinline__ void apply2c(const Mat2C<C> &m, C &a, C &b) {
    C o0 = cdot2(m.m00, a, m.m01, b);
    C o1 = cdot2(m.m10, a, m.m11, b);
    a = o0;
    b = o1;
}
template <class R> struct RegArith;
template <> struct RegArith<float> {
    typedef float2 T;
    static __device__ __forceinline__ T from_tile(float2 v) { return v; }
    static __device__ __forceinline__ float2 to_tile(T v) { return v; }
    static __device__ __forceinline__ T entry(const float *m, int k) {
        return make_float2(m[2 * k], m[2 * k + 1]);
    }
};
template <> struct RegArith<double> {
    typedef dfc T;
    static __device__ __forceinline__ T from_tile(double2 v) { return {df_from(v.x), df_from(v.y)}; }
    static __device__ __forceinline__ double2 to_tile(T v) {
        return make_double2(df_to(v.x), df_to(v.y));
    }
    // the host packs (h, l) into an entry's 8 bytes little-endian: h low, l high
    static __device__ __forceinline__ dfl unpack(double v) {
        const unsigned long long b = (unsigned long long)__double_as_longlong(v);
        return {__uint_as_float((unsigned)b), __uint_as_float((unsigned)(b >> 32))};
    }
    static __device__ __forceinline__ T entry(const double *m, int k) {
        return {unpack(m[2 * k]), unpack(m[2 * k + 1])};
    }
};

// Insert a zero bit at position p of k.
__device__ __forceinline__ idx_t insert_zero(idx_t k, int p) {
    idx_t lo = k & ((1LL << p) - 1);
    return ((k >> p) << (p + 1)) | lo;
}
__device__ __forceinline__ idx_t insert_zeros(idx_t k, const int *pos, int npos) {
    for (int i = 0; i < npos; ++i) k = insert_zero(k, pos[i]);
    return k;
}

}  // namespace qg
