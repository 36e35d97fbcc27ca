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
