// Building blocks of the register-resident stage kernels (forward gate
// stages and the adjoint engine's batched stages).
#pragma once

#include "qg_device.cuh"

namespace qg {
namespace rs {

// XOR swizzle of shared-memory element slots: a GF(2)-linear bijection that
// spreads the bits above the bank index into it, so that both "thread lanes
// low" and "register lanes low" access patterns hit distinct banks.  8-byte
// complex64 slots: 16 per 128-byte row; 16-byte complex128 slots: 8 per row.
template <class R> struct Swz;
template <> struct Swz<float> {
    __device__ __forceinline__ static unsigned f(unsigned e) {
        return e ^ (((e >> 4) ^ (e >> 8) ^ (e >> 12)) & 15u);
    }
};
template <> struct Swz<double> {
    __device__ __forceinline__ static unsigned f(unsigned e) {
        return e ^ (((e >> 3) ^ (e >> 6) ^ (e >> 9) ^ (e >> 12)) & 7u);
    }
};

__device__ __forceinline__ unsigned pdep_sw(unsigned x, unsigned mask) {
    unsigned r = 0;
    for (unsigned b = 1; mask; b <<= 1) {
        unsigned low = mask & (0u - mask);
        if (x & b) r |= low;
        mask &= mask - 1;
    }
    return r;
}

template <class C> __device__ __forceinline__ void cp_async_elem(C *smem, const C *gmem) {
    unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
    if (sizeof(C) == 16)
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(gmem) : "memory");
    else
        asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(sa), "l"(gmem) : "memory");
}

// Shared-memory slot of register j: P0 ^ (XOR of q[k] over the set bits k of j).
__device__ __forceinline__ void copy_sets(SetSlots *dst, const SetSlots *src, int nsets,
                                          unsigned tid, unsigned T) {
    static_assert(sizeof(SetSlots) % 4 == 0, "SetSlots size");
    const unsigned *s = (const unsigned *)src;
    unsigned *d = (unsigned *)dst;
    const int words = nsets * (int)(sizeof(SetSlots) / 4);
    for (int i = tid; i < words; i += T) d[i] = s[i];
}

template <int RL>
__device__ __forceinline__ unsigned reg_slot(unsigned P0, const unsigned (&q)[RL], int j) {
    unsigned a = P0;
#pragma unroll
    for (int k = 0; k < RL; ++k)
        if (j & (1 << k)) a ^= q[k];
    return a;
}

template <int I, int NR, class R, class C>
__device__ __forceinline__ void reg_gate(C (&a)[NR], const MatR<R> &m, unsigned jmask) {
    if (jmask == 0) {
#pragma unroll
        for (int j = 0; j < NR; ++j)
            if (!(j & (1 << I))) apply2<R>(m, a[j], a[j | (1 << I)]);
    } else {
#pragma unroll
        for (int j = 0; j < NR; ++j)
            if (!(j & (1 << I)) && (j & jmask) == jmask) apply2<R>(m, a[j], a[j | (1 << I)]);
    }
}

// reg_gate with the matrix in the register arithmetic's own type.
template <int I, int NR, class C>
__device__ __forceinline__ void reg_gate_c(C (&a)[NR], const Mat2C<C> &m, unsigned jmask) {
    if (jmask == 0) {
#pragma unroll
        for (int j = 0; j < NR; ++j)
            if (!(j & (1 << I))) apply2c(m, a[j], a[j | (1 << I)]);
    } else {
#pragma unroll
        for (int j = 0; j < NR; ++j)
            if (!(j & (1 << I)) && (j & jmask) == jmask) apply2c(m, a[j], a[j | (1 << I)]);
    }
}

template <int I, int NR, class C>
__device__ __forceinline__ void reg_swap(C (&a)[NR], unsigned jmask) {
#pragma unroll
    for (int j = 0; j < NR; ++j) {
        if (j & (1 << I)) continue;
        if ((j & jmask) != jmask) continue;
        C t = a[j];
        a[j] = a[j | (1 << I)];
        a[j | (1 << I)] = t;
    }
}

template <int I, int NR, class C>
__device__ __forceinline__ void reg_diag(C (&a)[NR], C d0, C d1, unsigned jmask) {
#pragma unroll
    for (int j = 0; j < NR; ++j) {
        if ((j & jmask) != jmask) continue;
        a[j] = cmul((j & (1 << I)) ? d1 : d0, a[j]);
    }
}

// Uniform if-chain over the register bit (no jump table).
#define QG_REG_DISPATCH(FN, REG, ...)                                         \
    do {                                                                      \
        const int _r = (REG);                                                 \
        if (_r == 0) FN<0, NR>(__VA_ARGS__);                                  \
        else if (RL > 1 && _r == 1) FN<(RL > 1 ? 1 : 0), NR>(__VA_ARGS__);    \
        else if (RL > 2 && _r == 2) FN<(RL > 2 ? 2 : 0), NR>(__VA_ARGS__);    \
        else if (RL > 3 && _r == 3) FN<(RL > 3 ? 3 : 0), NR>(__VA_ARGS__);    \
        else if (RL > 4) FN<(RL > 4 ? 4 : 0), NR>(__VA_ARGS__);               \
    } while (0)

}  // namespace rs
}  // namespace qg
