// Reductions, gathers and the sampling-pool kernels (sm_103a).
//
// All accumulations are FP64 regardless of the state's precision (the
// reference accumulates in the state's own precision:
// qgate/simulator/src/DeviceProcPrimitives.cu:36-54,
// qgate/simulator/src/CPUSamplingPool.cpp:16-49).  Reductions write one
// partial per block and a single-block pass sums the partials in a fixed
// order, so results are bit-reproducible run to run.
#include <algorithm>

#include "qg_bulk.cuh"
#include "qg_device.cuh"

namespace qg {

namespace {

constexpr int kRedThreads = 256;
// 8 CTAs of 256 threads on each of 152 SMs and 8 loads in flight per thread
// before any arithmetic: enough bytes in flight to cover HBM latency.
constexpr int kRedBlocks = 152 * 8;
constexpr int kUnroll = 8;

__device__ __forceinline__ double block_sum(double v) {
    __shared__ double warp_sums[32];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) warp_sums[warp] = v;
    __syncthreads();
    int nw = blockDim.x >> 5;
    v = (threadIdx.x < nw) ? warp_sums[threadIdx.x] : 0.;
    if (warp == 0)
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;  // valid in thread 0
}

__global__ void k_final_sum(const double *__restrict__ partials, int n, double *out) {
    double v = 0.;
    for (int i = threadIdx.x; i < n; i += blockDim.x) v += partials[i];
    v = block_sum(v);
    if (threadIdx.x == 0) *out = v;
}

template <class C> __device__ __forceinline__ double abs2d(C c) {
    return (double)c.x * (double)c.x + (double)c.y * (double)c.y;
}

// |c|^2 in the state's precision.  complex64 terms are formed and summed in
// FP32 over a short unrolled run (kUnroll items) and only that partial is
// added to the FP64 accumulator: GB300's FP64 rate is a small fraction of its
// FP32 rate, and a per-element FP64 multiply-add would make these HBM sweeps
// compute-bound.  The FP32 partial of a few terms carries a relative error of
// a few 1e-8, below the precision of the complex64 amplitudes themselves;
// the long accumulation is FP64.
template <class C> __device__ __forceinline__ auto abs2r(C c) { return c.x * c.x + c.y * c.y; }

// Pr(lane == 0): sum of |psi[i0]|^2 over the pair sweep's first members.
template <class R>
__global__ void __launch_bounds__(kRedThreads)
k_prob_scalar(const typename CT<R>::type *__restrict__ s, idx_t n_items, PairIdx pi,
              double *partials) {
    double acc = 0.;
    const idx_t stride = (idx_t)gridDim.x * blockDim.x;
    idx_t k = (idx_t)blockIdx.x * blockDim.x + threadIdx.x;
    for (; k + (kUnroll - 1) * stride < n_items; k += kUnroll * stride) {
        typename CT<R>::type v[kUnroll];
#pragma unroll
        for (int u = 0; u < kUnroll; ++u)
            v[u] = s[insert_zeros(k + u * stride, pi.pos, pi.npos) | (idx_t)pi.set_mask];
        R part = 0;
#pragma unroll
        for (int u = 0; u < kUnroll; ++u) part += abs2r(v[u]);
        acc += (double)part;
    }
    for (; k < n_items; k += stride)
        acc += (double)abs2r(s[insert_zeros(k, pi.pos, pi.npos) | (idx_t)pi.set_mask]);
    acc = block_sum(acc);
    if (threadIdx.x == 0) partials[blockIdx.x] = acc;
}

// complex64 with lane 0 outside the pattern: two amplitudes per float4.
__global__ void __launch_bounds__(kRedThreads)
k_prob_vec2_f32(const float4 *__restrict__ s, idx_t n_vec, PairIdx pi, double *partials) {
    double acc = 0.;
    const idx_t stride = (idx_t)gridDim.x * blockDim.x;
    idx_t v = (idx_t)blockIdx.x * blockDim.x + threadIdx.x;
    for (; v + (kUnroll - 1) * stride < n_vec; v += kUnroll * stride) {
        float4 a[kUnroll];
#pragma unroll
        for (int u = 0; u < kUnroll; ++u)
            a[u] = s[(insert_zeros(2 * (v + u * stride), pi.pos, pi.npos) | (idx_t)pi.set_mask) >> 1];
        float part = 0.f;
#pragma unroll
        for (int u = 0; u < kUnroll; ++u)
            part += a[u].x * a[u].x + a[u].y * a[u].y + a[u].z * a[u].z + a[u].w * a[u].w;
        acc += (double)part;
    }
    for (; v < n_vec; v += stride) {
        float4 a = s[(insert_zeros(2 * v, pi.pos, pi.npos) | (idx_t)pi.set_mask) >> 1];
        acc += (double)(a.x * a.x + a.y * a.y + a.z * a.z + a.w * a.w);
    }
    acc = block_sum(acc);
    if (threadIdx.x == 0) partials[blockIdx.x] = acc;
}

// w with its sign flipped when the parity bit par is 1.
__device__ __forceinline__ float sign_flip(float w, unsigned par) {
    return __int_as_float(__float_as_int(w) ^ (int)(par << 31));
}
__device__ __forceinline__ double sign_flip(double w, unsigned par) {
    return __longlong_as_double(__double_as_longlong(w) ^ (long long)((unsigned long long)par << 63));
}
__device__ __forceinline__ unsigned parity64(idx_t b) { return (unsigned)__popcll(b) & 1u; }

// <psi|P|psi>, diagonal Pauli string (x_mask == 0): sum of (-1)^parity(b & z) |psi[b]|^2.
template <class R>
__global__ void __launch_bounds__(kRedThreads)
k_pauli_diag(const typename CT<R>::type *__restrict__ s, idx_t n, unsigned long long z_mask,
             double *partials) {
    double acc = 0.;
    const idx_t stride = (idx_t)gridDim.x * blockDim.x;
    idx_t b = (idx_t)blockIdx.x * blockDim.x + threadIdx.x;
    for (; b + (kUnroll - 1) * stride < n; b += kUnroll * stride) {
        typename CT<R>::type v[kUnroll];
#pragma unroll
        for (int u = 0; u < kUnroll; ++u) v[u] = s[b + u * stride];
        R part = 0;
#pragma unroll
        for (int u = 0; u < kUnroll; ++u)
            part += sign_flip(abs2r(v[u]), parity64((b + u * stride) & (idx_t)z_mask));
        acc += (double)part;
    }
    for (; b < n; b += stride) acc += (double)sign_flip(abs2r(s[b]), parity64(b & (idx_t)z_mask));
    acc = block_sum(acc);
    if (threadIdx.x == 0) partials[blockIdx.x] = acc;
}

// <psi|P|psi> with x_mask != 0: pairs (b, b2 = b ^ x_mask), b with the highest
// x bit clear; ny = number of Y factors (x & z).  With w = conj(psi[b2]) psi[b]
// and s1, s2 the Z-signs of b and b2, the pair contributes
// Re(i^ny (s1 w + s2 conj(w))) (qgate/model/pauli_gates_diagonalizer.py
// gives the same operator as a basis change).  Since s2 = s1 (-1)^ny, that is
// coef * s1 * (Re w for even ny, Im w for odd ny) with coef = 2, -2, -2, 2 for
// ny mod 4 = 0..3: one parity per pair, applied as a sign flip, and coef
// multiplies the block's partial (exactly).
template <class R>
__global__ void __launch_bounds__(kRedThreads)
k_pauli_pair(const typename CT<R>::type *__restrict__ s, idx_t n_items, int hbit,
             unsigned long long x_mask, unsigned long long z_mask, int ny, double *partials) {
    typedef typename CT<R>::type C;
    const bool odd = ny & 1;
    double acc = 0.;
    const idx_t stride = (idx_t)gridDim.x * blockDim.x;
    idx_t k = (idx_t)blockIdx.x * blockDim.x + threadIdx.x;
    auto term = [&](idx_t b, C p, C q) -> R {
        const R w = odd ? q.x * p.y - q.y * p.x : q.x * p.x + q.y * p.y;
        return sign_flip(w, parity64(b & (idx_t)z_mask));
    };
    for (; k + (kUnroll - 1) * stride < n_items; k += kUnroll * stride) {
        // all loads first: 2 x kUnroll amplitudes in flight per thread
        idx_t b[kUnroll];
        C p[kUnroll], q[kUnroll];
#pragma unroll
        for (int u = 0; u < kUnroll; ++u) {
            b[u] = insert_zero(k + u * stride, hbit);
            p[u] = s[b[u]];
            q[u] = s[b[u] ^ (idx_t)x_mask];
        }
        R part = 0;
#pragma unroll
        for (int u = 0; u < kUnroll; ++u) part += term(b[u], p[u], q[u]);
        acc += (double)part;
    }
    for (; k < n_items; k += stride) {
        const idx_t b = insert_zero(k, hbit);
        acc += (double)term(b, s[b], s[b ^ (idx_t)x_mask]);
    }
    acc = block_sum(acc);
    if (threadIdx.x == 0) partials[blockIdx.x] = acc * ((ny + 1) & 2 ? -2. : 2.);
}

// ------------------------------------------------------------ gathers

__device__ __forceinline__ idx_t to_local(const GatherDesc &g, int q, idx_t ext) {
    idx_t local = 0;
    for (int l = g.lane_begin[q]; l < g.lane_begin[q + 1]; ++l)
        local |= ((ext >> g.ext[l]) & 1LL) << (l - g.lane_begin[q]);
    return local;
}

// value[i] = prod_q op(psi_q[local_q(start + step * i)]), 0 on empty lanes
// (qgate/simulator/pyruntime.py:186-214, qgate/simulator/src/DeviceGetStates.cu:185-204).
template <class R, int MATHOP>
__global__ void __launch_bounds__(256)
k_gather(void *__restrict__ out, idx_t count, idx_t start, idx_t step,
         unsigned long long empty_mask, const __grid_constant__ GatherDesc g) {
    typedef typename CT<R>::type C;
    const idx_t stride = (idx_t)gridDim.x * blockDim.x;
    for (idx_t i = (idx_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += stride) {
        idx_t ext = start + step * i;
        if (MATHOP == 0) {
            C v = cmk<C>(0., 0.);
            if ((ext & (idx_t)empty_mask) == 0) {
                v = cmk<C>(1., 0.);
                for (int q = 0; q < g.nqs; ++q)
                    v = cmul(v, ((const C *)g.ptr[q])[to_local(g, q, ext)]);
            }
            ((C *)out)[i] = v;
        } else {
            R v = 0;
            if ((ext & (idx_t)empty_mask) == 0) {
                v = 1;
                for (int q = 0; q < g.nqs; ++q) {
                    C c = ((const C *)g.ptr[q])[to_local(g, q, ext)];
                    v *= c.x * c.x + c.y * c.y;
                }
            }
            ((R *)out)[i] = v;
        }
    }
}

// Gather of one state in its own lane order over a contiguous range (the
// common full probability vector / state dump): out[i] = op(psi[start + i]),
// 4 items per thread with 16-byte loads where aligned.
template <class R, int MATHOP>
__global__ void __launch_bounds__(256)
k_gather_contig(void *__restrict__ out, const typename CT<R>::type *__restrict__ psi,
                idx_t count) {
    typedef typename CT<R>::type C;
    const idx_t stride = (idx_t)gridDim.x * blockDim.x;
    const idx_t quads = count / 4;
    for (idx_t q = (idx_t)blockIdx.x * blockDim.x + threadIdx.x; q < quads; q += stride) {
        const C a0 = psi[4 * q], a1 = psi[4 * q + 1], a2 = psi[4 * q + 2], a3 = psi[4 * q + 3];
        if (MATHOP == 0) {
            C *o = (C *)out + 4 * q;
            o[0] = a0;
            o[1] = a1;
            o[2] = a2;
            o[3] = a3;
        } else if (sizeof(R) == 4) {
            float4 p;
            p.x = a0.x * a0.x + a0.y * a0.y;
            p.y = a1.x * a1.x + a1.y * a1.y;
            p.z = a2.x * a2.x + a2.y * a2.y;
            p.w = a3.x * a3.x + a3.y * a3.y;
            ((float4 *)out)[q] = p;
        } else {
            R *o = (R *)out + 4 * q;
            o[0] = a0.x * a0.x + a0.y * a0.y;
            o[1] = a1.x * a1.x + a1.y * a1.y;
            o[2] = a2.x * a2.x + a2.y * a2.y;
            o[3] = a3.x * a3.x + a3.y * a3.y;
        }
    }
    for (idx_t i = 4 * quads + (idx_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += stride) {
        const C a = psi[i];
        if (MATHOP == 0)
            ((C *)out)[i] = a;
        else
            ((R *)out)[i] = a.x * a.x + a.y * a.y;
    }
}

// Marginal probabilities: out[o] = sum_c prod_q |psi_q[local_q(o | c << n_lanes)]|^2,
// FP64.  blockIdx.y splits the hidden range into groups written to scratch.
template <class R>
__global__ void __launch_bounds__(256)
k_marginal(double *__restrict__ out, int n_lanes, idx_t hidden_per_group,
           const __grid_constant__ GatherDesc g, int identity) {
    typedef typename CT<R>::type C;
    const idx_t n_out = (idx_t)1 << n_lanes;
    const idx_t stride = (idx_t)gridDim.x * blockDim.x;
    const idx_t c0 = (idx_t)blockIdx.y * hidden_per_group;
    for (idx_t o = (idx_t)blockIdx.x * blockDim.x + threadIdx.x; o < n_out; o += stride) {
        double acc = 0.;
        for (idx_t c = c0; c < c0 + hidden_per_group; ++c) {
            idx_t ext = o | (c << n_lanes);
            if (identity) {
                acc += (double)abs2r(((const C *)g.ptr[0])[ext]);
            } else {
                R v = 1;
                for (int q = 0; q < g.nqs; ++q)
                    v *= abs2r(((const C *)g.ptr[q])[to_local(g, q, ext)]);
                acc += (double)v;
            }
        }
        out[(idx_t)blockIdx.y * n_out + o] = acc;
    }
}

__global__ void k_sum_groups(double *__restrict__ out, const double *__restrict__ parts,
                             idx_t n_out, int n_groups) {
    const idx_t stride = (idx_t)gridDim.x * blockDim.x;
    for (idx_t o = (idx_t)blockIdx.x * blockDim.x + threadIdx.x; o < n_out; o += stride) {
        double acc = 0.;
        for (int gi = 0; gi < n_groups; ++gi) acc += parts[(idx_t)gi * n_out + o];
        out[o] = acc;
    }
}

template <class R>
__global__ void k_convert(R *__restrict__ dst, const double *__restrict__ src, idx_t n) {
    const idx_t stride = (idx_t)gridDim.x * blockDim.x;
    for (idx_t i = (idx_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
        dst[i] = (R)src[i];
}

// ------------------------------------------------------------ pool CDF
//
// The sampling pool's cumulative distribution is held as 64-bit fixed-point
// prefix sums.  Each probability p becomes q = round(p * 2^60) (exact for a
// complex64 |a|^2 >= 2^-37 and a complex128 |a|^2 >= 2^-8, else within
// 2^-61), and the prefix sums of q are integers: the scan rounds nowhere and
// every summation order gives the same bits.  A uniform u then selects the
// first i with P[i] > floor(u * T), T the total, which is the reference's
// upper_bound over its normalised FP64 CDF (cumsum / sum,
// qgate/simulator/src/CPUSamplingPool.cpp:16-49, 71-81) evaluated without
// rounding.  Keeping the per-item work in integers keeps it off GB300's FP64
// pipe (about 2 operations per clock per SM), which bounds an FP64 scan of
// 2^30 items at several milliseconds.  Sums saturate at 2^64 - 1 instead of
// wrapping, so a state far from unit norm still fails the norm check.

constexpr int kScanThreads = 256;
constexpr int kScanItems = 16;
constexpr idx_t kScanTile = kScanThreads * kScanItems;
constexpr int kFixBits = 60;                          // q = p * 2^60
constexpr unsigned long long kFixCap = 1ull << 62;    // FP64 p >= 4 (and NaN) reads as this

typedef unsigned long long u64;

__device__ __forceinline__ u64 sat_add(u64 a, u64 b) {
    const u64 s = a + b;
    return s < a ? ~0ull : s;
}

// round(p * 2^60) to nearest, ties to even, for 0 <= p < 4: with
// x = p * 2^28 (exact), q = floor(x) * 2^32 + rint((x - floor(x)) * 2^32),
// every step exact but the last rounding.  Both halves are single
// conversions, so the per-item cost is a few FP32-pipe instructions.
// p >= 16 saturates the high word; NaN reads as 0.
__device__ __forceinline__ u64 fix_from_f32(float p) {
    const float x = p * 268435456.f;  // 2^28
    const float f = floorf(x);
    const unsigned hi = __float2uint_rz(f);
    const unsigned lo = __float2uint_rn((x - f) * 4294967296.f);  // < 2^32
    return ((u64)hi << 32) | lo;
}

// round(p * 2^60) to nearest, ties to even; p = m * 2^(e - 1075).  Integer
// work only: FP64 operations are scarce on GB300.  p >= 4 saturates at 2^62.
__device__ __forceinline__ u64 fix_from_f64(double p) {
    const u64 b = (u64)__double_as_longlong(p);
    if ((b << 1) < (1ull << 53)) return 0;  // +-0 and subnormals
    const int e = (int)(b >> 52);           // the sign bit lifts negative p into saturation
    const u64 m = (b & ((1ull << 52) - 1)) | (1ull << 52);
    const int sh = e - (1075 - kFixBits);
    if (sh >= 0) return sh <= 9 ? m << sh : kFixCap;  // m << 9 < 2^62: p < 4
    const int r = -sh;
    if (r > 53) return 0;  // p * 2^60 < 1/2
    const u64 q = m >> r, rem = m & ((1ull << r) - 1), half = 1ull << (r - 1);
    return q + ((rem > half || (rem == half && (q & 1))) ? 1 : 0);
}

// floor(u * T) for 0 <= u (sign ignored: -0 reads as 0); u >= 1 gives 2^64 - 1.
__device__ __forceinline__ u64 fix_target(double u, u64 total) {
    const u64 b = (u64)__double_as_longlong(u) & ~(1ull << 63);
    const int e = (int)(b >> 52);
    if (e >= 1023) return ~0ull;
    if (e == 0) return 0;  // u < 2^-1022: u * T < 1
    const u64 m = (b & ((1ull << 52) - 1)) | (1ull << 52);
    const u64 lo = m * total, hi = __umul64hi(m, total);
    const int sh = 1075 - e;  // u * T = (m * T) >> sh, sh >= 53
    if (sh >= 128) return 0;
    if (sh >= 64) return hi >> (sh - 64);
    return (hi << (64 - sh)) | (lo >> sh);
}

// Item sources: the probability of item i as a fixed-point integer.
struct SrcStateF32 {
    const float2 *p;
    __device__ __forceinline__ u64 operator()(idx_t i) const {
        const float2 a = p[i];
        return fix_from_f32(a.x * a.x + a.y * a.y);
    }
};
struct SrcStateF64 {
    const double2 *p;
    __device__ __forceinline__ u64 operator()(idx_t i) const {
        const double2 a = p[i];
        return fix_from_f64(a.x * a.x + a.y * a.y);
    }
};
struct SrcProbF64 {
    const double *p;
    __device__ __forceinline__ u64 operator()(idx_t i) const { return fix_from_f64(p[i]); }
};
struct SrcFix {
    const u64 *p;
    __device__ __forceinline__ u64 operator()(idx_t i) const { return p[i]; }
};

// Guide table of a pool (Chen and Asau's guide-table method for inverse
// transform sampling): g[b] = the first i with P[i] > b * 2^shift, for the
// nb buckets with b * 2^shift below the total.  Buckets hold about 16 items
// on average, so a sample reads g[b], g[b + 1] and searches the few items
// between them instead of the whole CDF.  Item i with inclusive prefix P[i]
// and probability q starts the buckets ceil((P[i] - q) / 2^shift) ..
// (P[i] - 1) >> shift; the scan writes up to 8 of them inline and appends
// longer runs to a bounded list that k_guide_long fills (count > cap: the
// pool searches without the table).
typedef PoolGuide Guide;

// floor((incl - 1) / 2^shift) for shift >= 32, -1 for incl == 0: the bucket
// of the last CDF unit an item with inclusive prefix incl reaches.  Item i
// starts the buckets (bucket(P[i-1]), bucket(P[i])].
__device__ __forceinline__ int guide_bucket(u64 incl, int shift) {
    return (int)((incl - 1) >> 32) >> (shift - 32);
}

// Buckets b0..b1 of item i, when there is more than one (or bad bounds).
__device__ __noinline__ void guide_mark_slow(const Guide gd, unsigned i, long long b0,
                                             long long b1) {
    if (b0 < 0) b0 = 0;
    if (b1 >= (long long)gd.nb) b1 = (long long)gd.nb - 1;
    if (b0 > b1) return;
    const long long inl = b1 - b0 < 8 ? b1 : b0 + 7;
    for (long long b = b0; b <= inl; ++b) gd.g[b] = i;
    if (inl < b1) {
        const unsigned slot = atomicAdd(gd.long_count, 1u);
        if (slot < gd.long_cap)
            gd.long_list[slot] = make_uint4((unsigned)(inl + 1), (unsigned)((inl + 1) >> 32),
                                            (unsigned)b1, i);
    }
}

// Item i's bucket b after the previous item's bucket bp: usually equal (no
// bucket starts here) or one more (one store).  Entries hold i >> index_shift
// (0 up to 2^32 items), a lower bound of the item.
__device__ __forceinline__ void guide_mark(const Guide &gd, idx_t i, int bp, int b) {
    if (b == bp) return;
    if (b == bp + 1 && (unsigned)b < gd.nb)
        gd.g[b] = (unsigned)(i >> gd.index_shift);
    else
        guide_mark_slow(gd, (unsigned)(i >> gd.index_shift), (long long)bp + 1, b);
}

// Fills the long runs: every thread of the grid walks the list.
__global__ void __launch_bounds__(256)
k_guide_long(Guide gd) {
    const unsigned count = min(*gd.long_count, gd.long_cap);
    const u64 stride = (u64)gridDim.x * blockDim.x;
    for (unsigned j = 0; j < count; ++j) {
        const uint4 e = gd.long_list[j];
        const u64 b0 = (u64)e.x | ((u64)e.y << 32), b1 = e.z;
        for (u64 b = b0 + (u64)blockIdx.x * blockDim.x + threadIdx.x; b <= b1; b += stride)
            gd.g[b] = e.w;
    }
}

// Two 8-byte items from one 16-byte chunk of shared memory.
struct PairStateF32 {  // two complex64 amplitudes
    static __device__ __forceinline__ void get(uint4 c, u64 &q0, u64 &q1) {
        const float x0 = __uint_as_float(c.x), y0 = __uint_as_float(c.y);
        const float x1 = __uint_as_float(c.z), y1 = __uint_as_float(c.w);
        q0 = fix_from_f32(x0 * x0 + y0 * y0);
        q1 = fix_from_f32(x1 * x1 + y1 * y1);
    }
};
struct PairProbF64 {  // two FP64 probabilities
    static __device__ __forceinline__ void get(uint4 c, u64 &q0, u64 &q1) {
        q0 = fix_from_f64(__hiloint2double((int)c.y, (int)c.x));
        q1 = fix_from_f64(__hiloint2double((int)c.w, (int)c.z));
    }
};

__device__ __forceinline__ u64 warp_incl_scan(u64 v, int lane) {
    for (int o = 1; o < 32; o <<= 1) {
        const u64 t = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v = sat_add(v, t);
    }
    return v;
}

template <class Src>
__global__ void __launch_bounds__(kScanThreads)
k_fix_tile_sums(Src src, idx_t n, u64 *__restrict__ sums) {
    __shared__ u64 warp_sums[kScanThreads / 32];
    const idx_t base = (idx_t)blockIdx.x * kScanTile;
    u64 q[kScanItems];
#pragma unroll
    for (int j = 0; j < kScanItems; ++j) {
        const idx_t i = base + (idx_t)j * kScanThreads + threadIdx.x;
        q[j] = i < n ? src(i) : 0;
    }
    u64 v = 0;
#pragma unroll
    for (int j = 0; j < kScanItems; ++j) v = sat_add(v, q[j]);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int o = 16; o > 0; o >>= 1) v = sat_add(v, __shfl_xor_sync(0xffffffffu, v, o));
    if (lane == 0) warp_sums[warp] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        u64 t = 0;
        for (int w = 0; w < kScanThreads / 32; ++w) t = sat_add(t, warp_sums[w]);
        sums[blockIdx.x] = t;
    }
}

// Inclusive scan of one tile plus the inclusive prefix of the preceding
// tiles (incl_sums[tile - 1]).  Items pass through shared memory so that each
// thread scans a run of 16 consecutive ones; the padding of one word per 16
// puts a half-warp's runs in distinct banks.  out may alias the source.
__device__ __forceinline__ int pad16(int i) { return i + (i >> 4); }

template <class Src>
__global__ void __launch_bounds__(kScanThreads)
k_fix_tile_apply(Src src, u64 *out, idx_t n, const u64 *__restrict__ incl_sums, Guide gd) {
    __shared__ u64 tile[kScanTile + kScanTile / 16];
    __shared__ u64 warp_tot[kScanThreads / 32];
    const idx_t base = (idx_t)blockIdx.x * kScanTile;
    {
        u64 q[kScanItems];
#pragma unroll
        for (int j = 0; j < kScanItems; ++j) {
            const idx_t i = base + (idx_t)j * kScanThreads + threadIdx.x;
            q[j] = i < n ? src(i) : 0;
        }
#pragma unroll
        for (int j = 0; j < kScanItems; ++j) tile[pad16(j * kScanThreads + threadIdx.x)] = q[j];
    }
    __syncthreads();
    u64 loc[kScanItems];
    u64 run = 0;
#pragma unroll
    for (int j = 0; j < kScanItems; ++j) {
        run = sat_add(run, tile[pad16(threadIdx.x * kScanItems + j)]);
        loc[j] = run;
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const u64 inc = warp_incl_scan(run, lane);
    u64 excl = __shfl_up_sync(0xffffffffu, inc, 1);
    if (lane == 0) excl = 0;
    if (lane == 31) warp_tot[warp] = inc;
    __syncthreads();
    u64 off = blockIdx.x > 0 ? incl_sums[blockIdx.x - 1] : 0;
    for (int w = 0; w < warp; ++w) off = sat_add(off, warp_tot[w]);
    off = sat_add(off, excl);
    int bp = gd.g ? guide_bucket(off, gd.shift) : 0;
#pragma unroll
    for (int j = 0; j < kScanItems; ++j) {
        const int li = threadIdx.x * kScanItems + j;
        const u64 incl = sat_add(loc[j], off);
        if (gd.g && base + li < n) {
            const int b = guide_bucket(incl, gd.shift);
            guide_mark(gd, base + li, bp, b);
            bp = b;
        }
        tile[pad16(li)] = incl;
    }
    __syncthreads();
#pragma unroll
    for (int j = 0; j < kScanItems; ++j) {
        const idx_t i = base + (idx_t)j * kScanThreads + threadIdx.x;
        if (i < n) out[i] = tile[pad16(j * kScanThreads + threadIdx.x)];
    }
}

// Level 0 of the scan for 8-byte items, as persistent CTAs (two per SM)
// that stream 32 KB tiles (4096 items) through a 3-stage ring of shared
// memory with bulk async copies.  Thread t owns the run of items
// [16t, 16t + 16) of a tile: 8 chunks of 16 bytes, read in the rotated
// order c = (k + t) mod 8 so that the 8 lanes of each shared-memory phase
// hit distinct banks.  Waits are bounded; on a timeout the CTA records
// g_pool_status, drains its outstanding copies and stops.
constexpr int kBulkStages = 3;
constexpr unsigned kTileBytes = (unsigned)kScanTile * 8u;
constexpr size_t kBulkSmem = (size_t)kBulkStages * kTileBytes;

__device__ unsigned g_pool_status;

// Pass 1: tile sums (saturating).
template <class Pair>
__global__ void __launch_bounds__(kScanThreads, 2)
k_pool_sums_bulk(const unsigned char *__restrict__ src, idx_t tiles, u64 *__restrict__ sums) {
    extern __shared__ __align__(128) unsigned char ring[];
    __shared__ __align__(8) u64 bar[kBulkStages];
    __shared__ u64 red[2][kScanThreads / 32];
    __shared__ int abort_sh;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const idx_t my = tiles > (idx_t)blockIdx.x ? (tiles - 1 - blockIdx.x) / gridDim.x + 1 : 0;
    if (tid == 0) {
        for (int st = 0; st < kBulkStages; ++st) mbar_init(smem_u32(&bar[st]), 1);
        mbar_fence_init();
        abort_sh = 0;
    }
    __syncthreads();
    idx_t issued = 0;
    if (tid == 0)
        for (; issued < my && issued < kBulkStages; ++issued)
            bulk_load(smem_u32(ring + issued * kTileBytes),
                      src + (size_t)(blockIdx.x + issued * gridDim.x) * kTileBytes, kTileBytes,
                      smem_u32(&bar[issued]));
    idx_t i = 0;
    for (; i < my; ++i) {
        const int st = (int)(i % kBulkStages);
        if (!mbar_wait(smem_u32(&bar[st]), (unsigned)(i / kBulkStages) & 1u)) {
            atomicOr(&g_pool_status, 1u);
            abort_sh = 1;
        }
        const uint4 *row = (const uint4 *)(ring + st * kTileBytes) + 8 * tid;
        u64 v = 0;
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            u64 q0, q1;
            Pair::get(row[(k + tid) & 7], q0, q1);
            v = sat_add(v, sat_add(q0, q1));
        }
        for (int o = 16; o > 0; o >>= 1) v = sat_add(v, __shfl_xor_sync(0xffffffffu, v, o));
        if (lane == 0) red[i & 1][warp] = v;
        __syncthreads();
        if (abort_sh) break;
        if (tid == 0) {
            u64 t = 0;
            for (int w = 0; w < kScanThreads / 32; ++w) t = sat_add(t, red[i & 1][w]);
            sums[blockIdx.x + i * gridDim.x] = t;
            if (issued < my) {  // the stage just read is free again
                bulk_load(smem_u32(ring + st * kTileBytes),
                          src + (size_t)(blockIdx.x + issued * gridDim.x) * kTileBytes,
                          kTileBytes, smem_u32(&bar[st]));
                ++issued;
            }
        }
    }
    if (tid == 0)
        for (idx_t j = i; j < issued; ++j)  // copies still in flight after an abort
            mbar_wait(smem_u32(&bar[j % kBulkStages]), (unsigned)(j / kBulkStages) & 1u);
}

// Pass 2: the inclusive scan of each tile plus incl_sums[tile - 1], written
// back through shared memory and out with bulk stores.  The arithmetic wraps
// modulo 2^64, which is exact whenever the saturating total of pass 1 passes
// the norm check (all partial sums are then below 2^61).  In rotated order,
// with R_k the running sum of the chunks visited before k and W the sum of
// the chunks c0..7 (c0 = t mod 8, visited first), the exclusive prefix of
// chunk c_k within the run is R_k + (total - W) before the wrap to chunk 0
// and R_k - W after it.
template <class Pair>
__global__ void __launch_bounds__(kScanThreads, 2)
k_pool_scan_bulk(const unsigned char *src, idx_t tiles, u64 *cdf, const u64 *__restrict__ incl_sums,
                 Guide gd) {
    extern __shared__ __align__(128) unsigned char ring[];
    __shared__ __align__(8) u64 bar[kBulkStages];
    __shared__ u64 red[2][kScanThreads / 32];
    __shared__ int abort_sh;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, c0 = tid & 7;
    const idx_t my = tiles > (idx_t)blockIdx.x ? (tiles - 1 - blockIdx.x) / gridDim.x + 1 : 0;
    if (tid == 0) {
        for (int st = 0; st < kBulkStages; ++st) mbar_init(smem_u32(&bar[st]), 1);
        mbar_fence_init();
        abort_sh = 0;
    }
    __syncthreads();
    // Two tiles ahead; the third stage is refilled once its store has read it.
    idx_t issued = 0;
    if (tid == 0)
        for (; issued < my && issued < kBulkStages - 1; ++issued)
            bulk_load(smem_u32(ring + issued * kTileBytes),
                      src + (size_t)(blockIdx.x + issued * gridDim.x) * kTileBytes, kTileBytes,
                      smem_u32(&bar[issued]));
    idx_t i = 0;
    for (; i < my; ++i) {
        const idx_t tile = blockIdx.x + i * gridDim.x;
        const u64 base = tile > 0 ? incl_sums[tile - 1] : 0;
        const int st = (int)(i % kBulkStages);
        if (!mbar_wait(smem_u32(&bar[st]), (unsigned)(i / kBulkStages) & 1u)) {
            atomicOr(&g_pool_status, 1u);
            abort_sh = 1;
        }
        uint4 *row = (uint4 *)(ring + st * kTileBytes) + 8 * tid;
        u64 q[16], R[8];
        u64 tot = 0, W = 0;
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            Pair::get(row[(k + tid) & 7], q[2 * k], q[2 * k + 1]);
            R[k] = tot;
            const u64 sk = q[2 * k] + q[2 * k + 1];
            tot += sk;
            if (k < 8 - c0) W += sk;
        }
        u64 inc = tot;
        for (int o = 1; o < 32; o <<= 1) {
            const u64 t = __shfl_up_sync(0xffffffffu, inc, o);
            if (lane >= o) inc += t;
        }
        if (lane == 31) red[i & 1][warp] = inc;
        __syncthreads();
        if (abort_sh) break;
        u64 off = base + inc - tot;
        for (int w = 0; w < warp; ++w) off += red[i & 1][w];
        const u64 before = off + tot - W, after = off - W;
        int bq[16];
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            const u64 o0 = R[k] + (k < 8 - c0 ? before : after) + q[2 * k];
            const u64 o1 = o0 + q[2 * k + 1];
            bq[2 * k] = guide_bucket(o0, gd.shift);
            bq[2 * k + 1] = guide_bucket(o1, gd.shift);
            row[(k + tid) & 7] = make_uint4((unsigned)o0, (unsigned)(o0 >> 32), (unsigned)o1,
                                            (unsigned)(o1 >> 32));
        }
        if (gd.g) {
            // the item before chunk c's first is chunk c - 1's second (rotated
            // position k - 1), or the run's start for chunk 0
            const int brun = guide_bucket(off, gd.shift);
            const idx_t first = tile * kScanTile + 16 * tid;
#pragma unroll
            for (int k = 0; k < 8; ++k) {
                const int c = (k + tid) & 7;
                const int bp = c == 0 ? brun : bq[2 * ((k + 7) & 7) + 1];
                guide_mark(gd, first + 2 * c, bp, bq[2 * k]);
                guide_mark(gd, first + 2 * c + 1, bq[2 * k], bq[2 * k + 1]);
            }
        }
        fence_async_smem();
        __syncthreads();
        if (tid == 0) {
            bulk_store(cdf + (size_t)tile * kScanTile, smem_u32(ring + st * kTileBytes),
                       kTileBytes);
            bulk_commit();
            if (issued < my) {
                // stage issued % 3 last held tile i - 1: its store must have read it
                if (issued >= kBulkStages) bulk_wait_read<1>();
                const int sn = (int)(issued % kBulkStages);
                bulk_load(smem_u32(ring + sn * kTileBytes),
                          src + (size_t)(blockIdx.x + issued * gridDim.x) * kTileBytes,
                          kTileBytes, smem_u32(&bar[sn]));
                ++issued;
            }
        }
    }
    if (tid == 0) {
        for (idx_t j = i; j < issued; ++j)  // copies still in flight after an abort
            mbar_wait(smem_u32(&bar[j % kBulkStages]), (unsigned)(j / kBulkStages) & 1u);
        bulk_wait<0>();
    }
}

// upper_bound over the fixed-point CDF (first i with cdf[i] > floor(u * T)),
// clamped to n-1, then zero bits inserted at the empty lanes
// (qgate/simulator/src/CPUSamplingPool.cpp:71-81; spec:
// qgate/simulator/pyruntime.py:303-321).  A negative or NaN u selects 0, as
// the FP64 upper_bound does.
struct EmptyPos {
    int n;
    int pos[kMaxLanes];
};

// With a guide table, t = floor(u * T) < T lies in bucket b = t >> shift <=
// bmax = (T - 1) >> shift; the answer is in [g[b], g[b + 1]] (g[b + 1] read
// as n - 1 past bmax; entries widened by the index shift), where cdf[hi] > t
// holds, so a lower-bound search over that range finds it.
__global__ void __launch_bounds__(256)
k_search(const u64 *__restrict__ cdf, idx_t n, u64 total, const unsigned *__restrict__ guide,
         int shift, int index_shift, const double *__restrict__ u, long long *__restrict__ obs,
         idx_t m, EmptyPos ep) {
    const idx_t stride = (idx_t)gridDim.x * blockDim.x;
    const u64 bmax = (total - 1) >> shift;
    for (idx_t i = (idx_t)blockIdx.x * blockDim.x + threadIdx.x; i < m; i += stride) {
        const double x = u[i];
        idx_t lo = 0;
        if (x >= 1.) {
            lo = n - 1;
        } else if (guide && x >= 0.) {
            const u64 t = fix_target(x, total);
            const u64 b = t >> shift;
            lo = (idx_t)guide[b] << index_shift;
            idx_t hi = b + 1 <= bmax
                           ? ((idx_t)guide[b + 1] << index_shift) + ((1LL << index_shift) - 1)
                           : n - 1;
            if (hi > n - 1) hi = n - 1;
            while (lo < hi) {
                const idx_t mid = (lo + hi) >> 1;
                if (cdf[mid] <= t)
                    lo = mid + 1;
                else
                    hi = mid;
            }
        } else if (x >= 0.) {
            const u64 t = fix_target(x, total);
            idx_t hi = n;
            while (lo < hi) {
                const idx_t mid = (lo + hi) >> 1;
                if (cdf[mid] <= t)
                    lo = mid + 1;
                else
                    hi = mid;
            }
            if (lo > n - 1) lo = n - 1;
        }
        obs[i] = insert_zeros(lo, ep.pos, ep.n);
    }
}

inline unsigned sm_grid(idx_t items, int threads, int max_blocks) {
    idx_t g = (items + threads - 1) / threads;
    if (g > max_blocks) g = max_blocks;
    if (g < 1) g = 1;
    return (unsigned)g;
}

}  // namespace

int reduce_partials() { return kRedBlocks; }

void launch_prob(int prec, const void *state, idx_t n_items, const PairIdx &pi,
                 double *d_partials, double *d_out, cudaStream_t stream) {
    unsigned nb;
    bool vec = prec == kFP32 && (pi.set_mask & 1ULL) == 0 && pi.npos > 0 && pi.pos[0] >= 1 &&
               n_items % 2 == 0;
    if (vec) {
        nb = sm_grid(n_items / 2, kRedThreads, kRedBlocks);
        k_prob_vec2_f32<<<nb, kRedThreads, 0, stream>>>((const float4 *)state, n_items / 2, pi,
                                                        d_partials);
    } else if (prec == kFP32) {
        nb = sm_grid(n_items, kRedThreads, kRedBlocks);
        k_prob_scalar<float><<<nb, kRedThreads, 0, stream>>>((const float2 *)state, n_items, pi,
                                                             d_partials);
    } else {
        nb = sm_grid(n_items, kRedThreads, kRedBlocks);
        k_prob_scalar<double><<<nb, kRedThreads, 0, stream>>>((const double2 *)state, n_items, pi,
                                                              d_partials);
    }
    k_final_sum<<<1, 256, 0, stream>>>(d_partials, (int)nb, d_out);
    QG_CUDA(cudaGetLastError());
}

void launch_pauli(int prec, const void *state, int n_lanes, unsigned long long x_mask,
                  unsigned long long z_mask, double *d_partials, double *d_out,
                  cudaStream_t stream) {
    idx_t n = (idx_t)1 << n_lanes;
    unsigned nb;
    if (x_mask == 0) {
        nb = sm_grid(n, kRedThreads, kRedBlocks);
        if (prec == kFP32)
            k_pauli_diag<float><<<nb, kRedThreads, 0, stream>>>((const float2 *)state, n, z_mask,
                                                                d_partials);
        else
            k_pauli_diag<double><<<nb, kRedThreads, 0, stream>>>((const double2 *)state, n,
                                                                 z_mask, d_partials);
    } else {
        int hbit = 63 - __builtin_clzll(x_mask);
        int ny = __builtin_popcountll(x_mask & z_mask);
        idx_t items = n / 2;
        nb = sm_grid(items, kRedThreads, kRedBlocks);
        if (prec == kFP32)
            k_pauli_pair<float><<<nb, kRedThreads, 0, stream>>>(
                (const float2 *)state, items, hbit, x_mask, z_mask, ny, d_partials);
        else
            k_pauli_pair<double><<<nb, kRedThreads, 0, stream>>>(
                (const double2 *)state, items, hbit, x_mask, z_mask, ny, d_partials);
    }
    k_final_sum<<<1, 256, 0, stream>>>(d_partials, (int)nb, d_out);
    QG_CUDA(cudaGetLastError());
}

void launch_gather(int prec, int mathop, void *out, idx_t count, idx_t start, idx_t step,
                   unsigned long long empty_mask, const GatherDesc &g, cudaStream_t stream) {
    if (count <= 0) return;
    bool contig = g.nqs == 1 && step == 1 && empty_mask == 0 && start >= 0 &&
                  ((uintptr_t)out & 15u) == 0;
    for (int l = g.lane_begin[0]; contig && l < g.lane_begin[1]; ++l)
        contig = g.ext[l] == l - g.lane_begin[0];
    // the range must stay inside the state: bits above its lanes are not read
    contig = contig && start + count <= ((idx_t)1 << (g.lane_begin[1] - g.lane_begin[0]));
    if (contig) {
        const unsigned nq = sm_grid(count / 4 + 1, 256, 152 * 16);
        if (prec == kFP32) {
            const float2 *p = (const float2 *)g.ptr[0] + start;
            if (mathop == 0)
                k_gather_contig<float, 0><<<nq, 256, 0, stream>>>(out, p, count);
            else
                k_gather_contig<float, 1><<<nq, 256, 0, stream>>>(out, p, count);
        } else {
            const double2 *p = (const double2 *)g.ptr[0] + start;
            if (mathop == 0)
                k_gather_contig<double, 0><<<nq, 256, 0, stream>>>(out, p, count);
            else
                k_gather_contig<double, 1><<<nq, 256, 0, stream>>>(out, p, count);
        }
        QG_CUDA(cudaGetLastError());
        return;
    }
    unsigned nb = sm_grid(count, 256, 152 * 16);
    if (prec == kFP32) {
        if (mathop == 0)
            k_gather<float, 0><<<nb, 256, 0, stream>>>(out, count, start, step, empty_mask, g);
        else
            k_gather<float, 1><<<nb, 256, 0, stream>>>(out, count, start, step, empty_mask, g);
    } else {
        if (mathop == 0)
            k_gather<double, 0><<<nb, 256, 0, stream>>>(out, count, start, step, empty_mask, g);
        else
            k_gather<double, 1><<<nb, 256, 0, stream>>>(out, count, start, step, empty_mask, g);
    }
    QG_CUDA(cudaGetLastError());
}

static int marginal_groups(int n_lanes, int n_hidden) {
    // Enough threads to fill the GPU: split the hidden range when the output
    // alone is small.
    int groups_log2 = 0;
    while (n_lanes + groups_log2 < 20 && groups_log2 < n_hidden && groups_log2 < 15)
        ++groups_log2;
    return groups_log2;
}

size_t marginal_scratch_doubles(int n_lanes, int n_hidden) {
    int gl = marginal_groups(n_lanes, n_hidden);
    if (gl == 0) return 0;
    return ((size_t)1 << gl) << n_lanes;
}

void launch_marginal(int prec, double *out, int n_lanes, int n_hidden, const GatherDesc &g,
                     double *d_scratch, size_t scratch_doubles, cudaStream_t stream) {
    int gl = marginal_groups(n_lanes, n_hidden);
    idx_t n_out = (idx_t)1 << n_lanes;
    int identity = 0;
    if (g.nqs == 1) {
        identity = 1;
        for (int l = g.lane_begin[0]; l < g.lane_begin[1]; ++l)
            if (g.ext[l] != l - g.lane_begin[0]) identity = 0;
    }
    idx_t groups = (idx_t)1 << gl;
    idx_t per_group = ((idx_t)1 << n_hidden) / groups;
    double *dst = gl == 0 ? out : d_scratch;
    if (gl != 0 && scratch_doubles < (size_t)(groups * n_out)) fail(2, "marginal scratch too small");
    dim3 grid(sm_grid(n_out, 256, 152 * 16), (unsigned)groups);
    if (prec == kFP32)
        k_marginal<float><<<grid, 256, 0, stream>>>(dst, n_lanes, per_group, g, identity);
    else
        k_marginal<double><<<grid, 256, 0, stream>>>(dst, n_lanes, per_group, g, identity);
    if (gl != 0)
        k_sum_groups<<<sm_grid(n_out, 256, 152 * 16), 256, 0, stream>>>(out, d_scratch, n_out,
                                                                       (int)groups);
    QG_CUDA(cudaGetLastError());
}

void launch_convert_f64(int prec, void *dst, const double *src, idx_t n, cudaStream_t stream) {
    unsigned nb = sm_grid(n, 256, 152 * 16);
    if (prec == kFP32)
        k_convert<float><<<nb, 256, 0, stream>>>((float *)dst, src, n);
    else
        k_convert<double><<<nb, 256, 0, stream>>>((double *)dst, src, n);
    QG_CUDA(cudaGetLastError());
}

size_t pool_scratch_words(idx_t n) {
    size_t total = 0;
    idx_t len = n;
    while (len > 1) {
        idx_t tiles = (len + kScanTile - 1) / kScanTile;
        total += (size_t)tiles + 1;
        len = tiles;
    }
    return total + 2;
}

// Inclusive fixed-point scan of src into out (out may alias src's storage);
// the tile sums of each level are scanned in place one level up.
template <class Src>
static void fix_scan(Src src, idx_t n, u64 *out, u64 *scratch, const Guide &gd,
                     cudaStream_t stream) {
    const idx_t tiles = (n + kScanTile - 1) / kScanTile;
    u64 *sums = scratch;
    if (tiles > 1) {
        k_fix_tile_sums<Src><<<(unsigned)tiles, kScanThreads, 0, stream>>>(src, n, sums);
        fix_scan(SrcFix{sums}, tiles, sums, scratch + tiles + 1, Guide{}, stream);
    }
    k_fix_tile_apply<Src><<<(unsigned)tiles, kScanThreads, 0, stream>>>(src, out, n, sums, gd);
    QG_CUDA(cudaGetLastError());
}

static void guide_long(const Guide &gd, cudaStream_t stream) {
    if (gd.g) k_guide_long<<<152 * 4, 256, 0, stream>>>(gd);
    QG_CUDA(cudaGetLastError());
}

static int sm_count() {
    static int count = 0;
    if (!count) {
        int dev = 0;
        QG_CUDA(cudaGetDevice(&dev));
        QG_CUDA(cudaDeviceGetAttribute(&count, cudaDevAttrMultiProcessorCount, dev));
    }
    return count;
}

// Level 0 by the bulk-copy kernels (8-byte items, whole tiles, 16-byte
// aligned), upper levels by fix_scan.  Returns where the saturating total
// ends up.
template <class Pair>
static const u64 *bulk_scan(const void *src, idx_t n, u64 *cdf, u64 *scratch, const Guide &gd,
                            cudaStream_t stream) {
    static bool configured = false;
    if (!configured) {
        QG_CUDA(cudaFuncSetAttribute(k_pool_sums_bulk<Pair>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kBulkSmem));
        QG_CUDA(cudaFuncSetAttribute(k_pool_scan_bulk<Pair>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kBulkSmem));
        configured = true;
    }
    const idx_t tiles = n / kScanTile;
    const unsigned grid = (unsigned)std::min<idx_t>(tiles, 2 * (idx_t)sm_count());
    u64 *sums = scratch;
    k_pool_sums_bulk<Pair><<<grid, kScanThreads, kBulkSmem, stream>>>(
        (const unsigned char *)src, tiles, sums);
    if (tiles > 1) fix_scan(SrcFix{sums}, tiles, sums, scratch + tiles + 1, Guide{}, stream);
    k_pool_scan_bulk<Pair><<<grid, kScanThreads, kBulkSmem, stream>>>(
        (const unsigned char *)src, tiles, cdf, sums, gd);
    QG_CUDA(cudaGetLastError());
    guide_long(gd, stream);
    return sums + tiles - 1;
}

static bool bulk_ok(const void *p, idx_t n) {
    return n >= kScanTile && n % kScanTile == 0 && ((uintptr_t)p & 15u) == 0;
}

const unsigned long long *launch_pool_cdf_state(int prec, const void *state, idx_t n,
                                                unsigned long long *cdf,
                                                unsigned long long *scratch,
                                                const PoolGuide &gd, cudaStream_t stream) {
    if (prec == kFP32 && bulk_ok(state, n) && bulk_ok(cdf, n))
        return bulk_scan<PairStateF32>(state, n, cdf, scratch, gd, stream);
    if (prec == kFP32)
        fix_scan(SrcStateF32{(const float2 *)state}, n, cdf, scratch, gd, stream);
    else
        fix_scan(SrcStateF64{(const double2 *)state}, n, cdf, scratch, gd, stream);
    guide_long(gd, stream);
    return cdf + n - 1;
}

const unsigned long long *launch_pool_cdf_prob(const double *prob, idx_t n,
                                               unsigned long long *cdf,
                                               unsigned long long *scratch,
                                               const PoolGuide &gd, cudaStream_t stream) {
    if (bulk_ok(prob, n) && bulk_ok(cdf, n))
        return bulk_scan<PairProbF64>(prob, n, cdf, scratch, gd, stream);
    fix_scan(SrcProbF64{prob}, n, cdf, scratch, gd, stream);
    guide_long(gd, stream);
    return cdf + n - 1;
}

int pool_status(bool reset) {
    unsigned v = 0;
    QG_CUDA(cudaMemcpyFromSymbol(&v, g_pool_status, sizeof(v)));
    if (reset && v) {
        unsigned z = 0;
        QG_CUDA(cudaMemcpyToSymbol(g_pool_status, &z, sizeof(z)));
    }
    return (int)v;
}

void launch_search(const unsigned long long *cdf, idx_t n, unsigned long long total,
                   const unsigned *guide, int shift, int index_shift, const double *u,
                   long long *obs, idx_t n_samples, const int *empty_pos, int n_empty,
                   cudaStream_t stream) {
    if (n_samples <= 0) return;
    EmptyPos ep;
    ep.n = n_empty;
    for (int i = 0; i < n_empty; ++i) ep.pos[i] = empty_pos[i];
    k_search<<<sm_grid(n_samples, 256, 152 * 16), 256, 0, stream>>>(cdf, n, total, guide, shift, index_shift, u, obs,
                                                                   n_samples, ep);
    QG_CUDA(cudaGetLastError());
}

}  // namespace qg
