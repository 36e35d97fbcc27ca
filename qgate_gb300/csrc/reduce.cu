// Reductions, gathers and the sampling-pool kernels (sm_103a).
//
// All accumulations are FP64 regardless of the state's precision (the
// reference accumulates in the state's own precision:
// qgate/simulator/src/DeviceProcPrimitives.cu:36-54,
// qgate/simulator/src/CPUSamplingPool.cpp:16-49).  Reductions write one
// partial per block and a single-block pass sums the partials in a fixed
// order, so results are bit-reproducible run to run.
#include "qg_device.cuh"

namespace qg {

namespace {

constexpr int kRedThreads = 256;
constexpr int kRedBlocks = 152 * 4;  // 4 resident CTAs on each of 152 SMs
constexpr int kUnroll = 4;

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

template <class R> __device__ __forceinline__ R parity_sign_r(idx_t b) {
    return (__popcll((unsigned long long)b) & 1) ? R(-1) : R(1);
}

// <psi|P|psi>, diagonal Pauli string (x_mask == 0).
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
            part += parity_sign_r<R>((b + u * stride) & (idx_t)z_mask) * abs2r(v[u]);
        acc += (double)part;
    }
    for (; b < n; b += stride)
        acc += (double)(parity_sign_r<R>(b & (idx_t)z_mask) * abs2r(s[b]));
    acc = block_sum(acc);
    if (threadIdx.x == 0) partials[blockIdx.x] = acc;
}

// <psi|P|psi> with x_mask != 0: pairs (b, b ^ x_mask), b with the highest
// x bit clear; ny = number of Y factors (x & z).  With w = conj(psi[b^x]) psi[b]
// and s1, s2 the Z-signs of b and b^x, the pair contributes
// Re(i^ny (s1 w + s2 conj(w))).
template <class R>
__global__ void __launch_bounds__(kRedThreads)
k_pauli_pair(const typename CT<R>::type *__restrict__ s, idx_t n_items, int hbit,
             unsigned long long x_mask, unsigned long long z_mask, int ny, double *partials) {
    double acc = 0.;
    const idx_t stride = (idx_t)gridDim.x * blockDim.x;
    idx_t k = (idx_t)blockIdx.x * blockDim.x + threadIdx.x;
    auto term = [&](idx_t kk) -> R {
        idx_t b = insert_zero(kk, hbit);
        idx_t b2 = b ^ (idx_t)x_mask;
        typename CT<R>::type p = s[b], q = s[b2];
        R wr = q.x * p.x + q.y * p.y;
        R wi = q.x * p.y - q.y * p.x;
        R s1 = parity_sign_r<R>(b & (idx_t)z_mask), s2 = parity_sign_r<R>(b2 & (idx_t)z_mask);
        switch (ny & 3) {
        case 0: return (s1 + s2) * wr;
        case 1: return -(s1 - s2) * wi;
        case 2: return -(s1 + s2) * wr;
        default: return (s1 - s2) * wi;
        }
    };
    for (; k + (kUnroll - 1) * stride < n_items; k += kUnroll * stride) {
        R part = 0;
#pragma unroll
        for (int u = 0; u < kUnroll; ++u) part += term(k + u * stride);
        acc += (double)part;
    }
    for (; k < n_items; k += stride) acc += (double)term(k);
    acc = block_sum(acc);
    if (threadIdx.x == 0) partials[blockIdx.x] = acc;
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

// ------------------------------------------------------------ FP64 scan

constexpr int kScanThreads = 256;
constexpr int kScanItems = 16;
constexpr idx_t kScanTile = kScanThreads * kScanItems;

__global__ void __launch_bounds__(kScanThreads)
k_tile_sums(const double *__restrict__ x, idx_t n, double *__restrict__ sums) {
    const idx_t base = (idx_t)blockIdx.x * kScanTile;
    double v = 0.;
#pragma unroll
    for (int j = 0; j < kScanItems; ++j) {
        idx_t i = base + (idx_t)j * kScanThreads + threadIdx.x;
        if (i < n) v += x[i];
    }
    v = block_sum(v);
    if (threadIdx.x == 0) sums[blockIdx.x] = v;
}

// Inclusive scan of one tile in place, plus the inclusive prefix of the
// preceding tiles (incl_sums[tile - 1]), times norm.  Shared memory is padded
// by one double per 16 so that each thread's run of 16 consecutive items
// falls in distinct banks.
__device__ __forceinline__ int pad16(int i) { return i + (i >> 4); }

__global__ void __launch_bounds__(kScanThreads)
k_tile_apply(double *__restrict__ x, idx_t n, const double *__restrict__ incl_sums, double norm) {
    __shared__ double tile[kScanTile + kScanTile / 16];
    __shared__ double warp_tot[kScanThreads / 32];
    const idx_t base = (idx_t)blockIdx.x * kScanTile;
    for (int j = 0; j < kScanItems; ++j) {
        int li = j * kScanThreads + threadIdx.x;
        idx_t i = base + li;
        tile[pad16(li)] = i < n ? x[i] : 0.;
    }
    __syncthreads();
    double loc[kScanItems];
    double run = 0.;
#pragma unroll
    for (int j = 0; j < kScanItems; ++j) {
        run += tile[pad16(threadIdx.x * kScanItems + j)];
        loc[j] = run;
    }
    // exclusive scan of thread totals
    int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    double inc = run;
    for (int o = 1; o < 32; o <<= 1) {
        double t = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += t;
    }
    if (lane == 31) warp_tot[warp] = inc;
    __syncthreads();
    double warp_off = 0.;
    for (int w = 0; w < warp; ++w) warp_off += warp_tot[w];
    double off = warp_off + inc - run;
    if (blockIdx.x > 0) off += incl_sums[blockIdx.x - 1];
#pragma unroll
    for (int j = 0; j < kScanItems; ++j)
        tile[pad16(threadIdx.x * kScanItems + j)] = (loc[j] + off) * norm;
    __syncthreads();
    for (int j = 0; j < kScanItems; ++j) {
        int li = j * kScanThreads + threadIdx.x;
        idx_t i = base + li;
        if (i < n) x[i] = tile[pad16(li)];
    }
}

__global__ void k_copy_last(const double *x, idx_t n, double *out) { *out = x[n - 1]; }

// upper_bound(cdf, u) clamped to n-1, then zero bits inserted at the empty
// lanes (qgate/simulator/src/CPUSamplingPool.cpp:71-81; spec:
// qgate/simulator/pyruntime.py:303-321).
struct EmptyPos {
    int n;
    int pos[kMaxLanes];
};

__global__ void __launch_bounds__(256)
k_search(const double *__restrict__ cdf, idx_t n, const double *__restrict__ u,
         long long *__restrict__ obs, idx_t m, EmptyPos ep) {
    const idx_t stride = (idx_t)gridDim.x * blockDim.x;
    for (idx_t i = (idx_t)blockIdx.x * blockDim.x + threadIdx.x; i < m; i += stride) {
        double x = u[i];
        idx_t lo = 0, hi = n;
        while (lo < hi) {
            idx_t mid = (lo + hi) >> 1;
            if (cdf[mid] <= x)
                lo = mid + 1;
            else
                hi = mid;
        }
        if (lo > n - 1) lo = n - 1;
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

size_t scan_scratch_doubles(idx_t n) {
    size_t total = 0;
    idx_t len = n;
    while (len > 1) {
        idx_t tiles = (len + kScanTile - 1) / kScanTile;
        total += (size_t)tiles + 1;
        len = tiles;
    }
    return total + 2;
}

// Inclusive scan of every level above `data`; level-0 tiles are applied
// later by launch_scan_apply, once the caller knows the normalisation.
void launch_scan_sums(double *data, idx_t n, double *d_scratch, double *d_total,
                      cudaStream_t stream) {
    idx_t tiles = (n + kScanTile - 1) / kScanTile;
    double *sums = d_scratch;
    k_tile_sums<<<(unsigned)tiles, kScanThreads, 0, stream>>>(data, n, sums);
    if (tiles > 1) {
        double *next = d_scratch + tiles + 1;
        launch_scan_sums(sums, tiles, next, nullptr, stream);
        launch_scan_apply(sums, tiles, next, 1.0, stream);
    }
    if (d_total) k_copy_last<<<1, 1, 0, stream>>>(sums, tiles, d_total);
    QG_CUDA(cudaGetLastError());
}

void launch_scan_apply(double *data, idx_t n, double *d_scratch, double norm,
                       cudaStream_t stream) {
    idx_t tiles = (n + kScanTile - 1) / kScanTile;
    k_tile_apply<<<(unsigned)tiles, kScanThreads, 0, stream>>>(data, n, d_scratch, norm);
    QG_CUDA(cudaGetLastError());
}

void launch_search(const double *cdf, idx_t n, const double *u, long long *obs, idx_t n_samples,
                   const int *empty_pos, int n_empty, cudaStream_t stream) {
    if (n_samples <= 0) return;
    EmptyPos ep;
    ep.n = n_empty;
    for (int i = 0; i < n_empty; ++i) ep.pos[i] = empty_pos[i];
    k_search<<<sm_grid(n_samples, 256, 152 * 16), 256, 0, stream>>>(cdf, n, u, obs, n_samples, ep);
    QG_CUDA(cudaGetLastError());
}

}  // namespace qg
