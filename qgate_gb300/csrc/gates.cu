// Gate-apply, measurement and state-construction kernels (sm_103a).
//
// Every kernel here is a streaming sweep over the state and is bound by HBM
// bandwidth: the algorithmic traffic of a sweep is one read plus one write of
// each touched amplitude.  Loads and stores are 16-byte vectors wherever the
// lane pattern leaves amplitude pairs contiguous (two complex64 per float4,
// one complex128 per double2), and each thread keeps kILP independent work
// items in flight to cover HBM latency.
//
// Reference counterparts: the device lambdas of
// qgate/simulator/src/DeviceProcPrimitives.cu (applyGate :198-221,
// applyControlledGate :223-249, decohere :112-143, decohereAndShrink
// :146-172, applyReset :175-196, kron :56-109), each launched there as one
// thread per index with 128-thread blocks and scalar 8/16-byte accesses.
#include "qg_device.cuh"

namespace qg {

namespace {

constexpr int kThreads = 256;
constexpr int kILP = 4;

inline unsigned grid_for(idx_t items, int per_block) {
    idx_t g = (items + per_block - 1) / per_block;
    if (g < 1) g = 1;
    return (unsigned)g;
}

// ------------------------------------------------------------ pair ops

template <class R> struct GateOp {
    MatR<R> m;
    template <class C> __device__ __forceinline__ void operator()(C &a, C &b) const {
        apply2<R>(m, a, b);
    }
};

template <class R> struct DecohereOp {
    int value;
    R norm;
    template <class C> __device__ __forceinline__ void operator()(C &a, C &b) const {
        if (value == 0) {
            a = cscale(a, norm);
            b = cmk<C>(0., 0.);
        } else {
            a = cmk<C>(0., 0.);
            b = cscale(b, norm);
        }
    }
};

struct ResetOp {
    template <class C> __device__ __forceinline__ void operator()(C &a, C &b) const {
        a = b;
        b = cmk<C>(0., 0.);
    }
};

// Scalar pair sweep (any precision, any bit pattern).
template <class R, class Op>
__global__ void __launch_bounds__(kThreads)
k_pairs_scalar(typename CT<R>::type *__restrict__ s, idx_t n_items, PairIdx pi, Op op) {
    typedef typename CT<R>::type C;
    const idx_t base = (idx_t)blockIdx.x * (kThreads * kILP) + threadIdx.x;
    C a[kILP], b[kILP];
    idx_t i0[kILP];
#pragma unroll
    for (int u = 0; u < kILP; ++u) {
        idx_t k = base + (idx_t)u * kThreads;
        i0[u] = -1;
        if (k < n_items) {
            i0[u] = insert_zeros(k, pi.pos, pi.npos) | (idx_t)pi.set_mask;
            a[u] = s[i0[u]];
            b[u] = s[i0[u] | (idx_t)pi.partner];
        }
    }
#pragma unroll
    for (int u = 0; u < kILP; ++u) {
        if (i0[u] >= 0) {
            op(a[u], b[u]);
            s[i0[u]] = a[u];
            s[i0[u] | (idx_t)pi.partner] = b[u];
        }
    }
}

// complex64, lane 0 untouched by the pattern: work item v covers compressed
// indices 2v and 2v+1, which map to two adjacent amplitudes on each side of
// the pair, so each side is one float4.
template <class Op>
__global__ void __launch_bounds__(kThreads)
k_pairs_vec2_f32(float4 *__restrict__ s, idx_t n_items, PairIdx pi, Op op) {
    const idx_t base = (idx_t)blockIdx.x * (kThreads * kILP) + threadIdx.x;
    float4 a[kILP], b[kILP];
    idx_t v0[kILP], v1[kILP];
#pragma unroll
    for (int u = 0; u < kILP; ++u) {
        idx_t v = base + (idx_t)u * kThreads;
        v0[u] = -1;
        if (v < n_items) {
            idx_t i0 = insert_zeros(2 * v, pi.pos, pi.npos) | (idx_t)pi.set_mask;
            v0[u] = i0 >> 1;
            v1[u] = (i0 | (idx_t)pi.partner) >> 1;
            a[u] = s[v0[u]];
            b[u] = s[v1[u]];
        }
    }
#pragma unroll
    for (int u = 0; u < kILP; ++u) {
        if (v0[u] >= 0) {
            float2 a0 = make_float2(a[u].x, a[u].y), a1 = make_float2(a[u].z, a[u].w);
            float2 b0 = make_float2(b[u].x, b[u].y), b1 = make_float2(b[u].z, b[u].w);
            op(a0, b0);
            op(a1, b1);
            s[v0[u]] = make_float4(a0.x, a0.y, a1.x, a1.y);
            s[v1[u]] = make_float4(b0.x, b0.y, b1.x, b1.y);
        }
    }
}

// complex64, partner bit = lane 0: both members of a pair share one float4.
template <class Op>
__global__ void __launch_bounds__(kThreads)
k_pairs_adj_f32(float4 *__restrict__ s, idx_t n_items, PairIdx pi, Op op) {
    const idx_t base = (idx_t)blockIdx.x * (kThreads * kILP) + threadIdx.x;
    float4 a[kILP];
    idx_t vi[kILP];
#pragma unroll
    for (int u = 0; u < kILP; ++u) {
        idx_t k = base + (idx_t)u * kThreads;
        vi[u] = -1;
        if (k < n_items) {
            vi[u] = (insert_zeros(k, pi.pos, pi.npos) | (idx_t)pi.set_mask) >> 1;
            a[u] = s[vi[u]];
        }
    }
#pragma unroll
    for (int u = 0; u < kILP; ++u) {
        if (vi[u] >= 0) {
            float2 x = make_float2(a[u].x, a[u].y), y = make_float2(a[u].z, a[u].w);
            op(x, y);
            s[vi[u]] = make_float4(x.x, x.y, y.x, y.y);
        }
    }
}

template <class R, class Op>
void dispatch_pairs(void *state, idx_t n_items, const PairIdx &pi, const Op &op,
                    cudaStream_t stream) {
    if (n_items <= 0) return;
    const int per_block = kThreads * kILP;
    if constexpr (sizeof(R) == 4) {
        bool bit0_free = (pi.set_mask & 1ULL) == 0 && (pi.partner & 1ULL) == 0 &&
                         (pi.npos == 0 || pi.pos[0] >= 1);
        bool adj = pi.partner == 1ULL && (pi.set_mask & 1ULL) == 0;
        if (bit0_free && (n_items % 2) == 0) {
            idx_t nv = n_items / 2;
            k_pairs_vec2_f32<<<grid_for(nv, per_block), kThreads, 0, stream>>>(
                (float4 *)state, nv, pi, op);
            return;
        }
        if (adj) {
            // insertion pattern must have lane 0 among its positions.
            k_pairs_adj_f32<<<grid_for(n_items, per_block), kThreads, 0, stream>>>(
                (float4 *)state, n_items, pi, op);
            return;
        }
    }
    k_pairs_scalar<R, Op><<<grid_for(n_items, per_block), kThreads, 0, stream>>>(
        (typename CT<R>::type *)state, n_items, pi, op);
}

// ------------------------------------------------------------ init / shrink

template <class R>
__global__ void __launch_bounds__(kThreads)
k_init_basis(typename CT<R>::vec *__restrict__ s, idx_t n_vec) {
    typedef typename CT<R>::vec V;
    const idx_t base = (idx_t)blockIdx.x * (kThreads * kILP) + threadIdx.x;
#pragma unroll
    for (int u = 0; u < kILP; ++u) {
        idx_t v = base + (idx_t)u * kThreads;
        if (v < n_vec) {
            V z;
            memset(&z, 0, sizeof(V));
            if (v == 0) z.x = 1;
            s[v] = z;
        }
    }
}

// dst[k] = norm * src[insert_zero(k, lane) | value << lane]
template <class R>
__global__ void __launch_bounds__(kThreads)
k_shrink(typename CT<R>::type *__restrict__ dst, const typename CT<R>::type *__restrict__ src,
         idx_t n_items, PairIdx pi, R norm) {
    const idx_t base = (idx_t)blockIdx.x * (kThreads * kILP) + threadIdx.x;
#pragma unroll
    for (int u = 0; u < kILP; ++u) {
        idx_t k = base + (idx_t)u * kThreads;
        if (k < n_items) {
            idx_t i = insert_zeros(k, pi.pos, pi.npos) | (idx_t)pi.set_mask;
            dst[k] = cscale(src[i], norm);
        }
    }
}

__global__ void __launch_bounds__(kThreads)
k_shrink_vec2_f32(float4 *__restrict__ dst, const float4 *__restrict__ src, idx_t n_vec,
                  PairIdx pi, float norm) {
    const idx_t base = (idx_t)blockIdx.x * (kThreads * kILP) + threadIdx.x;
#pragma unroll
    for (int u = 0; u < kILP; ++u) {
        idx_t v = base + (idx_t)u * kThreads;
        if (v < n_vec) {
            idx_t i = insert_zeros(2 * v, pi.pos, pi.npos) | (idx_t)pi.set_mask;
            float4 a = src[i >> 1];
            dst[v] = make_float4(a.x * norm, a.y * norm, a.z * norm, a.w * norm);
        }
    }
}

// ------------------------------------------------------------ kron (join)

struct KronDesc {
    int n_src;
    const void *src[kMaxGetterStates];
    int shift[kMaxGetterStates];
    long long mask[kMaxGetterStates];
    long long basis[kMaxGetterStates];  // src == nullptr: the basis state |basis>
};

template <class C>
__device__ __forceinline__ C kron_factor(const KronDesc &kd, int g, idx_t d) {
    const idx_t i = (d >> kd.shift[g]) & kd.mask[g];
    if (kd.src[g]) return ((const C *)kd.src[g])[i];
    C v;
    v.x = i == kd.basis[g] ? 1 : 0;
    v.y = 0;
    return v;
}

// dst[d] = src[0][f0(d)] * ... * src[n-1][f_{n-1}(d)], the last source in the
// lowest bits (np.kron order, qgate/simulator/pyruntime.py:82-97).  The
// product is formed from the last source backwards, the order of the
// reference's pairwise kron (qgate/simulator/src/CPUQubitProcessor.cpp:166-205).
// A source without a buffer is a basis state (exact 0 / 1 factors).
template <class R>
__global__ void __launch_bounds__(kThreads)
k_kron(typename CT<R>::type *__restrict__ dst, idx_t n_dst, KronDesc kd) {
    typedef typename CT<R>::type C;
    const idx_t base = (idx_t)blockIdx.x * (kThreads * kILP) + threadIdx.x;
#pragma unroll
    for (int u = 0; u < kILP; ++u) {
        idx_t d = base + (idx_t)u * kThreads;
        if (d < n_dst) {
            int g = kd.n_src - 1;
            C v = kron_factor<C>(kd, g, d);
            for (g = kd.n_src - 2; g >= 0; --g) v = cmul(kron_factor<C>(kd, g, d), v);
            dst[d] = v;
        }
    }
}

// In-place removal of lane L at value v (decohere and separate): element k of
// the (n-1)-lane result is norm * s[k with bit v inserted at L].  In chunks
// of 2^L amplitudes, result chunk h comes from source chunk 2h + v >= h.
// Round 0 moves chunk v to chunk 0; round j >= 1 fills chunks
// [2^(j-1), 2^j) from chunks [2^j, 2^(j+1)): within a round sources and
// destinations are disjoint, a destination chunk was last read as a source
// in an earlier round, and no source chunk has been written yet.
template <class R>
__global__ void __launch_bounds__(kThreads)
k_shrink_round(typename CT<R>::type *s, int L, int v, idx_t h0, idx_t h1, R norm) {
    const idx_t n = (h1 - h0) << L;
    const idx_t lo_mask = ((idx_t)1 << L) - 1;
    for (idx_t k = (idx_t)blockIdx.x * kThreads + threadIdx.x; k < n;
         k += (idx_t)gridDim.x * kThreads) {
        const idx_t h = h0 + (k >> L), lo = k & lo_mask;
        s[(h << L) | lo] = cscale(s[(((h << 1) | (idx_t)v) << L) | lo], norm);
    }
}

// Rounds 0..j_last in one CTA (the first rounds are tiny), a barrier between
// rounds.
template <class R>
__global__ void __launch_bounds__(1024)
k_shrink_rounds_cta(typename CT<R>::type *s, int L, int v, int j_last, R norm) {
    const idx_t lo_mask = ((idx_t)1 << L) - 1;
    for (int j = 0; j <= j_last; ++j) {
        const idx_t h0 = j ? (idx_t)1 << (j - 1) : 0, h1 = (idx_t)1 << j;
        const idx_t n = (h1 - h0) << L;
        for (idx_t k = threadIdx.x; k < n; k += blockDim.x) {
            const idx_t h = h0 + (k >> L), lo = k & lo_mask;
            s[(h << L) | lo] = cscale(s[(((h << 1) | (idx_t)v) << L) | lo], norm);
        }
        __syncthreads();
    }
}

// ------------------------------------------------------------ dense multi-target

// One thread per group of 2^K amplitudes that share all non-target bits.
template <class R, int K>
__global__ void __launch_bounds__(128)
k_multi(typename CT<R>::type *__restrict__ s, idx_t n_items, MultiDesc d,
        const double *__restrict__ mat) {
    typedef typename CT<R>::type C;
    constexpr int D = 1 << K;
    __shared__ C sm[D * D];
    for (int i = threadIdx.x; i < D * D; i += blockDim.x)
        sm[i] = cmk<C>(mat[2 * i], mat[2 * i + 1]);
    __syncthreads();
    idx_t k = (idx_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n_items) return;
    idx_t base = insert_zeros(k, d.pos, d.npos) | (idx_t)d.cmask;
    idx_t off[D];
    C in[D];
#pragma unroll
    for (int j = 0; j < D; ++j) {
        idx_t o = 0;
#pragma unroll
        for (int t = 0; t < K; ++t)
            if (j & (1 << t)) o |= 1LL << d.tpos[t];
        off[j] = base | o;
        in[j] = s[off[j]];
    }
#pragma unroll
    for (int r = 0; r < D; ++r) {
        C acc = cmk<C>(0., 0.);
#pragma unroll
        for (int c = 0; c < D; ++c) acc = cadd(acc, cmul(sm[r * D + c], in[c]));
        s[off[r]] = acc;
    }
}

}  // namespace

// ------------------------------------------------------------ launchers

void launch_init_basis(int prec, void *state, idx_t n_amps, cudaStream_t stream) {
    const int per_block = kThreads * kILP;
    if (prec == kFP32) {
        if (n_amps == 1) {
            float2 one = make_float2(1.f, 0.f);
            QG_CUDA(cudaMemcpyAsync(state, &one, sizeof(one), cudaMemcpyHostToDevice, stream));
            return;
        }
        idx_t nv = n_amps / 2;
        k_init_basis<float><<<grid_for(nv, per_block), kThreads, 0, stream>>>((float4 *)state, nv);
    } else {
        k_init_basis<double><<<grid_for(n_amps, per_block), kThreads, 0, stream>>>(
            (double2 *)state, n_amps);
    }
    QG_CUDA(cudaGetLastError());
}

void launch_fill_zero(int prec, void *state, idx_t begin, idx_t end, cudaStream_t stream) {
    if (end <= begin) return;
    size_t cs = complex_size(prec);
    QG_CUDA(cudaMemsetAsync((char *)state + begin * cs, 0, (end - begin) * cs, stream));
}

void launch_apply_pairs(int prec, void *state, idx_t n_items, const PairIdx &pi, const Mat2 &m,
                        cudaStream_t stream) {
    // The matrix is converted on the device; pass it through the op by value.
    if (prec == kFP32) {
        GateOp<float> op;
        op.m.m00 = make_float2((float)m.v[0], (float)m.v[1]);
        op.m.m01 = make_float2((float)m.v[2], (float)m.v[3]);
        op.m.m10 = make_float2((float)m.v[4], (float)m.v[5]);
        op.m.m11 = make_float2((float)m.v[6], (float)m.v[7]);
        dispatch_pairs<float>(state, n_items, pi, op, stream);
    } else {
        GateOp<double> op;
        op.m.m00 = make_double2(m.v[0], m.v[1]);
        op.m.m01 = make_double2(m.v[2], m.v[3]);
        op.m.m10 = make_double2(m.v[4], m.v[5]);
        op.m.m11 = make_double2(m.v[6], m.v[7]);
        dispatch_pairs<double>(state, n_items, pi, op, stream);
    }
    QG_CUDA(cudaGetLastError());
}

void launch_decohere(int prec, void *state, idx_t n_items, const PairIdx &pi, int value,
                     double norm, cudaStream_t stream) {
    if (prec == kFP32) {
        DecohereOp<float> op{value, (float)norm};
        dispatch_pairs<float>(state, n_items, pi, op, stream);
    } else {
        DecohereOp<double> op{value, norm};
        dispatch_pairs<double>(state, n_items, pi, op, stream);
    }
    QG_CUDA(cudaGetLastError());
}

void launch_reset(int prec, void *state, idx_t n_items, const PairIdx &pi, cudaStream_t stream) {
    if (prec == kFP32)
        dispatch_pairs<float>(state, n_items, pi, ResetOp(), stream);
    else
        dispatch_pairs<double>(state, n_items, pi, ResetOp(), stream);
    QG_CUDA(cudaGetLastError());
}

void launch_shrink(int prec, void *dst, const void *src, idx_t n_items, const PairIdx &pi,
                   double norm, cudaStream_t stream) {
    if (n_items <= 0) return;
    const int per_block = kThreads * kILP;
    if (prec == kFP32) {
        bool vec = (pi.set_mask & 1ULL) == 0 && pi.npos > 0 && pi.pos[0] >= 1 && n_items % 2 == 0;
        if (vec) {
            idx_t nv = n_items / 2;
            k_shrink_vec2_f32<<<grid_for(nv, per_block), kThreads, 0, stream>>>(
                (float4 *)dst, (const float4 *)src, nv, pi, (float)norm);
        } else {
            k_shrink<float><<<grid_for(n_items, per_block), kThreads, 0, stream>>>(
                (float2 *)dst, (const float2 *)src, n_items, pi, (float)norm);
        }
    } else {
        k_shrink<double><<<grid_for(n_items, per_block), kThreads, 0, stream>>>(
            (double2 *)dst, (const double2 *)src, n_items, pi, norm);
    }
    QG_CUDA(cudaGetLastError());
}

void launch_kron(int prec, void *dst, idx_t n_dst, const void *const *srcs, const int *src_lanes,
                 int n_src, cudaStream_t stream, const long long *basis) {
    if (n_src > kMaxGetterStates) fail(2, "too many states to join (%d).", n_src);
    KronDesc kd;
    kd.n_src = n_src;
    int shift = 0;
    for (int g = n_src - 1; g >= 0; --g) {
        kd.src[g] = srcs[g];
        kd.shift[g] = shift;
        kd.mask[g] = (1LL << src_lanes[g]) - 1;
        kd.basis[g] = basis ? basis[g] : 0;
        if (!srcs[g] && !basis) fail(2, "join source without amplitudes.");
        shift += src_lanes[g];
    }
    const int per_block = kThreads * kILP;
    if (prec == kFP32)
        k_kron<float><<<grid_for(n_dst, per_block), kThreads, 0, stream>>>((float2 *)dst, n_dst, kd);
    else
        k_kron<double><<<grid_for(n_dst, per_block), kThreads, 0, stream>>>((double2 *)dst, n_dst,
                                                                            kd);
    QG_CUDA(cudaGetLastError());
}

void launch_shrink_inplace(int prec, void *state, int n_lanes, int lane, int value, double norm,
                           cudaStream_t stream) {
    if (lane < 0 || lane >= n_lanes || (value != 0 && value != 1))
        fail(2, "in-place shrink: bad lane or value.");
    const int L = lane, J = n_lanes - 1 - lane;  // rounds 0..J
    // rounds whose cumulative size stays within 2^16 amplitudes run in one CTA
    int j_small = -1;
    while (j_small < J && j_small + 1 + L <= 16) ++j_small;
    if (j_small >= 0) {
        if (prec == kFP32)
            k_shrink_rounds_cta<float><<<1, 1024, 0, stream>>>((float2 *)state, L, value, j_small,
                                                               (float)norm);
        else
            k_shrink_rounds_cta<double><<<1, 1024, 0, stream>>>((double2 *)state, L, value,
                                                                j_small, norm);
    }
    for (int j = j_small + 1; j <= J; ++j) {
        const idx_t h0 = j ? (idx_t)1 << (j - 1) : 0, h1 = (idx_t)1 << j;
        const idx_t n = (h1 - h0) << L;
        const unsigned grid = grid_for(n, kThreads);
        if (prec == kFP32)
            k_shrink_round<float><<<grid, kThreads, 0, stream>>>((float2 *)state, L, value, h0, h1,
                                                                 (float)norm);
        else
            k_shrink_round<double><<<grid, kThreads, 0, stream>>>((double2 *)state, L, value, h0,
                                                                  h1, norm);
    }
    QG_CUDA(cudaGetLastError());
}

template <class R>
static void multi_dispatch(void *state, idx_t n_items, const MultiDesc &d, const double *mat,
                           cudaStream_t stream) {
    typedef typename CT<R>::type C;
    unsigned grid = grid_for(n_items, 128);
    C *s = (C *)state;
    switch (d.k) {
    case 1: k_multi<R, 1><<<grid, 128, 0, stream>>>(s, n_items, d, mat); break;
    case 2: k_multi<R, 2><<<grid, 128, 0, stream>>>(s, n_items, d, mat); break;
    case 3: k_multi<R, 3><<<grid, 128, 0, stream>>>(s, n_items, d, mat); break;
    case 4: k_multi<R, 4><<<grid, 128, 0, stream>>>(s, n_items, d, mat); break;
    case 5: {
        auto f = k_multi<R, 5>;
        QG_CUDA(cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, 0));
        f<<<grid, 128, 0, stream>>>(s, n_items, d, mat);
        break;
    }
    default: fail(1, "dense multi-target gate supports 1..5 targets (got %d).", d.k);
    }
}

void launch_apply_multi(int prec, void *state, idx_t n_items, const MultiDesc &d,
                        const void *d_mat, cudaStream_t stream) {
    if (n_items <= 0) return;
    if (prec == kFP32)
        multi_dispatch<float>(state, n_items, d, (const double *)d_mat, stream);
    else
        multi_dispatch<double>(state, n_items, d, (const double *)d_mat, stream);
    QG_CUDA(cudaGetLastError());
}

}  // namespace qg
