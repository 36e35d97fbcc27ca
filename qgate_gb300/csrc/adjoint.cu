// Kernels of the adjoint-differentiation engine (sm_103a).
//
// A batch of B parameter vectors of one circuit shares one stage program;
// each CTA handles one tile of one batch element (grid = tiles x B) and reads
// that element's gate matrices from a per-element table.  The backward stage
// keeps the tiles of both psi and lambda = U^dagger ... H psi in registers,
// and for every parametrised rotation exp(-i c theta G) it first accumulates
// Im<lambda|P1 G|psi> (P1: its controls set) and then un-applies the gate to
// both states -- the gradient is 2c times that sum.  One HBM read and write of
// psi and lambda per stage, however many gates it holds.
//
// The reference has no differentiation path; its nearest composition is
// finite differences or parameter-shift over repeated runs
// (qgate/simulator/simulator.py:57-83 per evaluation).
#include "qg_regstage.cuh"

namespace qg {

namespace {

using namespace rs;

template <class C> __device__ __forceinline__ auto im_conj_mul(C l, C p) {  // Im(conj(l) p)
    return l.x * p.y - l.y * p.x;
}
template <class C> __device__ __forceinline__ auto re_conj_mul(C l, C p) {  // Re(conj(l) p)
    return l.x * p.x + l.y * p.y;
}

// Im<lam|P1 G|psi> over this thread's register pairs on register bit I.
template <int I, int NR, class C, class R>
__device__ __forceinline__ void reg_grad(const C (&a)[NR], const C (&l)[NR], unsigned jmask,
                                         int axis, R &out) {
    R acc = 0;
#pragma unroll
    for (int j = 0; j < NR; ++j) {
        if (j & (1 << I)) continue;
        if ((j & jmask) != jmask) continue;
        const C p0 = a[j], p1 = a[j | (1 << I)], l0 = l[j], l1 = l[j | (1 << I)];
        if (axis == 1)
            acc += im_conj_mul(l0, p1) + im_conj_mul(l1, p0);
        else if (axis == 2)
            acc += re_conj_mul(l1, p0) - re_conj_mul(l0, p1);
        else
            acc += im_conj_mul(l0, p0) - im_conj_mul(l1, p1);
    }
    out = acc;
}

// Shared-memory bytes of n register-set slot tables, rounded to 16.
__host__ __device__ constexpr unsigned adj_sets_bytes(int nsets) {
    return ((unsigned)nsets * (unsigned)sizeof(SetSlots) + 15u) & ~15u;
}

template <class R> __device__ __forceinline__ R warp_sum(R v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

template <class R, int RL, int MODE>
__global__ void __launch_bounds__(MODE == 1 ? 256 : 512)
k_adj_stage(typename CT<R>::type *__restrict__ psi_all, typename CT<R>::type *__restrict__ lam_all,
            const __grid_constant__ AdjStageDesc d, const R *__restrict__ mats_all,
            R *__restrict__ gpart) {
    typedef typename CT<R>::type C;
    constexpr int NR = 1 << RL;
    extern __shared__ __align__(16) unsigned char smraw[];
    const int m = d.m, n = d.n;
    const unsigned tid = threadIdx.x, T = blockDim.x;
    const int b = blockIdx.y;
    const idx_t tiles = (idx_t)gridDim.x;
    C *psi = psi_all + ((idx_t)b << n);
    C *lam = MODE == 1 ? lam_all + ((idx_t)b << n) : nullptr;

    C *sp = (C *)smraw;
    C *sl = sp + (MODE == 1 ? (1 << m) : 0);
    AdjOp *sops = (AdjOp *)(sp + ((MODE == 1 ? 2 : 1) << m));
    long long *sdep = (long long *)(sops + d.nops);
    SetSlots *sset = (SetSlots *)(sdep + NR);
    R *smat = (R *)((unsigned char *)sset + adj_sets_bytes(d.nsets));
    R *sgrad = smat + 8 * d.nmats;

    {
        const int4 *src = (const int4 *)d.ops;
        int4 *dst = (int4 *)sops;
        for (int i = tid; i < d.nops; i += T) dst[i] = src[i];
        if (tid < (unsigned)NR) sdep[tid] = d.dep_hi[tid];
        copy_sets(sset, d.sets, d.nsets, tid, T);
        const R *mats = mats_all + (size_t)b * d.nmats * 8;
        for (int i = tid; i < 8 * d.nmats; i += T) smat[i] = mats[i];
        if (MODE == 1)
            for (int i = tid; i < d.ngrads; i += T) sgrad[i] = 0;
    }
    const int t = m - RL;
    const idx_t base = insert_zeros((idx_t)blockIdx.x, d.ins_pos, d.nins);
    const int lr = d.lowrun < t ? d.lowrun : t;
    idx_t dt = (idx_t)(tid & ((1u << lr) - 1u));
    for (int bb = lr; bb < t; ++bb)
        if (tid & (1u << bb)) dt |= 1LL << d.hi_pos[bb - d.lowrun];
    const unsigned pt = Swz<R>::f(tid);
    __syncthreads();

#pragma unroll
    for (int i = 0; i < NR; ++i) {
        unsigned slot = pt ^ Swz<R>::f((unsigned)i << t);
        idx_t g = base | dt | sdep[i];
        cp_async_elem(&sp[slot], &psi[g]);
        if (MODE == 1) cp_async_elem(&sl[slot], &lam[g]);
    }
    asm volatile("cp.async.wait_all;\n" ::: "memory");
    __syncthreads();

    C a[NR], l[NR];
    unsigned e0 = 0, P0 = 0;
    unsigned q[RL];
#pragma unroll
    for (int k = 0; k < RL; ++k) q[k] = 0;
    const unsigned lane = tid & 31u;

    for (int oi = 0; oi < d.nops; ++oi) {
        const AdjOp o = sops[oi];
        if (o.kind == kOpTranspose) {
            if (oi > 0) {
                __syncthreads();
#pragma unroll
                for (int j = 0; j < NR; ++j) {
                    unsigned sl_ = reg_slot<RL>(P0, q, j);
                    sp[sl_] = a[j];
                    if (MODE == 1) sl[sl_] = l[j];
                }
                __syncthreads();
            }
            const SetSlots &ss = sset[o.reg];
            P0 = (unsigned)ss.lo[tid & 31u] ^ (unsigned)ss.hi[tid >> 5];
            e0 = Swz<R>::f(P0);
#pragma unroll
            for (int k = 0; k < RL; ++k) q[k] = ss.q[k];
#pragma unroll
            for (int j = 0; j < NR; ++j) {
                unsigned sl_ = reg_slot<RL>(P0, q, j);
                a[j] = sp[sl_];
                if (MODE == 1) l[j] = sl[sl_];
            }
            continue;
        }
        const bool act = (e0 & o.tmask) == o.tmask;
        if (MODE == 1 && o.gaxis) {
            R v = 0;
            if (act) {
                if (o.kind == kOpDiagThread) {
                    R acc = 0;
#pragma unroll
                    for (int j = 0; j < NR; ++j)
                        if ((j & o.jmask) == o.jmask) acc += im_conj_mul(l[j], a[j]);
                    v = (e0 & o.tbit) ? -acc : acc;
                } else {
                    QG_REG_DISPATCH(reg_grad, o.reg, a, l, (unsigned)o.jmask, (int)o.gaxis, v);
                }
            }
            v = warp_sum(v);
            if (lane == 0) atomicAdd(&sgrad[o.gslot], v);
        }
        if (!act) continue;
        const R *mm_ = smat + 8 * o.mat;
        if (o.kind == kOpGate) {
            MatR<R> mm;
            mm.m00 = cmk<C>(mm_[0], mm_[1]);
            mm.m01 = cmk<C>(mm_[2], mm_[3]);
            mm.m10 = cmk<C>(mm_[4], mm_[5]);
            mm.m11 = cmk<C>(mm_[6], mm_[7]);
            QG_REG_DISPATCH(reg_gate, o.reg, a, mm, (unsigned)o.jmask);
            if (MODE == 1) QG_REG_DISPATCH(reg_gate, o.reg, l, mm, (unsigned)o.jmask);
        } else if (o.kind == kOpSwapX) {
            QG_REG_DISPATCH(reg_swap, o.reg, a, (unsigned)o.jmask);
            if (MODE == 1) QG_REG_DISPATCH(reg_swap, o.reg, l, (unsigned)o.jmask);
        } else if (o.kind == kOpDiagReg) {
            C d0 = cmk<C>(mm_[0], mm_[1]), d1 = cmk<C>(mm_[6], mm_[7]);
            QG_REG_DISPATCH(reg_diag, o.reg, a, d0, d1, (unsigned)o.jmask);
            if (MODE == 1) QG_REG_DISPATCH(reg_diag, o.reg, l, d0, d1, (unsigned)o.jmask);
        } else {  // kOpDiagThread
            C ph = (e0 & o.tbit) ? cmk<C>(mm_[6], mm_[7]) : cmk<C>(mm_[0], mm_[1]);
#pragma unroll
            for (int j = 0; j < NR; ++j)
                if ((j & o.jmask) == o.jmask) {
                    a[j] = cmul(ph, a[j]);
                    if (MODE == 1) l[j] = cmul(ph, l[j]);
                }
        }
    }

    __syncthreads();
#pragma unroll
    for (int j = 0; j < NR; ++j) {
        unsigned sl_ = reg_slot<RL>(P0, q, j);
        sp[sl_] = a[j];
        if (MODE == 1) sl[sl_] = l[j];
    }
    __syncthreads();
#pragma unroll
    for (int i = 0; i < NR; ++i) {
        unsigned slot = pt ^ Swz<R>::f((unsigned)i << t);
        idx_t g = base | dt | sdep[i];
        psi[g] = sp[slot];
        if (MODE == 1) lam[g] = sl[slot];
    }
    if (MODE == 1)
        for (int i = tid; i < d.ngrads; i += T)
            gpart[((idx_t)b * d.ngrads + i) * tiles + blockIdx.x] = sgrad[i];
}

// grad[b * n_params + param[s]] += scale[s] * sum over tiles, FP64.
template <class R>
__global__ void k_adj_grad_reduce(const R *__restrict__ partials, int nslots, idx_t tiles,
                                  const int *__restrict__ param, const double *__restrict__ scale,
                                  double *__restrict__ grad, int n_params) {
    const int s = blockIdx.x, b = blockIdx.y;
    const R *p = partials + ((idx_t)b * nslots + s) * tiles;
    double acc = 0.;
    for (idx_t i = threadIdx.x; i < tiles; i += blockDim.x) acc += (double)p[i];
    __shared__ double ws[32];
    acc = warp_sum(acc);
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double v = 0.;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) v += ws[w];
        if (param[s] >= 0) grad[(idx_t)b * n_params + param[s]] += scale[s] * v;
    }
}

struct PauliTerms {
    int n;
    PauliTerm t[kMaxPauliTerms];
};

// lam[i] = sum_t coef_t i^ny_t (-1)^popcount((i ^ x_t) & z_t) psi[i ^ x_t]
// and the block partials of Re<psi|lam> (FP64 per block).
template <class R>
__global__ void __launch_bounds__(256)
k_pauli_sum_apply(const typename CT<R>::type *__restrict__ psi_all,
                  typename CT<R>::type *__restrict__ lam_all, int n,
                  const __grid_constant__ PauliTerms terms, double *__restrict__ e_partials) {
    typedef typename CT<R>::type C;
    const int b = blockIdx.y;
    const idx_t N = (idx_t)1 << n;
    const C *psi = psi_all + (idx_t)b * N;
    C *lam = lam_all + (idx_t)b * N;
    double acc = 0.;
    const idx_t stride = (idx_t)gridDim.x * blockDim.x;
    for (idx_t i = (idx_t)blockIdx.x * blockDim.x + threadIdx.x; i < N; i += stride) {
        R re = 0, im = 0;
        for (int k = 0; k < terms.n; ++k) {
            const PauliTerm &pt = terms.t[k];
            idx_t src = i ^ (idx_t)pt.x;
            C v = psi[src];
            R c = (R)pt.coef;
            if (__popcll((unsigned long long)(src & (idx_t)pt.z)) & 1) c = -c;
            int ny = __popcll(pt.x & pt.z) & 3;
            // multiply v by c * i^ny
            R vr = v.x * c, vi = v.y * c;
            if (ny == 0) {
                re += vr;
                im += vi;
            } else if (ny == 1) {
                re -= vi;
                im += vr;
            } else if (ny == 2) {
                re -= vr;
                im -= vi;
            } else {
                re += vi;
                im -= vr;
            }
        }
        C out;
        out.x = re;
        out.y = im;
        lam[i] = out;
        C p = psi[i];
        acc += (double)(p.x * re + p.y * im);
    }
    acc = warp_sum(acc);
    __shared__ double ws[8];
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double v = 0.;
        for (int w = 0; w < 8; ++w) v += ws[w];
        e_partials[(idx_t)b * gridDim.x + blockIdx.x] = v;
    }
}

__global__ void k_sum_rows(const double *__restrict__ partials, int cols, double *out) {
    double acc = 0.;
    for (int i = threadIdx.x; i < cols; i += blockDim.x) acc += partials[(idx_t)blockIdx.x * cols + i];
    acc = warp_sum(acc);
    __shared__ double ws[32];
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double v = 0.;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) v += ws[w];
        out[blockIdx.x] = v;
    }
}

constexpr int kPauliBlocks = 152 * 2;

template <class R, int MODE>
void adj_dispatch(void *psi, void *lam, const AdjStageDesc &d, const void *mats, void *gpart,
                  int batch, cudaStream_t stream) {
    typedef typename CT<R>::type C;
    const int NRmax = 1 << d.rl;
    size_t smem = ((size_t)sizeof(C) << d.m) * (MODE == 1 ? 2 : 1) + (size_t)d.nops * sizeof(AdjOp) +
                  sizeof(long long) * NRmax + adj_sets_bytes(d.nsets) +
                  sizeof(R) * (8 * (size_t)d.nmats + (size_t)d.ngrads);
    idx_t tiles = (idx_t)1 << (d.n - d.m);
    int threads = 1 << (d.m - d.rl);
    dim3 grid((unsigned)tiles, (unsigned)batch);
    auto launch = [&](auto kern) {
        QG_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        kern<<<grid, threads, smem, stream>>>((C *)psi, (C *)lam, d, (const R *)mats, (R *)gpart);
    };
    switch (d.rl) {
    case 3: launch(k_adj_stage<R, 3, MODE>); break;
    case 4: launch(k_adj_stage<R, 4, MODE>); break;
    case 5:
        // forward stages of complex64 only (the backward holds psi and
        // lambda: 2 x 32 amplitudes per thread would not fit)
        if constexpr (MODE == 0 && sizeof(R) == 4)
            launch(k_adj_stage<R, 5, MODE>);
        else
            fail(2, "adjoint stage: 5 register lanes only for complex64 forward stages");
        break;
    default: fail(2, "adjoint stage: unsupported register lanes %d", d.rl);
    }
    QG_CUDA(cudaGetLastError());
}

}  // namespace

void launch_adj_stage(int prec, int mode, void *psi, void *lam, const AdjStageDesc &d,
                      const void *mats, void *grad_partials, int batch, cudaStream_t stream) {
    if (prec == kFP32) {
        if (mode == 0)
            adj_dispatch<float, 0>(psi, lam, d, mats, grad_partials, batch, stream);
        else
            adj_dispatch<float, 1>(psi, lam, d, mats, grad_partials, batch, stream);
    } else {
        if (mode == 0)
            adj_dispatch<double, 0>(psi, lam, d, mats, grad_partials, batch, stream);
        else
            adj_dispatch<double, 1>(psi, lam, d, mats, grad_partials, batch, stream);
    }
}

void launch_adj_grad_reduce(int prec, const void *partials, int batch, int nslots, idx_t tiles,
                            const int *d_param, const double *d_scale, double *grad,
                            int n_params, cudaStream_t stream) {
    if (nslots == 0) return;
    dim3 grid((unsigned)nslots, (unsigned)batch);
    if (prec == kFP32)
        k_adj_grad_reduce<float><<<grid, 256, 0, stream>>>((const float *)partials, nslots, tiles,
                                                           d_param, d_scale, grad, n_params);
    else
        k_adj_grad_reduce<double><<<grid, 256, 0, stream>>>((const double *)partials, nslots,
                                                            tiles, d_param, d_scale, grad,
                                                            n_params);
    QG_CUDA(cudaGetLastError());
}

int pauli_sum_blocks() { return kPauliBlocks; }

void launch_pauli_sum_apply(int prec, const void *psi, void *lam, int n, int batch,
                            const PauliTerm *terms, int nterms, double *e_partials,
                            int blocks_per_batch, cudaStream_t stream) {
    if (nterms > kMaxPauliTerms) fail(1, "at most %d Pauli terms", kMaxPauliTerms);
    PauliTerms pt;
    pt.n = nterms;
    for (int i = 0; i < nterms; ++i) pt.t[i] = terms[i];
    dim3 grid((unsigned)blocks_per_batch, (unsigned)batch);
    if (prec == kFP32)
        k_pauli_sum_apply<float><<<grid, 256, 0, stream>>>((const float2 *)psi, (float2 *)lam, n, pt,
                                                           e_partials);
    else
        k_pauli_sum_apply<double><<<grid, 256, 0, stream>>>((const double2 *)psi, (double2 *)lam, n,
                                                            pt, e_partials);
    QG_CUDA(cudaGetLastError());
}

void launch_sum_rows(const double *partials, int rows, int cols, double *out, cudaStream_t stream) {
    k_sum_rows<<<rows, 256, 0, stream>>>(partials, cols, out);
    QG_CUDA(cudaGetLastError());
}

}  // namespace qg
