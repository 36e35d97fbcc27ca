// Fused multi-gate stage kernel (sm_103a).
//
// A stage is a run of gates whose lanes all lie in one set S of m lanes.
// The state is cut into 2^(n-m) tiles, each holding the 2^m amplitudes that
// share the bits outside S; one CTA stages one tile in shared memory, applies
// every gate of the stage there and writes the tile back, so a stage costs
// one HBM read and one write of the state however many gates it fuses.  The
// reference has no fusion: every gate is one full-state launch
// (qgate/simulator/src/DeviceProcPrimitives.cu:198-249).
#include "qg_device.cuh"
#include "qg_regstage.cuh"

namespace qg {

namespace {
using namespace rs;

// ------------------------------------------------------------ fused stage

// One CTA per tile of 2^m amplitudes whose global lanes are the stage's lane
// set.  The tile is copied into shared memory with cp.async 16-byte copies
// (runs of >= 2^lowrun contiguous amplitudes), every gate of the stage is
// applied in shared memory, and the tile is written back with 16-byte
// stores: one HBM read and one write of the state per stage, whatever the
// number of gates fused into it.
template <class R>
__device__ __forceinline__ idx_t tile_offset(const StageDesc &d, idx_t tile_base, int e) {
    idx_t g = tile_base | (idx_t)(e & ((1 << d.lowrun) - 1));
    int hi = e >> d.lowrun;
    for (int j = 0; j < d.nhi; ++j)
        if (hi & (1 << j)) g |= 1LL << d.hi_pos[j];
    return g;
}

__device__ __forceinline__ void cp_async16(void *smem, const void *gmem) {
    unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() {
    asm volatile("cp.async.wait_all;\n" ::: "memory");
}

template <class R>
__global__ void __launch_bounds__(512)
k_stage(typename CT<R>::type *__restrict__ s, const __grid_constant__ StageDesc d) {
    typedef typename CT<R>::type C;
    extern __shared__ __align__(16) unsigned char smraw[];
    C *sm = (C *)smraw;
    const int T = blockDim.x;
    const int tid = threadIdx.x;
    const int size = 1 << d.m;
    const idx_t tile_base = insert_zeros((idx_t)blockIdx.x, d.ins_pos, d.nins);
    // Elements per 16-byte copy: 2 for complex64 (needs lowrun >= 1), 1 for complex128.
    constexpr int EPV = sizeof(C) == 8 ? 2 : 1;
    for (int e = tid * EPV; e < size; e += T * EPV) {
        idx_t g = tile_offset<R>(d, tile_base, e);
        cp_async16(&sm[e], &s[g]);
    }
    cp_async_wait_all();
    __syncthreads();

    for (int gi = 0; gi < d.ngates; ++gi) {
        const StageGate &G = d.gates[gi];
        const MatR<R> m = to_matr<R>(G.m);
        if (G.diag) {
            for (int e = tid; e < size; e += T) {
                if ((e & G.cmask) == G.cmask) {
                    C v = sm[e];
                    sm[e] = (e & G.tbit) ? cmul(m.m11, v) : cmul(m.m00, v);
                }
            }
        } else {
            const int npairs = size >> G.npos;
            for (int k = tid; k < npairs; k += T) {
                int i0 = k;
                for (int p = 0; p < G.npos; ++p) {
                    int q = G.pos[p];
                    i0 = ((i0 >> q) << (q + 1)) | (i0 & ((1 << q) - 1));
                }
                i0 |= G.cmask;
                int i1 = i0 | G.tbit;
                C a = sm[i0], b = sm[i1];
                apply2<R>(m, a, b);
                sm[i0] = a;
                sm[i1] = b;
            }
        }
        __syncthreads();
    }

    typedef typename CT<R>::vec V;
    for (int e = tid * EPV; e < size; e += T * EPV) {
        idx_t g = tile_offset<R>(d, tile_base, e);
        *(V *)&s[g] = *(const V *)&sm[e];
    }
}

// ------------------------------------------------------------ register-resident stage

// Runs a stage program on the staged tile sm.  Registers hold the register
// arithmetic's type (FP32 complex for complex64, double-float for
// complex128): the first register load converts from the tile, later
// transposes move that type through shared memory unchanged.  Leaves the
// registers and their slots (P0, q) for the caller's final store.
template <class R, int RL, int TL>
__device__ __forceinline__ void run_program(typename CT<R>::type *sm, const RegOp<R> *sops,
                                            const SetSlots *sset, int nops, unsigned tid,
                                            typename RegArith<R>::T (&a)[1 << RL], unsigned &P0,
                                            unsigned (&q)[RL]) {
    typedef RegArith<R> RA;
    typedef typename RA::T RT;
    constexpr int NR = 1 << RL;
    RT *smr = (RT *)sm;
    unsigned e0 = 0;
    for (int oi = 0; oi < nops; ++oi) {
        const RegOp<R> o = sops[oi];
        if (o.kind == kOpTranspose) {
            if (oi > 0) {
                __syncthreads();
#pragma unroll
                for (int j = 0; j < NR; ++j) smr[reg_slot<RL>(P0, q, j)] = a[j];
                __syncthreads();
            }
            const SetSlots &ss = sset[o.reg];
            P0 = (unsigned)ss.lo[tid & 31u] ^ (unsigned)ss.hi[tid >> 5];
            e0 = Swz<R>::f(P0);  // the swizzle is an involution
#pragma unroll
            for (int k = 0; k < RL; ++k) q[k] = ss.q[k];
            if (oi == 0) {
#pragma unroll
                for (int j = 0; j < NR; ++j) a[j] = RA::from_tile(sm[reg_slot<RL>(P0, q, j)]);
            } else {
#pragma unroll
                for (int j = 0; j < NR; ++j) a[j] = smr[reg_slot<RL>(P0, q, j)];
            }
            continue;
        }
        if ((e0 & o.tmask) != o.tmask) continue;
        if (o.kind == kOpGate) {
            const Mat2C<RT> mm = {RA::entry(o.m, 0), RA::entry(o.m, 1), RA::entry(o.m, 2),
                                  RA::entry(o.m, 3)};
            QG_REG_DISPATCH(reg_gate_c, o.reg, a, mm, (unsigned)o.jmask);
        } else if (o.kind == kOpSwapX) {
            QG_REG_DISPATCH(reg_swap, o.reg, a, (unsigned)o.jmask);
        } else if (o.kind == kOpDiagReg) {
            const RT d0 = RA::entry(o.m, 0), d1 = RA::entry(o.m, 3);
            QG_REG_DISPATCH(reg_diag, o.reg, a, d0, d1, (unsigned)o.jmask);
        } else {  // kOpDiagThread
            const RT ph = (e0 & o.tbit) ? RA::entry(o.m, 3) : RA::entry(o.m, 0);
#pragma unroll
            for (int j = 0; j < NR; ++j)
                if ((j & o.jmask) == o.jmask) a[j] = cmul(ph, a[j]);
        }
    }
}

// One CTA per tile of 2^m amplitudes, 2^(m-rl) threads, 2^rl amplitudes per
// thread.  The stage program (ops, register sets, global offsets) is first
// copied from the kernel parameters to shared memory, so that every thread
// reads it with broadcast vector loads instead of per-field constant-bank
// loads.  Load (cp.async, coalesced, swizzled) -> run the program (register
// gates, diagonal phases, shared-memory transposes) -> store.
template <class R, int RL, int TL>
__global__ void __launch_bounds__(1 << TL)
k_rstage(typename CT<R>::type *__restrict__ s, const __grid_constant__ RStageDesc<R> d) {
    typedef typename CT<R>::type C;
    typedef RegOp<R> Op;
    constexpr int NR = 1 << RL;
    constexpr int t = TL;                 // thread lanes (tile lanes 0..t-1)
    constexpr int m = RL + TL;            // tile lanes
    constexpr unsigned T = 1u << TL;
    extern __shared__ __align__(16) unsigned char smraw[];
    C *sm = (C *)smraw;
    Op *sops = (Op *)(smraw + ((size_t)sizeof(C) << m));
    long long *sdep = (long long *)(sops + d.nops);
    SetSlots *sset = (SetSlots *)(sdep + NR);
    const unsigned tid = threadIdx.x;

    {
        const int4 *src = (const int4 *)d.ops;
        int4 *dst = (int4 *)sops;
        const int nvec = (int)(d.nops * sizeof(Op) / sizeof(int4));
        for (int i = tid; i < nvec; i += T) dst[i] = src[i];
        if (tid < (unsigned)NR) sdep[tid] = d.dep_hi[tid];
        copy_sets(sset, d.sets, d.nsets, tid, T);
    }
    const idx_t base = insert_zeros((idx_t)blockIdx.x, d.ins_pos, d.nins);
    // Global offset of tile element tid (tile lanes 0..t-1); the offsets of
    // the register-index parts (i << t) are disjoint from it, so element
    // (tid, i) lives at gp + dep_hi[i].
    const int lr = d.lowrun < t ? d.lowrun : t;
    idx_t dt = (idx_t)(tid & ((1u << lr) - 1u));
    for (int b = lr; b < t; ++b)
        if (tid & (1u << b)) dt |= 1LL << d.hi_pos[b - d.lowrun];
    C *const gp = s + (base | dt);
    const unsigned pt = Swz<R>::f(tid);
    __syncthreads();

#pragma unroll
    for (int i = 0; i < NR; ++i)
        cp_async_elem(&sm[pt ^ Swz<R>::f((unsigned)i << t)], gp + sdep[i]);
    asm volatile("cp.async.wait_all;\n" ::: "memory");
    __syncthreads();

    typename RegArith<R>::T a[NR];
    unsigned P0 = 0;
    unsigned q[RL];
#pragma unroll
    for (int k = 0; k < RL; ++k) q[k] = 0;
    run_program<R, RL, TL>(sm, sops, sset, d.nops, tid, a, P0, q);

    __syncthreads();
#pragma unroll
    for (int j = 0; j < NR; ++j) sm[reg_slot<RL>(P0, q, j)] = RegArith<R>::to_tile(a[j]);
    __syncthreads();
#pragma unroll
    for (int i = 0; i < NR; ++i) gp[sdep[i]] = sm[pt ^ Swz<R>::f((unsigned)i << t)];
}

// Persistent, double-buffered variant: a grid of (SMs x resident CTAs)
// walks the tiles; each CTA copies the stage program to shared memory once,
// then prefetches tile k+1 (cp.async into the other buffer) while it runs the
// program on tile k and writes tile k back, so HBM stays busy during the
// arithmetic.
template <class R, int RL, int TL>
__global__ void __launch_bounds__(1 << TL)
k_rstage_pipe(typename CT<R>::type *__restrict__ s, const __grid_constant__ RStageDesc<R> d,
              long long tiles) {
    typedef typename CT<R>::type C;
    typedef RegOp<R> Op;
    constexpr int NR = 1 << RL;
    constexpr int t = TL;
    constexpr int m = RL + TL;
    constexpr unsigned T = 1u << TL;
    extern __shared__ __align__(16) unsigned char smraw[];
    C *buf0 = (C *)smraw;
    C *buf1 = buf0 + (1 << m);
    Op *sops = (Op *)(smraw + ((size_t)sizeof(C) << (m + 1)));
    long long *sdep = (long long *)(sops + d.nops);
    SetSlots *sset = (SetSlots *)(sdep + NR);
    const unsigned tid = threadIdx.x;

    {
        const int4 *src = (const int4 *)d.ops;
        int4 *dst = (int4 *)sops;
        const int nvec = (int)(d.nops * sizeof(Op) / sizeof(int4));
        for (int i = tid; i < nvec; i += T) dst[i] = src[i];
        if (tid < (unsigned)NR) sdep[tid] = d.dep_hi[tid];
        copy_sets(sset, d.sets, d.nsets, tid, T);
    }
    const int lr = d.lowrun < t ? d.lowrun : t;
    idx_t dt = (idx_t)(tid & ((1u << lr) - 1u));
    for (int b = lr; b < t; ++b)
        if (tid & (1u << b)) dt |= 1LL << d.hi_pos[b - d.lowrun];
    const unsigned pt = Swz<R>::f(tid);
    __syncthreads();

    const long long G = gridDim.x;
    long long tile = blockIdx.x;
    if (tile >= tiles) return;
    auto issue = [&](long long tl, C *buf) {
        C *gp = s + (insert_zeros((idx_t)tl, d.ins_pos, d.nins) | dt);
#pragma unroll
        for (int i = 0; i < NR; ++i)
            cp_async_elem(&buf[pt ^ Swz<R>::f((unsigned)i << t)], gp + sdep[i]);
        asm volatile("cp.async.commit_group;\n" ::: "memory");
    };
    issue(tile, buf0);
    const int nops = d.nops;
    for (int k = 0; tile < tiles; ++k, tile += G) {
        C *sm = (k & 1) ? buf1 : buf0;
        const long long next = tile + G;
        if (next < tiles) {
            issue(next, (k & 1) ? buf0 : buf1);
            asm volatile("cp.async.wait_group 1;\n" ::: "memory");
        } else {
            asm volatile("cp.async.wait_group 0;\n" ::: "memory");
        }
        __syncthreads();

        typename RegArith<R>::T a[NR];
        unsigned P0 = 0;
        unsigned q[RL];
#pragma unroll
        for (int kk = 0; kk < RL; ++kk) q[kk] = 0;
        run_program<R, RL, TL>(sm, sops, sset, nops, tid, a, P0, q);
        __syncthreads();
#pragma unroll
        for (int j = 0; j < NR; ++j) sm[reg_slot<RL>(P0, q, j)] = RegArith<R>::to_tile(a[j]);
        __syncthreads();
        C *gp = s + (insert_zeros((idx_t)tile, d.ins_pos, d.nins) | dt);
#pragma unroll
        for (int i = 0; i < NR; ++i) gp[sdep[i]] = sm[pt ^ Swz<R>::f((unsigned)i << t)];
        __syncthreads();  // the buffer is refilled two iterations later
    }
}

template <class R>
void rstage_dispatch(void *state, const RStageDesc<R> &d, cudaStream_t stream, bool pipelined) {
    typedef typename CT<R>::type C;
    const size_t prog = (size_t)d.nops * sizeof(RegOp<R>) + sizeof(long long) * (1 << d.rl) +
                        sizeof(SetSlots) * (size_t)d.nsets;
    const size_t tile_bytes = ((size_t)1 << d.m) * sizeof(C);
    idx_t tiles = (idx_t)1 << (d.n - d.m);
    int threads = 1 << (d.m - d.rl);
    if (threads < 32 || threads > (d.rl >= 5 ? 256 : 512))
        fail(2, "register stage: bad tile shape m=%d rl=%d", d.m, d.rl);
    // Pipelining needs two tiles per CTA and several tiles per CTA to pay off.
    const size_t pipe_smem = 2 * tile_bytes + prog;
    if (pipelined && (pipe_smem > 227 * 1024 || tiles < 2 * 152)) pipelined = false;
    auto launch = [&](auto kern) {
        const size_t smem = tile_bytes + prog;
        QG_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        kern<<<(unsigned)tiles, threads, smem, stream>>>((C *)state, d);
    };
    auto launch_pipe = [&](auto kern) {
        QG_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)pipe_smem));
        int per_sm = 0, sms = 0, dev = 0;
        QG_CUDA(cudaGetDevice(&dev));
        QG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        QG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, threads, pipe_smem));
        if (per_sm < 1) per_sm = 1;
        long long grid = (long long)sms * per_sm;
        if (grid > tiles) grid = tiles;
        kern<<<(unsigned)grid, threads, pipe_smem, stream>>>((C *)state, d, (long long)tiles);
    };
    const int tl = d.m - d.rl;
#define QG_RS_CASE(RL_, TL_)                                        \
    if (d.rl == RL_ && tl == TL_) {                                 \
        if (pipelined)                                              \
            launch_pipe(k_rstage_pipe<R, RL_, TL_>);                \
        else                                                        \
            launch(k_rstage<R, RL_, TL_>);                          \
        QG_CUDA(cudaGetLastError());                                \
        return;                                                     \
    }
    QG_RS_CASE(3, 5) QG_RS_CASE(3, 6) QG_RS_CASE(3, 7) QG_RS_CASE(3, 8) QG_RS_CASE(3, 9)
    QG_RS_CASE(4, 5) QG_RS_CASE(4, 6) QG_RS_CASE(4, 7) QG_RS_CASE(4, 8) QG_RS_CASE(4, 9)
    if constexpr (sizeof(R) == 4) {
        QG_RS_CASE(5, 5) QG_RS_CASE(5, 6) QG_RS_CASE(5, 7) QG_RS_CASE(5, 8)
    }
#undef QG_RS_CASE
    fail(2, "register stage: unsupported shape m=%d rl=%d", d.m, d.rl);
}

}  // namespace

void launch_stage(int prec, void *state, const StageDesc &d, cudaStream_t stream) {
    size_t cs = complex_size(prec);
    size_t smem = ((size_t)1 << d.m) * cs;
    idx_t tiles = (idx_t)1 << (d.n - d.m);
    int threads = d.m >= 11 ? 512 : (d.m >= 9 ? 256 : 128);
    if (prec == kFP32) {
        QG_CUDA(cudaFuncSetAttribute(k_stage<float>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)smem));
        k_stage<float><<<(unsigned)tiles, threads, smem, stream>>>((float2 *)state, d);
    } else {
        QG_CUDA(cudaFuncSetAttribute(k_stage<double>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)smem));
        k_stage<double><<<(unsigned)tiles, threads, smem, stream>>>((double2 *)state, d);
    }
    QG_CUDA(cudaGetLastError());
}

void launch_rstage_f32(void *state, const RStageDesc<float> &d, cudaStream_t stream,
                       bool pipelined) {
    rstage_dispatch<float>(state, d, stream, pipelined);
}

void launch_rstage_f64(void *state, const RStageDesc<double> &d, cudaStream_t stream,
                       bool pipelined) {
    rstage_dispatch<double>(state, d, stream, pipelined);
}

}  // namespace qg
