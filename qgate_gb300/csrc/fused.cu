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

namespace qg {

namespace {

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

}  // namespace qg
