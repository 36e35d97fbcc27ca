// Batched execution of many small circuits of uneven qubit counts (complex64).
//
// Circuits of up to 13 qubits never touch HBM with their state: one CTA
// holds the whole 2^n-amplitude state in shared memory / registers, starts
// from |0...0>, runs the circuit's register program (read from global memory,
// L1-resident) and reduces sum_i <Z_i> in FP64.  Larger circuits live in a
// packed arena and advance one fused stage per round: a round is one launch
// over every (circuit, tile) work item of that round.  The host records the
// whole sequence once as a CUDA graph.
//
// The reference runs circuits one at a time, one Python call chain per gate
// (qgate/simulator/simulator.py:57-83, qgate/simulator/rop_executor.py:28-53).
#include <algorithm>

#include "qg_regstage.cuh"

namespace qg {

namespace {

using namespace rs;

typedef float R;
typedef float2 C;

// Runs ops[0..nops) on the register-resident tile; `sets` are the slot
// tables of the program's register sets.  On return, a[] holds the thread's
// amplitudes for the last register set (e0, P0, q; lanebit[k] = its lanes).
// `active` = false: the thread only takes part in the barriers (a CTA larger
// than the circuit's thread count).
template <int RL>
__device__ __forceinline__ void run_program(C (&a)[1 << RL], C *sm, const RegOp<R> *ops, int nops,
                                            const SetSlots *sets, unsigned tid, unsigned &e0,
                                            unsigned &P0, unsigned (&q)[RL],
                                            unsigned (&lanebit)[RL], bool active = true) {
    constexpr int NR = 1 << RL;
    for (int oi = 0; oi < nops; ++oi) {
        const RegOp<R> o = ops[oi];
        if (o.kind == kOpTranspose) {
            if (oi > 0) {
                __syncthreads();
                if (active) {
#pragma unroll
                    for (int j = 0; j < NR; ++j) sm[reg_slot<RL>(P0, q, j)] = a[j];
                }
                __syncthreads();
            }
            if (!active) continue;
            const SetSlots &ss = sets[o.reg];
            P0 = (unsigned)ss.lo[tid & 31u] ^ (unsigned)ss.hi[tid >> 5];
            e0 = Swz<R>::f(P0);
#pragma unroll
            for (int k = 0; k < RL; ++k) {
                q[k] = ss.q[k];
                lanebit[k] = Swz<R>::f(q[k]);
            }
#pragma unroll
            for (int j = 0; j < NR; ++j) a[j] = sm[reg_slot<RL>(P0, q, j)];
            continue;
        }
        if (!active || (e0 & o.tmask) != o.tmask) continue;
        if (o.kind == kOpGate) {
            MatR<R> mm;
            mm.m00 = cmk<C>(o.m[0], o.m[1]);
            mm.m01 = cmk<C>(o.m[2], o.m[3]);
            mm.m10 = cmk<C>(o.m[4], o.m[5]);
            mm.m11 = cmk<C>(o.m[6], o.m[7]);
            QG_REG_DISPATCH(reg_gate, o.reg, a, mm, (unsigned)o.jmask);
        } else if (o.kind == kOpSwapX) {
            QG_REG_DISPATCH(reg_swap, o.reg, a, (unsigned)o.jmask);
        } else if (o.kind == kOpDiagReg) {
            C d0 = cmk<C>(o.m[0], o.m[1]), d1 = cmk<C>(o.m[6], o.m[7]);
            QG_REG_DISPATCH(reg_diag, o.reg, a, d0, d1, (unsigned)o.jmask);
        } else {
            C ph = (e0 & o.tbit) ? cmk<C>(o.m[6], o.m[7]) : cmk<C>(o.m[0], o.m[1]);
#pragma unroll
            for (int j = 0; j < NR; ++j)
                if ((j & o.jmask) == o.jmask) a[j] = cmul(ph, a[j]);
        }
    }
}

__device__ __forceinline__ double block_sum_d(double v, double *ws) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane == 0) ws[w] = v;
    __syncthreads();
    double r = 0.;
    if (threadIdx.x == 0)
        for (int i = 0; i < (int)((blockDim.x + 31) >> 5); ++i) r += ws[i];
    return r;  // thread 0
}

template <int RL>
__global__ void __launch_bounds__(512)
k_batch_resident(int n, const ResidentCircuit *__restrict__ circuits,
                 const RegOp<R> *__restrict__ ops_all, const SetSlots *__restrict__ sets_all,
                 double *__restrict__ out) {
    constexpr int NR = 1 << RL;
    extern __shared__ __align__(16) unsigned char smraw[];
    __shared__ double ws[16];
    C *sm = (C *)smraw;
    const ResidentCircuit c = circuits[blockIdx.x];
    const unsigned tid = threadIdx.x, T = blockDim.x;
    const int size = 1 << n;
    for (int e = tid; e < size; e += T) sm[e] = make_float2(0.f, 0.f);
    __syncthreads();
    if (tid == 0) sm[0] = make_float2(1.f, 0.f);  // slot of element 0 is 0
    __syncthreads();
    C a[NR];
    unsigned e0 = 0, P0 = 0, q[RL], lanebit[RL];
#pragma unroll
    for (int k = 0; k < RL; ++k) q[k] = lanebit[k] = 0;
    run_program<RL>(a, sm, ops_all + c.ops_off, c.nops, sets_all + c.sets_off, tid, e0, P0, q,
                    lanebit);
    // sum_i <Z_i> = sum_b |psi_b|^2 (n - 2 popcount(b))
    float part = 0.f;
#pragma unroll
    for (int j = 0; j < NR; ++j) {
        unsigned e = e0;
#pragma unroll
        for (int k = 0; k < RL; ++k)
            if (j & (1 << k)) e |= lanebit[k];
        part += (a[j].x * a[j].x + a[j].y * a[j].y) * (float)(n - 2 * __popc(e));
    }
    double tot = block_sum_d((double)part, ws);
    if (tid == 0) out[c.out_index] = tot;
}

// One CTA per (stage, tile) work item of a round; tile of 2^12 amplitudes,
// 16 per thread in registers (256 threads).
__global__ void __launch_bounds__(256)
k_batch_stage(const BatchStage *__restrict__ stages, const int2 *__restrict__ items,
              const RegOp<R> *__restrict__ ops_all, const SetSlots *__restrict__ sets_all,
              C *__restrict__ arena) {
    constexpr int RL = 4, NR = 16;
    extern __shared__ __align__(16) unsigned char smraw[];
    C *sm = (C *)smraw;
    const int2 it = items[blockIdx.x];
    const BatchStage &st = stages[it.x];
    C *s = arena + st.state_off;
    const int t = st.m - RL;
    const unsigned tid = threadIdx.x;
    const idx_t base = insert_zeros((idx_t)it.y, st.ins_pos, st.nins);
    const int lr = st.lowrun < t ? st.lowrun : t;
    idx_t dt = (idx_t)(tid & ((1u << lr) - 1u));
    for (int b = lr; b < t; ++b)
        if (tid & (1u << b)) dt |= 1LL << st.hi_pos[b - st.lowrun];
    const unsigned pt = Swz<R>::f(tid);
#pragma unroll
    for (int i = 0; i < NR; ++i) {
        unsigned slot = pt ^ Swz<R>::f((unsigned)i << t);
        cp_async_elem(&sm[slot], &s[base | dt | st.dep_hi[i]]);
    }
    asm volatile("cp.async.wait_all;\n" ::: "memory");
    __syncthreads();
    C a[NR];
    unsigned e0 = 0, P0 = 0, q[RL], lanebit[RL];
#pragma unroll
    for (int k = 0; k < RL; ++k) q[k] = lanebit[k] = 0;
    run_program<RL>(a, sm, ops_all + st.ops_off, st.nops, sets_all + st.sets_off, tid, e0, P0,
                    q, lanebit);
    __syncthreads();
#pragma unroll
    for (int j = 0; j < NR; ++j) sm[reg_slot<RL>(P0, q, j)] = a[j];
    __syncthreads();
#pragma unroll
    for (int i = 0; i < NR; ++i) {
        unsigned slot = pt ^ Swz<R>::f((unsigned)i << t);
        s[base | dt | st.dep_hi[i]] = sm[slot];
    }
}

constexpr int kSumzChunks = 16;

__global__ void __launch_bounds__(256)
k_batch_sumz(const C *__restrict__ arena, const long long *__restrict__ off,
             const int *__restrict__ nq, double *__restrict__ partials) {
    __shared__ double ws[8];
    const int c = blockIdx.y, n = nq[c];
    const C *s = arena + off[c];
    const idx_t N = (idx_t)1 << n;
    const idx_t chunk = N / kSumzChunks;
    const idx_t b0 = (idx_t)blockIdx.x * chunk;
    double acc = 0.;
    for (idx_t b = b0 + threadIdx.x; b < b0 + chunk; b += 4 * blockDim.x) {
        float part = 0.f;
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            idx_t bb = b + (idx_t)u * blockDim.x;
            if (bb < b0 + chunk) {
                C v = s[bb];
                part += (v.x * v.x + v.y * v.y) * (float)(n - 2 * __popcll((unsigned long long)bb));
            }
        }
        acc += (double)part;
    }
    double tot = block_sum_d(acc, ws);
    if (threadIdx.x == 0) partials[(idx_t)c * kSumzChunks + blockIdx.x] = tot;
}

__global__ void k_batch_sumz_final(const double *__restrict__ partials, const int *__restrict__ idx,
                                   int count, double *__restrict__ out) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= count) return;
    double v = 0.;
    for (int k = 0; k < kSumzChunks; ++k) v += partials[(idx_t)c * kSumzChunks + k];
    out[idx[c]] = v;
}

__global__ void k_batch_init(C *arena, const long long *__restrict__ off, int count) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c < count) arena[off[c]] = make_float2(1.f, 0.f);
}

// ---------------------------------------------------------------- one launch

constexpr unsigned kBatchThreads = 256;
// a 12-qubit resident state, or two tiles (the one running, the next
// loading) and the running stage's program: its ops and register sets, read
// by every op of every tile of an item (from global memory they would come
// from L2 whenever the tile loads have pushed them out of L1)
constexpr int kBatchProgOps = 192, kBatchProgSets = 64;
constexpr size_t kBatchTileBytes = sizeof(C) << 13;
constexpr size_t kBatchSmem = kBatchTileBytes + kBatchProgOps * sizeof(RegOp<R>) +
                              kBatchProgSets * sizeof(SetSlots);
constexpr long long kBatchWaitTries = 1LL << 22;  // x ~100 ns sleeps: ~0.5 s

// Waits (thread 0) until counter >= need; bounded: a wait that gives up
// sets bit 0 of *status and lets the item run on whatever is there (the host
// reports the failure).
__device__ __forceinline__ void wait_count(const int *counter, int need, unsigned *status) {
    long long tries = 0;
    while (*(volatile const int *)counter < need) {
        if (++tries > kBatchWaitTries) {
            atomicOr(status, 1u);
            break;
        }
        __nanosleep(100);
    }
    __threadfence();
}

template <int RL>
__device__ __forceinline__ double resident_sum_z(const ResidentCircuit &c, C *sm,
                                                 const RegOp<R> *ops_all,
                                                 const SetSlots *sets_all, double *ws) {
    constexpr int NR = 1 << RL;
    const unsigned tid = threadIdx.x;
    const int n = c.n;
    const bool active = tid < (1u << (n - RL));
    for (int e = tid; e < (1 << n); e += kBatchThreads) sm[e] = make_float2(0.f, 0.f);
    __syncthreads();
    if (tid == 0) sm[0] = make_float2(1.f, 0.f);  // slot of element 0 is 0
    __syncthreads();
    C a[NR];
    unsigned e0 = 0, P0 = 0, q[RL], lanebit[RL];
#pragma unroll
    for (int k = 0; k < RL; ++k) q[k] = lanebit[k] = 0;
    run_program<RL>(a, sm, ops_all + c.ops_off, c.nops, sets_all + c.sets_off, tid, e0, P0, q,
                    lanebit, active);
    float part = 0.f;
    if (active) {
#pragma unroll
        for (int j = 0; j < NR; ++j) {
            unsigned e = e0;
#pragma unroll
            for (int k = 0; k < RL; ++k)
                if (j & (1 << k)) e |= lanebit[k];
            part += (a[j].x * a[j].x + a[j].y * a[j].y) * (float)(n - 2 * __popc(e));
        }
    }
    return block_sum_d((double)part, ws);
}

// The bits of k placed, in order, at the set bits of mask.
__device__ __forceinline__ int deposit(int k, unsigned mask) {
    unsigned r = 0;
    for (unsigned b = 1; mask; b <<= 1) {
        const unsigned low = mask & (0u - mask);
        if ((unsigned)k & b) r |= low;
        mask ^= low;
    }
    return (int)r;
}

// The whole batch in one persistent launch.  CTAs take work items in queue
// order (an atomic head): a whole small circuit (resident in shared memory),
// a run of tiles of one fused stage of a large circuit (in the arena), or one
// chunk of a large circuit's final sum_i <Z_i>.  An item that needs earlier
// items of its circuit waits (bounded) on the circuit's completion counter;
// every such item comes later in the queue than all it waits for, so the
// launch always progresses (the dequeue comment below has the argument).  Round-0 tiles start from |0...0>
// (nothing is read).  The last chunk of a circuit's sum adds the partials in
// order and writes the result.
__global__ void __launch_bounds__(kBatchThreads, 2)
k_batch_persistent(const BatchItem *__restrict__ items, int n_items, int *head, int *done,
                   int *sdone, unsigned *status, const ResidentCircuit *__restrict__ res,
                   const BatchStage *__restrict__ stages, const RegOp<R> *__restrict__ ops_all,
                   const SetSlots *__restrict__ sets_all, C *__restrict__ arena,
                   const BigCircuit *__restrict__ big, double *__restrict__ partials,
                   double *__restrict__ out) {
    constexpr int RL = 4, NR = 16;
    extern __shared__ __align__(16) unsigned char smraw[];
    __shared__ double ws[kBatchThreads / 32];
    __shared__ int item_sh;
    __shared__ int last_sh;
    C *sm = (C *)smraw;
    const unsigned tid = threadIdx.x;
    // The next item is taken while the current one runs (thread 0 reads the
    // atomic's result only at the end), which hides the dequeue latency.  A
    // reserved but unstarted item never blocks progress: the lowest-indexed
    // unfinished item that any CTA holds is always some CTA's current item,
    // and everything it waits for comes earlier in the queue, so is finished.
    if (tid == 0) item_sh = atomicAdd(head, 1);
    __syncthreads();
    for (;;) {
        const int it = item_sh;
        __syncthreads();
        if (it >= n_items) break;
        int next = 0;
        if (tid == 0) next = atomicAdd(head, 1);
        const BatchItem w = items[it];
        if (w.dep >= 0) {
            if (tid == 0) wait_count(&done[w.dep], w.need, status);
            __syncthreads();
        }
        if (w.kind == 0) {
            const ResidentCircuit c = res[w.index];
            double tot;
            if (c.rl == 3)
                tot = resident_sum_z<3>(c, sm, ops_all, sets_all, ws);
            else
                tot = resident_sum_z<4>(c, sm, ops_all, sets_all, ws);
            if (tid == 0) out[c.out_index] = tot;
            __syncthreads();
        } else if (w.kind == 1) {
            // tiles [w.tile, w.tile + w.ntiles) of one stage, the next tile's
            // loads in flight (into the other half of shared memory) while
            // the current one runs
            const BatchStage &st = stages[w.index];
            C *s = arena + st.state_off;
            const int t = st.m - RL;
            const int lr = st.lowrun < t ? st.lowrun : t;
            idx_t dt = (idx_t)(tid & ((1u << lr) - 1u));
            for (int b = lr; b < t; ++b)
                if (tid & (1u << b)) dt |= 1LL << st.hi_pos[b - st.lowrun];
            const unsigned pt = Swz<R>::f(tid);
            // the stage's program into shared memory (when it fits)
            const RegOp<R> *prog_ops = ops_all + st.ops_off;
            const SetSlots *prog_sets = sets_all + st.sets_off;
            if (st.nops <= kBatchProgOps && st.nsets <= kBatchProgSets) {
                RegOp<R> *sops = (RegOp<R> *)(smraw + kBatchTileBytes);
                SetSlots *ssets = (SetSlots *)(sops + kBatchProgOps);
                const int4 *go = (const int4 *)prog_ops;
                int4 *so = (int4 *)sops;
                const int n16 = st.nops * (int)(sizeof(RegOp<R>) / 16);
                for (int i = (int)tid; i < n16; i += (int)kBatchThreads) so[i] = go[i];
                const unsigned *gs = (const unsigned *)prog_sets;
                unsigned *ss = (unsigned *)ssets;
                const int n4 = st.nsets * (int)(sizeof(SetSlots) / 4);
                for (int i = (int)tid; i < n4; i += (int)kBatchThreads) ss[i] = gs[i];
                prog_ops = sops;
                prog_sets = ssets;
                // made visible to every thread by the barrier before the first op
            }
            auto load_tile = [&](C *buf, int tile) {
                const idx_t base = insert_zeros((idx_t)tile, st.ins_pos, st.nins);
#pragma unroll
                for (int i = 0; i < NR; ++i)
                    cp_async_elem(&buf[pt ^ Swz<R>::f((unsigned)i << t)],
                                  &s[base | dt | st.dep_hi[i]]);
                asm volatile("cp.async.commit_group;\n" ::: "memory");
            };
            if (w.round > 0) load_tile(sm, deposit(w.tile, w.live));
            for (int j = 0; j < w.ntiles; ++j) {
                C *cur = sm + ((j & 1) << 12);
                const int tile = deposit(w.tile + j, w.live);
                if (w.round == 0 && tile != 0) {
                    // round 0 from |0...0>: every tile but tile 0 stays zero
                    const idx_t base = insert_zeros((idx_t)tile, st.ins_pos, st.nins);
#pragma unroll
                    for (int i = 0; i < NR; ++i)
                        __stcg(&s[base | dt | st.dep_hi[i]], make_float2(0.f, 0.f));
                    continue;
                }
                if (w.round == 0) {
                    // |0...0>: only element 0 of tile 0 is 1 (its slot is 0)
#pragma unroll
                    for (int i = 0; i < NR; ++i)
                        cur[pt ^ Swz<R>::f((unsigned)i << t)] = make_float2(0.f, 0.f);
                    __syncthreads();
                    if (tile == 0 && tid == 0) cur[0] = make_float2(1.f, 0.f);
                } else if (j + 1 < w.ntiles) {
                    load_tile(sm + (((j + 1) & 1) << 12), deposit(w.tile + j + 1, w.live));
                    asm volatile("cp.async.wait_group 1;\n" ::: "memory");
                } else {
                    asm volatile("cp.async.wait_group 0;\n" ::: "memory");
                }
                __syncthreads();
                C a[NR];
                unsigned e0 = 0, P0 = 0, q[RL], lanebit[RL];
#pragma unroll
                for (int k = 0; k < RL; ++k) q[k] = lanebit[k] = 0;
                run_program<RL>(a, cur, prog_ops, st.nops, prog_sets, tid, e0, P0, q, lanebit);
                __syncthreads();
#pragma unroll
                for (int i = 0; i < NR; ++i) cur[reg_slot<RL>(P0, q, i)] = a[i];
                __syncthreads();
                const idx_t base = insert_zeros((idx_t)tile, st.ins_pos, st.nins);
#pragma unroll
                for (int i = 0; i < NR; ++i)
                    __stcg(&s[base | dt | st.dep_hi[i]], cur[pt ^ Swz<R>::f((unsigned)i << t)]);
                // the half just read is the target of the loads issued next
                __syncthreads();
            }
            // Publish the tiles: the barrier above orders the CTA's stores
            // before thread 0's fence, whose release covers them.
            if (tid == 0) {
                __threadfence();
                atomicAdd(&done[w.dep_done], w.ntiles);
            }
        } else {
            // one chunk of sum_i <Z_i> of a large circuit
            const BigCircuit b = big[w.index];
            const C *s = arena + b.off;
            const idx_t chunk = ((idx_t)1 << b.n) / kSumzChunks;
            const idx_t b0 = (idx_t)w.tile * chunk;
            double acc = 0.;
            for (idx_t x = b0 + tid; x < b0 + chunk; x += 4 * kBatchThreads) {
                float part = 0.f;
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const idx_t xx = x + (idx_t)u * kBatchThreads;
                    if (xx < b0 + chunk) {
                        const C v = __ldcg(&s[xx]);
                        part += (v.x * v.x + v.y * v.y) *
                                (float)(b.n - 2 * __popcll((unsigned long long)xx));
                    }
                }
                acc += (double)part;
            }
            const double tot = block_sum_d(acc, ws);
            if (tid == 0) {
                partials[(idx_t)w.index * kSumzChunks + w.tile] = tot;
                __threadfence();
                last_sh = atomicAdd(&sdone[w.index], 1) == kSumzChunks - 1;
            }
            __syncthreads();
            if (last_sh && tid == 0) {
                __threadfence();
                double v = 0.;
                for (int k = 0; k < kSumzChunks; ++k)
                    v += *(volatile const double *)&partials[(idx_t)w.index * kSumzChunks + k];
                out[b.out_index] = v;
            }
            __syncthreads();
        }
        if (tid == 0) item_sh = next;
        __syncthreads();
    }
}

}  // namespace

void launch_batch_persistent(const BatchItem *d_items, int n_items, int *d_counters,
                             int n_big, unsigned *d_status, const ResidentCircuit *d_res,
                             const BatchStage *d_stages, const RegOp<float> *d_ops,
                             const SetSlots *d_sets, float2 *arena, const BigCircuit *d_big,
                             double *d_partials, double *d_out, int ctas, cudaStream_t stream) {
    if (n_items <= 0) return;
    // counters: [0] the queue head, [1, 1 + n_big) stage items done per
    // circuit, then sum chunks done per circuit
    int *head = d_counters, *done = d_counters + 1, *sdone = d_counters + 1 + n_big;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)ctas);
    cfg.blockDim = dim3(kBatchThreads);
    cfg.dynamicSmemBytes = kBatchSmem;
    cfg.stream = stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;  // its blocks wait on one another
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    QG_CUDA(cudaLaunchKernelEx(&cfg, k_batch_persistent, d_items, n_items, head, done, sdone,
                               d_status, d_res, d_stages, d_ops, d_sets, (C *)arena, d_big,
                               d_partials, d_out));
}

int batch_persistent_ctas() {
    int dev = 0, sms = 0, per_sm = 0;
    QG_CUDA(cudaGetDevice(&dev));
    QG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    QG_CUDA(cudaFuncSetAttribute(k_batch_persistent, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)kBatchSmem));
    QG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_batch_persistent,
                                                          (int)kBatchThreads, kBatchSmem));
    return std::max(1, per_sm) * sms;
}

void launch_batch_resident(int n, int rl, const ResidentCircuit *d_circuits, int count,
                           const RegOp<float> *d_ops, const SetSlots *d_sets, double *d_out,
                           cudaStream_t stream) {
    if (count <= 0) return;
    size_t smem = sizeof(C) << n;
    int threads = 1 << (n - rl);
    auto launch = [&](auto kern) {
        kern<<<count, threads, smem, stream>>>(n, d_circuits, d_ops, d_sets, d_out);
    };
    switch (rl) {
    case 3: launch(k_batch_resident<3>); break;
    case 4: launch(k_batch_resident<4>); break;
    case 5: launch(k_batch_resident<5>); break;
    default: fail(2, "batch: unsupported register lanes %d", rl);
    }
    QG_CUDA(cudaGetLastError());
}

void launch_batch_stage(const BatchStage *d_stages, const int2 *d_items, int n_items,
                        const RegOp<float> *d_ops, const SetSlots *d_sets, float2 *arena,
                        cudaStream_t stream) {
    if (n_items <= 0) return;
    size_t smem = sizeof(C) << 12;
    k_batch_stage<<<n_items, 256, smem, stream>>>(d_stages, d_items, d_ops, d_sets, arena);
    QG_CUDA(cudaGetLastError());
}

size_t batch_sumz_partials(int count) { return (size_t)kSumzChunks * count; }

void launch_batch_sumz(const float2 *arena, const long long *d_off, const int *d_n,
                       const int *d_out_index, int count, double *d_partials, double *d_out,
                       cudaStream_t stream) {
    if (count <= 0) return;
    dim3 grid(kSumzChunks, count);
    k_batch_sumz<<<grid, 256, 0, stream>>>(arena, d_off, d_n, d_partials);
    k_batch_sumz_final<<<(count + 127) / 128, 128, 0, stream>>>(d_partials, d_out_index, count,
                                                                d_out);
    QG_CUDA(cudaGetLastError());
}

// Shared-memory opt-in for every batch kernel; called before a graph capture
// (no attribute changes while capturing).
void batch_prepare() {
    QG_CUDA(cudaFuncSetAttribute(k_batch_resident<3>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)(sizeof(C) << 13)));
    QG_CUDA(cudaFuncSetAttribute(k_batch_resident<4>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)(sizeof(C) << 13)));
    QG_CUDA(cudaFuncSetAttribute(k_batch_resident<5>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)(sizeof(C) << 13)));
    QG_CUDA(cudaFuncSetAttribute(k_batch_stage, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)(sizeof(C) << 12)));
}

void launch_batch_init(float2 *arena, const long long *d_off, int count, cudaStream_t stream) {
    if (count <= 0) return;
    k_batch_init<<<(count + 127) / 128, 128, 0, stream>>>(arena, d_off, count);
    QG_CUDA(cudaGetLastError());
}

}  // namespace qg
