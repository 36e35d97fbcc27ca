// Tensor-core stage kernel (complex64): a tile of m = 12 or 13 lanes stays
// on chip while a sequence of ops is applied to it: fused 5-lane blocks, each
// a 32x32 complex unitary, as tcgen05 matrix products (dense ops), and runs of
// diagonal gates as one table of phases multiplied in registers (phase ops:
// each thread multiplies its amplitudes by their entries, found through a
// slot table like the operand slots below; the layout stays).
//
// For a block on tile lanes L[0..4] the tile is a 2^(m-5) x 32 complex matrix
// V (row = the other m-5 lanes, column = the block's amplitude index); the
// block computes V U^T.  In real form that is D[rows x 64] = A[rows x 64]
// B[64 x 64] with A[r][2i + c] = (Re, Im) of V[r][i] and B the real 64x64
// form of U^T: per 128 rows an M=128, N=64, K=64 product, 4 MMAs of K=16 in
// kind::f16 (FP16 operands, FP32 accumulator).
//
// Precision: the state is carried scaled by 2^12 (exact; amplitudes of a
// normalised state are <= 1, so |A| <= 2^12 stays far below the FP16 range
// and typical amplitudes sit in its normal range).  Each operand is split
// into two FP16 parts rounded to nearest, Ah = f16(A), Al = f16(A - Ah),
// so |A - Ah - Al| <= 2^-24 |A| + 2^-25 (subnormal spacing), the same for B,
// and D = Ah Bh + Ah Bl + Al Bh in FP32 (the dropped Al Bl term is <= 2^-24
// relative): about FP32 accuracy per block.  The accumulator rounds toward
// zero at every MMA, so the correction products are issued first and the
// four main-product K-steps last, and the host scales each block's rows by
// the expected shrink of those roundings (tc_compensate).
//
// Data path per block: thread r holds row r of the previous layout in
// registers (64 floats; 32 with two threads per row); it splits each
// amplitude and stores Ah/Al straight
// into the block's canonical 128-byte-swizzled K-major operand layout (B:
// no swizzle, written on the host) - the map from
// (row, register) to operand slot is GF(2)-linear, so it is a precomputed
// slot table (SetSlots), and no separate transpose pass exists.  One thread
// issues the 12 MMAs per 128 rows and commits them to an mbarrier; every
// thread then reads its row of D back from tensor memory (tcgen05.ld
// 32x32b), which is the next block's source layout.  The blocks' B
// operands (Bh, Bl: 16 KB per block) arrive once per CTA by bulk async
// copies (cp.async.bulk) and stay in shared memory.
//
// Every wait is bounded; a wait that gives up sets g_tc_status, later CTAs
// skip their work, and the CTA still frees its tensor memory.
#include <algorithm>
#include <cstdint>

#include "qg_bulk.cuh"
#include "qg_device.cuh"
#include "qg_internal.h"
#include "qg_regstage.cuh"

namespace qg {

__device__ unsigned g_tc_status;

namespace {


// Shared-memory matrix descriptor: start address, leading-dimension byte
// offset (between core matrices along K; unused by swizzled K-major
// layouts), stride-dimension byte offset (between 8-row groups), descriptor
// version 1, layout type (0 = no swizzle, 2 = 128-byte swizzle).
__device__ __forceinline__ uint64_t smem_desc(unsigned saddr, unsigned lbo, unsigned sbo,
                                              unsigned layout = 0) {
    return (uint64_t)((saddr & 0x3FFFFu) >> 4) | ((uint64_t)(lbo >> 4) << 16) |
           ((uint64_t)(sbo >> 4) << 32) | (1ull << 46) | ((uint64_t)layout << 61);
}

// Instruction descriptor of kind::f16: D = F32, A = B = F16, both K-major,
// N = 64, M = 128.
constexpr unsigned kIdescF16 = (1u << 4) | (0u << 7) | (0u << 10) | ((64u >> 3) << 17) |
                               ((128u >> 4) << 24);

__device__ __forceinline__ void mma_f16(unsigned dtmem, uint64_t a, uint64_t b, unsigned acc) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %3, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %4, p;\n\t}\n" ::"r"(dtmem),
        "l"(a), "l"(b), "r"(acc), "r"(kIdescF16)
        : "memory");
}

__device__ __forceinline__ void mma_commit(unsigned bar) {
    asm volatile(
        "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(bar)
        : "memory");
}

__device__ __forceinline__ void tc_fence_before() {
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
}

__device__ __forceinline__ void tmem_ld_x64(unsigned taddr, unsigned (&u)[64]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x64.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31, %32, %33, %34, %35, %36, %37, %38, %39, %40, %41, %42, %43, %44, %45, %46, %47, %48, %49, %50, %51, %52, %53, %54, %55, %56, %57, %58, %59, %60, %61, %62, %63}, [%64];\n"
        : "=r"(u[0]), "=r"(u[1]), "=r"(u[2]), "=r"(u[3]), "=r"(u[4]), "=r"(u[5]), "=r"(u[6]), "=r"(u[7]),
          "=r"(u[8]), "=r"(u[9]), "=r"(u[10]), "=r"(u[11]), "=r"(u[12]), "=r"(u[13]), "=r"(u[14]), "=r"(u[15]),
          "=r"(u[16]), "=r"(u[17]), "=r"(u[18]), "=r"(u[19]), "=r"(u[20]), "=r"(u[21]), "=r"(u[22]), "=r"(u[23]),
          "=r"(u[24]), "=r"(u[25]), "=r"(u[26]), "=r"(u[27]), "=r"(u[28]), "=r"(u[29]), "=r"(u[30]), "=r"(u[31]),
          "=r"(u[32]), "=r"(u[33]), "=r"(u[34]), "=r"(u[35]), "=r"(u[36]), "=r"(u[37]), "=r"(u[38]), "=r"(u[39]),
          "=r"(u[40]), "=r"(u[41]), "=r"(u[42]), "=r"(u[43]), "=r"(u[44]), "=r"(u[45]), "=r"(u[46]), "=r"(u[47]),
          "=r"(u[48]), "=r"(u[49]), "=r"(u[50]), "=r"(u[51]), "=r"(u[52]), "=r"(u[53]), "=r"(u[54]), "=r"(u[55]),
          "=r"(u[56]), "=r"(u[57]), "=r"(u[58]), "=r"(u[59]), "=r"(u[60]), "=r"(u[61]), "=r"(u[62]), "=r"(u[63])
        : "r"(taddr));
}

__device__ __forceinline__ void tmem_ld_x32(unsigned taddr, unsigned (&u)[32]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];\n"
        : "=r"(u[0]), "=r"(u[1]), "=r"(u[2]), "=r"(u[3]), "=r"(u[4]), "=r"(u[5]), "=r"(u[6]), "=r"(u[7]),
          "=r"(u[8]), "=r"(u[9]), "=r"(u[10]), "=r"(u[11]), "=r"(u[12]), "=r"(u[13]), "=r"(u[14]), "=r"(u[15]),
          "=r"(u[16]), "=r"(u[17]), "=r"(u[18]), "=r"(u[19]), "=r"(u[20]), "=r"(u[21]), "=r"(u[22]), "=r"(u[23]),
          "=r"(u[24]), "=r"(u[25]), "=r"(u[26]), "=r"(u[27]), "=r"(u[28]), "=r"(u[29]), "=r"(u[30]), "=r"(u[31])
        : "r"(taddr));
}

__device__ __forceinline__ void tmem_wait_ld() {
    asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
}

// (hi, lo) FP16 split of a complex amplitude (x, y): hi = f16x2(x, y)
// rounded to nearest, lo = f16x2 of the residuals.
__device__ __forceinline__ void split_f16x2(float x, float y, unsigned &hi, unsigned &lo) {
    asm("{\n\t.reg .f32 hx, hy;\n\t.reg .b16 bx, by;\n\t"
        "cvt.rn.f16x2.f32 %0, %3, %2;\n\t"
        "mov.b32 {bx, by}, %0;\n\t"
        "cvt.f32.f16 hx, bx;\n\t"
        "cvt.f32.f16 hy, by;\n\t"
        "sub.f32 hx, %2, hx;\n\t"
        "sub.f32 hy, %3, hy;\n\t"
        "cvt.rn.f16x2.f32 %1, hy, hx;\n\t}\n"
        : "=r"(hi), "=r"(lo)
        : "f"(x), "f"(y));
}

// Bit in which the Gray codes of i - 1 and i differ (ctz(i)), at compile
// time once the loops are unrolled.
__host__ __device__ constexpr int gray_bit(int i) {
    return (i & 1) ? 0 : (i & 2) ? 1 : (i & 4) ? 2 : (i & 8) ? 3 : 4;
}
// Inverse Gray code of j (5 bits).
__host__ __device__ constexpr int gray_index(int j) {
    return j ^ (j >> 1) ^ (j >> 2) ^ (j >> 3) ^ (j >> 4);
}

// Visits the 2^NB registers of a thread in Gray-code order: f(j, p) with
// p = base + offset of register j, where register j's offset is the sum of
// e[k] over the set bits k of j.
template <int NB, class P, class F>
__device__ __forceinline__ void gray_walk(P *base, const long long (&e)[5], F f) {
    P *p = base;
#pragma unroll
    for (int i = 0; i < (1 << NB); ++i) {
        const int j = i ^ (i >> 1);
        if (i > 0) {
            const int k = gray_bit(i);
            p = (j >> k & 1) ? p + e[k] : p - e[k];
        }
        f(j, p);
    }
}

// The state is carried scaled by 2^12 through the blocks of a stage.
constexpr float kScale = 4096.f, kUnscale = 1.f / 4096.f;

}  // namespace

__device__ __forceinline__ void group_sync(unsigned id, unsigned threads) {
    asm volatile("bar.sync %0, %1;\n" ::"r"(id), "r"(threads) : "memory");
}

// Persistent kernel, one CTA per SM.  The CTA holds every block operand of
// the stage in shared memory (loaded once) and G independent tile groups;
// each group walks its own tiles with its own operand buffers, tensor-memory
// columns and mbarrier, so the groups overlap one another's loads, splits
// and products on the SM's tensor core.  RT = 128-row groups per tile (tile
// lanes m = 12 for RT = 1, 13 for RT = 2); H = threads per row (each thread
// holds 32 / H amplitudes of its row; H = 2 halves the registers per thread
// so that twice the warps fit); PH = the launch has phase ops (without them
// the kernel keeps the registers of the dense path alone).
template <int RT, int G, int H, bool PH>
__global__ void __launch_bounds__(128 * RT * G * H, 1)
k_tstage(float2 *__restrict__ s, const __grid_constant__ TcStageDesc d, int tiles) {
    constexpr int m = RT == 1 ? 12 : 13;
    constexpr int t = m - 5;
    constexpr int NA = 32 / H;                          // amplitudes per thread
    constexpr int NB = H == 1 ? 5 : 4;                  // register bits per thread
    constexpr unsigned TR = 128u * RT;                  // rows per tile
    constexpr unsigned TG = TR * H;                     // threads per group
    constexpr unsigned T = TG * G;
    constexpr unsigned kColsGroup = 64u * RT;
    constexpr unsigned kCols = kColsGroup * G <= 32 ? 32 : (kColsGroup * G <= 64 ? 64 :
                               (kColsGroup * G <= 128 ? 128 : (kColsGroup * G <= 256 ? 256 : 512)));
    constexpr unsigned kBBytes = 2u * 64u * 64u * 2u;   // Bh, Bl of one dense op in FP16
    constexpr unsigned kABytes = 4u << m;               // one FP16 operand of a tile
    static_assert(H == 1 || H == 2, "threads per row");
    extern __shared__ __align__(1024) unsigned char smraw[];
    const int nb = d.nblocks;
    unsigned char *Bs = smraw + (size_t)G * 2 * kABytes;  // the ops' operands
    SetSlots *sset = (SetSlots *)(Bs + d.ops_bytes);
    __shared__ __align__(8) unsigned long long bar_mma[G], bar_b;
    __shared__ unsigned tmem_sh;
    __shared__ int abort_sh[G];
    const unsigned tid = threadIdx.x;
    const unsigned warp = tid >> 5;
    const unsigned g = tid / TG, lt = tid % TG;
    const unsigned r = lt % TR, hh = lt / TR;           // row, half of the row
    const unsigned wg = (lt >> 5) % (4u * RT);          // warp within the rows
    unsigned *Ah = (unsigned *)(smraw + (size_t)g * 2 * kABytes);  // f16x2 per amplitude
    unsigned *Al = Ah + (1 << m);
    float2 *tile_sm = (float2 *)Ah;                     // natural tile (aliases Ah, Al)

    // The operand atoms must be 1024-byte aligned for the 128-byte swizzle.
    if ((smem_u32(smraw) & 1023u) != 0u) {
        if (tid == 0) atomicOr(&g_tc_status, 4u);
        return;
    }
    if (tid == 0) abort_sh[0] = *(volatile unsigned *)&g_tc_status != 0u;
    __syncthreads();
    if (abort_sh[0]) return;
    __syncthreads();

    const unsigned bb = smem_u32(&bar_b), bmma = smem_u32(&bar_mma[g]);
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(
                         smem_u32(&tmem_sh)),
                     "r"(kCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
    }
    if (tid < G) {
        mbar_init(smem_u32(&bar_mma[tid]), 1);
        abort_sh[tid] = 0;
    }
    if (tid == 0) {
        mbar_init(bb, 1);
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    rs::copy_sets(sset, d.sets, nb + 2, tid, T);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    // This warp's lanes (row quadrant) and columns (128-row group, half).
    const unsigned tmem = tmem_sh + g * kColsGroup + 64u * (wg >> 2) + 32u * hh +
                          ((32u * (wg & 3u)) << 16);
    const unsigned dcol0 = tmem_sh + g * kColsGroup;       // the group's accumulator
    if (tid == 0) bulk_load(smem_u32(Bs), d.bmats, d.ops_bytes, bb);

    // Load layout: row bit b at global lane row_lane[b], amplitude bit k at
    // the lane of e[k] (chosen per stage on the host; lanes 0..3 of the tile
    // are among the warp's row bits, so accesses come in 128-byte runs).  A
    // thread holds amplitudes hh * NA + j of its row, j < NA.
    const long long(&e)[5] = d.in_e;  // read from the parameter space where used
    // This thread's row offset in the load layout (recomputed where used,
    // which keeps it out of the registers the ops need).
    auto row_offset = [&]() {
        idx_t o = 0;
        for (int b = 0; b < t; ++b)
            if (r & (1u << b)) o |= 1LL << d.row_lane[b];
        if (H == 2 && hh) o += e[4];
        return o;
    };
    const unsigned gbar = 1u + g;                          // the group's named barrier
    unsigned phase = 0;
    bool ok = true, b_ready = false, t_ready = false;
    const int tstep = (int)gridDim.x * G;

    // The next tile's loads are issued into v once the finished tile has
    // been staged in shared memory, before it is copied out, so they are in
    // flight during the copy-out; the scale is applied after.
    unsigned v[2 * NA];  // floats (bits): this thread's part of row r
    auto load_raw = [&](int tl) {
        const float2 *gp0 = s + (insert_zeros((idx_t)tl, d.ins_pos, d.nins) | row_offset());
        gray_walk<NB>(gp0, e, [&](int j, const float2 *p) {
            const float2 x = *p;
            v[2 * j] = __float_as_uint(x.x);
            v[2 * j + 1] = __float_as_uint(x.y);
        });
    };
    if ((int)blockIdx.x * G + (int)g < tiles) load_raw((int)blockIdx.x * G + (int)g);
    for (int tl = (int)blockIdx.x * G + (int)g; tl < tiles && ok; tl += tstep) {
#pragma unroll
        for (int i = 0; i < 2 * NA; ++i) v[i] = __float_as_uint(__uint_as_float(v[i]) * kScale);
        for (int b = 0; b < nb; ++b) {
            const SetSlots &ss = sset[b];
            unsigned slot = (unsigned)ss.lo[r & 31u] ^ (unsigned)ss.hi[r >> 5];
            if (H == 2 && hh) slot ^= ss.q[4];
            if (PH && d.op_kind[b] == 2) {
                // Cross op: per tile, every amplitude's phase is a scalar
                // times one factor per tile lane (picked by the lane's bit),
                // from the records' angles and the tile's bits outside the
                // tile lanes.  Scratch: the group's operand buffer, free
                // between dense ops (U at [0, m], V at [16, 16 + m]); the
                // register table lives in the warps' lanes.
                if (!t_ready) {
                    t_ready = mbar_wait(bb, 0u);
                    if (!t_ready) atomicOr(&g_tc_status, 1u);
                }
                const TcCrossHdr &xh = *(const TcCrossHdr *)(Bs + d.op_off[b]);
                const TcCrossRec *xr = (const TcCrossRec *)(Bs + d.op_off[b] + sizeof(TcCrossHdr));
                float2 *xf = (float2 *)Ah;
                const int nrec = min(max(xh.nrec, 0),
                                     (int)((d.ops_bytes - d.op_off[b] - sizeof(TcCrossHdr)) /
                                           sizeof(TcCrossRec)));
                {
                    // position p's factors, one 8-lane group per position
                    // (TG / 8 >= 16 groups cover the m + 1 <= 14 positions in
                    // one round): its lanes take the position's records in
                    // turn, then a fixed shuffle tree sums the angles (the
                    // same order every run; every lane runs it, so the
                    // shuffles are uniform), and the group's lanes 0 and 1
                    // form the two factors
                    static_assert(TG / 8u >= (unsigned)m + 1u, "one round of positions");
                    const long long g0 = insert_zeros((idx_t)tl, d.ins_pos, d.nins);
                    const int p = (int)(lt >> 3);
                    const unsigned ql = lt & 7u;
                    const int k0 = p <= m ? min(max(xh.start[p], 0), nrec) : 0;
                    const int k1 = p < m ? min(xh.start[p + 1], nrec) : (p == m ? nrec : 0);
                    float a0 = 0.f, a1 = 0.f;
                    for (int k = k0 + (int)ql; k < k1; k += 8) {
                        const TcCrossRec x = xr[k];
                        if ((g0 & x.need) != x.need) continue;
                        if (x.tgt == 0) {
                            a0 += x.a0;
                            a1 += x.a1;
                        } else {
                            a1 += (g0 & x.tgt) ? x.a1 : x.a0;
                        }
                    }
#pragma unroll
                    for (int o = 4; o > 0; o >>= 1) {
                        a0 += __shfl_xor_sync(0xffffffffu, a0, o);
                        a1 += __shfl_xor_sync(0xffffffffu, a1, o);
                    }
                    if (ql < 2u && p <= m) {
                        constexpr float kTwoPi = 6.283185307f;
                        float a = ql ? a1 : a0;
                        a -= kTwoPi * rintf(a * (1.f / kTwoPi));
                        float sa, ca;
                        sincosf(a, &sa, &ca);
                        xf[16 * ql + p] = make_float2(ca, sa);
                    }
                }
                group_sync(gbar, TG);
                // (labels as in the kernel's load layout) this thread's row
                // factor, and lane l of every warp holds register entry l
                float2 tab = make_float2(1.f, 0.f);
#pragma unroll
                for (int k = 0; k < 5; ++k)
                    tab = cmul(tab, xf[((lt & 31u) >> k & 1u) ? 16 + xh.amps[k] : xh.amps[k]]);
                float2 base = xf[16 + m];  // the scalar
                for (int bb2 = 0; bb2 < t; ++bb2)
                    base = cmul(base, xf[(r >> bb2 & 1u) ? 16 + xh.rows[bb2] : xh.rows[bb2]]);
#pragma unroll
                for (int j = 0; j < NA; ++j) {
                    const int src = (H == 2 && hh) ? (j | 16) : j;
                    const float2 e = make_float2(__shfl_sync(0xffffffffu, tab.x, src),
                                                 __shfl_sync(0xffffffffu, tab.y, src));
                    const float2 f = cmul(base, e);
                    const float x = __uint_as_float(v[2 * j]), y = __uint_as_float(v[2 * j + 1]);
                    v[2 * j] = __float_as_uint(fmaf(x, f.x, -y * f.y));
                    v[2 * j + 1] = __float_as_uint(fmaf(x, f.y, y * f.x));
                }
                group_sync(gbar, TG);  // the scratch is read before the next split
                continue;
            }
            if (PH && d.op_kind[b] == 1) {
                // Phase op: each amplitude times its table entry, in place
                // (the layout stays).  Every thread waits for the operands
                // itself (bounded; a wait that gives up is reported).
                if (!t_ready) {
                    t_ready = mbar_wait(bb, 0u);
                    if (!t_ready) atomicOr(&g_tc_status, 1u);
                }
                const float2 *tab = (const float2 *)(Bs + d.op_off[b]);
#pragma unroll
                for (int i = 0; i < NA; ++i) {
                    const int j = i ^ (i >> 1);
                    if (i > 0) slot ^= ss.q[gray_bit(i)];
                    const float2 p = tab[slot];
                    const float x = __uint_as_float(v[2 * j]), y = __uint_as_float(v[2 * j + 1]);
                    v[2 * j] = __float_as_uint(fmaf(x, p.x, -y * p.y));
                    v[2 * j + 1] = __float_as_uint(fmaf(x, p.y, y * p.x));
                }
                continue;
            }
            unsigned q[NB];
#pragma unroll
            for (int k = 0; k < NB; ++k) q[k] = ss.q[k];
#pragma unroll
            for (int i = 0; i < NA; ++i) {  // Gray-code order: one XOR per slot
                const int j = i ^ (i >> 1);
                if (i > 0) slot ^= q[gray_bit(i)];
                unsigned h, l;
                split_f16x2(__uint_as_float(v[2 * j]), __uint_as_float(v[2 * j + 1]), h, l);
                Ah[slot] = h;
                Al[slot] = l;
            }
            asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
            group_sync(gbar, TG);
            if (lt == 0) {
                if (!b_ready) b_ready = mbar_wait(bb, 0u);
                if (b_ready) {
                    tc_fence_after();
                    const unsigned ah = smem_u32(Ah), al = smem_u32(Al),
                                   bh = smem_u32(Bs + d.op_off[b]), bl = bh + kBBytes / 2;
                    // The tensor core rounds its FP32 accumulator toward zero
                    // at every MMA, which shrinks magnitudes: the correction
                    // products go first (small values), the main product's
                    // four K-steps last, so that only those round at full
                    // magnitude (the host scales each block's rows to cancel
                    // the expected shrink of those four roundings).
#pragma unroll
                    for (int mt = 0; mt < RT; ++mt) {
                        const unsigned dcol = dcol0 + 64u * mt;
#pragma unroll
                        for (int ks = 0; ks < 4; ++ks) {
                            // A: 128-byte swizzled K-major, 8-row atoms of
                            // 1024 bytes, K-step ks at +32 bytes in the atom.
                            const unsigned aoff = 16384u * mt + 32u * ks, boff = 2048u * ks;
                            const uint64_t dah = smem_desc(ah + aoff, 16, 1024, 2);
                            const uint64_t dal = smem_desc(al + aoff, 16, 1024, 2);
                            const uint64_t dbh = smem_desc(bh + boff, 1024, 128);
                            const uint64_t dbl = smem_desc(bl + boff, 1024, 128);
                            mma_f16(dcol, dah, dbl, ks > 0 ? 1u : 0u);
                            mma_f16(dcol, dal, dbh, 1u);
                        }
#pragma unroll
                        for (int ks = 0; ks < 4; ++ks) {
                            const unsigned aoff = 16384u * mt + 32u * ks, boff = 2048u * ks;
                            mma_f16(dcol, smem_desc(ah + aoff, 16, 1024, 2),
                                    smem_desc(bh + boff, 1024, 128), 1u);
                        }
                    }
                    mma_commit(bmma);
                } else {
                    atomicOr(&g_tc_status, 1u);
                    abort_sh[g] = 1;
                    mbar_arrive(bmma);
                }
            }
            const bool got = mbar_wait(bmma, phase);
            phase ^= 1u;
            if (!got) {
                abort_sh[g] = 1;
                atomicOr(&g_tc_status, 2u);
            }
            // One decision for the whole group, so that its threads leave
            // together.
            group_sync(gbar, TG);
            if (abort_sh[g]) {
                ok = false;
                break;
            }
            tc_fence_after();
            if constexpr (H == 1)
                tmem_ld_x64(tmem, v);
            else
                tmem_ld_x32(tmem, v);
            tmem_wait_ld();
        }
        tc_fence_before();
        group_sync(gbar, TG);  // every thread's products read: the buffers are free
        if (!ok) break;
        if (d.direct_out) {
            // The final layout's warp rows cover whole 128-byte lines: rows
            // go straight from the registers to the state, then the next
            // tile's loads.
            idx_t o = 0;
            for (int b = 0; b < t; ++b)
                if (r & (1u << b)) o |= 1LL << d.out_row_lane[b];
            if (H == 2 && hh) o += d.out_e[4];
            float2 *gp = s + (insert_zeros((idx_t)tl, d.ins_pos, d.nins) | o);
            gray_walk<NB>(gp, d.out_e, [&](int j, float2 *p) {
                *p = make_float2(__uint_as_float(v[2 * j]) * kUnscale,
                                 __uint_as_float(v[2 * j + 1]) * kUnscale);
            });
            if (tl + tstep < tiles) load_raw(tl + tstep);
            continue;
        }
        // Last layout -> swizzled natural tile -> load layout -> global.
        {
            const SetSlots &ss = sset[nb];
            unsigned slot = (unsigned)ss.lo[r & 31u] ^ (unsigned)ss.hi[r >> 5];
            if (H == 2 && hh) slot ^= ss.q[4];
            unsigned q[NB];
#pragma unroll
            for (int k = 0; k < NB; ++k) q[k] = ss.q[k];
#pragma unroll
            for (int i = 0; i < NA; ++i) {
                const int j = i ^ (i >> 1);
                if (i > 0) slot ^= q[gray_bit(i)];
                tile_sm[slot] = make_float2(__uint_as_float(v[2 * j]) * kUnscale,
                                            __uint_as_float(v[2 * j + 1]) * kUnscale);
            }
        }
        group_sync(gbar, TG);
        if (tl + tstep < tiles) load_raw(tl + tstep);
        {
            // the natural tile read in the load layout
            const SetSlots &nat = sset[nb + 1];
            unsigned slot = (unsigned)nat.lo[r & 31u] ^ (unsigned)nat.hi[r >> 5];
            if (H == 2 && hh) slot ^= nat.q[4];
            float2 *gp = s + (insert_zeros((idx_t)tl, d.ins_pos, d.nins) | row_offset());
            gray_walk<NB>(gp, e, [&](int j, float2 *p) {
                const int i = gray_index(j);
                if (i > 0) slot ^= nat.q[gray_bit(i)];
                *p = tile_sm[slot];
            });
        }
        group_sync(gbar, TG);  // the natural tile is read before the next splits
    }
    // A group whose bulk-copy wait never ran still owns an outstanding copy
    // only if it never issued an MMA; the CTA waits for it before exiting.
    if (tid == 0 && !b_ready) mbar_wait(bb, 0u);
    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem_sh),
                     "r"(kCols)
                     : "memory");
    }
}

// Shared memory of the persistent kernel: G tiles' operand pairs, the
// stage's op operands and the slot tables.
static size_t tstage_smem(int m, int groups, size_t ops_bytes, int nops) {
    return (size_t)groups * 2 * ((size_t)4 << m) + ops_bytes +
           sizeof(SetSlots) * (size_t)(nops + 2);
}

// Groups per CTA: 4 for 12-lane tiles (of 128 threads, or of 256 with two
// threads per row), 2 of 256 threads for 13-lane tiles.
static int tstage_groups(int m) { return m == 12 ? 4 : 2; }

void launch_tstage(void *state, const TcStageDesc &d, cudaStream_t stream, bool two_per_row) {
    if (d.m != 12 && d.m != 13) fail(2, "tensor stage: tile lanes must be 12 or 13 (got %d)", d.m);
    if (d.nblocks < 1 || d.nblocks > kMaxTcBlocks) fail(2, "tensor stage: bad op count %d", d.nblocks);
    if (((uintptr_t)d.bmats & 15u) != 0 || (d.ops_bytes & 15u) != 0)
        fail(2, "tensor stage: operand array misaligned");
    // Every slot a thread forms (an XOR of table entries) is at most the OR
    // of the table's entries: it must stay inside the tile operand (dense
    // ops), the op's table (phase ops) or the natural tile.
    auto reach = [](const SetSlots &ss) {
        unsigned any = 0;
        for (unsigned short x : ss.lo) any |= x;
        for (unsigned short x : ss.hi) any |= x;
        for (unsigned short x : ss.q) any |= x;
        return any;
    };
    for (int b = 0; b < d.nblocks + 2; ++b) {
        const unsigned any = reach(d.sets[b]);
        const bool phase = b < d.nblocks && d.op_kind[b] == 1;
        const bool cross = b < d.nblocks && d.op_kind[b] == 2;
        if (b < d.nblocks && d.op_kind[b] > 2) fail(2, "tensor stage: op %d of unknown kind", b);
        if (!phase && any >= (1u << d.m)) fail(2, "tensor stage: slot table %d outside the tile", b);
        if (b >= d.nblocks) continue;
        // (a cross op's records are bounded by the operand array in the kernel)
        const unsigned need = phase ? 8u * (any + 1u)
                                    : (cross ? (unsigned)sizeof(TcCrossHdr) : 2u * 64u * 64u * 2u);
        if ((d.op_off[b] & 15u) != 0 || d.op_off[b] + need > d.ops_bytes)
            fail(2, "tensor stage: op %d operands outside the operand array", b);
    }
    if (tstage_smem(d.m, tstage_groups(d.m), d.ops_bytes, d.nblocks) + 2048 > 227 * 1024)
        fail(2, "tensor stage: %u bytes of operands do not fit in shared memory", d.ops_bytes);
    if (d.n - d.m > 30) fail(2, "tensor stage: %d lanes are too many", d.n);
    const int tiles = 1 << (d.n - d.m);
    int dev = 0, sms = 0;
    QG_CUDA(cudaGetDevice(&dev));
    QG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    auto launch = [&](auto kern, int groups, int threads) {
        const size_t smem = tstage_smem(d.m, groups, d.ops_bytes, d.nblocks);
        QG_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        const int ctas = std::min((tiles + groups - 1) / groups, sms);
        kern<<<(unsigned)ctas, threads, smem, stream>>>((float2 *)state, d, tiles);
    };
    bool phases = false;  // phase or cross ops
    for (int b = 0; b < d.nblocks; ++b) phases = phases || d.op_kind[b] != 0;
    if (d.m == 12 && two_per_row)
        phases ? launch(k_tstage<1, 3, 2, true>, 3, 768) : launch(k_tstage<1, 3, 2, false>, 3, 768);
    else if (d.m == 12)
        phases ? launch(k_tstage<1, 4, 1, true>, 4, 512) : launch(k_tstage<1, 4, 1, false>, 4, 512);
    else
        phases ? launch(k_tstage<2, 2, 1, true>, 2, 512) : launch(k_tstage<2, 2, 1, false>, 2, 512);
    QG_CUDA(cudaGetLastError());
}

int tstage_status(bool reset) {
    unsigned v = 0;
    QG_CUDA(cudaMemcpyFromSymbol(&v, g_tc_status, sizeof(v)));
    if (reset && v) {
        unsigned z = 0;
        QG_CUDA(cudaMemcpyToSymbol(g_tc_status, &z, sizeof(z)));
    }
    return (int)v;
}

}  // namespace qg
