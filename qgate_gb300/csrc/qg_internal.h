// Internal declarations shared by the engine's translation units.
//
// State layout in HBM: one contiguous buffer of 2^n interleaved complex
// amplitudes (float2 for complex64, double2 for complex128); bit i of an
// amplitude index is local lane i.  This is the reference's layout
// (qgate/simulator/src/DeviceTypes.h:18-58), kept so that lane numbering and
// index conventions are identical; the reference's multi-device chunking
// (qgate/simulator/src/MultiChunkPtr.h:28-41) is dropped: one GPU holds the
// whole state in a single allocation.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <string>
#include <vector>

namespace qg {

typedef long long idx_t;

constexpr int kMaxLanes = 62;        // index bits an amplitude index may carry
constexpr int kMaxStageGates = 96;   // gates one fused stage may apply
constexpr int kMaxTileLanes = 14;    // lanes one shared-memory tile may hold
constexpr int kMaxGetterStates = 63; // states objects one gather may combine
constexpr int kMaxMultiTargets = 6;  // targets of a dense multi-target gate

enum Prec { kFP64 = 1, kFP32 = 2 };

inline size_t complex_size(int prec) { return prec == kFP64 ? 16 : 8; }

// Thrown inside the engine, caught at the extern "C" boundary.
struct Error {
    int code;
    std::string msg;
};
[[noreturn]] void fail(int code, const char *fmt, ...);
void cuda_check(cudaError_t err, const char *what);
// Sets the message returned by qg_last_error() on this thread.
void set_last_error(const std::string &msg);
#define QG_CUDA(call) ::qg::cuda_check((call), #call)

// ---------------------------------------------------------------- kernels

// Pair-sweep index pattern: the k-th work item is the amplitude index made by
// inserting zero bits at pos[0..npos) (ascending) into k, then OR-ing
// set_mask; its partner is that index | partner.
struct PairIdx {
    int npos;
    int pos[kMaxLanes];
    unsigned long long set_mask;
    unsigned long long partner;
};

// Row-major 2x2 complex matrix in FP64 (converted to the state's precision
// inside the kernels, as the reference does:
// qgate/simulator/src/CPUQubitProcessor.cpp:311).
struct Mat2 {
    double v[8];
};

// One gate of a fused stage, in tile-local lane numbering.
struct StageGate {
    int npos;               // inserted zero bits (controls + target)
    signed char pos[kMaxTileLanes];
    unsigned cmask;         // tile-local control bits
    unsigned tbit;          // tile-local target bit
    int diag;               // matrix is diagonal
    double m[8];
};

struct StageDesc {
    int n;                  // lanes of the state
    int m;                  // lanes per tile
    int lowrun;             // tile lanes 0..lowrun-1 are global lanes 0..lowrun-1
    int nhi;                // tile lanes lowrun..m-1
    int hi_pos[kMaxTileLanes];       // their global lanes
    int nins;               // = m when m < n: global lanes of the tile, ascending
    int ins_pos[kMaxTileLanes];
    int ngates;
    StageGate gates[kMaxStageGates];
};

// Register-resident fused stage.  Each thread holds 2^rl amplitudes of the
// tile in registers: those whose tile index differs only in the tile lanes of
// the current register set.  Gates whose target is in the register set are
// applied in registers; diagonal gates need no data movement at all; a
// transpose (through shared memory) switches to another register set.
constexpr int kMaxRegOps = 192;
constexpr int kMaxRegSets = 64;
constexpr int kMaxRegLanes = 5;

enum RegOpKind {
    kOpGate = 0,        // dense 2x2 on register bit `reg`
    kOpSwapX = 1,       // X (swap) on register bit `reg`
    kOpDiagReg = 2,     // diagonal on register bit `reg`
    kOpDiagThread = 3,  // diagonal whose target is a thread lane (tile mask `tbit`)
    kOpTranspose = 4    // switch to register set `reg`
};

// 48 bytes (complex64) / 80 bytes (complex128): a whole number of 16-byte
// vectors, so a stage program copies to shared memory as int4s.
template <class R> struct alignas(16) RegOp {
    unsigned char kind;
    unsigned char reg;
    unsigned short jmask;  // controls among register-index bits
    unsigned tmask;        // controls among thread lanes (tile-lane mask)
    unsigned tbit;         // kOpDiagThread: the target's tile-lane mask
    unsigned pad;
    R m[8];                // row-major 2x2 matrix, interleaved re/im
};
static_assert(sizeof(RegOp<float>) == 48, "RegOp<float> layout");
static_assert(sizeof(RegOp<double>) == 80, "RegOp<double> layout");

// Shared-memory slot tables of one register set (host-precomputed): the
// swizzled slot of a thread's element 0 is lo[tid & 31] ^ hi[tid >> 5];
// register j adds the XOR of q[k] over the set bits k of j.
struct SetSlots {
    unsigned short lo[32];
    unsigned short hi[16];
    unsigned short q[kMaxRegLanes + 1];
};

template <class R> struct RStageDesc {
    int n, m, rl;              // lanes of the state, tile lanes, register lanes
    int lowrun, nhi;
    int hi_pos[kMaxTileLanes];
    int nins;
    int ins_pos[kMaxTileLanes];
    long long dep_hi[1 << kMaxRegLanes];  // global offset of tile element (i << (m - rl))
    int nops, nsets;
    // Per register set: the swizzled shared-memory slot of the thread's
    // element 0 is slot_lo[tid & 31] ^ slot_hi[tid >> 5] (the bit deposit of
    // the thread index into the thread lanes, and the swizzle, are both
    // linear over GF(2)), and register j adds the XOR of slot_q[k] over the
    // set bits k of j.  Precomputed on the host.
    SetSlots sets[kMaxRegSets];
    RegOp<R> ops[kMaxRegOps];                     // 16-byte aligned
};

// Tensor-core stage (complex64): a sequence of ops on a tile of m = 12 or 13
// lanes - fused 5-lane blocks applied as tcgen05 products (dense ops) and
// diagonal phase tables applied elementwise (phase ops).  Load layout:
// thread bit b holds global lane row_lane[b], register bit k global lane
// log2(dep_hi[1 << k]).  sets[b] maps the registers of the layout before op
// b (the load layout for b = 0) to the slots of dense op b's operand layout,
// or to the entries of phase op b's table (a phase op keeps the layout);
// sets[nblocks] maps the layout after the last op, sets[nblocks + 1] the load
// layout, to the swizzled natural tile.  bmats holds the ops' operands, op b
// at byte op_off[b]: a dense op's split operands Bh, Bl (2 x 4096 FP16
// values, canonical K-major layout), a phase op's table of complex64 phases
// (ops_bytes in all, a multiple of 16).
constexpr int kMaxTcBlocks = 24;
// Operands of a cross op (op_kind 2): this header, then `nrec` records
// sorted by tile position.  Records of position p < m are [start[p],
// start[p + 1]); records [start[m], nrec) act on no tile lane (a per-tile
// scalar).  A record applies when the tile's amplitude index has every bit
// of `need` set; with tgt == 0 (the gate's target is at p) it adds angle a0
// to the phase of bit p = 0 and a1 to bit p = 1; otherwise (the target is
// outside the tile, at the lanes of tgt) it adds (tile bit tgt ? a1 : a0) to
// bit p = 1 (or to the scalar).  rows / amps: tile positions of the row bits
// and register bits of the layout the op runs in.
struct TcCrossHdr {
    int nrec;
    int start[15];
    signed char rows[8];
    signed char amps[5];
    signed char pad[3];
};
struct TcCrossRec {
    long long need, tgt;
    float a0, a1;  // in (-pi, pi]
    float pad[2];
};
static_assert(sizeof(TcCrossHdr) % 16 == 0 && sizeof(TcCrossRec) == 32, "cross op layout");

struct TcStageDesc {
    int n, m;
    int row_lane[8];
    int nins;
    int ins_pos[kMaxTileLanes];
    long long dep_hi[32];
    long long in_e[5];                    // dep_hi[1 << k]
    // direct_out = 1: the final layout's warp rows hold tile positions 0..3
    // (whole 128-byte lines), so rows are stored straight to the state:
    // row bit b at global lane out_row_lane[b], amplitude bit k at out_e[k].
    // Otherwise rows go through the natural tile (sets[nb], sets[nb + 1]).
    int direct_out;
    int out_row_lane[8];
    long long out_e[5];
    int nblocks;                          // ops
    unsigned ops_bytes;
    unsigned op_off[kMaxTcBlocks];        // byte offset of op b's operands
    unsigned char op_kind[kMaxTcBlocks];  // 0: dense block, 1: phase table, 2: cross
    const unsigned char *bmats;
    SetSlots sets[kMaxTcBlocks + 2];
};
// two_per_row: the 12-lane variant with two threads per tile row (twice the
// warps per SM, half the registers per thread).
void launch_tstage(void *state, const TcStageDesc &d, cudaStream_t stream, bool two_per_row);
// Status word of the tensor stage kernels (nonzero: a bounded wait gave up).
int tstage_status(bool reset);

// XOR swizzle of shared-memory element slots (see qg_regstage.cuh):
// 16 slots per 128-byte row for complex64, 8 for complex128.  An involution.
inline unsigned host_swz(unsigned e, int prec);
inline unsigned host_pdep(unsigned x, unsigned mask);
// Slot tables of a register set with tile lanes rb[0..rl) in an m-lane tile.
inline SetSlots make_set_slots(const int *rb, int rl, int m, int prec);

inline unsigned host_swz(unsigned e, int prec) {
    return prec == kFP32 ? e ^ (((e >> 4) ^ (e >> 8) ^ (e >> 12)) & 15u)
                         : e ^ (((e >> 3) ^ (e >> 6) ^ (e >> 9) ^ (e >> 12)) & 7u);
}
inline unsigned host_pdep(unsigned x, unsigned mask) {
    unsigned r = 0;
    for (unsigned b = 1; mask; b <<= 1) {
        unsigned low = mask & (0u - mask);
        if (x & b) r |= low;
        mask &= mask - 1;
    }
    return r;
}

// pipelined: persistent grid with double-buffered tiles (when the state has
// enough tiles and two fit in shared memory).
void launch_rstage_f32(void *state, const RStageDesc<float> &d, cudaStream_t stream,
                       bool pipelined);
void launch_rstage_f64(void *state, const RStageDesc<double> &d, cudaStream_t stream,
                       bool pipelined);

// ---------------------------------------------------------------- adjoint

// One op of a batched stage program (forward apply, or backward un-apply with
// gradient partials).  Matrices live in a per-batch-element table in device
// memory (rotation matrices differ per parameter vector); `mat` indexes it.
struct AdjOp {
    unsigned char kind;   // RegOpKind
    unsigned char reg;
    unsigned short jmask;
    unsigned tmask;
    unsigned tbit;
    unsigned short mat;   // matrix slot
    unsigned char gaxis;  // 0: no gradient; 1/2/3: generator X/Y/Z of a rotation
    unsigned char gslot;  // gradient slot within the stage
};
static_assert(sizeof(AdjOp) == 16, "AdjOp layout");

constexpr int kMaxAdjOps = 256;
constexpr int kMaxAdjSlots = 128;

struct AdjStageDesc {
    int n, m, rl;
    int lowrun, nhi;
    int hi_pos[kMaxTileLanes];
    int nins;
    int ins_pos[kMaxTileLanes];
    long long dep_hi[1 << kMaxRegLanes];
    int nops, nmats, ngrads, nsets;
    SetSlots sets[kMaxRegSets];
    AdjOp ops[kMaxAdjOps];
};

// mode 0: apply ops to psi.  mode 1: for each op, first accumulate the
// gradient term Im<lam|P1 G|psi> of its slot (if any), then apply the op's
// (adjoint) matrix to both psi and lam.  mats: [batch][nmats][8] in the
// state's precision; grad_partials: [batch][ngrads][tiles] in the state's
// precision.  States of batch element b start at b * 2^n.
void launch_adj_stage(int prec, int mode, void *psi, void *lam, const AdjStageDesc &d,
                      const void *mats, void *grad_partials, int batch, cudaStream_t stream);
// grad[b * n_params + param[s]] += scale[s] * sum_t partials[b][s][t]  (FP64)
void launch_adj_grad_reduce(int prec, const void *partials, int batch, int nslots, idx_t tiles,
                            const int *d_param, const double *d_scale, double *grad,
                            int n_params, cudaStream_t stream);

struct PauliTerm {
    double coef;
    unsigned long long x, z;
};
constexpr int kMaxPauliTerms = 256;
// lam = sum_t coef_t P_t psi and e_partials[b][block] for E_b = Re<psi|lam>.
void launch_pauli_sum_apply(int prec, const void *psi, void *lam, int n, int batch,
                            const PauliTerm *terms, int nterms, double *e_partials,
                            int blocks_per_batch, cudaStream_t stream);
int pauli_sum_blocks();
void launch_sum_rows(const double *partials, int rows, int cols, double *out, cudaStream_t stream);

// ---------------------------------------------------------------- batches

// Tile mapping of one stage of one circuit of a batch (the RStageDesc header
// without the program), in device memory.
struct BatchStage {
    long long state_off;  // element offset of the circuit's state in the arena
    int n, m, rl, lowrun, nhi, nins, nops;
    int hi_pos[kMaxTileLanes];
    int ins_pos[kMaxTileLanes];
    long long dep_hi[1 << kMaxRegLanes];
    long long ops_off;    // index of the stage's first RegOp in the program buffer
    int sets_off;         // index of the stage's first register set
    int nsets;            // register sets of the stage
};

// Circuits that fit one CTA: 2^n amplitudes of complex64 in shared memory,
// whole gate program, then sum_i <Z_i> (FP64) to out[circuit].
struct ResidentCircuit {
    long long ops_off;
    int nops, sets_off, out_index, n, rl, pad;
};
// A large circuit of a batch: its state's element offset in the arena, its
// qubits, and where its result goes.
struct BigCircuit {
    long long off;
    int n, out_index;
};
// A work item of the one-launch batch: kind 0 = resident circuit res[index];
// kind 1 = tiles k = tile .. tile + ntiles - 1 of stage stages[index] (round
// `round`), where k counts the tiles whose index bits lie in `live` (tile
// index = the bits of k deposited at the set bits of live); it adds ntiles to
// done[dep_done] when finished; kind 2 = chunk `tile` of big[index]'s final
// sum.  It waits until done[dep] >= need first (dep = -1: no wait).
struct BatchItem {
    int kind, index, tile, round, dep, need, dep_done, ntiles;
    unsigned live;
    int pad[3];
};

void launch_batch_resident(int n, int rl, const ResidentCircuit *d_circuits, int count,
                           const RegOp<float> *d_ops, const SetSlots *d_sets, double *d_out,
                           cudaStream_t stream);
// One round: every (stage, tile) work item of the round.  d_items[i] =
// {stage index, tile index}.
void launch_batch_stage(const BatchStage *d_stages, const int2 *d_items, int n_items,
                        const RegOp<float> *d_ops, const SetSlots *d_sets, float2 *arena,
                        cudaStream_t stream);
// out[out_index[c]] = sum_i <Z_i> over 2^n_c amplitudes at arena + off[c];
// FP64; d_partials holds batch_sumz_partials(count) doubles.
size_t batch_sumz_partials(int count);
void launch_batch_sumz(const float2 *arena, const long long *d_off, const int *d_n,
                       const int *d_out_index, int count, double *d_partials, double *d_out,
                       cudaStream_t stream);
void launch_batch_init(float2 *arena, const long long *d_off, int count, cudaStream_t stream);
void batch_prepare();
// The whole batch as one persistent (cooperative) launch of `ctas` CTAs over
// the work items; d_counters: 1 + 2 n_big zeroed ints; *d_status nonzero if a
// bounded wait gave up; partials: batch_sumz_partials(n_big) doubles.
void launch_batch_persistent(const BatchItem *d_items, int n_items, int *d_counters,
                             int n_big, unsigned *d_status, const ResidentCircuit *d_res,
                             const BatchStage *d_stages, const RegOp<float> *d_ops,
                             const SetSlots *d_sets, float2 *arena, const BigCircuit *d_big,
                             double *d_partials, double *d_out, int ctas, cudaStream_t stream);
// CTAs of the persistent launch that fit on the device at once.
int batch_persistent_ctas();

// Engine services for other translation units.
cudaStream_t engine_stream();
void *engine_alloc(size_t bytes);
void engine_free(void *p);

// Descriptor of a lane-permuted gather over a product of states.
struct GatherDesc {
    int nqs;
    const void *ptr[kMaxGetterStates];
    int lane_begin[kMaxGetterStates + 1];  // into ext[]
    signed char ext[kMaxLanes + 2];        // external bit of each local lane
};

// Dense multi-target gate descriptor.
struct MultiDesc {
    int k;                       // targets
    int tpos[kMaxMultiTargets];  // target lanes (matrix bit order)
    int npos;                    // sorted insertion positions (targets + controls)
    int pos[kMaxLanes];
    unsigned long long cmask;
};

// All launchers run asynchronously on `stream`.
void launch_init_basis(int prec, void *state, idx_t n_amps, cudaStream_t stream);
void launch_fill_zero(int prec, void *state, idx_t begin, idx_t end, cudaStream_t stream);
void launch_apply_pairs(int prec, void *state, idx_t n_items, const PairIdx &pi, const Mat2 &m,
                        cudaStream_t stream);
void launch_decohere(int prec, void *state, idx_t n_items, const PairIdx &pi, int value,
                     double norm, cudaStream_t stream);
void launch_reset(int prec, void *state, idx_t n_items, const PairIdx &pi, cudaStream_t stream);
void launch_shrink(int prec, void *dst, const void *src, idx_t n_items, const PairIdx &pi,
                   double norm, cudaStream_t stream);
// srcs[g] == nullptr with basis != nullptr: source g is the basis state
// |basis[g]> (no buffer).
void launch_kron(int prec, void *dst, idx_t n_dst, const void *const *srcs, const int *src_lanes,
                 int n_src, cudaStream_t stream, const long long *basis = nullptr);
// Decohere-and-separate in place: the first 2^(n_lanes-1) amplitudes of
// `state` become norm * (the amplitudes with lane `lane` = value), in order.
void launch_shrink_inplace(int prec, void *state, int n_lanes, int lane, int value, double norm,
                           cudaStream_t stream);
void launch_apply_multi(int prec, void *state, idx_t n_items, const MultiDesc &d,
                        const void *d_mat, cudaStream_t stream);
void launch_stage(int prec, void *state, const StageDesc &d, cudaStream_t stream);

// Reductions: write one FP64 value to d_out (device), using d_partials as
// scratch of at least reduce_partials() doubles.
int reduce_partials();
void launch_prob(int prec, const void *state, idx_t n_items, const PairIdx &pi,
                 double *d_partials, double *d_out, cudaStream_t stream);
void launch_pauli(int prec, const void *state, int n_lanes, unsigned long long x_mask,
                  unsigned long long z_mask, double *d_partials, double *d_out,
                  cudaStream_t stream);

// Getter / pool.
void launch_gather(int prec, int mathop, void *out, idx_t count, idx_t start, idx_t step,
                   unsigned long long empty_mask, const GatherDesc &g, cudaStream_t stream);
// Marginal probabilities (FP64) over 2^n_lanes outputs with n_hidden hidden
// lanes placed above them in the external index.
void launch_marginal(int prec, double *out, int n_lanes, int n_hidden, const GatherDesc &g,
                     double *d_scratch, size_t scratch_doubles, cudaStream_t stream);
size_t marginal_scratch_doubles(int n_lanes, int n_hidden);
void launch_convert_f64(int prec, void *dst, const double *src, idx_t n, cudaStream_t stream);
// Sampling-pool CDF: inclusive prefix sums of round(p * 2^60) as 64-bit
// integers, from a state's |a|^2 in its own lane order or from an FP64
// probability array (cdf may alias prob).  Both return the device address
// of the total, which saturates at 2^64 - 1; pool_status reports a bounded
// wait of the bulk-copy kernels that gave up.
// The scan also fills the pool's guide table when g is set: g[b] = the first
// i with cdf[i] > b * 2^shift, shifted right by index_shift, for b < nb (nb
// must exceed (total - 1) >> shift),
// with runs of more than 8 buckets per item passed through long_list (at most
// long_cap entries; *long_count, zeroed by the caller, above long_cap means
// the table is incomplete and must not be used).
struct PoolGuide {
    unsigned *g;
    unsigned long long nb;
    int shift;
    int index_shift;  // entries hold item >> index_shift (lower bounds)
    unsigned *long_count;
    uint4 *long_list;
    unsigned long_cap;
};
size_t pool_scratch_words(idx_t n);
const unsigned long long *launch_pool_cdf_state(int prec, const void *state, idx_t n,
                                                unsigned long long *cdf,
                                                unsigned long long *scratch,
                                                const PoolGuide &guide, cudaStream_t stream);
const unsigned long long *launch_pool_cdf_prob(const double *prob, idx_t n,
                                               unsigned long long *cdf,
                                               unsigned long long *scratch,
                                               const PoolGuide &guide, cudaStream_t stream);
int pool_status(bool reset);
// guide: the pool's table (nullptr: plain binary search over cdf).
void launch_search(const unsigned long long *cdf, idx_t n, unsigned long long total,
                   const unsigned *guide, int shift, int index_shift, const double *u,
                   long long *obs, idx_t n_samples, const int *empty_pos, int n_empty,
                   cudaStream_t stream);

inline SetSlots make_set_slots(const int *rb, int rl, int m, int prec) {
    SetSlots ss;
    for (auto &v : ss.q) v = 0;
    unsigned mask = 0;
    for (int k = 0; k < rl; ++k) {
        mask |= 1u << rb[k];
        ss.q[k] = (unsigned short)host_swz(1u << rb[k], prec);
    }
    const unsigned tb = ((1u << m) - 1) & ~mask;
    for (unsigned x = 0; x < 32; ++x) ss.lo[x] = (unsigned short)host_swz(host_pdep(x, tb), prec);
    for (unsigned x = 0; x < 16; ++x)
        ss.hi[x] = (unsigned short)host_swz(host_pdep(x << 5, tb), prec);
    return ss;
}

}  // namespace qg

namespace qg {
// Kernel parameters are limited to 32764 bytes (CUDA 12.1+).
static_assert(sizeof(RStageDesc<double>) + 16 <= 32764, "stage descriptor too large");
static_assert(sizeof(AdjStageDesc) + 64 <= 32764, "adjoint descriptor too large");
static_assert(sizeof(TcStageDesc) + 16 <= 32764, "tensor stage descriptor too large");
static_assert(sizeof(StageDesc) + 16 <= 32764, "stage descriptor too large");
}  // namespace qg
