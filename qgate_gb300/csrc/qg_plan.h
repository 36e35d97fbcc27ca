// Host-side planning shared by the gate queue (api.cpp) and the adjoint
// engine (adjoint_host.cpp).
#pragma once

#include <utility>
#include <vector>

#include "qg_internal.h"

namespace qg {

struct PendingGate {
    int target;
    std::vector<int> controls;
    Mat2 m;
    bool diag;
};

// The lanes of a stage's tile: ascending global lanes, the tile position of
// each global lane (-1 outside), and how many lowest lanes are contiguous.
struct TileLanes {
    std::vector<int> lanes;
    int local_of[64];
    int lowrun;
};

unsigned long long gate_qmask(const PendingGate &g);
bool is_diag(const Mat2 &m);
TileLanes tile_lanes_of(unsigned long long S, int n);

// Whether a diagonal gate with unit-modulus entries that has lanes outside
// S and at most one lane in S (a "cross" gate) can run in a stage on lane set
// S: on a tile the lanes outside S are fixed, so it acts as a per-tile phase
// on its one lane in the tile (or a per-tile scalar).
bool cross_gate(const PendingGate &g, unsigned long long S);

// Gates (in order) a stage on lane set S takes, commutation-safe; at most
// `limit` scanned and `max_take` taken.  With `cross`, cross gates count as
// fitting S.  Returns the count; fills take/keep when given.
int stage_take(const std::vector<const PendingGate *> &gates, unsigned long long S, size_t limit,
               std::vector<const PendingGate *> *take, std::vector<const PendingGate *> *keep,
               bool cross = false, int max_take = kMaxStageGates);

// Lane set of the next tensor-core stage over `remaining`: `base` and the
// first gate's lanes, grown to M lanes by the lookahead (multi-start, swap);
// `cross` and `max_take` as for stage_take.
unsigned long long plan_stage_lanes(const std::vector<const PendingGate *> &remaining,
                                    unsigned long long base, int M, bool cross = false,
                                    int max_take = kMaxStageGates);

// Gates a tensor stage of the gate queue may take (its ops hold them as
// block matrices, phase tables and cross records, not as a gate list).
constexpr int kMaxTensorStageGates = 1024;

// Fused 5-lane blocks of a stage's gates: (tile-position lane mask, gates).
// Gates with lanes outside the tile (cross gates) form their own blocks,
// marked by kCrossBlock in the mask (the rest of the mask: their lanes in
// the tile).
typedef std::vector<std::pair<unsigned, std::vector<const PendingGate *>>> TcBlocks;
constexpr unsigned kCrossBlock = 1u << 31;
TcBlocks tc_blocks(const std::vector<const PendingGate *> &gates, const TileLanes &tl);

// Ops of a tensor stage: each fused block is a dense op (a 32x32 unitary on
// the tensor cores); with `phases`, every run of consecutive blocks whose
// gates are all diagonal becomes one phase op instead (their product, a
// diagonal over the union of their lanes, applied elementwise).
// A cross op applies a run of cross gates: per tile, the phase of every
// amplitude is a product of one factor per tile lane (which of two by the
// lane's bit) and a scalar, formed on the GPU from the gates' angles and the
// tile's bits outside the tile lanes.
struct TcOp {
    bool phase;
    unsigned lanes;  // tile-position mask
    std::vector<const PendingGate *> gates;
    bool cross = false;
};
typedef std::vector<TcOp> TcOps;
TcOps tc_ops(const TcBlocks &blocks, bool phases);
inline bool tc_dense(const TcOp &op) { return !op.phase && !op.cross; }
// Operand bytes of an op: 16 KB for a dense op (Bh, Bl), 8 bytes per entry of
// a phase table (2^lanes complex64 phases), a header and 32 bytes per gate
// for a cross op.
size_t tc_op_bytes(const TcOp &op);
// How many ops from ops[b0] one launch holds (their operands and slot tables
// in the shared memory a tensor-stage launch leaves for them).
int tc_ops_per_launch(const TcOps &ops, size_t b0);

// Host plan of one tensor-stage launch over ops [b0, b0 + nb): the
// descriptor (all but the operand pointer) and the ops' operands in `buf`
// (dense ops first, then the phase tables; desc.ops_bytes in all).
void tc_plan_launch(const TileLanes &tl, int n, const TcOps &ops, size_t b0, int nb,
                    TcStageDesc &desc, unsigned char *buf);

// Whether complex64 stages run on the tensor cores (the gate queue's setting).
bool tensor_stages_enabled();

}  // namespace qg
