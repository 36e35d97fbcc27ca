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

// Gates (in order) a stage on lane set S takes, commutation-safe; at most
// `limit` scanned.  Returns the count; fills take/keep when given.
int stage_take(const std::vector<const PendingGate *> &gates, unsigned long long S, size_t limit,
               std::vector<const PendingGate *> *take, std::vector<const PendingGate *> *keep);

// Lane set of the next tensor-core stage over `remaining`: `base` and the
// first gate's lanes, grown to M lanes by the lookahead (multi-start, swap).
unsigned long long plan_stage_lanes(const std::vector<const PendingGate *> &remaining,
                                    unsigned long long base, int M);

// Fused 5-lane blocks of a stage's gates: (tile-position lane mask, gates).
typedef std::vector<std::pair<unsigned, std::vector<const PendingGate *>>> TcBlocks;
TcBlocks tc_blocks(const std::vector<const PendingGate *> &gates, const TileLanes &tl);

// Ops of a tensor stage: each fused block is a dense op (a 32x32 unitary on
// the tensor cores); with `phases`, every run of consecutive blocks whose
// gates are all diagonal becomes one phase op instead (their product, a
// diagonal over the union of their lanes, applied elementwise).
struct TcOp {
    bool phase;
    unsigned lanes;  // tile-position mask
    std::vector<const PendingGate *> gates;
};
typedef std::vector<TcOp> TcOps;
TcOps tc_ops(const TcBlocks &blocks, bool phases);
// Operand bytes of an op: 16 KB for a dense op (Bh, Bl), 8 bytes per entry of
// a phase table (2^lanes complex64 phases).
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
