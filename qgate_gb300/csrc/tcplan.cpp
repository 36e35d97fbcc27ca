// Host-side planning shared by the gate queue (api.cpp) and the adjoint
// engine (adjoint_host.cpp): tiles, stage lane sets, and the fused 5-lane
// blocks of tensor-core stages with their split FP16 operands.
#include "qg_plan.h"

#include <algorithm>
#include <complex>
#include <cstring>
#include <cmath>

namespace qg {

unsigned long long gate_qmask(const PendingGate &g) {
    unsigned long long q = 1ULL << g.target;
    for (int c : g.controls) q |= 1ULL << c;
    return q;
}

bool is_diag(const Mat2 &m) {
    return m.v[2] == 0. && m.v[3] == 0. && m.v[4] == 0. && m.v[5] == 0.;
}


TileLanes tile_lanes_of(unsigned long long S, int n) {
    TileLanes tl;
    for (int q = 0; q < n; ++q)
        if (S & (1ULL << q)) tl.lanes.push_back(q);
    for (int i = 0; i < 64; ++i) tl.local_of[i] = -1;
    for (int i = 0; i < (int)tl.lanes.size(); ++i) tl.local_of[tl.lanes[i]] = i;
    tl.lowrun = 0;
    while (tl.lowrun < (int)tl.lanes.size() && tl.lanes[tl.lowrun] == tl.lowrun) ++tl.lowrun;
    return tl;
}


// A diagonal gate whose two entries have modulus 1 (so they are phases).
static bool unit_diag(const PendingGate &g) {
    if (!g.diag) return false;
    auto unit = [](double re, double im) { return std::fabs(re * re + im * im - 1.) < 1e-12; };
    return unit(g.m.v[0], g.m.v[1]) && unit(g.m.v[6], g.m.v[7]);
}

bool cross_gate(const PendingGate &g, unsigned long long S) {
    const unsigned long long q = gate_qmask(g);
    return (q & ~S) && __builtin_popcountll(q & S) <= 1 && unit_diag(g);
}

// Gates of `gates` (in order) that a stage on lane set S takes: a gate is
// taken when its lanes lie in S (or, with `cross`, it is a cross gate) and
// no earlier gate that was left out shares a lane with it (so it commutes
// with everything left out before it).  At most `limit` gates are scanned
// and `max_take` taken; returns the count.
int stage_take(const std::vector<const PendingGate *> &gates, unsigned long long S,
               size_t limit, std::vector<const PendingGate *> *take,
               std::vector<const PendingGate *> *keep, bool cross, int max_take) {
    unsigned long long blocked = 0;
    int count = 0;
    for (size_t i = 0; i < gates.size(); ++i) {
        const PendingGate *g = gates[i];
        if (i >= limit) {
            if (!keep) break;
            keep->push_back(g);
            continue;
        }
        const unsigned long long q = gate_qmask(*g);
        const bool fits = !(q & ~S) || (cross && cross_gate(*g, S));
        if ((q & blocked) || !fits || count >= max_take) {
            blocked |= q;
            if (keep) keep->push_back(g);
            continue;
        }
        ++count;
        if (take) take->push_back(g);
    }
    return count;
}


// stage_take's count over precomputed lane masks (xd: the gate is a
// unit-modulus diagonal, so a cross gate wherever at most one of its lanes
// is in S): the same walk, stopped once every lane of S is blocked (without
// cross gates no later gate can be taken then).
static int take_count(const std::vector<unsigned long long> &q, const std::vector<char> &xd,
                      unsigned long long S, bool cross, int max_take) {
    unsigned long long blocked = 0;
    int count = 0;
    for (size_t i = 0; i < q.size(); ++i) {
        const unsigned long long g = q[i];
        const bool fits = !(g & ~S) || (cross && xd[i] && __builtin_popcountll(g & S) <= 1);
        if ((g & blocked) || !fits || count >= max_take) {
            blocked |= g;
            if (!cross && (blocked & S) == S) break;
            continue;
        }
        ++count;
    }
    return count;
}

// Lane set (M lanes, including `base` and the first gate's lanes) of the next
// tensor-core stage over `remaining` (see flush_lookahead).
unsigned long long plan_stage_lanes(const std::vector<const PendingGate *> &remaining,
                                    unsigned long long base, int M, bool cross, int max_take) {
    const size_t kWindow = 512;
    const unsigned long long q0 = gate_qmask(*remaining[0]);
    unsigned long long cand_all = 0;
    std::vector<unsigned long long> qw;
    std::vector<char> xd;
    qw.reserve(std::min(remaining.size(), kWindow));
    for (size_t i = 0; i < remaining.size() && i < kWindow; ++i) {
        qw.push_back(gate_qmask(*remaining[i]));
        xd.push_back(cross && unit_diag(*remaining[i]));
        cand_all |= qw.back();
    }
    auto stage_take = [&](const std::vector<const PendingGate *> &, unsigned long long S, size_t,
                          std::nullptr_t, std::nullptr_t) {
        return take_count(qw, xd, S, cross, max_take);
    };
    const unsigned long long fixed = base | q0;
    // Greedy growth from `S0`: add the lane that lets the stage take the
    // most gates until the stage has M lanes.
    auto grow = [&](unsigned long long S0) {
        unsigned long long S = S0;
        while (__builtin_popcountll(S) < M) {
            const unsigned long long cand = cand_all & ~S;
            if (!cand) break;
            int best = -1, best_lane = -1;
            for (unsigned long long c = cand; c; c &= c - 1) {
                const int lane = __builtin_ctzll(c);
                const int got =
                    stage_take(remaining, S | (1ULL << lane), kWindow, nullptr, nullptr);
                if (got > best) {
                    best = got;
                    best_lane = lane;
                }
            }
            S |= 1ULL << best_lane;
        }
        return S;
    };
    // Multi-start: the plain greedy growth, and growths seeded with each
    // of the few lanes that take the most gates on their own; keep the
    // best.
    unsigned long long S = grow(fixed);
    int cur = stage_take(remaining, S, kWindow, nullptr, nullptr);
    {
        std::vector<std::pair<int, int>> seeds;
        for (unsigned long long c = cand_all & ~fixed; c; c &= c - 1) {
            const int lane = __builtin_ctzll(c);
            seeds.emplace_back(
                -stage_take(remaining, fixed | (1ULL << lane), kWindow, nullptr, nullptr), lane);
        }
        std::sort(seeds.begin(), seeds.end());
        for (size_t k = 0; k < seeds.size() && k < 6 && __builtin_popcountll(fixed) < M; ++k) {
            const unsigned long long T = grow(fixed | (1ULL << seeds[k].second));
            const int got = stage_take(remaining, T, kWindow, nullptr, nullptr);
            if (got > cur) {
                S = T;
                cur = got;
            }
        }
    }
    // Swap pass: replace a chosen lane (not a low lane or one of the
    // first gate's) by an outside lane while that lets the stage take
    // more gates.
    {
        const unsigned long long cand = cand_all;
        for (int iter = 0; iter < 16; ++iter) {
            bool improved = false;
            for (unsigned long long o = S & ~fixed; o && !improved; o &= o - 1) {
                const unsigned long long out = o & (0ULL - o);
                for (unsigned long long c = cand & ~S; c; c &= c - 1) {
                    const unsigned long long in = c & (0ULL - c);
                    const unsigned long long T = (S & ~out) | in;
                    const int got = stage_take(remaining, T, kWindow, nullptr, nullptr);
                    if (got > cur) {
                        S = T;
                        cur = got;
                        improved = true;
                        break;
                    }
                }
            }
            if (!improved) break;
        }
    }
    return S;
}

// ------------------------------------------------------------ tensor-core stages

// Register layout of a tile: thread r holds row r (bits i of r at tile
// positions rows[i]), register pair j holds amplitude j (bits k of j at
// tile positions amps[k]).
struct TcLayout {
    int rows[8];
    int amps[5];
};

// Operand layout of a block (tile index -> operand slot; a slot is one
// complex amplitude as f16x2, 4 bytes): the canonical K-major layout with the
// 128-byte swizzle.  Before the swizzle, row r of a 128-row group is 128
// contiguous bytes (its 32 amplitudes: amps[0..4] -> slot bits 0..4), rows
// r % 8 -> bits 5..7 (128 bytes apart), r / 8 -> bits 8..11 (8-row atoms of
// 1024 bytes, the stride byte offset), rows[7] -> bit 12 (second 128-row
// group, 16384 bytes); r's bits are rows[0..6].  The swizzle XORs the 16-byte
// chunk index (slot bits 2..4) with r % 8 (slot bits 5..7).  All of it is a
// GF(2)-linear map of the tile index.
static unsigned tc_operand_slot(const TcLayout &L, unsigned tidx) {
    unsigned c = 0;
    for (int k = 0; k < 5; ++k)
        if (tidx >> L.amps[k] & 1u) c |= 1u << k;
    for (int i = 0; i < 8; ++i)
        if (L.rows[i] >= 0 && (tidx >> L.rows[i] & 1u)) c |= 1u << (i < 7 ? 5 + i : 12);
    return c ^ (((c >> 5) & 7u) << 2);
}

template <class F> static SetSlots tc_slots(const TcLayout &src, int t, F dst) {
    SetSlots ss;
    memset(&ss, 0, sizeof(ss));
    auto dep = [&](unsigned x) {
        unsigned ti = 0;
        for (int i = 0; i < t; ++i)
            if (x >> i & 1u) ti |= 1u << src.rows[i];
        return ti;
    };
    for (unsigned x = 0; x < 32; ++x) ss.lo[x] = (unsigned short)dst(dep(x));
    for (unsigned x = 0; x < 16 && (x << 5) < (1u << t); ++x)
        ss.hi[x] = (unsigned short)dst(dep(x << 5));
    for (int k = 0; k < 5; ++k) ss.q[k] = (unsigned short)dst(1u << src.amps[k]);
    return ss;
}

// IEEE binary16 bits of x, rounded to nearest even (subnormals kept).
static unsigned short f16_bits(float x) {
    unsigned f;
    memcpy(&f, &x, 4);
    const unsigned sign = (f >> 16) & 0x8000u;
    const unsigned a = f & 0x7fffffffu;
    if (a - 0x38800000u < 0x477ff000u - 0x38800000u) {
        // normal binary16 range (2^-14 <= |x| < 65520): round to nearest
        // even at bit 13 with one add, then rebias the exponent (127 -> 15)
        const unsigned r = a + 0xfffu + ((a >> 13) & 1u);
        return (unsigned short)(sign | ((r - 0x38000000u) >> 13));
    }
    const int e = (int)((f >> 23) & 0xffu) - 127 + 15;
    unsigned mant = f & 0x7fffffu;
    if (e >= 31) return (unsigned short)(sign | 0x7c00u);
    if (e <= 0) {
        if (e < -10) return (unsigned short)sign;
        mant |= 0x800000u;
        const int shift = 14 - e;
        unsigned hm = mant >> shift;
        const unsigned rem = mant & ((1u << shift) - 1u), half = 1u << (shift - 1);
        if (rem > half || (rem == half && (hm & 1u))) ++hm;
        return (unsigned short)(sign | hm);
    }
    unsigned out = ((unsigned)e << 10) | (mant >> 13);
    const unsigned rem = mant & 0x1fffu;
    if (rem > 0x1000u || (rem == 0x1000u && (out & 1u))) ++out;
    return (unsigned short)(sign | out);
}

static double f16_value(unsigned short h) {
    const unsigned e = (h >> 10) & 31u, mant = h & 1023u;
    float v;
    if (e == 0) {
        v = (float)mant * 5.9604644775390625e-8f;  // subnormal: mant * 2^-24, exact
    } else {
        const unsigned bits = ((e + 112u) << 23) | (mant << 13);  // rebias 15 -> 127
        memcpy(&v, &bits, 4);
    }
    return (h & 0x8000u) ? -(double)v : (double)v;
}

// Split operand of a 32x32 complex block U (row-major, amplitude order of
// the block layout): B[k][n] of D = A B with A[r][2i + c] = (Re, Im) V[r][i]
// and D[r][2o + c] = (Re, Im) (U V[r])[o], stored K-major (row n holds its
// K elements) in the canonical no-swizzle layout: element (n, k) at FP16
// index (k / 16) * 1024 + (k % 16 / 8) * 512 + (n / 8) * 64 + (n % 8) * 8 +
// k % 8.  Bh = f16(B), Bl = f16(B - Bh), both rounded to nearest.
static void tc_operand(const std::complex<double> *U, unsigned short *bh, unsigned short *bl) {
    for (int o = 0; o < 32; ++o)
        for (int i = 0; i < 32; ++i) {
            const double re = U[o * 32 + i].real(), im = U[o * 32 + i].imag();
            const double val[2][2] = {{re, -im}, {im, re}};  // [c_out][c_in]
            for (int co = 0; co < 2; ++co)
                for (int ci = 0; ci < 2; ++ci) {
                    const int n = 2 * o + co, k = 2 * i + ci;
                    const size_t at = (size_t)(k / 16) * 1024 + (k % 16 / 8) * 512 +
                                      (n / 8) * 64 + (n % 8) * 8 + k % 8;
                    const double x = val[co][ci];
                    const unsigned short h = f16_bits((float)x);
                    bh[at] = h;
                    bl[at] = f16_bits((float)(x - f16_value(h)));
                }
        }
}

// Bias compensation for the tensor core's accumulator.  The FP32 accumulator
// of tcgen05.mma rounds toward zero at every MMA, so each output shrinks in
// magnitude by half an ulp per rounding on average; the kernel orders the
// MMAs so that only the main product's K-steps round at full magnitude, and
// an output whose inputs span c of the four K-steps sees roundings at about
// 1/c, 2/c, ..., 1 of its final value: an expected relative shrink of
// (c + 1) / 4 * kRzShrink, kRzShrink being the mean relative shrink of one
// rounding at full magnitude.  Model: a truncation of x with a uniform
// discarded part loses ulp(x) / 2; weighted by |x|^2 over mantissas m in
// [1, 2) of density 1 / (m ln 2), one truncation loses 2^-24 E[m] / E[m^2] =
// 2^-24 * 2/3 = 4.0e-8 of the norm's magnitude, and a dense row (c = 4) about
// 2.5 of those (9.9e-8).  Measured on GB300 from the norm drift of dense
// blocks: 7.25e-8 per block for c = 4 (0.73 of the model; the accumulator
// keeps some guard bits), which fixes the constant below.  Each row of U is
// scaled up by that amount, which removes the drift (it would otherwise
// shrink the norm by ~1.5e-7 per block); the remaining error is unbiased.
// Diagonal runs never reach this path: they become phase ops, which do not
// round in the tensor core.
constexpr double kRzShrink = 5.8e-8;

static void tc_compensate(std::complex<double> *U) {
    for (int o = 0; o < 32; ++o) {
        int c = 0;
        for (int ks = 0; ks < 4; ++ks) {
            bool nz = false;
            for (int i = 8 * ks; i < 8 * ks + 8; ++i) nz |= U[o * 32 + i] != 0.;
            c += nz;
        }
        if (c == 0) continue;
        const double f = 1. + 0.25 * (c + 1) * kRzShrink;
        for (int i = 0; i < 32; ++i) U[o * 32 + i] *= f;
    }
}

// Greedy 5-lane blocks over a stage's gates in order: a gate joins the open
// block when its lanes fit and no earlier deferred gate shares a lane (so it
// commutes with everything deferred); the rest start the next block.
// Cross gates (lanes outside the tile) never join a block; a cross gate
// keeps the later non-diagonal gates of its tile lane out of the blocks
// (diagonal gates commute with it).  Cross gates are left as late as
// possible, so that few cross ops hold them all: only when no block can take
// a gate, every cross gate that no earlier remaining non-diagonal gate shares
// its tile lane with forms a cross block.  Without cross gates this is the
// plain greedy walk.
TcBlocks tc_blocks(const std::vector<const PendingGate *> &gates, const TileLanes &tl) {
    std::vector<std::pair<unsigned, std::vector<const PendingGate *>>> out;
    std::vector<const PendingGate *> rem(gates);
    // tile-position mask of g's lanes in the tile; false if some lane is outside
    auto tile_mask = [&](const PendingGate *g, unsigned &q) {
        bool in = true;
        q = 0;
        const int pt = tl.local_of[g->target];
        if (pt < 0) in = false;
        else q |= 1u << pt;
        for (int c : g->controls) {
            const int pc = tl.local_of[c];
            if (pc < 0) in = false;
            else q |= 1u << pc;
        }
        return in;
    };
    while (!rem.empty()) {
        unsigned L = 0, blocked = 0, blocked_nd = 0;
        std::vector<const PendingGate *> take, keep;
        for (auto *g : rem) {
            unsigned q;
            if (!tile_mask(g, q)) {
                keep.push_back(g);
                blocked_nd |= q;
                continue;
            }
            if ((q & blocked) || (!g->diag && (q & blocked_nd)) || __builtin_popcount(L | q) > 5) {
                keep.push_back(g);
                blocked |= q;
                continue;
            }
            L |= q;
            take.push_back(g);
        }
        if (!take.empty()) {
            out.emplace_back(L, std::move(take));
            rem.swap(keep);
            continue;
        }
        // no block can take a gate: the cross gates that can go now
        unsigned nd = 0;
        L = 0;
        take.clear();
        keep.clear();
        for (auto *g : rem) {
            unsigned q;
            if (tile_mask(g, q)) {
                if (!g->diag) nd |= q;
                keep.push_back(g);
            } else if (q & nd) {
                keep.push_back(g);
            } else {
                L |= q;
                take.push_back(g);
            }
        }
        out.emplace_back(L | kCrossBlock, std::move(take));
        rem.swap(keep);
    }
    return out;
}

// Orders a block's lanes and rows so that the stores into its operand hit
// distinct banks.  The bank of a slot is bits 0..4 of tc_operand_slot:
// amps[0], amps[1], amps[2] ^ rows[0], amps[3] ^ rows[1], amps[4] ^ rows[2];
// a warp's threads differ in the source layout's rows[0..4] (W), so the
// stores are conflict-free when W's lanes drive the five bank bits one each:
// two W lanes of the block as amps[0..1], further W lanes of the block as
// amps[2..4], and W's other lanes as the rows[k] whose amps[k + 2] is not a W
// lane.  That works whenever the block holds at least two W lanes.  rows[3..4]
// are then chosen so that the next block can do the same (at least two of
// this layout's rows[0..4] among its lanes).
static TcLayout tc_choose_layout(unsigned lanes, unsigned next_lanes, const TcLayout &src, int m) {
    unsigned W = 0;
    for (int x = 0; x < 5; ++x) W |= 1u << src.rows[x];
    auto in_w = [&](int p) { return (W >> p & 1u) != 0; };
    auto nxt = [&](int p) { return (next_lanes >> p & 1u) != 0; };
    std::vector<int> Lw, Lo, Rw, Ro;
    for (int p = 0; p < m; ++p) {
        if (lanes >> p & 1u) (in_w(p) ? Lw : Lo).push_back(p);
        else (in_w(p) ? Rw : Ro).push_back(p);
    }
    // Rows outside W: lanes outside the next block first (they keep the next
    // block's choice free); W rows: lanes of the next block last.
    std::stable_sort(Ro.begin(), Ro.end(), [&](int p, int q) { return !nxt(p) && nxt(q); });
    TcLayout c;
    for (int x = 0; x < 8; ++x) c.rows[x] = -1;
    // amps: W lanes first (the first two are amps[0..1]).
    std::vector<int> A(Lw);
    A.insert(A.end(), Lo.begin(), Lo.end());
    for (int k = 0; k < 5; ++k) c.amps[k] = A[k];
    // rows[0..2]: a W row where amps[k + 2] is not a W lane, else a non-W row.
    size_t iw = 0, io = 0;
    std::vector<bool> used_o(Ro.size(), false);
    for (int k = 0; k < 3; ++k) {
        if (!in_w(c.amps[k + 2]) && iw < Rw.size()) {
            c.rows[k] = Rw[iw++];
        } else if (io < Ro.size()) {
            used_o[io] = true;
            c.rows[k] = Ro[io++];
        } else {
            c.rows[k] = Rw[iw++];
        }
    }
    std::vector<int> rest;
    for (; iw < Rw.size(); ++iw) rest.push_back(Rw[iw]);
    for (size_t x = io; x < Ro.size(); ++x) rest.push_back(Ro[x]);
    // rows[3..4]: top up to two lanes of the next block among rows[0..4].
    int inext = 0;
    for (int x = 0; x < 3; ++x) inext += nxt(c.rows[x]);
    std::stable_sort(rest.begin(), rest.end(), [&](int p, int q) {
        return inext < 2 ? (nxt(p) && !nxt(q)) : (!nxt(p) && nxt(q));
    });
    for (size_t x = 0; x < rest.size(); ++x) c.rows[3 + x] = rest[x];
    return c;
}

// U (32x32, row-major) of a block's gates in the amplitude order of `lay`.
static void tc_block_matrix(const std::vector<const PendingGate *> &gates, const TileLanes &tl,
                            const TcLayout &lay, std::complex<double> *U) {
    typedef std::complex<double> cd;
    int bit_of[64];
    for (int p = 0; p < 64; ++p) bit_of[p] = -1;
    for (int k = 0; k < 5; ++k) bit_of[lay.amps[k]] = k;
    for (int i = 0; i < 1024; ++i) U[i] = (i / 32 == i % 32) ? cd(1, 0) : cd(0, 0);
    for (auto *g : gates) {
        const int tb = 1 << bit_of[tl.local_of[g->target]];
        int cm = 0;
        for (int c : g->controls) cm |= 1 << bit_of[tl.local_of[c]];
        const cd m00(g->m.v[0], g->m.v[1]), m01(g->m.v[2], g->m.v[3]), m10(g->m.v[4], g->m.v[5]),
            m11(g->m.v[6], g->m.v[7]);
        for (int r = 0; r < 32; ++r) {
            if ((r & tb) || (r & cm) != cm) continue;
            for (int c = 0; c < 32; ++c) {
                cd a0 = U[r * 32 + c], a1 = U[(r | tb) * 32 + c];
                U[r * 32 + c] = m00 * a0 + m01 * a1;
                U[(r | tb) * 32 + c] = m10 * a0 + m11 * a1;
            }
        }
    }
}

// Fills a block of fewer than 5 lanes: lanes of the source layout's warp
// bits first (two of them keep its operand stores conflict-free), then the
// lowest free positions.
static unsigned tc_fill_lanes(unsigned lanes, const TcLayout &src, int m) {
    for (int x = 0; x < 5 && __builtin_popcount(lanes) < 5; ++x) {
        unsigned in_warp = 0;
        for (int y = 0; y < 5; ++y) in_warp += lanes >> src.rows[y] & 1u;
        if (in_warp >= 2) break;
        lanes |= 1u << src.rows[x];
    }
    for (int p = 0; p < m && __builtin_popcount(lanes) < 5; ++p) lanes |= 1u << p;
    return lanes;
}

// Tile positions 0..3 (global lanes 0..3: the sixteen amplitudes of a
// 128-byte line) on a warp's row bits make its row stores two whole lines
// per instruction, as the load layout's loads are.  (Positions 0 and 1 alone,
// eight whole 32-byte sectors per instruction, measured slower than the trip
// through the natural tile.)
constexpr unsigned kDirectLow = 15u;

// tc_fill_lanes that never adds the positions in `avoid`.
static unsigned tc_fill_lanes_avoiding(unsigned lanes, const TcLayout &src, int m,
                                       unsigned avoid) {
    for (int x = 0; x < 5 && __builtin_popcount(lanes) < 5; ++x) {
        unsigned in_warp = 0;
        for (int y = 0; y < 5; ++y) in_warp += lanes >> src.rows[y] & 1u;
        if (in_warp >= 2) break;
        if (avoid >> src.rows[x] & 1u) continue;
        lanes |= 1u << src.rows[x];
    }
    for (int p = 0; p < m && __builtin_popcount(lanes) < 5; ++p)
        if (!(avoid >> p & 1u)) lanes |= 1u << p;
    return lanes;
}

// Moves tile position p to rows[x] (swapping with whatever was there).
static void tc_place_row(TcLayout &c, int p, int x) {
    for (int i = 0; i < 8; ++i)
        if (c.rows[i] == p) {
            std::swap(c.rows[i], c.rows[x]);
            return;
        }
}

// Shared-memory wavefronts of one warp-wide 4-byte store through slot
// tables: the largest number of threads on one bank.
static int tc_store_cost(const SetSlots &ss) {
    int cnt[32] = {0};
    int mx = 0;
    for (int i = 0; i < 32; ++i) mx = std::max(mx, ++cnt[ss.lo[i] & 31]);
    return mx;
}

// Wavefronts of one warp-wide 8-byte store through slot tables (two half
// warps; per half, the largest number of threads on one 8-byte bank pair).
static int tc_store_cost8(const SetSlots &ss) {
    int cost = 0;
    for (int h = 0; h < 2; ++h) {
        int cnt[16] = {0}, mx = 0;
        for (int i = 0; i < 16; ++i) mx = std::max(mx, ++cnt[ss.lo[16 * h + i] & 15]);
        cost += mx;
    }
    return cost;
}

// ---------------------------------------------------------------- stage ops

TcOps tc_ops(const TcBlocks &blocks, bool phases) {
    TcOps out;
    for (const auto &bl : blocks) {
        if (bl.first & kCrossBlock) {
            const unsigned lanes = bl.first & ~kCrossBlock;
            if (!out.empty() && out.back().cross) {
                out.back().lanes |= lanes;
                out.back().gates.insert(out.back().gates.end(), bl.second.begin(), bl.second.end());
                continue;
            }
            TcOp op;
            op.phase = false;
            op.cross = true;
            op.lanes = lanes;
            op.gates = bl.second;
            out.push_back(std::move(op));
            continue;
        }
        bool diag = phases;
        for (auto *g : bl.second) diag = diag && g->diag;
        if (diag && !out.empty() && out.back().phase) {
            out.back().lanes |= bl.first;
            out.back().gates.insert(out.back().gates.end(), bl.second.begin(), bl.second.end());
            continue;
        }
        TcOp op;
        op.phase = diag;
        op.lanes = bl.first;
        op.gates = bl.second;
        out.push_back(std::move(op));
    }
    return out;
}

size_t tc_op_bytes(const TcOp &op) {
    if (op.cross) return sizeof(TcCrossHdr) + sizeof(TcCrossRec) * op.gates.size();
    return op.phase ? (size_t)8 << __builtin_popcount(op.lanes) : (size_t)2 * 64 * 64 * 2;
}

// Shared memory a launch has for its ops' operands and slot tables: the
// opt-in maximum (227 KB) less 2 KB of static shared memory, 128 KB of tile
// operands (4 groups x 2 x 16 KB for 12-lane tiles, 2 x 2 x 32 KB for 13-lane
// tiles; 3 groups of the two-threads-per-row variant take less) and the two
// natural-tile slot tables.
constexpr size_t kTcOpsBudget = 227 * 1024 - 2048 - 128 * 1024 - 2 * sizeof(SetSlots);

int tc_ops_per_launch(const TcOps &ops, size_t b0) {
    size_t used = 0;
    int nb = 0;
    while (b0 + nb < ops.size() && nb < kMaxTcBlocks) {
        const size_t add = tc_op_bytes(ops[b0 + nb]) + sizeof(SetSlots);
        if (nb > 0 && used + add > kTcOpsBudget) break;
        used += add;
        ++nb;
    }
    return nb;
}

// Table of a phase op: entry idx (bit k of idx = tile position order[k]) is
// the product of the op's diagonal gates' entries at that assignment of
// their lanes (m00 or m11 of a gate whose controls are all set, else 1),
// computed in FP64 and rounded to complex64.
static void tc_phase_table(const TcOp &op, const TileLanes &tl, const std::vector<int> &order,
                           float *table) {
    typedef std::complex<double> cd;
    const int u = (int)order.size();
    int bit_of[64];
    for (int p = 0; p < 64; ++p) bit_of[p] = -1;
    for (int k = 0; k < u; ++k) bit_of[order[k]] = k;
    for (unsigned idx = 0; idx < (1u << u); ++idx) {
        cd ph(1., 0.);
        for (auto *g : op.gates) {
            bool on = true;
            for (int c : g->controls) on = on && (idx >> bit_of[tl.local_of[c]] & 1u);
            if (!on) continue;
            ph *= (idx >> bit_of[tl.local_of[g->target]] & 1u) ? cd(g->m.v[6], g->m.v[7])
                                                               : cd(g->m.v[0], g->m.v[1]);
        }
        table[2 * idx] = (float)ph.real();
        table[2 * idx + 1] = (float)ph.imag();
    }
}

// Host plan of one tensor-stage launch: ops [b0, b0 + nb) of a stage on tile
// `tl` -> the descriptor (all but the operand pointer) and the ops' operands
// in `buf`.
static void tc_plan_launch_ordered(const TileLanes &tl, int n, const TcOps &ops, size_t b0,
                                   int nb, TcStageDesc &desc, unsigned char *buf);

// Header and records of a cross op in the layout `lay` it runs in: one record
// per gate (its two phases as angles), by the tile position of its one lane
// in the tile (the scalar records last).
static void tc_cross_records(const TcOp &op, const TileLanes &tl, const TcLayout &lay,
                             unsigned char *out) {
    const int m = (int)tl.lanes.size();
    TcCrossHdr hdr;
    memset(&hdr, 0, sizeof(hdr));
    std::vector<std::vector<TcCrossRec>> bucket(m + 1);
    for (const PendingGate *g : op.gates) {
        TcCrossRec r;
        memset(&r, 0, sizeof(r));
        r.a0 = (float)std::atan2(g->m.v[1], g->m.v[0]);
        r.a1 = (float)std::atan2(g->m.v[7], g->m.v[6]);
        int p = m;
        if (tl.local_of[g->target] >= 0) {
            p = tl.local_of[g->target];
        } else {
            r.tgt = 1LL << g->target;
        }
        for (int c : g->controls) {
            if (tl.local_of[c] >= 0) p = tl.local_of[c];
            else r.need |= 1LL << c;
        }
        bucket[p].push_back(r);
    }
    TcCrossRec *rec = (TcCrossRec *)(out + sizeof(TcCrossHdr));
    int k = 0;
    for (int p = 0; p <= m; ++p) {
        hdr.start[p] = k;
        for (const TcCrossRec &r : bucket[p]) rec[k++] = r;
    }
    for (int p = m + 1; p < 15; ++p) hdr.start[p] = k;
    hdr.nrec = k;
    for (int b = 0; b < 8; ++b) hdr.rows[b] = (signed char)lay.rows[b];
    for (int j = 0; j < 5; ++j) hdr.amps[j] = (signed char)lay.amps[j];
    memcpy(out, &hdr, sizeof(hdr));
}

void tc_plan_launch(const TileLanes &tl, int n, const TcOps &ops, size_t b0, int nb,
                    TcStageDesc &desc, unsigned char *buf) {
    // The launch's ops in an order that ends with a dense op leaving tile
    // positions 0..3 to the rows (its rows then go straight to the state):
    // a dense op moves to the end when it shares no lane with any op after
    // it (disjoint ops commute), the latest such op first.
    TcOps slice(ops.begin() + b0, ops.begin() + b0 + nb);
    int last = -1;
    for (int b = nb - 1; b >= 0 && last < 0; --b)
        if (tc_dense(slice[b])) last = b;
    if (last >= 0 && (slice[last].lanes & kDirectLow)) {
        for (int x = last - 1; x >= 0; --x) {
            if (!tc_dense(slice[x]) || (slice[x].lanes & kDirectLow)) continue;
            bool disjoint = true;
            for (int y = x + 1; y < nb && disjoint; ++y) disjoint = !(slice[y].lanes & slice[x].lanes);
            if (disjoint) {
                TcOp mv = slice[x];
                slice.erase(slice.begin() + x);
                slice.push_back(mv);
                break;
            }
        }
    }
    tc_plan_launch_ordered(tl, n, slice, 0, nb, desc, buf);
}

static void tc_plan_launch_ordered(const TileLanes &tl, int n, const TcOps &ops, size_t b0,
                                   int nb, TcStageDesc &desc, unsigned char *buf) {
    const int m = (int)tl.lanes.size();
    const int t = m - 5;
    memset(&desc, 0, sizeof(desc));
    desc.n = n;
    desc.m = m;
    desc.nins = m < n ? m : 0;
    for (int j = 0; j < desc.nins; ++j) desc.ins_pos[j] = tl.lanes[j];
    desc.nblocks = nb;
    {
        // operand offsets: dense ops first (16 KB each, keeping the 1024-byte
        // alignment of their swizzled operands), then the cross ops' records,
        // then the phase tables
        unsigned off = 0;
        auto kind = [&](const TcOp &op) { return tc_dense(op) ? 0 : (op.cross ? 1 : 2); };
        for (int pass = 0; pass < 3; ++pass)
            for (int b = 0; b < nb; ++b)
                if (kind(ops[b0 + b]) == pass) {
                    desc.op_off[b] = off;
                    off += (unsigned)tc_op_bytes(ops[b0 + b]);
                }
        desc.ops_bytes = off;
    }
    auto next_dense = [&](int b) -> int {
        for (int x = b + 1; x < nb; ++x)
            if (tc_dense(ops[b0 + x])) return x;
        return -1;
    };
    const int first_dense = !tc_dense(ops[b0]) ? next_dense(0) : 0;
    int last_dense = -1;
    for (int b = 0; b < nb; ++b)
        if (tc_dense(ops[b0 + b])) last_dense = b;
    // Load layout: tile positions 0..3 (the contiguous low lanes) plus one
    // more position p on the warp's thread bits, chosen so that the first
    // dense op's operand stores hit the fewest banks twice.
    auto load_layout = [&](int p) {
        TcLayout L;
        for (int i = 0; i < 8; ++i) L.rows[i] = -1;
        int r = 0, a = 0;
        for (int q = 0; q < 4; ++q) L.rows[r++] = q;
        L.rows[r++] = p;
        for (int q = 4; q < m; ++q) {
            if (q == p) continue;
            if (a < 5) L.amps[a++] = q;
            else L.rows[r++] = q;
        }
        return L;
    };
    TcLayout cur = load_layout(4);
    if (first_dense >= 0) {
        const int nd = next_dense(first_dense);
        const unsigned next0 = nd >= 0 ? ops[b0 + nd].lanes : 0u;
        int best = 1 << 30;
        for (int p = 4; p < m; ++p) {
            TcLayout L = load_layout(p);
            unsigned l0 = tc_fill_lanes(ops[b0 + first_dense].lanes, L, m);
            TcLayout lay = tc_choose_layout(l0, next0, L, m);
            int c = tc_store_cost(tc_slots(L, t, [&](unsigned ti) { return tc_operand_slot(lay, ti); }));
            if (c < best) {
                best = c;
                cur = L;
            }
        }
    }
    // phase-only launches end in the load layout (coalesced by construction)
    bool direct_out = last_dense < 0;
    for (int b = 0; b < t; ++b) desc.row_lane[b] = tl.lanes[cur.rows[b]];
    for (int j = 0; j < 32; ++j) {
        long long off = 0;
        for (int k = 0; k < 5; ++k)
            if (j >> k & 1) off |= 1LL << tl.lanes[cur.amps[k]];
        desc.dep_hi[j] = off;
    }
    for (int k = 0; k < 5; ++k) desc.in_e[k] = desc.dep_hi[1 << k];
    desc.sets[nb + 1] = tc_slots(cur, t, [&](unsigned ti) { return host_swz(ti, kFP32); });
    std::complex<double> U[1024];
    for (int b = 0; b < nb; ++b) {
        const TcOp &op = ops[b0 + b];
        if (op.cross) {
            desc.op_kind[b] = 2;
            tc_cross_records(op, tl, cur, (unsigned char *)(buf + desc.op_off[b]));
            continue;
        }
        if (op.phase) {
            // table index bits: the op's lanes on the warp's thread bits
            // first (a warp then reads few distinct banks), then the others
            std::vector<int> order;
            for (int x = 0; x < 5; ++x)
                if (op.lanes >> cur.rows[x] & 1u) order.push_back(cur.rows[x]);
            for (int p = 0; p < m; ++p)
                if ((op.lanes >> p & 1u) && std::find(order.begin(), order.end(), p) == order.end())
                    order.push_back(p);
            desc.op_kind[b] = 1;
            desc.sets[b] = tc_slots(cur, t, [&](unsigned ti) {
                unsigned idx = 0;
                for (size_t k = 0; k < order.size(); ++k)
                    if (ti >> order[k] & 1u) idx |= 1u << k;
                return idx;
            });
            tc_phase_table(op, tl, order, (float *)(buf + desc.op_off[b]));
            continue;
        }
        // The last dense op stores its rows straight to the state when its
        // block leaves tile positions 0..3 (the low lanes of a 128-byte line)
        // to the rows: those four then go among the warp's row bits.
        const unsigned low = b == last_dense && !(op.lanes & kDirectLow) ? kDirectLow : 0u;
        const bool direct = low != 0u;
        unsigned lanes = direct ? tc_fill_lanes_avoiding(op.lanes, cur, m, low)
                                : tc_fill_lanes(op.lanes, cur, m);
        const int nd = next_dense(b);
        const unsigned next = nd >= 0 ? ops[b0 + nd].lanes : 0u;
        TcLayout lay = tc_choose_layout(lanes, next, cur, m);
        if (direct) {
            // positions 0..3 into rows[0..4], in every choice of slots and
            // order, where the operand stores of this op hit the fewest banks
            // twice
            const int np = __builtin_popcount(low);
            int best = 1 << 30;
            const TcLayout keep = lay;
            for (unsigned mask = 0; mask < 32u; ++mask) {
                if (__builtin_popcount(mask) != np) continue;
                int slots[4], k = 0;
                for (int x = 0; x < 5; ++x)
                    if (mask >> x & 1u) slots[k++] = x;
                int perm[4] = {0, 1, 2, 3};
                do {
                    TcLayout c = keep;
                    for (int i = 0; i < np; ++i) tc_place_row(c, perm[i], slots[i]);
                    const int cost = tc_store_cost(
                        tc_slots(cur, t, [&](unsigned ti) { return tc_operand_slot(c, ti); }));
                    if (cost < best) {
                        best = cost;
                        lay = c;
                    }
                } while (std::next_permutation(perm, perm + np));
            }
            direct_out = true;
        } else if (b == last_dense) {
            // Last dense op: rows[3..4] only feed the 8-byte stores into the
            // natural tile; pick them for the fewest wavefronts there.
            int best = 1 << 30;
            TcLayout keep = lay;
            for (int x = 3; x < t; ++x)
                for (int y = 3; y < t; ++y) {
                    if (x == y) continue;
                    TcLayout c = keep;
                    std::swap(c.rows[3], c.rows[x]);
                    std::swap(c.rows[4], c.rows[y == 3 ? x : y]);
                    const int cost = tc_store_cost8(
                        tc_slots(c, t, [&](unsigned ti) { return host_swz(ti, kFP32); }));
                    if (cost < best) {
                        best = cost;
                        lay = c;
                    }
                }
        }
        desc.op_kind[b] = 0;
        desc.sets[b] = tc_slots(cur, t, [&](unsigned ti) { return tc_operand_slot(lay, ti); });
        tc_block_matrix(op.gates, tl, lay, U);
        tc_compensate(U);
        unsigned short *o = (unsigned short *)(buf + desc.op_off[b]);
        tc_operand(U, o, o + 64 * 64);
        cur = lay;
    }
    desc.sets[nb] = tc_slots(cur, t, [&](unsigned ti) { return host_swz(ti, kFP32); });
    desc.direct_out = direct_out ? 1 : 0;
    for (int b = 0; b < 8; ++b) desc.out_row_lane[b] = b < t ? tl.lanes[cur.rows[b]] : 0;
    for (int k = 0; k < 5; ++k) desc.out_e[k] = 1LL << tl.lanes[cur.amps[k]];
}


}  // namespace qg
