// Host side of the adjoint-differentiation engine: stage planning for a
// batch of parameter vectors, the forward sweep with checkpoints, the
// Pauli-sum observable, and the backward sweep that re-anchors psi at every
// checkpoint.
//
// For U_k = exp(-i c theta_k G) (G a Pauli X/Y/Z on the target, optional
// controls P1):  dE/dtheta_k = 2 c Im<lambda_k| P1 G |psi_k>, where psi_k is
// the state after gate k and lambda_k = U_{k+1}^dagger ... U_N^dagger H psi_N.
// The backward sweep starts from (psi_N, H psi_N) and, gate by gate in
// reverse, takes that inner product and un-applies U_k from both states.
// Rx/Ry/Rz(theta) = exp(-i theta/2 {X,Y,Z}) (c = 1/2) and
// ExpiZ(theta) = exp(+i theta Z) (c = -1) follow the reference's matrices
// (qgate/simulator/src/GateMatrix.cpp:114-141); U3 is Rz(phi) Ry(theta)
// Rz(lambda) (GateMatrix.cpp:14-25) and is decomposed by the caller.
#include "qg_internal.h"
#include "qg_plan.h"
#include "../../include/qgate_gb300.h"

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstring>
#include <vector>

namespace qg {

namespace {

struct Op {
    int kind;  // 0 fixed, 1 rotation
    int target;
    std::vector<int> controls;
    int axis;
    int param;
    double coef;
    double mat[8];
    unsigned long long qmask() const {
        unsigned long long q = 1ULL << target;
        for (int c : controls) q |= 1ULL << c;
        return q;
    }
};

void rotation(int axis, double angle, double *m) {  // exp(-i angle G)
    double c = std::cos(angle), s = std::sin(angle);
    for (int i = 0; i < 8; ++i) m[i] = 0.;
    if (axis == 1) {  // [[c, -is], [-is, c]]
        m[0] = c;
        m[3] = -s;
        m[5] = -s;
        m[6] = c;
    } else if (axis == 2) {  // [[c, -s], [s, c]]
        m[0] = c;
        m[2] = -s;
        m[4] = s;
        m[6] = c;
    } else {  // diag(e^{-i angle}, e^{i angle})
        m[0] = c;
        m[1] = -s;
        m[6] = c;
        m[7] = s;
    }
}

void adjoint_of(const double *m, double *out) {
    out[0] = m[0];
    out[1] = -m[1];
    out[2] = m[4];
    out[3] = -m[5];
    out[4] = m[2];
    out[5] = -m[3];
    out[6] = m[6];
    out[7] = -m[7];
}

bool mat_is_diag(const double *m) { return m[2] == 0. && m[3] == 0. && m[4] == 0. && m[5] == 0.; }
bool mat_is_x(const double *m) {
    static const double x[8] = {0., 0., 1., 0., 1., 0., 0., 0.};
    for (int i = 0; i < 8; ++i)
        if (m[i] != x[i]) return false;
    return true;
}

int op_kind(const Op &o) {
    if (o.kind == 1) return o.axis == 3 ? kOpDiagReg : kOpGate;
    if (mat_is_diag(o.mat)) return kOpDiagReg;
    if (mat_is_x(o.mat)) return kOpSwapX;
    return kOpGate;
}

int op_cost(int kind) { return kind == kOpDiagReg ? 4 : (kind == kOpSwapX ? 2 : 9); }

// Greedy stage packing with commutation-safe deferral (as in the gate queue's
// planner): returns, per stage, its lane set and op indices (in `order`).
struct StagePlan {
    unsigned long long S;
    std::vector<int> ops;
};

std::vector<StagePlan> plan(const std::vector<Op> &ops, const std::vector<int> &order, int n,
                            int M, int rl, int budget, int maxops) {
    std::vector<StagePlan> out;
    const int low = std::min(n, 4);
    const unsigned long long all = n >= 64 ? ~0ULL : ((1ULL << n) - 1);
    const unsigned long long base = (n <= M) ? all : ((1ULL << low) - 1);
    std::vector<int> remaining(order);
    while (!remaining.empty()) {
        unsigned long long S = base, blocked = 0, dense = 0;
        int cost = 0;
        StagePlan st;
        std::vector<int> deferred;
        for (int idx : remaining) {
            const Op &o = ops[idx];
            unsigned long long q = o.qmask();
            int k = op_kind(o);
            unsigned long long dt = dense;
            if (k != kOpDiagReg) dt |= 1ULL << o.target;
            int est = cost + op_cost(k) + 7 * (int)((__builtin_popcountll(dt) + rl - 1) / rl);
            bool over = budget > 0 && !st.ops.empty() && est > budget;
            if ((q & blocked) || (int)st.ops.size() >= maxops || over ||
                __builtin_popcountll(S | q) > M) {
                deferred.push_back(idx);
                blocked |= q;
                continue;
            }
            S |= q;
            cost += op_cost(k);
            dense = dt;
            st.ops.push_back(idx);
        }
        if (st.ops.empty()) fail(QG_ERR_VALUE, "gate wider than a tile.");
        for (int qq = 0; qq < n && __builtin_popcountll(S) < M; ++qq) S |= 1ULL << qq;
        st.S = S;
        out.push_back(st);
        remaining.swap(deferred);
    }
    return out;
}

// Register program of one stage.  Returns false when it does not fit.
template <class R>
bool schedule(const std::vector<Op> &ops, const std::vector<int> &idxs, unsigned long long S,
              int n, int rl, int mode, AdjStageDesc &d, std::vector<int> &mat_src,
              std::vector<int> &grad_op) {
    std::vector<int> lanes;
    for (int q = 0; q < n; ++q)
        if (S & (1ULL << q)) lanes.push_back(q);
    const int m = (int)lanes.size();
    int local_of[64];
    for (int i = 0; i < 64; ++i) local_of[i] = -1;
    for (int i = 0; i < m; ++i) local_of[lanes[i]] = i;
    int lowrun = 0;
    while (lowrun < m && lanes[lowrun] == lowrun) ++lowrun;
    const int t = m - rl;
    memset(&d, 0, sizeof(d));
    d.n = n;
    d.m = m;
    d.rl = rl;
    d.lowrun = lowrun;
    d.nhi = m - lowrun;
    for (int j = 0; j < d.nhi; ++j) d.hi_pos[j] = lanes[lowrun + j];
    d.nins = m < n ? m : 0;
    for (int j = 0; j < d.nins; ++j) d.ins_pos[j] = lanes[j];
    for (int i = 0; i < (1 << rl); ++i) {
        long long off = 0;
        for (int k = 0; k < rl; ++k)
            if (i & (1 << k)) off |= 1LL << lanes[t + k];
        d.dep_hi[i] = off;
    }
    mat_src.clear();
    grad_op.clear();
    const int ng = (int)idxs.size();
    std::vector<int> tgt(ng), kind(ng);
    std::vector<unsigned> cm(ng);
    for (int i = 0; i < ng; ++i) {
        const Op &o = ops[idxs[i]];
        tgt[i] = local_of[o.target];
        unsigned c = 0;
        for (int q : o.controls) c |= 1u << local_of[q];
        cm[i] = c;
        kind[i] = op_kind(o);
    }
    int nsets = 0;
    std::vector<int> RB;
    auto upcoming = [&](int from) {
        std::vector<int> out;
        for (int i = from; i < ng && (int)out.size() < rl; ++i) {
            bool needs_reg = kind[i] != kOpDiagReg;
            if (!needs_reg) continue;
            if (std::find(out.begin(), out.end(), tgt[i]) == out.end()) out.push_back(tgt[i]);
        }
        return out;
    };
    auto emit_set = [&](std::vector<int> want) -> bool {
        for (int b : RB)
            if ((int)want.size() < rl && std::find(want.begin(), want.end(), b) == want.end())
                want.push_back(b);
        for (int b = 0; b < m && (int)want.size() < rl; ++b)
            if (std::find(want.begin(), want.end(), b) == want.end()) want.push_back(b);
        if (nsets >= kMaxRegSets || d.nops >= kMaxAdjOps) return false;
        d.sets[nsets] = make_set_slots(want.data(), rl, m, sizeof(R) == 4 ? kFP32 : kFP64);
        d.nsets = nsets + 1;
        AdjOp &o = d.ops[d.nops++];
        memset(&o, 0, sizeof(o));
        o.kind = kOpTranspose;
        o.reg = (unsigned char)nsets++;
        RB = want;
        return true;
    };
    if (!emit_set(upcoming(0))) return false;
    for (int i = 0; i < ng; ++i) {
        const Op &src = ops[idxs[i]];
        auto pos_in = [&](int b) {
            for (int k = 0; k < rl; ++k)
                if (RB[k] == b) return k;
            return -1;
        };
        int k = pos_in(tgt[i]);
        int kd = kind[i];
        if (kd != kOpDiagReg && k < 0) {
            if (!emit_set(upcoming(i))) return false;
            k = pos_in(tgt[i]);
        }
        if (d.nops >= kMaxAdjOps) return false;
        AdjOp &o = d.ops[d.nops++];
        memset(&o, 0, sizeof(o));
        unsigned rbmask = 0;
        for (int b : RB) rbmask |= 1u << b;
        unsigned jm = 0;
        for (int kk = 0; kk < rl; ++kk)
            if (cm[i] & (1u << RB[kk])) jm |= 1u << kk;
        o.jmask = (unsigned short)jm;
        o.tmask = cm[i] & ~rbmask;
        if (kd == kOpDiagReg && k < 0) {
            o.kind = kOpDiagThread;
            o.tbit = 1u << tgt[i];
        } else {
            o.kind = (unsigned char)kd;
            o.reg = (unsigned char)k;
        }
        if (kd != kOpSwapX) {
            if ((int)mat_src.size() >= 0xffff) return false;
            o.mat = (unsigned short)mat_src.size();
            mat_src.push_back(idxs[i]);
        }
        if (mode == 1 && src.kind == 1) {
            if ((int)grad_op.size() >= kMaxAdjSlots) return false;
            o.gaxis = (unsigned char)src.axis;
            o.gslot = (unsigned char)grad_op.size();
            grad_op.push_back(idxs[i]);
        }
    }
    d.nmats = (int)mat_src.size();
    d.ngrads = (int)grad_op.size();
    return true;
}

struct Launch {
    AdjStageDesc desc;
    int mode;
    size_t mat_off;    // element offset (in R) of this stage's [batch][nmats][8] table
    size_t slot_off;   // offset into the param / scale tables
    int ckpt_before;   // backward: restore psi from this checkpoint first (-1: none)
    int ckpt_after;    // forward: save psi to this checkpoint after (-1: none)
};

template <class R>
void build_launches(const std::vector<Op> &ops, const std::vector<int> &order, int n, int M,
                    int rl, int budget, int mode, int batch, int n_params, const double *params,
                    std::vector<Launch> &launches, std::vector<R> &mats,
                    std::vector<int> &slot_param, std::vector<double> &slot_scale) {
    std::vector<StagePlan> stages = plan(ops, order, n, M, rl, budget, kMaxAdjOps / 2);
    std::vector<int> mat_src, grad_op;
    for (size_t si = 0; si < stages.size(); ++si) {
        std::vector<std::vector<int>> pieces{stages[si].ops};
        while (!pieces.empty()) {
            std::vector<int> piece = pieces.front();
            pieces.erase(pieces.begin());
            Launch L;
            if (!schedule<R>(ops, piece, stages[si].S, n, rl, mode, L.desc, mat_src, grad_op)) {
                if (piece.size() < 2) fail(QG_ERR_RUNTIME, "adjoint stage program does not fit.");
                size_t h = piece.size() / 2;
                pieces.insert(pieces.begin(), std::vector<int>(piece.begin() + h, piece.end()));
                pieces.insert(pieces.begin(), std::vector<int>(piece.begin(), piece.begin() + h));
                continue;
            }
            L.mode = mode;
            L.mat_off = mats.size();
            L.slot_off = slot_param.size();
            L.ckpt_before = -1;
            L.ckpt_after = -1;
            const int nm = (int)mat_src.size();
            mats.resize(mats.size() + (size_t)batch * nm * 8);
            for (int b = 0; b < batch; ++b) {
                for (int k = 0; k < nm; ++k) {
                    const Op &o = ops[mat_src[k]];
                    double m[8];
                    if (o.kind == 1)
                        rotation(o.axis, o.coef * params[(size_t)b * n_params + o.param], m);
                    else
                        memcpy(m, o.mat, sizeof(m));
                    double mm[8];
                    if (mode == 1)
                        adjoint_of(m, mm);
                    else
                        memcpy(mm, m, sizeof(mm));
                    R *dst = &mats[L.mat_off + ((size_t)b * nm + k) * 8];
                    for (int v = 0; v < 8; ++v) dst[v] = (R)mm[v];
                }
            }
            for (int g : grad_op) {
                slot_param.push_back(ops[g].param);
                slot_scale.push_back(2. * ops[g].coef);
            }
            launches.push_back(L);
        }
    }
}

// Forward sweep on the tensor cores (complex64 states of >= 13 qubits, when
// tensor-core stages are on).  The stages of each checkpoint segment are
// planned like the gate queue's (plan_stage_lanes over 12-lane tiles); the
// lanes, blocks and layouts depend only on the gates' lanes, so they are the
// same for every parameter vector, and only the block unitaries differ: one
// k_tstage launch per stage and vector, each with that vector's operands.
struct TcForward {
    struct Step {
        TcStageDesc desc;     // bmats filled at launch
        size_t ops_off;       // byte offset of batch element 0's operands
        size_t ops_stride;    // operand bytes per batch element
        int ckpt_after;       // save psi to this checkpoint after the step (-1: none)
    };
    std::vector<Step> steps;
    std::vector<unsigned char> ops;  // [step][batch][nb][Bh | Bl]
};

void plan_tc_forward(const std::vector<Op> &ops, const std::vector<int> &bounds, int n, int batch,
                     int n_params, const double *params, TcForward &out) {
    const int M = 12;
    const unsigned long long base = (1ULL << 4) - 1;
    auto gate_of = [&](const Op &o, int b) {
        PendingGate g;
        g.target = o.target;
        g.controls = o.controls;
        if (o.kind == 1)
            rotation(o.axis, o.coef * params[(size_t)b * n_params + o.param], g.m.v);
        else
            memcpy(g.m.v, o.mat, sizeof(g.m.v));
        g.diag = is_diag(g.m);
        return g;
    };
    const int nseg = (int)bounds.size() - 1;
    for (int sgi = 0; sgi < nseg; ++sgi) {
        // planning on batch element 0's gates (only their lanes matter)
        std::vector<PendingGate> g0;
        for (int j = bounds[sgi]; j < bounds[sgi + 1]; ++j) g0.push_back(gate_of(ops[j], 0));
        std::vector<const PendingGate *> remaining;
        for (auto &g : g0) remaining.push_back(&g);
        while (!remaining.empty()) {
            unsigned long long S = plan_stage_lanes(remaining, base, M);
            std::vector<const PendingGate *> chosen, deferred;
            stage_take(remaining, S, remaining.size(), &chosen, &deferred);
            for (int q = 0; q < n && __builtin_popcountll(S) < M; ++q) S |= 1ULL << q;
            const TileLanes tl = tile_lanes_of(S, n);
            const TcBlocks blocks0 = tc_blocks(chosen, tl);
            // the blocks as indices into the segment's gates
            std::vector<std::pair<unsigned, std::vector<int>>> bidx;
            for (auto &bl : blocks0) {
                std::vector<int> ix;
                for (auto *g : bl.second) ix.push_back((int)(g - g0.data()));
                bidx.emplace_back(bl.first, ix);
            }
            // dense ops only: whether a rotation is diagonal depends on its
            // angle, which differs between parameter vectors
            const TcOps ops0 = tc_ops(blocks0, false);
            for (size_t b0 = 0; b0 < bidx.size();) {
                const int nb = tc_ops_per_launch(ops0, b0);
                TcForward::Step st;
                st.ops_off = out.ops.size();
                st.ops_stride = (size_t)nb * tc_op_bytes(ops0[b0]);
                st.ckpt_after = -1;
                out.ops.resize(out.ops.size() + (size_t)batch * st.ops_stride);
                std::vector<TcStageDesc> descs(batch);
#pragma omp parallel for schedule(dynamic, 1)
                for (int b = 0; b < batch; ++b) {
                    std::vector<PendingGate> gb;
                    gb.reserve(g0.size());
                    for (int j = bounds[sgi]; j < bounds[sgi + 1]; ++j) gb.push_back(gate_of(ops[j], b));
                    TcBlocks blocks;
                    for (auto &bi : bidx) {
                        std::vector<const PendingGate *> ptrs;
                        for (int ix : bi.second) ptrs.push_back(&gb[ix]);
                        blocks.emplace_back(bi.first, ptrs);
                    }
                    tc_plan_launch(tl, n, tc_ops(blocks, false), b0, nb, descs[b],
                                   out.ops.data() + st.ops_off + (size_t)b * st.ops_stride);
                }
                st.desc = descs[0];
                out.steps.push_back(st);
                b0 += nb;
            }
            remaining.swap(deferred);
        }
        if (sgi + 1 < nseg && !out.steps.empty()) out.steps.back().ckpt_after = sgi;
    }
}

}  // namespace

template <class R>
static void adjoint_run(int prec, int n, std::vector<Op> &ops, const double *params, int n_params,
                        int batch, const std::vector<PauliTerm> &terms, int ck_every,
                        double *E_out, double *G_out) {
    cudaStream_t st = engine_stream();
    const int N = (int)ops.size();
    const size_t cs = sizeof(R) * 2;
    const size_t state_bytes = cs << n;
    const int rl = n >= 9 ? 4 : 3;
    // complex64 forward stages keep 32 amplitudes per thread (256 threads
    // per 13-lane tile); everything else 16 (or 8 on small states)
    const int rl_fwd = (sizeof(R) == 4 && n >= 13) ? 5 : rl;
    const int M_fwd = std::min(n, rl == 4 ? 13 : 12);
    // complex64 backward stages keep 8 amplitudes of psi and of lambda per
    // thread (11-lane tiles): measured 6 % faster than 16 on the 24-qubit
    // ansatz (less register pressure at the same shared-memory traffic)
    const int rl_b = sizeof(R) == 4 ? 3 : rl;
    const int M_bwd = std::min(n, rl_b == 4 ? 12 : 11);
    const int budget = 0;

    // segments between checkpoints
    std::vector<int> bounds;  // op index boundaries, including 0 and N
    bounds.push_back(0);
    if (ck_every > 0)
        for (int j = ck_every; j < N; j += ck_every) bounds.push_back(j);
    bounds.push_back(N);
    const int nseg = (int)bounds.size() - 1;

    std::vector<Launch> launches;
    std::vector<R> mats;
    std::vector<int> slot_param;
    std::vector<double> slot_scale;
    // complex64 forward sweeps of >= 13 qubits run on the tensor cores
    const bool tc_fwd = sizeof(R) == 4 && n >= 13 && tensor_stages_enabled();
    TcForward tcf;
    if (tc_fwd) {
        plan_tc_forward(ops, bounds, n, batch, n_params, params, tcf);
    } else {
        for (int s = 0; s < nseg; ++s) {
            std::vector<int> order;
            for (int j = bounds[s]; j < bounds[s + 1]; ++j) order.push_back(j);
            size_t first = launches.size();
            build_launches<R>(ops, order, n, M_fwd, rl_fwd, budget, 0, batch, n_params, params,
                              launches, mats, slot_param, slot_scale);
            if (s + 1 < nseg && launches.size() > first) launches.back().ckpt_after = s;
            if (s + 1 < nseg && launches.size() == first) fail(QG_ERR_VALUE, "empty segment.");
        }
    }
    const size_t n_fwd = launches.size();
    if (G_out) {
        for (int s = nseg - 1; s >= 0; --s) {
            std::vector<int> order;
            for (int j = bounds[s + 1] - 1; j >= bounds[s]; --j) order.push_back(j);
            size_t first = launches.size();
            build_launches<R>(ops, order, n, M_bwd, rl_b, budget, 1, batch, n_params, params,
                              launches, mats, slot_param, slot_scale);
            if (s + 1 < nseg && launches.size() > first) launches[first].ckpt_before = s;
        }
    }

    const int nck = nseg - 1;
    std::vector<void *> owned;
    auto alloc = [&](size_t bytes) {
        void *p = engine_alloc(bytes);
        owned.push_back(p);
        return p;
    };
    try {
        void *psi = alloc(state_bytes * batch);
        void *lam = alloc(state_bytes * batch);
        void *ck = nck > 0 && G_out ? alloc(state_bytes * batch * nck) : nullptr;
        void *dmats = alloc(std::max<size_t>(mats.size() * sizeof(R), 16));
        QG_CUDA(cudaMemcpyAsync(dmats, mats.data(), mats.size() * sizeof(R), cudaMemcpyHostToDevice,
                                st));
        const int nslot = (int)slot_param.size();
        int *dparam = (int *)alloc(std::max<size_t>(nslot * sizeof(int), 16));
        double *dscale = (double *)alloc(std::max<size_t>(nslot * sizeof(double), 16));
        if (nslot) {
            QG_CUDA(cudaMemcpyAsync(dparam, slot_param.data(), nslot * sizeof(int),
                                    cudaMemcpyHostToDevice, st));
            QG_CUDA(cudaMemcpyAsync(dscale, slot_scale.data(), nslot * sizeof(double),
                                    cudaMemcpyHostToDevice, st));
        }
        double *dgrad = G_out ? (double *)alloc(sizeof(double) * batch * std::max(n_params, 1))
                              : nullptr;
        if (dgrad) QG_CUDA(cudaMemsetAsync(dgrad, 0, sizeof(double) * batch * n_params, st));
        int max_grads = 0;
        for (auto &L : launches) max_grads = std::max(max_grads, L.desc.ngrads);
        const idx_t tiles_max = (idx_t)1 << (n - std::min(n, M_bwd));
        void *gpart = G_out && max_grads
                          ? alloc(sizeof(R) * (size_t)batch * max_grads * (size_t)tiles_max)
                          : nullptr;
        const int pb = pauli_sum_blocks();
        double *epart = (double *)alloc(sizeof(double) * (size_t)batch * pb);
        double *dE = (double *)alloc(sizeof(double) * batch);

        // |0...0> for every batch element
        for (int b = 0; b < batch; ++b)
            launch_init_basis(prec, (char *)psi + state_bytes * b, (idx_t)1 << n, st);

        if (tc_fwd) {
            unsigned char *dops = (unsigned char *)alloc(std::max<size_t>(tcf.ops.size(), 16));
            QG_CUDA(cudaMemcpyAsync(dops, tcf.ops.data(), tcf.ops.size(),
                                    cudaMemcpyHostToDevice, st));
            for (auto &step : tcf.steps) {
                TcStageDesc d = step.desc;
                for (int b = 0; b < batch; ++b) {
                    d.bmats = dops + step.ops_off + (size_t)b * step.ops_stride;
                    launch_tstage((char *)psi + state_bytes * b, d, st, false);
                }
                if (step.ckpt_after >= 0 && ck)
                    QG_CUDA(cudaMemcpyAsync((char *)ck + state_bytes * batch * step.ckpt_after,
                                            psi, state_bytes * batch, cudaMemcpyDeviceToDevice,
                                            st));
            }
        }

        for (size_t li = 0; li < launches.size(); ++li) {
            Launch &L = launches[li];
            if (li == n_fwd) {
                // lambda = H psi_N, E = Re<psi|lambda>
                launch_pauli_sum_apply(prec, psi, lam, n, batch, terms.data(), (int)terms.size(),
                                       epart, pb, st);
                launch_sum_rows(epart, batch, pb, dE, st);
            }
            if (L.ckpt_before >= 0)
                QG_CUDA(cudaMemcpyAsync(psi, (char *)ck + state_bytes * batch * L.ckpt_before,
                                        state_bytes * batch, cudaMemcpyDeviceToDevice, st));
            launch_adj_stage(prec, L.mode, psi, lam, L.desc, (const R *)dmats + L.mat_off, gpart,
                             batch, st);
            if (L.mode == 1 && L.desc.ngrads)
                launch_adj_grad_reduce(prec, gpart, batch, L.desc.ngrads,
                                       (idx_t)1 << (n - L.desc.m), dparam + L.slot_off,
                                       dscale + L.slot_off, dgrad, n_params, st);
            if (L.ckpt_after >= 0 && ck)
                QG_CUDA(cudaMemcpyAsync((char *)ck + state_bytes * batch * L.ckpt_after, psi,
                                        state_bytes * batch, cudaMemcpyDeviceToDevice, st));
        }
        if (launches.size() == n_fwd) {
            launch_pauli_sum_apply(prec, psi, lam, n, batch, terms.data(), (int)terms.size(), epart,
                                   pb, st);
            launch_sum_rows(epart, batch, pb, dE, st);
        }
        QG_CUDA(cudaMemcpyAsync(E_out, dE, sizeof(double) * batch, cudaMemcpyDeviceToHost, st));
        if (G_out)
            QG_CUDA(cudaMemcpyAsync(G_out, dgrad, sizeof(double) * batch * n_params,
                                    cudaMemcpyDeviceToHost, st));
        QG_CUDA(cudaStreamSynchronize(st));
    } catch (...) {
        cudaStreamSynchronize(st);
        for (void *p : owned) engine_free(p);
        throw;
    }
    for (void *p : owned) engine_free(p);
}

}  // namespace qg

using namespace qg;

extern "C" int qg_adjoint_expectation(int prec, int n_qubits, const qg_circuit_op *cops, int n_ops,
                                      const double *params, int n_params, int batch,
                                      const qg_pauli_term *cterms, int n_terms,
                                      int checkpoint_every, double *expectations,
                                      double *gradients) {
    try {
        if (prec != kFP32 && prec != kFP64) fail(QG_ERR_VALUE, "unexpected dtype.");
        if (n_qubits < 1 || n_qubits > 34) fail(QG_ERR_VALUE, "n_qubits out of range.");
        if (batch < 1) fail(QG_ERR_VALUE, "batch must be >= 1.");
        if (n_terms < 1 || n_terms > kMaxPauliTerms) fail(QG_ERR_VALUE, "1..256 Pauli terms.");
        // States narrower than a warp-sized tile get idle |0> lanes above the
        // used ones; they change neither the expectation nor the gradient.
        const int n = std::max(n_qubits, 8);
        std::vector<Op> ops(n_ops);
        for (int i = 0; i < n_ops; ++i) {
            const qg_circuit_op &c = cops[i];
            Op &o = ops[i];
            o.kind = c.kind;
            o.target = c.target;
            if (c.kind != 0 && c.kind != 1) fail(QG_ERR_VALUE, "op %d: unknown kind.", i);
            if (c.target < 0 || c.target >= n_qubits) fail(QG_ERR_VALUE, "op %d: bad target.", i);
            if (c.n_controls < 0 || c.n_controls > 4) fail(QG_ERR_VALUE, "op %d: 0..4 controls.", i);
            unsigned long long seen = 1ULL << c.target;
            for (int k = 0; k < c.n_controls; ++k) {
                int q = c.controls[k];
                if (q < 0 || q >= n_qubits || (seen & (1ULL << q)))
                    fail(QG_ERR_VALUE, "op %d: bad control.", i);
                seen |= 1ULL << q;
                o.controls.push_back(q);
            }
            o.axis = c.axis;
            o.param = c.param;
            o.coef = c.coef;
            memcpy(o.mat, c.mat, sizeof(o.mat));
            if (c.kind == 1) {
                if (c.axis < 1 || c.axis > 3) fail(QG_ERR_VALUE, "op %d: axis must be 1..3.", i);
                if (c.param < 0 || c.param >= n_params)
                    fail(QG_ERR_VALUE, "op %d: parameter index out of range.", i);
            }
        }
        std::vector<PauliTerm> terms(n_terms);
        const unsigned long long all = (1ULL << n_qubits) - 1;
        for (int i = 0; i < n_terms; ++i) {
            if ((cterms[i].x_mask | cterms[i].z_mask) & ~all)
                fail(QG_ERR_VALUE, "Pauli term %d outside the qubits.", i);
            terms[i] = PauliTerm{cterms[i].coef, cterms[i].x_mask, cterms[i].z_mask};
        }
        if (prec == kFP32)
            adjoint_run<float>(prec, n, ops, params, n_params, batch, terms, checkpoint_every,
                               expectations, gradients);
        else
            adjoint_run<double>(prec, n, ops, params, n_params, batch, terms, checkpoint_every,
                                expectations, gradients);
    } catch (const Error &e) {
        set_last_error(e.msg);
        return e.code;
    } catch (const std::bad_alloc &) {
        set_last_error("host allocation failed");
        return QG_ERR_NOMEM;
    }
    set_last_error("");
    return QG_OK;
}
