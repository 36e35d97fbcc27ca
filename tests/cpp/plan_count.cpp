// CPU check of the tensor-stage planning of whole circuits, built and run by
// tests/test_cpu_planner.py::test_bench_circuit_plans.  Reads circuits (gate
// lanes and 2x2 matrices, written by the test from the bench's workloads),
// plans each as the gate queue does for complex64 states on 12-lane
// tensor-core tiles (merge_runs, then the loop of flush_lookahead in
// qgate_gb300/csrc/api.cpp over plan_stage_lanes / stage_take, then tc_blocks
// / tc_ops / tc_ops_per_launch per stage) and prints, per circuit,
// "<label> <gates> <passes> <single-gate passes> <dense ops> <phase ops> <cross ops>".
#include "tcplan.cpp"

#include <cstdio>

using namespace qg;

bool qg::tensor_stages_enabled() { return true; }

namespace {

void mat_mul(const Mat2 &a, const Mat2 &b, Mat2 &out) {  // out = a * b
    for (int r = 0; r < 2; ++r)
        for (int c = 0; c < 2; ++c) {
            double re = 0., im = 0.;
            for (int k = 0; k < 2; ++k) {
                const double ar = a.v[2 * (2 * r + k)], ai = a.v[2 * (2 * r + k) + 1];
                const double br = b.v[2 * (2 * k + c)], bi = b.v[2 * (2 * k + c) + 1];
                re += ar * br - ai * bi;
                im += ar * bi + ai * br;
            }
            out.v[2 * (2 * r + c)] = re;
            out.v[2 * (2 * r + c) + 1] = im;
        }
}

// The gate queue's merge of consecutive uncontrolled gates on one lane.
void merge_runs(std::vector<PendingGate> &gates) {
    std::vector<PendingGate> out;
    int last[64];
    for (int i = 0; i < 64; ++i) last[i] = -1;
    for (auto &g : gates) {
        const int prev = last[g.target];
        if (g.controls.empty() && prev >= 0 && out[prev].controls.empty() &&
            out[prev].target == g.target) {
            Mat2 prod;
            mat_mul(g.m, out[prev].m, prod);
            out[prev].m = prod;
            out[prev].diag = is_diag(prod);
            continue;
        }
        out.push_back(g);
        const int idx = (int)out.size() - 1;
        last[g.target] = idx;
        for (int c : g.controls) last[c] = idx;
    }
    gates.swap(out);
}

void plan(const char *label, int n, std::vector<PendingGate> gates, int M) {
    const size_t n_in = gates.size();
    merge_runs(gates);
    std::vector<const PendingGate *> remaining;
    for (auto &g : gates) remaining.push_back(&g);
    const unsigned long long base = (1ULL << std::min(n, 4)) - 1;
    int passes = 0, singles = 0, dense = 0, phase = 0, cross = 0;
    while (!remaining.empty()) {
        if (__builtin_popcountll(gate_qmask(*remaining[0]) | base) > M) {
            ++singles;
            ++passes;
            remaining.erase(remaining.begin());
            continue;
        }
        unsigned long long S = plan_stage_lanes(remaining, base, M, true, kMaxTensorStageGates);
        std::vector<const PendingGate *> chosen, deferred;
        stage_take(remaining, S, remaining.size(), &chosen, &deferred, true, kMaxTensorStageGates);
        if (chosen.size() == 1) {
            ++singles;
            ++passes;
        } else {
            for (int q = 0; q < n && __builtin_popcountll(S) < M; ++q) S |= 1ULL << q;
            const TileLanes tl = tile_lanes_of(S, n);
            const TcOps ops = tc_ops(tc_blocks(chosen, tl), true);
            for (const TcOp &op : ops) {
                if (op.cross) ++cross;
                else if (op.phase) ++phase;
                else ++dense;
            }
            for (size_t b0 = 0; b0 < ops.size(); ++passes) b0 += tc_ops_per_launch(ops, b0);
        }
        remaining.swap(deferred);
    }
    printf("%s %zu %d %d %d %d %d\n", label, n_in, passes, singles, dense, phase, cross);
}

}  // namespace

// argv[i]: a circuit file: "label n count", then per gate "target n_controls
// controls... m00re m00im m01re m01im m10re m10im m11re m11im".
int main(int argc, char **argv) {
    for (int a = 1; a < argc; ++a) {
        FILE *f = fopen(argv[a], "r");
        if (!f) return 2;
        char label[64];
        int n = 0, count = 0;
        if (fscanf(f, "%63s %d %d", label, &n, &count) != 3) return 3;
        std::vector<PendingGate> gates;
        for (int i = 0; i < count; ++i) {
            PendingGate g;
            int nc = 0;
            if (fscanf(f, "%d %d", &g.target, &nc) != 2) return 3;
            g.controls.resize(nc);
            for (int k = 0; k < nc; ++k)
                if (fscanf(f, "%d", &g.controls[k]) != 1) return 3;
            for (int k = 0; k < 8; ++k)
                if (fscanf(f, "%lf", &g.m.v[k]) != 1) return 3;
            g.diag = is_diag(g.m);
            gates.push_back(g);
        }
        fclose(f);
        plan(label, n, gates, 12);
    }
    return 0;
}
