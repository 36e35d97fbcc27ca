// CPU checks of the tensor-stage host planner (qgate_gb300/csrc/tcplan.cpp),
// built and run by tests/test_cpu_planner.py.  The planner file is included
// whole so that its file-local helpers can be checked directly.  Prints
// "<check> <value>" lines; FP16 rounding pairs go to the file named by argv[1]
// for comparison with numpy.
#include "tcplan.cpp"

#include <cstdio>
#include <random>
#include <map>
#include <set>

using namespace qg;
typedef std::complex<double> cd;

static PendingGate make_gate(int t, std::vector<int> c, cd a, cd b, cd cc, cd d) {
    PendingGate g;
    g.target = t;
    g.controls = c;
    const double v[8] = {a.real(), a.imag(), b.real(), b.imag(), cc.real(), cc.imag(), d.real(), d.imag()};
    memcpy(g.m.v, v, sizeof(v));
    g.diag = is_diag(g.m);
    return g;
}

static std::vector<PendingGate> random_gates(std::mt19937 &rng, int n, int count,
                                             int dense_in_4 = 3) {
    std::uniform_real_distribution<double> U(0, 6.283185307179586);
    std::vector<PendingGate> out;
    for (int i = 0; i < count; ++i) {
        const int t = (int)(rng() % n);
        std::vector<int> c;
        const int nc = (int)(rng() % 3);
        while ((int)c.size() < nc) {
            int x = (int)(rng() % n);
            if (x != t && std::find(c.begin(), c.end(), x) == c.end()) c.push_back(x);
        }
        const double th = U(rng), ph = U(rng), la = U(rng);
        if ((int)(rng() % 4) >= dense_in_4)  // diagonal: a controlled phase or an Rz
            out.push_back(make_gate(t, c, rng() % 2 ? std::polar(1., -la) : cd(1., 0.), 0., 0.,
                                    std::polar(1., ph)));
        else
            out.push_back(make_gate(t, c, std::cos(th / 2), -std::polar(std::sin(th / 2), la),
                                    std::polar(std::sin(th / 2), ph),
                                    std::polar(std::cos(th / 2), ph + la)));
    }
    return out;
}

int main(int argc, char **argv) {
    std::mt19937 rng(2024);
    // FP16 rounding: (float bits, f16 bits) pairs for numpy to check
    {
        FILE *f = fopen(argv[1], "wb");
        std::uniform_real_distribution<double> u(-1, 1);
        for (int i = 0; i < 200000; ++i) {
            float x = (float)(u(rng) * std::ldexp(1.0, -(int)(rng() % 30)));
            if (i % 5 == 0) {
                unsigned b = (unsigned)rng();
                memcpy(&x, &b, 4);
                if (!std::isfinite(x) || std::fabs(x) > 6.0e4f) x = 0.f;
            }
            unsigned short h = f16_bits(x);
            fwrite(&x, 4, 1, f);
            fwrite(&h, 2, 1, f);
        }
        fclose(f);
    }
    // Split operands: Bh + Bl against the real form of a random unitary.
    {
        std::normal_distribution<double> g(0, 1);
        static cd U[1024];
        for (int i = 0; i < 32; ++i) {  // Gram-Schmidt rows of a random complex matrix
            for (int k = 0; k < 32; ++k) U[i * 32 + k] = cd(g(rng), g(rng));
            for (int j = 0; j < i; ++j) {
                cd dot = 0;
                for (int k = 0; k < 32; ++k) dot += std::conj(U[j * 32 + k]) * U[i * 32 + k];
                for (int k = 0; k < 32; ++k) U[i * 32 + k] -= dot * U[j * 32 + k];
            }
            double nrm = 0;
            for (int k = 0; k < 32; ++k) nrm += std::norm(U[i * 32 + k]);
            for (int k = 0; k < 32; ++k) U[i * 32 + k] /= std::sqrt(nrm);
        }
        static unsigned short bh[4096], bl[4096];
        tc_operand(U, bh, bl);
        double worst = 0;
        for (int o = 0; o < 32; ++o)
            for (int i = 0; i < 32; ++i) {
                const double val[2][2] = {{U[o * 32 + i].real(), -U[o * 32 + i].imag()},
                                          {U[o * 32 + i].imag(), U[o * 32 + i].real()}};
                for (int co = 0; co < 2; ++co)
                    for (int ci = 0; ci < 2; ++ci) {
                        const int n = 2 * o + co, k = 2 * i + ci;
                        const size_t at = (size_t)(k / 16) * 1024 + (k % 16 / 8) * 512 +
                                          (n / 8) * 64 + (n % 8) * 8 + k % 8;
                        worst = std::max(worst, std::fabs(f16_value(bh[at]) + f16_value(bl[at]) -
                                                          val[co][ci]));
                    }
            }
        printf("operand_split_max_abs_err %.3e\n", worst);
    }
    // stage_take / plan_stage_lanes / tc_blocks on random gate lists.
    int bad_partition = 0, bad_commute = 0, bad_count = 0, bad_lanes = 0, bad_blocks = 0;
    int cross_taken = 0;
    for (int trial = 0; trial < 40; ++trial) {
        const int n = 16 + (int)(rng() % 10), M = 12;
        // odd trials: cross gates allowed, and mostly diagonal gates
        const bool cross = trial % 2 == 1;
        const int cap = cross ? kMaxTensorStageGates : kMaxStageGates;
        auto gates = random_gates(rng, n, 200 + (int)(rng() % 400), cross ? 2 : 3);
        std::vector<const PendingGate *> rem;
        for (auto &g : gates) rem.push_back(&g);
        const unsigned long long base = 15;
        while (!rem.empty()) {
            const unsigned long long q0 = gate_qmask(*rem[0]);
            if (__builtin_popcountll(q0 | base) > M) {
                rem.erase(rem.begin());
                continue;
            }
            const unsigned long long S = plan_stage_lanes(rem, base, M, cross, cap);
            if (__builtin_popcountll(S) > M || (S & (base | q0)) != (base | q0)) ++bad_lanes;
            // the fast count equals stage_take's over the window, for S and neighbours
            std::vector<unsigned long long> qw;
            std::vector<char> xd;
            for (size_t i = 0; i < rem.size() && i < 512; ++i) {
                qw.push_back(gate_qmask(*rem[i]));
                xd.push_back(cross && unit_diag(*rem[i]));
            }
            for (int v = 0; v < 4; ++v) {
                const unsigned long long T = v == 0 ? S : (S ^ (1ULL << (rng() % n)));
                if (take_count(qw, xd, T, cross, cap) !=
                    stage_take(rem, T, 512, nullptr, nullptr, cross, cap))
                    ++bad_count;
            }
            std::vector<const PendingGate *> take, keep;
            stage_take(rem, S, rem.size(), &take, &keep, cross, cap);
            // partition in order, taken gates inside S, nothing taken past a
            // deferred gate that shares a lane with it
            size_t it = 0, ik = 0;
            unsigned long long blocked = 0;
            for (auto *g : rem) {
                const unsigned long long q = gate_qmask(*g);
                if (it < take.size() && take[it] == g) {
                    ++it;
                    if ((q & ~S) && !(cross && cross_gate(*g, S))) ++bad_lanes;
                    if (q & blocked) ++bad_commute;
                    cross_taken += (q & ~S) != 0;
                } else if (ik < keep.size() && keep[ik] == g) {
                    ++ik;
                    blocked |= q;
                } else {
                    ++bad_partition;
                }
            }
            if (it != take.size() || ik != keep.size()) ++bad_partition;
            if (take.size() > 1) {
                unsigned long long SS = S;
                for (int q = 0; q < n && __builtin_popcountll(SS) < M; ++q) SS |= 1ULL << q;
                TileLanes tl = tile_lanes_of(SS, n);
                auto blocks = tc_blocks(take, tl);
                std::vector<const PendingGate *> seq;
                for (auto &b : blocks) {
                    const bool xb = (b.first & kCrossBlock) != 0;
                    const unsigned bl = b.first & ~kCrossBlock;
                    if (!xb && __builtin_popcount(bl) > 5) ++bad_blocks;
                    for (auto *g : b.second) {
                        unsigned q = 0;
                        bool in = true;
                        for (int x : g->controls)
                            if (tl.local_of[x] >= 0) q |= 1u << tl.local_of[x]; else in = false;
                        if (tl.local_of[g->target] >= 0) q |= 1u << tl.local_of[g->target];
                        else in = false;
                        // a cross block holds gates with a lane outside the
                        // tile and at most one inside; other blocks in-tile gates
                        if (in == xb || (q & ~bl) || (xb && __builtin_popcount(q) > 1)) ++bad_blocks;
                        seq.push_back(g);
                    }
                }
                // the block order is a commutation-safe reordering of `take`
                // (gates on common lanes keep their order unless both are diagonal)
                for (size_t a = 0; a < seq.size(); ++a)
                    for (size_t b2 = a + 1; b2 < seq.size(); ++b2) {
                        const auto pa = std::find(take.begin(), take.end(), seq[a]) - take.begin();
                        const auto pb = std::find(take.begin(), take.end(), seq[b2]) - take.begin();
                        if (pa > pb && (gate_qmask(*seq[a]) & gate_qmask(*seq[b2])) &&
                            !(seq[a]->diag && seq[b2]->diag))
                            ++bad_blocks;
                    }
            }
            rem.swap(keep);
        }
    }
    printf("bad_partition %d\nbad_commute %d\nbad_count %d\nbad_lanes %d\nbad_blocks %d\n"
           "cross_taken %d\n",
           bad_partition, bad_commute, bad_count, bad_lanes, bad_blocks, cross_taken);
    // Operand slots of random layouts are bijections of the 4096 tile indices,
    // and a launch plan's slot tables address every slot once per layout.
    {
        int bad_slots = 0;
        for (int trial = 0; trial < 50; ++trial) {
            std::vector<int> pos(12);
            for (int i = 0; i < 12; ++i) pos[i] = i;
            std::shuffle(pos.begin(), pos.end(), rng);
            TcLayout L;
            for (int i = 0; i < 8; ++i) L.rows[i] = i < 7 ? pos[i] : -1;
            for (int k = 0; k < 5; ++k) L.amps[k] = pos[7 + k];
            std::set<unsigned> seen;
            for (unsigned ti = 0; ti < 4096; ++ti) seen.insert(tc_operand_slot(L, ti));
            if (seen.size() != 4096 || *seen.rbegin() >= 4096) ++bad_slots;
        }
        int bad_tables = 0, launches = 0, phase_ops = 0, dense_ops = 0, direct_launches = 0,
            cross_ops = 0;
        double worst_emul = 0.;
        auto b_index = [](int k, int nn) {  // the FP16 index of B[k][n] in Bh (Bl: + 4096)
            return (size_t)(k / 16) * 1024 + (k % 16 / 8) * 512 + (nn / 8) * 64 + (nn % 8) * 8 + k % 8;
        };
        for (int trial = 0; trial < 24; ++trial) {
            const int m = trial % 3 == 2 ? 13 : 12, t = m - 5, TR = 1 << t;
            const int n = 20;
            auto gates = random_gates(rng, n, 160, trial % 2 ? 1 : 3);  // odd: mostly diagonal
            std::vector<const PendingGate *> rem;
            for (auto &g : gates) rem.push_back(&g);
            const unsigned long long base = 15;
            // trials 1, 3 mod 4: cross gates allowed (as the gate queue plans)
            const bool cross = trial % 4 == 1 || trial % 4 == 3;
            const int cap = cross ? kMaxTensorStageGates : kMaxStageGates;
            const unsigned long long S0 = plan_stage_lanes(rem, base, m, cross, cap);
            std::vector<const PendingGate *> take, keep;
            stage_take(rem, S0, rem.size(), &take, &keep, cross, cap);
            if (take.size() < 2) continue;
            unsigned long long SS = S0;
            for (int q = 0; q < n && __builtin_popcountll(SS) < m; ++q) SS |= 1ULL << q;
            // the tile: random bits on the lanes outside it
            const long long g0 = (long long)(rng() & ((1u << n) - 1)) & ~(long long)SS;
            TileLanes tl = tile_lanes_of(SS, n);
            const TcOps ops = tc_ops(tc_blocks(take, tl), true);
            const int nb = tc_ops_per_launch(ops, 0);
            static TcStageDesc desc;
            static unsigned char buf[128 * 1024];
            tc_plan_launch(tl, n, ops, 0, nb, desc, buf);
            ++launches;
            auto slot_of = [&](const SetSlots &ss, unsigned r, unsigned j) {
                unsigned slot = (unsigned)ss.lo[r & 31u] ^ (unsigned)ss.hi[r >> 5];
                for (int k = 0; k < 5; ++k)
                    if (j >> k & 1u) slot ^= ss.q[k];
                return slot;
            };
            // dense ops and the natural tile: TR rows x 32 registers onto the
            // tile's slots once; phase ops: onto the table entries equally often
            // (the launch may order its ops differently from `ops`: every
            // check here reads the descriptor)
            for (int b = 0; b < nb + 2; ++b) {
                const int kind = b < nb ? desc.op_kind[b] : 0;
                if (b < nb && desc.op_off[b] % 16) ++bad_tables;
                if (kind == 2) {
                    // cross op: header and records inside the operand array
                    ++cross_ops;
                    TcCrossHdr hdr;
                    memcpy(&hdr, buf + desc.op_off[b], sizeof(hdr));
                    if (desc.op_off[b] + sizeof(hdr) + sizeof(TcCrossRec) * (size_t)hdr.nrec >
                        desc.ops_bytes)
                        ++bad_tables;
                    for (int p = 0; p < m; ++p)
                        if (hdr.start[p] > hdr.start[p + 1] || hdr.start[p + 1] > hdr.nrec)
                            ++bad_tables;
                    continue;
                }
                const bool phase = kind == 1;
                if (b < nb) (phase ? phase_ops : dense_ops) += 1;
                std::map<unsigned, int> seen;
                for (unsigned r = 0; r < (unsigned)TR; ++r)
                    for (unsigned j = 0; j < 32; ++j) seen[slot_of(desc.sets[b], r, j)] += 1;
                const size_t entries = phase ? seen.size() : (size_t)1 << m;
                if (phase && (entries & (entries - 1))) ++bad_tables;
                if (b < nb && desc.op_off[b] + (phase ? 8 * entries : (size_t)16384) > desc.ops_bytes)
                    ++bad_tables;
                if (seen.size() != entries || seen.rbegin()->first >= entries) ++bad_tables;
                for (auto &kv : seen)
                    if (kv.second != (int)(((size_t)1 << m) / entries)) ++bad_tables;
            }
            // Emulation of the kernel's data flow in FP64 on a random tile:
            // load layout -> per op (dense: scatter through the slot table,
            // D = A (Bh + Bl) from the operand buffer, rows back in the new
            // layout; phase: times the table entry) -> natural tile ->
            // load layout; against the ops' gates applied to the tile directly.
            std::map<long long, cd> want;
            std::normal_distribution<double> gauss(0, 1);
            auto load_off = [&](unsigned r, unsigned j) {
                long long lo = desc.dep_hi[j] | g0;
                for (int b = 0; b < t; ++b)
                    if (r >> b & 1u) lo |= 1LL << desc.row_lane[b];
                return lo;
            };
            std::vector<std::vector<cd>> V(TR, std::vector<cd>(32));
            for (unsigned r = 0; r < (unsigned)TR; ++r)
                for (unsigned j = 0; j < 32; ++j)
                    want[load_off(r, j)] = V[r][j] = cd(gauss(rng), gauss(rng));
            if (want.size() != ((size_t)1 << m)) ++bad_tables;
            for (int b = 0; b < nb; ++b) {
                const SetSlots &ss = desc.sets[b];
                if (desc.op_kind[b] == 2) {
                    // cross op: per-position angles from the records and the
                    // tile's outside bits, then every amplitude's phase
                    TcCrossHdr hdr;
                    memcpy(&hdr, buf + desc.op_off[b], sizeof(hdr));
                    const TcCrossRec *rec = (const TcCrossRec *)(buf + desc.op_off[b] + sizeof(hdr));
                    std::vector<double> A0(m + 1, 0.), A1(m + 1, 0.);
                    for (int p = 0; p <= m; ++p)
                        for (int k = hdr.start[p]; k < (p < m ? hdr.start[p + 1] : hdr.nrec); ++k) {
                            const TcCrossRec &x = rec[k];
                            if ((g0 & x.need) != x.need) continue;
                            if (x.tgt == 0) {
                                A0[p] += x.a0;
                                A1[p] += x.a1;
                            } else {
                                A1[p] += (g0 & x.tgt) ? x.a1 : x.a0;
                            }
                        }
                    for (unsigned r = 0; r < (unsigned)TR; ++r)
                        for (unsigned j = 0; j < 32; ++j) {
                            double ph = A1[m];
                            for (int bb = 0; bb < t; ++bb)
                                ph += (r >> bb & 1u) ? A1[hdr.rows[bb]] : A0[hdr.rows[bb]];
                            for (int k = 0; k < 5; ++k)
                                ph += (j >> k & 1u) ? A1[hdr.amps[k]] : A0[hdr.amps[k]];
                            V[r][j] *= std::polar(1., ph);
                        }
                    continue;
                }
                if (desc.op_kind[b] == 1) {
                    const float *tab = (const float *)(buf + desc.op_off[b]);
                    for (unsigned r = 0; r < (unsigned)TR; ++r)
                        for (unsigned j = 0; j < 32; ++j) {
                            const unsigned e = slot_of(ss, r, j);
                            V[r][j] *= cd(tab[2 * e], tab[2 * e + 1]);
                        }
                    continue;
                }
                std::vector<cd> A((size_t)1 << m);
                for (unsigned r = 0; r < (unsigned)TR; ++r)
                    for (unsigned j = 0; j < 32; ++j) A[slot_of(ss, r, j)] = V[r][j];
                const unsigned short *B = (const unsigned short *)(buf + desc.op_off[b]);
                for (unsigned row = 0; row < (unsigned)TR; ++row) {
                    // unswizzled slot (row << 5) | i holds amplitude i of the
                    // operand row; the 128-byte swizzle XORs bits 2..4 with 5..7
                    double arow[64];
                    for (unsigned i = 0; i < 32; ++i) {
                        const unsigned c = (row << 5) | i;
                        const unsigned cs = c ^ (((c >> 5) & 7u) << 2);
                        arow[2 * i] = A[cs].real();
                        arow[2 * i + 1] = A[cs].imag();
                    }
                    for (int o = 0; o < 32; ++o) {
                        double re = 0, im = 0;
                        for (int k = 0; k < 64; ++k) {
                            const size_t i0 = b_index(k, 2 * o), i1 = b_index(k, 2 * o + 1);
                            re += arow[k] * (f16_value(B[i0]) + f16_value(B[4096 + i0]));
                            im += arow[k] * (f16_value(B[i1]) + f16_value(B[4096 + i1]));
                        }
                        V[row][o] = cd(re, im);
                    }
                }
            }
            // copy-out: final layout -> natural tile -> load layout, or
            // (direct_out) final layout straight to the state's offsets
            std::map<long long, cd> got;
            if (desc.direct_out) {
                ++direct_launches;
                std::map<long long, int> hit;
                for (unsigned r = 0; r < (unsigned)TR; ++r) {
                    long long ro = g0;
                    for (int b = 0; b < t; ++b)
                        if (r >> b & 1u) ro |= 1LL << desc.out_row_lane[b];
                    // a warp's rows cover whole 128-byte lines (lanes 0..3)
                    for (unsigned j = 0; j < 32; ++j) {
                        long long off = ro;
                        for (int k = 0; k < 5; ++k)
                            if (j >> k & 1u) off |= desc.out_e[k];
                        got[off] = V[r][j];
                        hit[off] += 1;
                    }
                }
                // every amplitude of the tile written once
                if (hit.size() != want.size()) ++bad_tables;
                for (auto &kv : hit)
                    if (kv.second != 1 || !want.count(kv.first)) ++bad_tables;
                unsigned wl = 0;
                for (int b = 0; b < 5; ++b) wl |= 1u << desc.out_row_lane[b];
                if ((wl & 15u) != 15u) ++bad_tables;
            } else {
                std::vector<cd> nat((size_t)1 << m);
                for (unsigned r = 0; r < (unsigned)TR; ++r)
                    for (unsigned j = 0; j < 32; ++j) nat[slot_of(desc.sets[nb], r, j)] = V[r][j];
                for (unsigned r = 0; r < (unsigned)TR; ++r)
                    for (unsigned j = 0; j < 32; ++j)
                        got[load_off(r, j)] = nat[slot_of(desc.sets[nb + 1], r, j)];
            }
            for (int b = 0; b < nb; ++b)
                for (auto *g : ops[b].gates) {
                    const long long tb = 1LL << g->target;
                    long long cm = 0;
                    for (int c : g->controls) cm |= 1LL << c;
                    const cd m00(g->m.v[0], g->m.v[1]), m01(g->m.v[2], g->m.v[3]),
                        m10(g->m.v[4], g->m.v[5]), m11(g->m.v[6], g->m.v[7]);
                    if (g->diag) {  // elementwise (its lanes may lie outside the tile)
                        for (auto &kv : want)
                            if ((kv.first & cm) == cm) kv.second *= (kv.first & tb) ? m11 : m00;
                        continue;
                    }
                    for (auto &kv : want) {
                        const long long off = kv.first;
                        if ((off & tb) || (off & cm) != cm) continue;
                        const cd a0 = want[off], a1 = want[off | tb];
                        want[off] = m00 * a0 + m01 * a1;
                        want[off | tb] = m10 * a0 + m11 * a1;
                    }
                }
            double nrm = 0;
            for (auto &kv : want) nrm = std::max(nrm, std::abs(kv.second));
            for (auto &kv : want)
                worst_emul = std::max(worst_emul, std::abs(got[kv.first] - kv.second) / nrm);
        }
        printf("emulated_stage_max_rel_err %.3e\nphase_ops %d\ndense_ops %d\ncross_ops %d\n",
               worst_emul, phase_ops, dense_ops, cross_ops);
        printf("bad_slots %d\nbad_tables %d\nlaunches_checked %d\ndirect_out_launches %d\n",
               bad_slots, bad_tables, launches, direct_launches);
    }
    return 0;
}
