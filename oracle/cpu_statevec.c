/*
 * CPU port of the reference's state-vector primitives, in plain C with
 * OpenMP threads.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the oracle's compiled restatement: it
 * times the reference's CPU algorithm on the host cores (the "cpu_baseline"
 * of bench.py and its `--impl reference` arm) and checks the GPU engine at
 * sizes where numpy would be slow.  It is never linked into or called by the
 * product.
 *
 * Each routine restates the reference file:line it names (qgate 0.2.2).  The
 * reference distributes the same per-pair loops over std::threads
 * (qgate/simulator/src/Parallel.h:10-117) with a byte-table index permutation
 * (qgate/simulator/src/BitPermTable.h:11-75); here the pair index is formed
 * by inserting zero bits, which yields the same index sequence.
 *
 *   gcc -O3 -fopenmp -fPIC -shared cpu_statevec.c -o libcpu_statevec.so
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef long long idx_t;

static inline idx_t insert_zero(idx_t k, int p) {
    idx_t lo = k & (((idx_t)1 << p) - 1);
    return ((k >> p) << (p + 1)) | lo;
}

static idx_t insert_zeros(idx_t k, const int *pos, int npos) {
    for (int i = 0; i < npos; ++i) k = insert_zero(k, pos[i]);
    return k;
}

static void sort_ints(int *a, int n) {
    for (int i = 1; i < n; ++i) {
        int v = a[i], j = i - 1;
        while (j >= 0 && a[j] > v) {
            a[j + 1] = a[j];
            --j;
        }
        a[j + 1] = v;
    }
}

int cs_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* |0...0>: qgate/simulator/src/CPUQubitProcessor.cpp:61-73.  prec: 1 = FP64
 * (complex128), 2 = FP32 (complex64). */
void cs_init_basis(void *state, int n, int prec) {
    idx_t N = (idx_t)1 << n;
    size_t cs = prec == 1 ? 16 : 8;
#pragma omp parallel for schedule(static)
    for (idx_t b = 0; b < N; b += 4096) {
        idx_t e = b + 4096 < N ? b + 4096 : N;
        memset((char *)state + b * cs, 0, (e - b) * cs);
    }
    if (prec == 1)
        ((double *)state)[0] = 1.;
    else
        ((float *)state)[0] = 1.f;
}

/* Controlled (n_ctrl >= 0) 2x2 update on pairs differing in `target`:
 * qgate/simulator/src/CPUQubitProcessor.cpp:307-362.  The matrix is 8 doubles
 * {re00, im00, re01, im01, re10, im10, re11, im11}, converted to the state's
 * precision as the reference does (CPUQubitProcessor.cpp:311). */
#define APPLY_BODY(R)                                                                  \
    R *s = (R *)state;                                                                 \
    const R m00r = (R)m[0], m00i = (R)m[1], m01r = (R)m[2], m01i = (R)m[3];           \
    const R m10r = (R)m[4], m10i = (R)m[5], m11r = (R)m[6], m11i = (R)m[7];           \
    _Pragma("omp parallel for schedule(static)")                                       \
    for (idx_t k = 0; k < n_items; ++k) {                                              \
        idx_t i0 = insert_zeros(k, pos, npos) | cmask;                                 \
        idx_t i1 = i0 | tbit;                                                          \
        R ar = s[2 * i0], ai = s[2 * i0 + 1], br = s[2 * i1], bi = s[2 * i1 + 1];      \
        s[2 * i0] = m00r * ar - m00i * ai + m01r * br - m01i * bi;                     \
        s[2 * i0 + 1] = m00r * ai + m00i * ar + m01r * bi + m01i * br;                 \
        s[2 * i1] = m10r * ar - m10i * ai + m11r * br - m11i * bi;                     \
        s[2 * i1 + 1] = m10r * ai + m10i * ar + m11r * bi + m11i * br;                 \
    }

void cs_apply_gate(void *state, int n, int prec, const double *m, const int *ctrl, int n_ctrl,
                   int target) {
    int pos[64];
    idx_t cmask = 0;
    for (int i = 0; i < n_ctrl; ++i) {
        pos[i] = ctrl[i];
        cmask |= (idx_t)1 << ctrl[i];
    }
    pos[n_ctrl] = target;
    int npos = n_ctrl + 1;
    sort_ints(pos, npos);
    idx_t tbit = (idx_t)1 << target;
    idx_t n_items = (idx_t)1 << (n - npos);
    if (prec == 1) {
        APPLY_BODY(double)
    } else {
        APPLY_BODY(float)
    }
}

/* A whole circuit, in passes over blocks of the state that stay in the
 * core's cache: consecutive gates whose lanes, together with lanes 0..3, fit
 * in `max_lanes` lanes form a pass; the pass's lane set is padded with the
 * lowest free lanes, and for every assignment of the other lanes the pass
 * applies its gates in order to that 2^max_lanes-amplitude block.  Each
 * amplitude pair sees exactly the updates of cs_apply_gate (the same
 * expressions, qgate/simulator/src/CPUQubitProcessor.cpp:307-362) in the
 * same gate order, so the result equals one cs_apply_gate sweep per gate; it
 * only moves the state through memory once per pass instead of once per
 * gate.  Gate g: matrix mats[8g..8g+8) (as cs_apply_gate), target
 * targets[g], controls ctrls[ctrl_off[g]..ctrl_off[g+1]). */
#define PAIR_UPDATE(R, i0, i1)                                                           \
    {                                                                                    \
        R ar = s[2 * (i0)], ai = s[2 * (i0) + 1], br = s[2 * (i1)], bi = s[2 * (i1) + 1];     \
        s[2 * (i0)] = m00r * ar - m00i * ai + m01r * br - m01i * bi;                     \
        s[2 * (i0) + 1] = m00r * ai + m00i * ar + m01r * bi + m01i * br;                 \
        s[2 * (i1)] = m10r * ar - m10i * ai + m11r * br - m11i * bi;                     \
        s[2 * (i1) + 1] = m10r * ai + m10i * ar + m11r * bi + m11i * br;                 \
    }
/* Local index i = h * 2^L + l: l runs over the block's L contiguous low
 * lanes (consecutive amplitudes), h over its other lanes (dep[h << L]). */
#define PASS_BODY(R)                                                                     \
    R *s = (R *)state;                                                                   \
    _Pragma("omp parallel for schedule(static)")                                         \
    for (idx_t o = 0; o < n_outer; ++o) {                                                \
        const idx_t base = insert_zeros(o, pos, K);                                      \
        for (int g = g0; g < g1; ++g) {                                                  \
            const double *m = mats + 8 * (size_t)g;                                      \
            SETUP(R)                                                                     \
            const idx_t tl = ltb[g - g0], cm = lcm[g - g0];                              \
            const idx_t cmh = cm >> L, cml = cm & (nlow - 1);                            \
            if (tl >= nlow) {                                                            \
                const idx_t th = tl >> L;                                                \
                for (idx_t h = 0; h < nhigh; ++h) {                                      \
                    if ((h & th) || (h & cmh) != cmh) continue;                          \
                    const idx_t p0 = base + dep[h << L], p1 = base + dep[(h | th) << L];  \
                    if (cml) {                                                           \
                        for (idx_t l = 0; l < nlow; ++l)                                 \
                            if ((l & cml) == cml) PAIR_UPDATE(R, p0 + l, p1 + l)         \
                    } else {                                                             \
                        for (idx_t l = 0; l < nlow; ++l) PAIR_UPDATE(R, p0 + l, p1 + l)  \
                    }                                                                    \
                }                                                                        \
            } else {                                                                     \
                for (idx_t h = 0; h < nhigh; ++h) {                                      \
                    if ((h & cmh) != cmh) continue;                                      \
                    const idx_t p = base + dep[h << L];                                  \
                    if (cml) {                                                           \
                        for (idx_t l0 = 0; l0 < nlow; l0 += 2 * tl)                       \
                            for (idx_t l = l0; l < l0 + tl; ++l)                         \
                                if ((l & cml) == cml) PAIR_UPDATE(R, p + l, p + l + tl)  \
                    } else if (tl == 1) {                                                \
                        for (idx_t l = 0; l < nlow; l += 2) PAIR_UPDATE(R, p + l, p + l + 1) \
                    } else {                                                             \
                        for (idx_t l0 = 0; l0 < nlow; l0 += 2 * tl)                       \
                            for (idx_t l = l0; l < l0 + tl; ++l)                         \
                                PAIR_UPDATE(R, p + l, p + l + tl)                        \
                    }                                                                    \
                }                                                                        \
            }                                                                            \
        }                                                                                \
    }

static idx_t gate_lanes(const int *targets, const int *ctrl_off, const int *ctrls, int g) {
    idx_t q = (idx_t)1 << targets[g];
    for (int c = ctrl_off[g]; c < ctrl_off[g + 1]; ++c) q |= (idx_t)1 << ctrls[c];
    return q;
}

int cs_run_circuit(void *state, int n, int prec, int n_gates, const double *mats,
                   const int *targets, const int *ctrl_off, const int *ctrls, int max_lanes) {
    if (max_lanes > n) max_lanes = n;
    if (max_lanes < 5 || max_lanes > 20) return -1;
    const idx_t low = ((idx_t)1 << (n < 4 ? n : 4)) - 1;
    int passes = 0;
    idx_t *dep = (idx_t *)malloc(sizeof(idx_t) << max_lanes);
    idx_t *ltb = (idx_t *)malloc(sizeof(idx_t) * (size_t)(n_gates > 0 ? n_gates : 1));
    idx_t *lcm = (idx_t *)malloc(sizeof(idx_t) * (size_t)(n_gates > 0 ? n_gates : 1));
    for (int g0 = 0; g0 < n_gates;) {
        idx_t S = low;
        int g1 = g0;
        while (g1 < n_gates) {
            const idx_t q = gate_lanes(targets, ctrl_off, ctrls, g1);
            if (__builtin_popcountll(S | q) > max_lanes) break;
            S |= q;
            ++g1;
        }
        if (g1 == g0) { /* a gate wider than the pass: its lanes alone */
            S = gate_lanes(targets, ctrl_off, ctrls, g0);
            g1 = g0 + 1;
        }
        for (int q = 0; q < n && __builtin_popcountll(S) < max_lanes; ++q) S |= (idx_t)1 << q;
        int pos[64], K = 0, local_of[64];
        for (int q = 0; q < n; ++q) {
            local_of[q] = -1;
            if (S >> q & 1) {
                local_of[q] = K;
                pos[K++] = q;
            }
        }
        const idx_t nloc = (idx_t)1 << K, n_outer = (idx_t)1 << (n - K);
        int L = 0;
        while (L < K && pos[L] == L) ++L;
        const idx_t nlow = (idx_t)1 << L, nhigh = (idx_t)1 << (K - L);
        for (idx_t i = 0; i < nloc; ++i) {
            idx_t off = 0;
            for (int k = 0; k < K; ++k)
                if (i >> k & 1) off |= (idx_t)1 << pos[k];
            dep[i] = off;
        }
        for (int g = g0; g < g1; ++g) {
            ltb[g - g0] = (idx_t)1 << local_of[targets[g]];
            idx_t cm = 0;
            for (int c = ctrl_off[g]; c < ctrl_off[g + 1]; ++c) cm |= (idx_t)1 << local_of[ctrls[c]];
            lcm[g - g0] = cm;
        }
#define SETUP(R)                                                                \
    const R m00r = (R)m[0], m00i = (R)m[1], m01r = (R)m[2], m01i = (R)m[3];     \
    const R m10r = (R)m[4], m10i = (R)m[5], m11r = (R)m[6], m11i = (R)m[7];
        if (prec == 1) {
            PASS_BODY(double)
        } else {
            PASS_BODY(float)
        }
#undef SETUP
        ++passes;
        g0 = g1;
    }
    free(dep);
    free(ltb);
    free(lcm);
    return passes;
}

/* Pr(lane == 0): qgate/simulator/src/CPUQubitProcessor.cpp:75-125 (the
 * reference accumulates per thread in the state's precision; FP64 here). */
double cs_calc_probability(const void *state, int n, int prec, int lane) {
    idx_t n_items = (idx_t)1 << (n - 1);
    double sum = 0.;
    if (prec == 1) {
        const double *s = (const double *)state;
#pragma omp parallel for reduction(+ : sum) schedule(static)
        for (idx_t k = 0; k < n_items; ++k) {
            idx_t i = insert_zero(k, lane);
            sum += s[2 * i] * s[2 * i] + s[2 * i + 1] * s[2 * i + 1];
        }
    } else {
        const float *s = (const float *)state;
#pragma omp parallel for reduction(+ : sum) schedule(static)
        for (idx_t k = 0; k < n_items; ++k) {
            idx_t i = insert_zero(k, lane);
            sum += (double)s[2 * i] * s[2 * i] + (double)s[2 * i + 1] * s[2 * i + 1];
        }
    }
    return sum;
}

/* |psi|^2 of every amplitude (lane order = external order): the prob array
 * of qgate/simulator/src/CPUQubitsStatesGetter.cpp:159-254 for one state with
 * the identity lane transform and no hidden lanes. */
void cs_probabilities(const void *state, int n, int prec, double *out) {
    idx_t N = (idx_t)1 << n;
    if (prec == 1) {
        const double *s = (const double *)state;
#pragma omp parallel for schedule(static)
        for (idx_t i = 0; i < N; ++i) out[i] = s[2 * i] * s[2 * i] + s[2 * i + 1] * s[2 * i + 1];
    } else {
        const float *s = (const float *)state;
#pragma omp parallel for schedule(static)
        for (idx_t i = 0; i < N; ++i)
            out[i] = (double)s[2 * i] * s[2 * i] + (double)s[2 * i + 1] * s[2 * i + 1];
    }
}

/* In-place prefix sum normalised by the total, threads' partial sums first
 * (qgate/simulator/src/CPUSamplingPool.cpp:8-49).  Returns the total. */
double cs_prefix_sum_normalise(double *p, idx_t N) {
    int nt = cs_num_threads();
    double *part = (double *)calloc((size_t)nt + 1, sizeof(double));
    idx_t span = (N + nt - 1) / nt;
#pragma omp parallel num_threads(nt)
    {
        int t = 0;
#ifdef _OPENMP
        t = omp_get_thread_num();
#endif
        idx_t b = (idx_t)t * span, e = b + span < N ? b + span : N;
        double v = 0.;
        for (idx_t i = b; i < e; ++i) {
            v += p[i];
            p[i] = v;
        }
        part[t + 1] = v;
    }
    for (int t = 1; t <= nt; ++t) part[t] += part[t - 1];
    double total = part[nt];
    double norm = 1. / total;
#pragma omp parallel num_threads(nt)
    {
        int t = 0;
#ifdef _OPENMP
        t = omp_get_thread_num();
#endif
        idx_t b = (idx_t)t * span, e = b + span < N ? b + span : N;
        double off = part[t];
        for (idx_t i = b; i < e; ++i) p[i] = (p[i] + off) * norm;
    }
    free(part);
    return total;
}

/* upper_bound per uniform, clamped to N-1, then empty-lane zero bits
 * inserted: qgate/simulator/src/CPUSamplingPool.cpp:71-81. */
void cs_sample(const double *cdf, idx_t N, const double *u, long long *obs, idx_t m,
               const int *empty, int n_empty) {
    int pos[64];
    for (int i = 0; i < n_empty; ++i) pos[i] = empty[i];
    sort_ints(pos, n_empty);
#pragma omp parallel for schedule(static)
    for (idx_t i = 0; i < m; ++i) {
        idx_t lo = 0, hi = N;
        double x = u[i];
        while (lo < hi) {
            idx_t mid = (lo + hi) >> 1;
            if (cdf[mid] <= x)
                lo = mid + 1;
            else
                hi = mid;
        }
        if (lo > N - 1) lo = N - 1;
        obs[i] = insert_zeros(lo, pos, n_empty);
    }
}
