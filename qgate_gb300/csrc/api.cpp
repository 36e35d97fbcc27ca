// extern "C" boundary of the GB300 state-vector engine: device context,
// caching arena, states / processor / getter / pool objects, the gate queue
// with its fusion planner, and the host side of every entry point declared
// in include/qgate_gb300.h.
//
// One GPU, one non-blocking stream: every launch is stream-ordered, so a
// buffer returned to the arena can be handed out again without waiting.
// The host synchronises only where a value must come back (probabilities,
// expectations, gathers, sampling), as the reference's CUDA runtime does
// (qgate/simulator/src/CUDAQubitProcessor.cpp:40-50,
// qgate/simulator/src/DeviceSum.h:16-23).
#include "qg_internal.h"
#include "qg_plan.h"
#include "../../include/qgate_gb300.h"

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <set>
#include <unordered_map>
#include <unordered_set>
#include <unistd.h>

namespace qg {

static thread_local std::string t_last_error;

void set_last_error(const std::string &msg) { t_last_error = msg; }

void fail(int code, const char *fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    throw Error{code, std::string(buf)};
}

void cuda_check(cudaError_t err, const char *what) {
    if (err == cudaSuccess) return;
    if (err == cudaErrorMemoryAllocation) fail(QG_ERR_NOMEM, "Out of device memory. (%s)", what);
    fail(QG_ERR_CUDA, "CUDA error %d (%s) in %s", (int)err, cudaGetErrorString(err), what);
}

// ------------------------------------------------------------ arena

// Caching allocator with power-of-two size classes, the single-device
// counterpart of the reference's chunk cache
// (qgate/simulator/src/MultiDeviceMemoryStore.cpp:164-201).
struct Arena {
    std::map<size_t, std::vector<void *>> free_lists;
    std::unordered_map<void *, size_t> live;
    size_t in_use = 0, cached = 0;
    long long limit = -1;

    static size_t size_class(size_t bytes) {
        size_t c = 256;
        while (c < bytes) c <<= 1;
        return c;
    }
    void trim() {
        for (auto &kv : free_lists)
            for (void *p : kv.second) cudaFree(p);
        free_lists.clear();
        cached = 0;
    }
    void *alloc(size_t bytes) {
        size_t cls = size_class(bytes);
        auto it = free_lists.find(cls);
        if (it != free_lists.end() && !it->second.empty()) {
            void *p = it->second.back();
            it->second.pop_back();
            cached -= cls;
            in_use += cls;
            live[p] = cls;
            return p;
        }
        if (limit >= 0 && (long long)(in_use + cls) > limit)
            fail(QG_ERR_NOMEM, "Out of device memory. (arena limit %lld bytes, requested %zu)",
                 limit, cls);
        if (limit >= 0 && (long long)(in_use + cached + cls) > limit) trim();
        void *p = nullptr;
        cudaError_t err = cudaMalloc(&p, cls);
        if (err != cudaSuccess) {
            cudaGetLastError();
            trim();
            err = cudaMalloc(&p, cls);
            if (err != cudaSuccess) {
                cudaGetLastError();
                fail(QG_ERR_NOMEM, "Out of device memory. (requested %zu bytes)", cls);
            }
        }
        in_use += cls;
        live[p] = cls;
        return p;
    }
    void release(void *p) {
        if (!p) return;
        auto it = live.find(p);
        if (it == live.end()) return;
        size_t cls = it->second;
        live.erase(it);
        in_use -= cls;
        cached += cls;
        free_lists[cls].push_back(p);
    }
};

// ------------------------------------------------------------ objects

// A device buffer of amplitudes.  Shared between a states object and the
// lazy states objects that read it (a product formed by join, a view left by
// decohere_and_separate); returned to the arena when the last holder drops it.
struct Buf {
    void *d = nullptr;
    size_t bytes = 0;
    Buf() = default;
    Buf(const Buf &) = delete;
    Buf &operator=(const Buf &) = delete;
    ~Buf();
};
typedef std::shared_ptr<Buf> BufPtr;

// One factor of a lazy product: a buffer of 2^n_lanes amplitudes, or (buf
// null) the basis state |basis> on n_lanes lanes.
struct Factor {
    BufPtr buf;
    int n_lanes = 0;
    long long basis = 0;
};

// Qubit-grouping policy.  The front-end allocates, joins and separates
// states objects as its qubit groups change (qgate/simulator/
// qubits_handler.py:34-122); the amplitudes are formed only when something
// reads them:
//  - initialize / reset leave a product of one basis factor (no buffer yet);
//  - join leaves a product of the sources' buffers (shared, not copied) and
//    their pending gates moved up to the joined lanes: a chain of joins
//    between two reads costs one kron pass, or none when every factor is
//    still a basis state (the joined gates then run on a fresh |0...0>);
//  - decohere_and_separate leaves the remaining lanes as a view of the
//    source's buffer; when it is read and the source is gone, the lane is
//    removed in place and the view adopts the buffer (no allocation).
// A buffer shared with a lazy object is copied before it is written.
struct States {
    int prec;
    int n_lanes = -1;
    void *d = nullptr;  // buf->d once materialized
    BufPtr buf;
    std::vector<PendingGate> pending;
    bool streamed = false;  // part of the pending run was launched by the streaming flush
    enum { kDense = 0, kProduct = 1, kView = 2 };
    int lazy = kDense;
    std::vector<Factor> factors;  // kProduct: the last factor at the lowest lanes
    BufPtr parent;                // kView: the n_lanes + 1 lane source
    int sep_lane = 0, sep_value = 0;
    double sep_norm = 1.;
};

struct Processor {
    int prec;
};
struct Getter {
    int prec;
};
struct Pool {
    unsigned long long *cdf = nullptr;  // fixed-point prefix sums, 2^-60 units
    unsigned long long total = 0;       // cdf[n - 1]
    unsigned *guide = nullptr;          // guide table (nullptr: plain search)
    int guide_shift = 0, guide_index_shift = 0;
    idx_t n = 0;
    std::vector<int> empty_pos;  // ascending
};

// A compiled circuit: a gate list handed over once and applied in one call.
// With graph replay on, the first run on a states buffer plans and launches
// the gates under stream capture; later runs on the same buffer (same lanes,
// same fusion settings) replay that CUDA graph without host planning.  The
// tensor stages' block operands of a captured graph live in chunks the
// circuit owns (pinned staging + device copy), so replays re-read them.
struct Circuit {
    int prec;
    int min_lanes = 0;
    std::vector<PendingGate> gates;
    bool graph = false;
    cudaGraph_t g = nullptr;
    cudaGraphExec_t exec = nullptr;
    void *state = nullptr;  // what the graph was captured for
    int n_lanes = -1;
    unsigned version = 0;
    long long passes = 0, bytes = 0;
    static constexpr size_t kChunkBytes = 8ull << 20;
    std::vector<std::pair<unsigned char *, unsigned char *>> chunks;
    size_t chunk_off = 0;
};

struct Device {
    bool initialized = false;
    int dev = 0;
    cudaStream_t stream = nullptr;
    Arena arena;
    int guide_index_shift = -1;    // pools' guide entries: -1 = automatic
    unsigned settings_version = 1;  // bumped by every change of the fusion settings
    struct Circuit *capturing = nullptr;  // set while a compiled circuit is captured
    double *d_partials = nullptr;  // reduce_partials() + 8
    double *h_result = nullptr;    // pinned, 16 doubles
    static constexpr size_t kStageBytes = 64ull << 20;
    void *h_stage[2] = {nullptr, nullptr};
    cudaEvent_t ev[2] = {nullptr, nullptr};
    // Fusion parameters, indexed by prec ([1] fp64, [2] fp32): lanes per
    // shared-memory tile, lanes per thread's registers, per-amplitude cost
    // budget of a stage (0 = unlimited).
    int tile_lanes[3] = {0, 12, 12};
    int reg_lanes[3] = {0, 3, 4};  // complex128 (double-float registers): 3
    int cost_budget[3] = {0, 0, 0};
    bool pipelined = false;  // persistent double-buffered stage kernel (opt-in)
    // batched circuits as one persistent launch over a work queue (default),
    // or as one launch per round of stages
    bool batch_one_launch = true;
    // Kernels may write results straight into the caller's (pageable) host
    // buffers where the device accesses pageable memory through the host
    // page tables (Grace + NVLink-C2C), which skips the pinned staging.
    // Opt-in: measured on GB300 it is faster into buffers already touched
    // (4 GiB: 36 ms vs 46 ms) but first touch of a fresh buffer through GPU
    // page faults costs ~1.8 s, and callers such as the front-end's prob
    // getter allocate a fresh array per call.
    bool host_direct = false;
    bool host_direct_supported = false;
    // Large device -> host results: produced into one device buffer, the
    // destination's pages touched by all host threads, then one copy into
    // the pageable buffer (on Grace + NVLink-C2C, where such copies run at
    // ~190 GB/s into touched pages).  Set where pageable access is supported.
    bool pageable_copy = false;
    // complex64 stages on 12- or 13-lane tiles as fused 5-lane blocks on the
    // tensor cores (default; 0 selects the register-resident CUDA-core stage).
    bool tensor_blocks = true;
    // Ring of split block operands: pinned host staging and its device copy.
    static constexpr size_t kBRingBytes = 32ull << 20;
    unsigned char *h_bring = nullptr, *d_bring = nullptr;
    // Pinned staging of a batch's programs (grown on demand; reused by the
    // next batch, which starts after this one's results are read).
    unsigned char *h_batch = nullptr;
    size_t h_batch_bytes = 0;
    size_t bring_off = 0;
    long long n_gates = 0, n_passes = 0, n_bytes = 0;
    // qubit-grouping counters: join calls, kron passes, state buffers
    // allocated, decohere_and_separate calls, separations done in place / by
    // copy, copies of shared buffers before a write
    long long g_joins = 0, g_krons = 0, g_allocs = 0, g_separates = 0, g_inplace = 0,
              g_copies = 0, g_cow = 0;
    // Per-kernel-class launch timing with CUDA events on the engine's stream.
    bool timing = false;
    struct TimedClass {
        long long launches = 0;
        double ms = 0.;
        std::vector<std::pair<cudaEvent_t, cudaEvent_t>> pending;
    };
    std::map<std::string, TimedClass> timers;
    std::vector<cudaEvent_t> event_pool;
    std::unordered_set<States *> states;
    std::unordered_set<Processor *> procs;
    std::unordered_set<Getter *> getters;
    std::unordered_set<Pool *> pools;
    std::unordered_set<struct Circuit *> circuits;
    // Trace replay: gate runs that recur between observations (the same
    // gates on the same lanes, e.g. a circuit run again through the plugin
    // API) are kept as circuits and replayed from a captured CUDA graph.
    bool trace_replay = true;
    struct Trace {
        unsigned long long hash = 0;
        long long used = 0;
        struct Circuit *c = nullptr;
    };
    std::vector<Trace> traces;
    long long trace_clock = 0, trace_hits = 0, trace_captures = 0;
    std::recursive_mutex mu;
};

static Device g_dev;

static void device_init(int device_id, long long limit) {
    Device &d = g_dev;
    if (d.initialized) return;
    int count = 0;
    QG_CUDA(cudaGetDeviceCount(&count));
    if (count < 1) fail(QG_ERR_CUDA, "no CUDA device");
    if (device_id < 0) QG_CUDA(cudaGetDevice(&device_id));
    QG_CUDA(cudaSetDevice(device_id));
    d.dev = device_id;
    QG_CUDA(cudaStreamCreateWithFlags(&d.stream, cudaStreamNonBlocking));
    QG_CUDA(cudaMalloc(&d.d_partials, sizeof(double) * (reduce_partials() + 8)));
    QG_CUDA(cudaMallocHost(&d.h_result, sizeof(double) * 16));
    for (int i = 0; i < 2; ++i) {
        QG_CUDA(cudaMallocHost(&d.h_stage[i], Device::kStageBytes));
        QG_CUDA(cudaEventCreateWithFlags(&d.ev[i], cudaEventDisableTiming));
    }
    d.arena.limit = limit;
    int pageable = 0, host_tables = 0;
    QG_CUDA(cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, device_id));
    QG_CUDA(cudaDeviceGetAttribute(&host_tables, cudaDevAttrPageableMemoryAccessUsesHostPageTables,
                                   device_id));
    d.host_direct_supported = pageable == 1 && host_tables == 1;
    d.pageable_copy = d.host_direct_supported;
    d.initialized = true;
}

Buf::~Buf() { g_dev.arena.release(d); }

static Device &dev() {
    if (!g_dev.initialized) device_init(-1, -1);
    QG_CUDA(cudaSetDevice(g_dev.dev));
    return g_dev;
}

cudaStream_t engine_stream() { return dev().stream; }
void *engine_alloc(size_t bytes) { return dev().arena.alloc(bytes); }
bool tensor_stages_enabled() { return dev().tensor_blocks; }
void engine_free(void *p) { g_dev.arena.release(p); }

template <class T> static T *lookup(std::unordered_set<T *> &set, qg_handle h, const char *what) {
    T *p = reinterpret_cast<T *>(h);
    if (!p || set.find(p) == set.end()) fail(QG_ERR_VALUE, "invalid %s handle.", what);
    return p;
}
static States *get_states(qg_handle h) { return lookup(g_dev.states, h, "qubit states"); }
static States *get_alloc_states(qg_handle h) {
    States *s = get_states(h);
    if (!s->d && s->lazy == States::kDense) fail(QG_ERR_RUNTIME, "qubit states not initialized.");
    return s;
}

static void check_lane(const States *s, int lane) {
    if (lane < 0 || lane >= s->n_lanes)
        fail(QG_ERR_VALUE, "lane %d out of range [0, %d).", lane, s->n_lanes);
}

static cudaEvent_t take_event(Device &d) {
    if (!d.event_pool.empty()) {
        cudaEvent_t e = d.event_pool.back();
        d.event_pool.pop_back();
        return e;
    }
    cudaEvent_t e;
    QG_CUDA(cudaEventCreate(&e));
    return e;
}

// Runs `launch` (which enqueues kernels on d.stream) and, when timing is on,
// brackets it with CUDA events attributed to kernel class `cls`.
template <class F> static void timed(Device &d, const char *cls, F launch) {
    if (!d.timing) {
        launch();
        return;
    }
    cudaEvent_t a = take_event(d), b = take_event(d);
    QG_CUDA(cudaEventRecord(a, d.stream));
    launch();
    QG_CUDA(cudaEventRecord(b, d.stream));
    d.timers[cls].pending.emplace_back(a, b);
}

// ------------------------------------------------------------ grouping

static PairIdx pair_pattern(const std::vector<int> &fixed, unsigned long long set_mask,
                            unsigned long long partner);

static BufPtr new_buffer(Device &d, int prec, int n_lanes) {
    BufPtr b = std::make_shared<Buf>();
    b->bytes = ((size_t)1 << n_lanes) * complex_size(prec);
    b->d = d.arena.alloc(b->bytes);
    d.g_allocs += 1;
    return b;
}

static void set_buffer(States *s, BufPtr b) {
    s->buf = std::move(b);
    s->d = s->buf ? s->buf->d : nullptr;
}

// Forget the amplitudes (not the pending gates or the lane count).
static void drop_contents(States *s) {
    set_buffer(s, nullptr);
    s->lazy = States::kDense;
    s->factors.clear();
    s->parent.reset();
}

static void set_basis(States *s, long long basis) {
    drop_contents(s);
    s->lazy = States::kProduct;
    Factor f;
    f.n_lanes = s->n_lanes;
    f.basis = basis;
    s->factors.push_back(f);
}

// Adjacent basis factors multiply to one basis factor.
static void coalesce_factors(std::vector<Factor> &fs) {
    std::vector<Factor> out;
    for (auto &f : fs) {
        if (!f.buf && !out.empty() && !out.back().buf) {
            out.back().basis = (out.back().basis << f.n_lanes) | f.basis;
            out.back().n_lanes += f.n_lanes;
        } else {
            out.push_back(f);
        }
    }
    fs.swap(out);
}

// Kron of factors (the last at the lowest lanes) into a fresh buffer.
static BufPtr kron_factors(Device &d, int prec, std::vector<Factor> fs) {
    while ((int)fs.size() > kMaxGetterStates) {
        // the lowest factors first into one buffer
        std::vector<Factor> low(fs.end() - kMaxGetterStates, fs.end());
        fs.resize(fs.size() - kMaxGetterStates);
        Factor f;
        for (auto &x : low) f.n_lanes += x.n_lanes;
        f.buf = kron_factors(d, prec, low);
        fs.push_back(f);
    }
    int n = 0;
    std::vector<const void *> srcs;
    std::vector<int> lanes;
    std::vector<long long> basis;
    for (auto &f : fs) {
        srcs.push_back(f.buf ? f.buf->d : nullptr);
        lanes.push_back(f.n_lanes);
        basis.push_back(f.basis);
        n += f.n_lanes;
    }
    BufPtr b = new_buffer(d, prec, n);
    bool any_buffer = false;
    for (auto &f : fs) any_buffer = any_buffer || f.buf != nullptr;
    if (fs.size() == 1 && !fs[0].buf && fs[0].basis == 0) {
        timed(d, "init", [&] { launch_init_basis(prec, b->d, (idx_t)1 << n, d.stream); });
    } else if (!any_buffer) {
        // a basis state: written, nothing read
        timed(d, "init", [&] {
            launch_kron(prec, b->d, (idx_t)1 << n, srcs.data(), lanes.data(), (int)srcs.size(),
                        d.stream, basis.data());
        });
    } else {
        d.g_krons += 1;
        timed(d, "join", [&] {
            launch_kron(prec, b->d, (idx_t)1 << n, srcs.data(), lanes.data(), (int)srcs.size(),
                        d.stream, basis.data());
        });
    }
    return b;
}

// Forms the amplitudes of a lazy states object (its pending gates stay
// pending).
static void materialize(Device &d, States *s) {
    if (s->lazy == States::kProduct) {
        BufPtr b = kron_factors(d, s->prec, s->factors);  // (s unchanged if this throws)
        s->factors.clear();
        s->lazy = States::kDense;
        set_buffer(s, b);
    } else if (s->lazy == States::kView) {
        // (s changes only once the new amplitudes are formed: an allocation
        // that fails leaves the view as it was)
        if (s->parent.use_count() == 1) {
            // the source is gone: remove the lane in place and keep its buffer
            d.g_inplace += 1;
            timed(d, "measure", [&] {
                launch_shrink_inplace(s->prec, s->parent->d, s->n_lanes + 1, s->sep_lane,
                                      s->sep_value, s->sep_norm, d.stream);
            });
            BufPtr par = std::move(s->parent);
            s->lazy = States::kDense;
            set_buffer(s, par);
        } else {
            BufPtr b = new_buffer(d, s->prec, s->n_lanes);
            d.g_copies += 1;
            PairIdx pi = pair_pattern({s->sep_lane}, (unsigned long long)s->sep_value << s->sep_lane,
                                      0);
            timed(d, "measure", [&] {
                launch_shrink(s->prec, b->d, s->parent->d, (idx_t)1 << s->n_lanes, pi,
                              s->sep_norm, d.stream);
            });
            s->parent.reset();
            s->lazy = States::kDense;
            set_buffer(s, b);
        }
    }
}

// Materializes s and makes its buffer its own (copied if a lazy object still
// reads it), before an in-place write.
static void prepare_write(Device &d, States *s) {
    materialize(d, s);
    if (s->buf && s->buf.use_count() > 1) {
        d.g_cow += 1;
        BufPtr b = new_buffer(d, s->prec, s->n_lanes);
        QG_CUDA(cudaMemcpyAsync(b->d, s->d, ((size_t)1 << s->n_lanes) * complex_size(s->prec),
                                cudaMemcpyDeviceToDevice, d.stream));
        set_buffer(s, b);
    }
}

static void settle_timers(Device &d) {
    bool any = false;
    for (auto &kv : d.timers) any = any || !kv.second.pending.empty();
    if (!any) return;
    QG_CUDA(cudaStreamSynchronize(d.stream));
    for (auto &kv : d.timers) {
        for (auto &pr : kv.second.pending) {
            float ms = 0.f;
            QG_CUDA(cudaEventElapsedTime(&ms, pr.first, pr.second));
            kv.second.ms += ms;
            kv.second.launches += 1;
            d.event_pool.push_back(pr.first);
            d.event_pool.push_back(pr.second);
        }
        kv.second.pending.clear();
    }
}

// ------------------------------------------------------------ gate queue

static PairIdx pair_pattern(const std::vector<int> &fixed, unsigned long long set_mask,
                            unsigned long long partner) {
    PairIdx pi;
    std::vector<int> pos(fixed);
    std::sort(pos.begin(), pos.end());
    pi.npos = (int)pos.size();
    for (int i = 0; i < pi.npos; ++i) pi.pos[i] = pos[i];
    pi.set_mask = set_mask;
    pi.partner = partner;
    return pi;
}

static void run_single_gate(Device &d, States *s, const PendingGate &g) {
    std::vector<int> pos(g.controls);
    pos.push_back(g.target);
    unsigned long long cmask = 0;
    for (int c : g.controls) cmask |= 1ULL << c;
    PairIdx pi = pair_pattern(pos, cmask, 1ULL << g.target);
    idx_t n_items = (idx_t)1 << (s->n_lanes - (int)pos.size());
    timed(d, "gate", [&] { launch_apply_pairs(s->prec, s->d, n_items, pi, g.m, d.stream); });
    d.n_passes += 1;
    d.n_bytes += 4 * n_items * (long long)complex_size(s->prec);
}

// Shared-memory stage (generic, any tile size): used for tiles too small for
// the register-resident kernel.
static void run_stage_smem(Device &d, States *s, unsigned long long S,
                           const std::vector<const PendingGate *> &gates) {
    StageDesc sd;
    memset(&sd, 0, sizeof(sd));
    const int n = s->n_lanes;
    TileLanes tl = tile_lanes_of(S, n);
    const int m = (int)tl.lanes.size();
    sd.n = n;
    sd.m = m;
    sd.lowrun = tl.lowrun;
    sd.nhi = m - tl.lowrun;
    for (int j = 0; j < sd.nhi; ++j) sd.hi_pos[j] = tl.lanes[tl.lowrun + j];
    sd.nins = m < n ? m : 0;
    for (int j = 0; j < sd.nins; ++j) sd.ins_pos[j] = tl.lanes[j];
    sd.ngates = (int)gates.size();
    for (int gi = 0; gi < sd.ngates; ++gi) {
        const PendingGate &g = *gates[gi];
        StageGate &G = sd.gates[gi];
        std::vector<int> pos;
        unsigned cmask = 0;
        for (int c : g.controls) {
            pos.push_back(tl.local_of[c]);
            cmask |= 1u << tl.local_of[c];
        }
        pos.push_back(tl.local_of[g.target]);
        std::sort(pos.begin(), pos.end());
        G.npos = (int)pos.size();
        for (int i = 0; i < G.npos; ++i) G.pos[i] = (signed char)pos[i];
        G.cmask = cmask;
        G.tbit = 1u << tl.local_of[g.target];
        G.diag = g.diag ? 1 : 0;
        memcpy(G.m, g.m.v, sizeof(G.m));
    }
    timed(d, "stage", [&] { launch_stage(s->prec, s->d, sd, d.stream); });
    d.n_passes += 1;
    d.n_bytes += 2 * ((long long)1 << n) * (long long)complex_size(s->prec);
}

static bool is_x(const Mat2 &m) {
    static const double x[8] = {0., 0., 1., 0., 1., 0., 0., 0.};
    for (int i = 0; i < 8; ++i)
        if (m.v[i] != x[i]) return false;
    return true;
}

// Builds the register program of one stage: walks the gates in order and
// keeps the targets of dense gates in the register set, inserting a
// shared-memory transpose (to the next rl distinct targets) when a target is
// not resident.  Diagonal gates never need one.  `sets` receives, per
// register set, its rl tile lanes.
template <class R>
static void build_program(const std::vector<const PendingGate *> &gates, const TileLanes &tl,
                          int rl, std::vector<RegOp<R>> &ops,
                          std::vector<std::vector<int>> &sets) {
    const int m = (int)tl.lanes.size();
    ops.clear();
    sets.clear();
    const int ng = (int)gates.size();
    std::vector<int> tgt(ng), kind(ng);
    std::vector<unsigned> cm(ng);
    for (int i = 0; i < ng; ++i) {
        const PendingGate &g = *gates[i];
        tgt[i] = tl.local_of[g.target];
        unsigned c = 0;
        for (int q : g.controls) c |= 1u << tl.local_of[q];
        cm[i] = c;
        kind[i] = g.diag ? kOpDiagReg : (is_x(g.m) ? kOpSwapX : kOpGate);
    }
    std::vector<int> RB;
    auto upcoming = [&](int from) {
        std::vector<int> out;
        for (int i = from; i < ng && (int)out.size() < rl; ++i) {
            if (kind[i] == kOpDiagReg) continue;
            if (std::find(out.begin(), out.end(), tgt[i]) == out.end()) out.push_back(tgt[i]);
        }
        return out;
    };
    auto emit_set = [&](std::vector<int> want) {
        for (int b : RB)
            if ((int)want.size() < rl && std::find(want.begin(), want.end(), b) == want.end())
                want.push_back(b);
        for (int b = 0; b < m && (int)want.size() < rl; ++b)
            if (std::find(want.begin(), want.end(), b) == want.end()) want.push_back(b);
        RegOp<R> o;
        memset(&o, 0, sizeof(o));
        o.kind = kOpTranspose;
        o.reg = (unsigned char)std::min<size_t>(sets.size(), 255);
        ops.push_back(o);
        sets.push_back(want);
        RB = want;
    };
    emit_set(upcoming(0));
    for (int i = 0; i < ng; ++i) {
        auto pos_in = [&](int b) {
            for (int k = 0; k < rl; ++k)
                if (RB[k] == b) return k;
            return -1;
        };
        int k = pos_in(tgt[i]);
        int kd = kind[i];
        if (kd != kOpDiagReg && k < 0) {
            emit_set(upcoming(i));
            k = pos_in(tgt[i]);
        }
        RegOp<R> o;
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
            o.reg = 0;
        } else {
            o.kind = (unsigned char)kd;
            o.reg = (unsigned char)k;
        }
        for (int v = 0; v < 8; ++v) o.m[v] = (R)gates[i]->m.v[v];
        ops.push_back(o);
    }
}

static void fill_tile_header(const TileLanes &tl, int n, int rl, int &lowrun, int &nhi, int *hi_pos,
                             int &nins, int *ins_pos, long long *dep_hi) {
    const int m = (int)tl.lanes.size();
    const int t = m - rl;
    lowrun = tl.lowrun;
    nhi = m - tl.lowrun;
    for (int j = 0; j < nhi; ++j) hi_pos[j] = tl.lanes[tl.lowrun + j];
    nins = m < n ? m : 0;
    for (int j = 0; j < nins; ++j) ins_pos[j] = tl.lanes[j];
    for (int i = 0; i < (1 << rl); ++i) {
        long long off = 0;
        for (int k = 0; k < rl; ++k)
            if (i & (1 << k)) off |= 1LL << tl.lanes[t + k];
        dep_hi[i] = off;
    }
}

// Register program of one stage in a kernel-parameter descriptor.  Returns
// false if it does not fit.
template <class R>
static bool schedule_rstage(const std::vector<const PendingGate *> &gates, const TileLanes &tl,
                            int n, int rl, RStageDesc<R> &d) {
    std::vector<RegOp<R>> ops;
    std::vector<std::vector<int>> sets;
    build_program<R>(gates, tl, rl, ops, sets);
    if ((int)ops.size() > kMaxRegOps || (int)sets.size() > kMaxRegSets) return false;
    const int m = (int)tl.lanes.size();
    memset(&d, 0, sizeof(d));
    d.n = n;
    d.m = m;
    d.rl = rl;
    fill_tile_header(tl, n, rl, d.lowrun, d.nhi, d.hi_pos, d.nins, d.ins_pos, d.dep_hi);
    d.nops = (int)ops.size();
    d.nsets = (int)sets.size();
    for (int i = 0; i < d.nops; ++i) d.ops[i] = ops[i];
    const int prec = sizeof(R) == 4 ? kFP32 : kFP64;
    for (size_t si = 0; si < sets.size(); ++si)
        d.sets[si] = make_set_slots(sets[si].data(), rl, m, prec);
    return true;
}

static void run_tstage(Device &d, States *s, const TileLanes &tl,
                       const std::vector<const PendingGate *> &gates) {
    const int n = s->n_lanes;
    const TcOps ops = tc_ops(tc_blocks(gates, tl), true);
    if (!d.h_bring) {
        QG_CUDA(cudaMallocHost(&d.h_bring, Device::kBRingBytes));
        QG_CUDA(cudaMalloc(&d.d_bring, Device::kBRingBytes));
        d.bring_off = 0;
    }
    for (size_t b0 = 0; b0 < ops.size();) {
        const int nb = tc_ops_per_launch(ops, b0);
        size_t bytes = 0;
        for (int b = 0; b < nb; ++b) bytes += tc_op_bytes(ops[b0 + b]);
        unsigned char *hb, *db;
        if (d.capturing) {
            // operands a captured graph re-reads: chunks owned by the circuit
            Circuit *c = d.capturing;
            if (c->chunks.empty() || c->chunk_off + bytes > Circuit::kChunkBytes) {
                unsigned char *h = nullptr, *dv = nullptr;
                QG_CUDA(cudaMallocHost(&h, Circuit::kChunkBytes));
                if (cudaMalloc(&dv, Circuit::kChunkBytes) != cudaSuccess) {
                    cudaFreeHost(h);
                    fail(QG_ERR_NOMEM, "circuit operand chunk: device allocation failed.");
                }
                c->chunks.emplace_back(h, dv);
                c->chunk_off = 0;
            }
            hb = c->chunks.back().first + c->chunk_off;
            db = c->chunks.back().second + c->chunk_off;
            c->chunk_off += bytes;
        } else {
            if (d.bring_off + bytes > Device::kBRingBytes) {
                QG_CUDA(cudaStreamSynchronize(d.stream));  // the staging is reused
                d.bring_off = 0;
            }
            hb = d.h_bring + d.bring_off;
            db = d.d_bring + d.bring_off;
            d.bring_off += bytes;
        }
        static TcStageDesc desc;
        tc_plan_launch(tl, n, ops, b0, nb, desc, hb);
        desc.bmats = db;
        QG_CUDA(cudaMemcpyAsync(db, hb, bytes, cudaMemcpyHostToDevice, d.stream));
        timed(d, "tstage", [&] { launch_tstage(s->d, desc, d.stream, d.pipelined); });
        d.n_passes += 1;
        d.n_bytes += 2 * ((long long)1 << n) * (long long)complex_size(s->prec);
        b0 += nb;
    }
}

static void pack_double_float(RStageDesc<double> &desc) {
    for (int i = 0; i < desc.nops; ++i) {
        RegOp<double> &o = desc.ops[i];
        if (o.kind == kOpTranspose || o.kind == kOpSwapX) continue;
        for (int k = 0; k < 8; ++k) {
            const double v = o.m[k];
            const float hl[2] = {(float)v, (float)(v - (double)(float)v)};
            memcpy(&o.m[k], hl, sizeof(hl));
        }
    }
}

static void run_stage(Device &d, States *s, unsigned long long S,
                      const std::vector<const PendingGate *> &gates) {
    const int n = s->n_lanes;
    TileLanes tl = tile_lanes_of(S, n);
    const int m = (int)tl.lanes.size();
    // Valid shapes: 32..512 threads (256 with 5 register lanes), 3..5
    // register lanes (complex128 at most 4).
    if (d.tensor_blocks && s->prec == kFP32 && (m == 12 || m == 13) && n >= m) {
        run_tstage(d, s, tl, gates);
        return;
    }
    const int max_rl = s->prec == kFP64 ? 4 : 5;
    auto max_t = [](int r) { return r >= 5 ? 8 : 9; };
    int rl = std::min(d.reg_lanes[s->prec], max_rl);
    while (rl < max_rl && m - rl > max_t(rl)) ++rl;
    while (rl > 3 && m - rl < 5) --rl;
    if (m - rl > max_t(rl) || m - rl < 5) {
        run_stage_smem(d, s, S, gates);
        return;
    }
    bool ok;
    if (s->prec == kFP32) {
        static RStageDesc<float> desc;
        ok = schedule_rstage(gates, tl, n, rl, desc);
        if (ok) timed(d, "stage", [&] { launch_rstage_f32(s->d, desc, d.stream, d.pipelined); });
    } else {
        static RStageDesc<double> desc;
        ok = schedule_rstage(gates, tl, n, rl, desc);
        if (ok) {
            pack_double_float(desc);
            timed(d, "stage", [&] { launch_rstage_f64(s->d, desc, d.stream, d.pipelined); });
        }
    }
    if (!ok) {
        // Program too long for one descriptor: split the stage.
        size_t h = gates.size() / 2;
        std::vector<const PendingGate *> a(gates.begin(), gates.begin() + h),
            b(gates.begin() + h, gates.end());
        run_stage(d, s, S, a);
        run_stage(d, s, S, b);
        return;
    }
    d.n_passes += 1;
    d.n_bytes += 2 * ((long long)1 << n) * (long long)complex_size(s->prec);
}

static void mat_mul(const Mat2 &a, const Mat2 &b, Mat2 &out) {  // out = a * b
    for (int r = 0; r < 2; ++r)
        for (int c = 0; c < 2; ++c) {
            double re = 0., im = 0.;
            for (int k = 0; k < 2; ++k) {
                double ar = a.v[2 * (2 * r + k)], ai = a.v[2 * (2 * r + k) + 1];
                double br = b.v[2 * (2 * k + c)], bi = b.v[2 * (2 * k + c) + 1];
                re += ar * br - ai * bi;
                im += ar * bi + ai * br;
            }
            out.v[2 * (2 * r + c)] = re;
            out.v[2 * (2 * r + c) + 1] = im;
        }
}

// Merges each uncontrolled single-lane gate into the previous gate on its lane
// when that gate is also uncontrolled on the same lane (no gate in between
// touches the lane), so the pair costs one 2x2 update.
static void merge_runs(std::vector<PendingGate> &gates) {
    std::vector<PendingGate> out;
    out.reserve(gates.size());
    int last[64];
    for (int i = 0; i < 64; ++i) last[i] = -1;
    for (auto &g : gates) {
        int prev = last[g.target];
        if (g.controls.empty() && prev >= 0 && out[prev].controls.empty() &&
            out[prev].target == g.target) {
            Mat2 prod;
            mat_mul(g.m, out[prev].m, prod);
            out[prev].m = prod;
            out[prev].diag = is_diag(prod);
            continue;
        }
        const int idx = (int)out.size();
        last[g.target] = idx;
        for (int c : g.controls) last[c] = idx;
        out.push_back(std::move(g));  // (`gates` is replaced by `out` below)
    }
    gates.swap(out);
}

// Per-amplitude instruction estimate of a gate inside a register stage.
static int gate_cost(const PendingGate &g) {
    if (g.diag) return 4;
    if (is_x(g.m)) return 2;
    return 9;
}

// Planner for tensor-core stages: instead of growing a stage's lane set in
// gate order, it starts from the low lanes and the first pending gate's
// lanes and adds, one at a time up to M lanes, the lane that lets the stage
// take the most gates (counted over a window of the next 512 gates; also
// from a few seeded starts, keeping the best), then swaps lanes in and out
// while that takes more.  On the 30-qubit random circuit this takes 32
// stages of 12 lanes instead of 47 (and fewer fused blocks per gate), i.e.
// 32 % fewer passes over the state.
static void flush_lookahead(Device &d, States *s, std::vector<const PendingGate *> &remaining,
                            unsigned long long base, int M, int max_stages = 1 << 30) {
    const int n = s->n_lanes;
    for (int done = 0; !remaining.empty() && done < max_stages; ++done) {
        const unsigned long long q0 = gate_qmask(*remaining[0]);
        if (__builtin_popcountll(q0 | base) > M) {
            run_single_gate(d, s, *remaining[0]);
            remaining.erase(remaining.begin());
            continue;
        }
        // cross gates (diagonal gates with at most one lane in the tile) run
        // in any stage as per-tile phases
        unsigned long long S = plan_stage_lanes(remaining, base, M, true, kMaxTensorStageGates);
        std::vector<const PendingGate *> chosen, deferred;
        stage_take(remaining, S, remaining.size(), &chosen, &deferred, true, kMaxTensorStageGates);
        if (chosen.size() == 1) {
            run_single_gate(d, s, *chosen[0]);
        } else {
            for (int q = 0; q < n && __builtin_popcountll(S) < M; ++q) S |= 1ULL << q;
            run_stage(d, s, S, chosen);
        }
        remaining.swap(deferred);
    }
}

// Whether a states object's pending gates go to the lookahead planner of
// tensor-core stages, and its tile size M and always-present lanes `base`.
static bool lookahead_params(const Device &d, const States *s, int &M, unsigned long long &base) {
    const int n = s->n_lanes;
    M = std::min(d.tile_lanes[s->prec], kMaxTileLanes);
    if (!(d.tensor_blocks && s->prec == kFP32 && (M == 12 || M == 13) && n > M)) return false;
    base = (1ULL << std::min(n, 4)) - 1;
    return true;
}

// Streaming flush: once a states object holds kStreamAt pending gates, the
// first stage is planned and launched right away (the planner looks 512
// gates ahead, so it decides as a full flush would), so the GPU works while
// the caller is still enqueueing the rest of the circuit.
constexpr size_t kStreamAt = 640;

// X gates (any controls) that reach a basis state before every other gate
// on their lanes permute it: while a states object is a product of basis
// factors, such gates are applied to the basis value (exactly; no pass), and
// the other gates keep their order.  A gate is taken only when no gate kept
// before it touches its lanes, so it commutes with all of those.  (A circuit
// that prepares its input with X gates - the QFT of |x> - then plans as if
// it started from |x>: the prepared lanes no longer hold back the per-tile
// phases of their controlled phase gates.)
static void absorb_basis_flips(States *s) {
    if (s->lazy != States::kProduct || s->pending.empty() || s->n_lanes > 62) return;
    for (const Factor &f : s->factors)
        if (f.buf) return;
    unsigned long long b = 0;  // factors[0] at the highest lanes
    for (const Factor &f : s->factors) b = (b << f.n_lanes) | (unsigned long long)f.basis;
    unsigned long long touched = 0;
    std::vector<PendingGate> keep;
    keep.reserve(s->pending.size());
    bool any = false;
    for (PendingGate &g : s->pending) {
        unsigned long long lanes = 1ULL << g.target;
        for (int c : g.controls) lanes |= 1ULL << c;
        if (!(lanes & touched) && is_x(g.m)) {
            bool on = true;
            for (int c : g.controls) on = on && ((b >> c) & 1ULL);
            if (on) b ^= 1ULL << g.target;
            any = true;
            continue;
        }
        touched |= lanes;
        keep.push_back(std::move(g));
    }
    s->pending.swap(keep);  // (the kept gates were moved out of the list)
    if (any) set_basis(s, (long long)b);
}

static void stream_flush(States *s) {
    Device &d = dev();
    int M;
    unsigned long long base;
    if (s->pending.size() < kStreamAt || !lookahead_params(d, s, M, base)) return;
    absorb_basis_flips(s);
    if (s->pending.size() < kStreamAt) return;
    prepare_write(d, s);
    merge_runs(s->pending);
    std::vector<const PendingGate *> remaining;
    for (auto &g : s->pending) remaining.push_back(&g);
    s->streamed = true;
    flush_lookahead(d, s, remaining, base, M, 1);
    std::vector<PendingGate> rest;
    rest.reserve(remaining.size());
    for (auto *g : remaining) rest.push_back(*g);
    s->pending.swap(rest);
}

// Fusion planner.  Walks the pending gates in order and packs them into
// stages whose lane set S has at most M lanes; a gate that does not fit, or
// that touches a lane of an earlier deferred gate, is deferred to the next
// stage (it then commutes with everything moved ahead of it, because their
// lane sets are disjoint).  The lowest lanes are always in S so that each
// tile is made of >= 128-byte contiguous runs.  A per-amplitude cost budget
// closes a stage before its arithmetic outgrows its HBM time.
static bool replay_trace(Device &d, States *s);

static void flush(States *s) {
    absorb_basis_flips(s);
    if (s->pending.empty()) {
        s->streamed = false;
        if (s->lazy != States::kDense) materialize(dev(), s);
        return;
    }
    Device &d = dev();
    prepare_write(d, s);
    if (replay_trace(d, s)) return;
    s->streamed = false;
    const int n = s->n_lanes;
    int M = d.tile_lanes[s->prec];
    if (M <= 1) {
        for (auto &g : s->pending) run_single_gate(d, s, g);
        s->pending.clear();
        return;
    }
    merge_runs(s->pending);
    std::vector<const PendingGate *> remaining;
    for (auto &g : s->pending) remaining.push_back(&g);
    if (M > kMaxTileLanes) M = kMaxTileLanes;
    if (s->prec == kFP64 && M > 13) M = 13;
    const int budget = d.cost_budget[s->prec];
    const int rl = d.reg_lanes[s->prec];
    const int low = std::min(n, s->prec == kFP32 ? 4 : 3);
    const unsigned long long all = n >= 64 ? ~0ULL : ((1ULL << n) - 1);
    if (n <= M) M = n;
    const unsigned long long base = (n <= M) ? all : ((1ULL << low) - 1);
    if (d.tensor_blocks && s->prec == kFP32 && (M == 12 || M == 13) && n > M) {
        flush_lookahead(d, s, remaining, base, M);
        s->pending.clear();
        return;
    }
    while (!remaining.empty()) {
        unsigned long long S = base, blocked = 0, dense_targets = 0;
        int cost = 0;
        std::vector<const PendingGate *> chosen, deferred;
        // A gate wider than a tile runs on its own.
        if (__builtin_popcountll(gate_qmask(*remaining[0]) | base) > M) {
            run_single_gate(d, s, *remaining[0]);
            remaining.erase(remaining.begin());
            continue;
        }
        for (auto *g : remaining) {
            unsigned long long q = gate_qmask(*g);
            int c = gate_cost(*g);
            unsigned long long dt = dense_targets;
            if (!g->diag) dt |= 1ULL << g->target;
            int est = cost + c + 7 * (int)((__builtin_popcountll(dt) + rl - 1) / rl);
            bool over = budget > 0 && !chosen.empty() && est > budget;
            if ((q & blocked) || (int)chosen.size() >= kMaxStageGates || over ||
                __builtin_popcountll(S | q) > M) {
                deferred.push_back(g);
                blocked |= q;
                continue;
            }
            S |= q;
            cost += c;
            dense_targets = dt;
            chosen.push_back(g);
        }
        if (chosen.size() == 1) {
            run_single_gate(d, s, *chosen[0]);
        } else {
            for (int q = 0; q < n && __builtin_popcountll(S) < M; ++q) S |= 1ULL << q;
            run_stage(d, s, S, chosen);
        }
        remaining.swap(deferred);
    }
    s->pending.clear();
}

static void flush_all() {
    for (States *s : g_dev.states) flush(s);
}

static double read_result(Device &d, double *d_val) {
    QG_CUDA(cudaMemcpyAsync(d.h_result, d_val, sizeof(double), cudaMemcpyDeviceToHost, d.stream));
    QG_CUDA(cudaStreamSynchronize(d.stream));
    return d.h_result[0];
}


// ------------------------------------------------------------ transfers

// Host-side copy between pinned staging and the caller's (pageable) buffer,
// split over OpenMP threads: one host thread copies ~10-20 GB/s, well below
// what NVLink-C2C delivers into the staging buffers.
static void host_copy(void *dst, const void *src, size_t bytes) {
    const size_t kSlice = 4u << 20;
    if (bytes < 2 * kSlice) {
        memcpy(dst, src, bytes);
        return;
    }
    const long long nslices = (long long)((bytes + kSlice - 1) / kSlice);
#pragma omp parallel for schedule(static)
    for (long long i = 0; i < nslices; ++i) {
        size_t off = (size_t)i * kSlice;
        size_t len = std::min(kSlice, bytes - off);
        memcpy((char *)dst + off, (const char *)src + off, len);
    }
}

// Device buffer -> host, through two pinned staging buffers so that the
// host-side copy of one chunk overlaps the transfer of the next.
// `produce(chunk_begin, chunk_count, dbuf)` fills dbuf on the stream.
// Device -> host transfer of `count` items that `produce(begin, cnt, dst)`
// writes with kernels on the engine stream: straight into the host buffer
// when the device writes pageable host memory (kernel_output and
// host_direct), else through the pinned staging buffers in chunks (two in
// flight), each copied into the host buffer by host threads.
// The host's page size (one write per page faults a destination in; 64 KB
// pages on some Arm hosts make 4 KB steps 16 times too many).
static size_t host_page_bytes() {
    static const size_t bytes = [] {
        const long v = sysconf(_SC_PAGESIZE);
        return v >= 4096 ? (size_t)v : (size_t)4096;
    }();
    return bytes;
}

template <class F>
static void staged_d2h(Device &d, void *host, idx_t count, size_t item, F produce,
                       bool kernel_output = true) {
    if (count <= 0) return;
    if (kernel_output && d.host_direct) {
        produce(0, count, host);
        QG_CUDA(cudaStreamSynchronize(d.stream));
        return;
    }
    const size_t bytes = (size_t)count * item;
    if (d.pageable_copy && bytes >= ((size_t)64 << 20) && bytes <= ((size_t)16 << 30)) {
        void *dbuf = d.arena.alloc(bytes);
        try {
            produce(0, count, dbuf);
            // Touch every page of the destination in parallel while the
            // kernels run (the copy overwrites all of it).
            char *h = (char *)host;
            const size_t kPage = host_page_bytes();
#pragma omp parallel for schedule(static)
            for (long long i = 0; i < (long long)((bytes + kPage - 1) / kPage); ++i)
                ((volatile char *)h)[(size_t)i * kPage] = 0;
            QG_CUDA(cudaMemcpyAsync(host, dbuf, bytes, cudaMemcpyDeviceToHost, d.stream));
            QG_CUDA(cudaStreamSynchronize(d.stream));
        } catch (...) {
            cudaStreamSynchronize(d.stream);
            d.arena.release(dbuf);
            throw;
        }
        d.arena.release(dbuf);
        return;
    }
    idx_t chunk = (idx_t)(Device::kStageBytes / item);
    void *dbuf[2] = {d.arena.alloc(chunk * item), nullptr};
    idx_t nchunks = (count + chunk - 1) / chunk;
    if (nchunks > 1) dbuf[1] = d.arena.alloc(chunk * item);
    idx_t pend_begin[2] = {0, 0}, pend_cnt[2] = {0, 0};
    try {
        for (idx_t c = 0; c < nchunks + 2; ++c) {
            int b = (int)(c & 1);
            if (c >= 2 && pend_cnt[b] > 0) {
                QG_CUDA(cudaEventSynchronize(d.ev[b]));
                host_copy((char *)host + pend_begin[b] * item, d.h_stage[b], pend_cnt[b] * item);
                pend_cnt[b] = 0;
            }
            if (c < nchunks) {
                idx_t begin = c * chunk, cnt = std::min(chunk, count - begin);
                produce(begin, cnt, dbuf[b]);
                QG_CUDA(cudaMemcpyAsync(d.h_stage[b], dbuf[b], cnt * item, cudaMemcpyDeviceToHost,
                                        d.stream));
                QG_CUDA(cudaEventRecord(d.ev[b], d.stream));
                pend_begin[b] = begin;
                pend_cnt[b] = cnt;
            }
        }
    } catch (...) {
        cudaStreamSynchronize(d.stream);
        d.arena.release(dbuf[0]);
        d.arena.release(dbuf[1]);
        throw;
    }
    d.arena.release(dbuf[0]);
    d.arena.release(dbuf[1]);
}

// ------------------------------------------------------------ gather descriptors

static GatherDesc make_gather(const int *lane_tables, const int *lane_counts,
                              const qg_handle *qstates_list, int n_qstates, int prec) {
    if (n_qstates > kMaxGetterStates) fail(QG_ERR_VALUE, "too many qubit states (%d).", n_qstates);
    GatherDesc g;
    memset(&g, 0, sizeof(g));
    g.nqs = n_qstates;
    int off = 0;
    for (int q = 0; q < n_qstates; ++q) {
        States *s = get_alloc_states(qstates_list[q]);
        if (s->prec != prec) fail(QG_ERR_VALUE, "precision mismatch between getter and states.");
        flush(s);
        if (lane_counts[q] != s->n_lanes)
            fail(QG_ERR_VALUE, "lane table size %d != n_lanes %d.", lane_counts[q], s->n_lanes);
        g.ptr[q] = s->d;
        g.lane_begin[q] = off;
        for (int l = 0; l < lane_counts[q]; ++l) {
            if (off >= kMaxLanes) fail(QG_ERR_VALUE, "too many lanes.");
            int e = lane_tables[off];
            if (e < 0 || e >= kMaxLanes) fail(QG_ERR_VALUE, "external lane %d out of range.", e);
            g.ext[off] = (signed char)e;
            ++off;
        }
    }
    g.lane_begin[n_qstates] = off;
    return g;
}

// ------------------------------------------------------------ gate matrices

typedef std::complex<double> cd;

static void put(double *mat, cd a00, cd a01, cd a10, cd a11) {
    cd v[4] = {a00, a01, a10, a11};
    for (int i = 0; i < 4; ++i) {
        mat[2 * i] = v[i].real();
        mat[2 * i + 1] = v[i].imag();
    }
}

// The gate set and conventions of qgate/simulator/src/GateMatrix.cpp:13-158
// (U = Rz(phi) Ry(theta) Rz(lambda) exactly, i.e. OpenQASM's U up to the
// global phase exp(i(lambda+phi)/2)).
static void gate_matrix(const char *name, const double *a, int na, double *mat) {
    const cd j(0., 1.);
    const double r = std::sqrt(0.5);
    auto need = [&](int k) {
        if (na < k) fail(QG_ERR_VALUE, "gate %s needs %d argument(s).", name, k);
    };
    std::string nm(name);
    if (nm == "U") {
        need(3);
        double t2 = a[0] * 0.5, p2 = a[1] * 0.5, l2 = a[2] * 0.5;
        put(mat, std::exp(j * (-l2 - p2)) * std::cos(t2), -std::exp(j * (l2 - p2)) * std::sin(t2),
            std::exp(j * (-l2 + p2)) * std::sin(t2), std::exp(j * (l2 + p2)) * std::cos(t2));
    } else if (nm == "U2") {
        need(2);
        double p2 = a[0] * 0.5, l2 = a[1] * 0.5;
        put(mat, std::exp(j * (-l2 - p2)) * r, -std::exp(j * (l2 - p2)) * r,
            std::exp(j * (-l2 + p2)) * r, std::exp(j * (l2 + p2)) * r);
    } else if (nm == "U1") {
        need(1);
        put(mat, 1., 0., 0., std::exp(j * a[0]));
    } else if (nm == "ID") {
        put(mat, 1., 0., 0., 1.);
    } else if (nm == "X") {
        put(mat, 0., 1., 1., 0.);
    } else if (nm == "Y") {
        put(mat, 0., -j, j, 0.);
    } else if (nm == "Z") {
        put(mat, 1., 0., 0., -1.);
    } else if (nm == "H") {
        put(mat, r, r, r, -r);
    } else if (nm == "S") {
        put(mat, 1., 0., 0., j);
    } else if (nm == "T") {
        put(mat, 1., 0., 0., std::exp(j * (M_PI * 0.25)));
    } else if (nm == "RX") {
        need(1);
        double c = std::cos(a[0] / 2.), s = std::sin(a[0] / 2.);
        put(mat, c, -j * s, -j * s, c);
    } else if (nm == "RY") {
        need(1);
        double c = std::cos(a[0] / 2.), s = std::sin(a[0] / 2.);
        put(mat, c, -s, s, c);
    } else if (nm == "RZ") {
        need(1);
        double t2 = a[0] / 2.;
        put(mat, std::exp(-j * t2), 0., 0., std::exp(j * t2));
    } else if (nm == "ExpiI") {
        need(1);
        cd e = std::exp(j * a[0]);
        put(mat, e, 0., 0., e);
    } else if (nm == "ExpiZ") {
        need(1);
        put(mat, std::exp(j * a[0]), 0., 0., std::exp(-j * a[0]));
    } else if (nm == "SH") {
        put(mat, r, r, j * r, -j * r);
    } else {
        fail(QG_ERR_RUNTIME, "Unknown gate type.");
    }
}

static void adjoint2(double *m) {
    // conj(transpose)
    double t[8];
    memcpy(t, m, sizeof(t));
    m[0] = t[0];
    m[1] = -t[1];
    m[2] = t[4];
    m[3] = -t[5];
    m[4] = t[2];
    m[5] = -t[3];
    m[6] = t[6];
    m[7] = -t[7];
}

// ------------------------------------------------------------ compiled circuits

static void drop_graph(Device &d, Circuit *c) {
    if (c->exec || !c->chunks.empty()) QG_CUDA(cudaStreamSynchronize(d.stream));
    if (c->exec) cudaGraphExecDestroy(c->exec);
    if (c->g) cudaGraphDestroy(c->g);
    for (auto &ch : c->chunks) {
        cudaFreeHost(ch.first);
        cudaFree(ch.second);
    }
    c->chunks.clear();
    c->chunk_off = 0;
    c->exec = nullptr;
    c->g = nullptr;
    c->state = nullptr;
    c->n_lanes = -1;
}

// Plans the circuit's gates on s under stream capture (nothing runs) and
// instantiates the graph.  The states object's queue must be empty.
static void capture_circuit(Device &d, Circuit *c, States *s) {
    const bool timing = d.timing;
    const long long p0 = d.n_passes, b0 = d.n_bytes;
    d.timing = false;
    d.capturing = c;
    cudaGraph_t graph = nullptr;
    auto restore = [&] {
        d.capturing = nullptr;
        d.timing = timing;
        d.n_passes = p0;
        d.n_bytes = b0;
        s->pending.clear();
    };
    QG_CUDA(cudaStreamBeginCapture(d.stream, cudaStreamCaptureModeRelaxed));
    try {
        s->pending = c->gates;
        flush(s);
    } catch (...) {
        cudaStreamEndCapture(d.stream, &graph);
        if (graph) cudaGraphDestroy(graph);
        restore();
        throw;
    }
    const cudaError_t ec = cudaStreamEndCapture(d.stream, &graph);
    c->passes = d.n_passes - p0;
    c->bytes = d.n_bytes - b0;
    restore();
    cuda_check(ec, "cudaStreamEndCapture");
    cudaGraphExec_t exec = nullptr;
    const cudaError_t ei = cudaGraphInstantiate(&exec, graph, 0);
    if (ei != cudaSuccess) {
        cudaGraphDestroy(graph);
        cuda_check(ei, "cudaGraphInstantiate");
    }
    c->g = graph;
    c->exec = exec;
    c->state = s->d;
    c->n_lanes = s->n_lanes;
    c->version = d.settings_version;
}

// ------------------------------------------------------------ trace replay

constexpr size_t kTraceMinGates = 8, kTraceSlots = 8;

static unsigned long long trace_hash(const States *s, const std::vector<PendingGate> &gates) {
    unsigned long long h = 1469598103934665603ULL;  // FNV-1a
    auto mix = [&](const void *p, size_t n) {
        const unsigned char *b = (const unsigned char *)p;
        for (size_t i = 0; i < n; ++i) h = (h ^ b[i]) * 1099511628211ULL;
    };
    mix(&s->prec, sizeof(s->prec));
    mix(&s->n_lanes, sizeof(s->n_lanes));
    for (const auto &g : gates) {
        mix(&g.target, sizeof(g.target));
        const int nc = (int)g.controls.size();
        mix(&nc, sizeof(nc));
        if (nc) mix(g.controls.data(), sizeof(int) * (size_t)nc);
        mix(g.m.v, sizeof(g.m.v));
    }
    return h;
}

static bool same_gates(const std::vector<PendingGate> &a, const std::vector<PendingGate> &b) {
    if (a.size() != b.size()) return false;
    for (size_t i = 0; i < a.size(); ++i)
        if (a[i].target != b[i].target || a[i].controls != b[i].controls ||
            memcmp(a[i].m.v, b[i].m.v, sizeof(a[i].m.v)) != 0)
            return false;
    return true;
}

// Called by flush() with the states object's pending gates (a whole run
// since the last flush, none of it launched yet).  A run seen before is
// applied from its circuit: the second time it is planned under stream
// capture into a CUDA graph, every later time the graph is replayed with no
// host planning; the plan is the same, so the state is the same.  A new run
// is remembered (the least recently used of kTraceSlots is forgotten) and
// planned as usual.  Returns whether the run was applied here.
static bool replay_trace(Device &d, States *s) {
    if (!d.trace_replay || d.capturing || s->streamed || s->pending.size() < kTraceMinGates)
        return false;
    const unsigned long long h = trace_hash(s, s->pending);
    Device::Trace *hit = nullptr;
    for (auto &t : d.traces)
        if (t.hash == h && t.c->prec == s->prec && same_gates(t.c->gates, s->pending)) {
            hit = &t;
            break;
        }
    if (!hit) {
        Circuit *c = new Circuit();
        c->prec = s->prec;
        c->graph = true;
        c->gates = s->pending;
        Device::Trace t;
        t.hash = h;
        t.c = c;
        t.used = ++d.trace_clock;
        if (d.traces.size() < kTraceSlots) {
            d.traces.push_back(t);
        } else {
            auto lru = std::min_element(d.traces.begin(), d.traces.end(),
                                        [](const Device::Trace &a, const Device::Trace &b) {
                                            return a.used < b.used;
                                        });
            if (lru->c->exec || !lru->c->chunks.empty()) drop_graph(d, lru->c);
            delete lru->c;
            *lru = t;
        }
        return false;  // planned as usual
    }
    hit->used = ++d.trace_clock;
    Circuit *c = hit->c;
    std::vector<PendingGate> run;
    run.swap(s->pending);  // capture_circuit wants the queue empty
    if (c->exec && (c->state != s->d || c->n_lanes != s->n_lanes ||
                    c->version != d.settings_version))
        drop_graph(d, c);
    if (!c->exec) {
        capture_circuit(d, c, s);
        d.trace_captures += 1;
    } else {
        d.trace_hits += 1;
    }
    QG_CUDA(cudaGraphLaunch(c->exec, d.stream));
    d.n_passes += c->passes;
    d.n_bytes += c->bytes;
    return true;
}

static void drop_traces(Device &d) {
    for (auto &t : d.traces) {
        if (t.c->exec || !t.c->chunks.empty()) drop_graph(d, t.c);
        delete t.c;
    }
    d.traces.clear();
}

}  // namespace qg

using namespace qg;

#define QG_BEGIN                                      \
    try {                                             \
        std::lock_guard<std::recursive_mutex> _lk(g_dev.mu);
#define QG_END                                                 \
    }                                                          \
    catch (const qg::Error &e) {                               \
        t_last_error = e.msg;                                  \
        return e.code;                                         \
    }                                                          \
    catch (const std::bad_alloc &) {                           \
        t_last_error = "host allocation failed";               \
        return QG_ERR_NOMEM;                                   \
    }                                                          \
    catch (...) {                                              \
        t_last_error = "unknown error";                        \
        return QG_ERR_RUNTIME;                                 \
    }                                                          \
    t_last_error.clear();                                      \
    return QG_OK;

static void check_prec(int prec) {
    if (prec != kFP64 && prec != kFP32) fail(QG_ERR_VALUE, "unexpected dtype.");
}

extern "C" {

const char *qg_last_error(void) { return t_last_error.c_str(); }

int qg_devices_initialize(int device_id, int64_t memory_limit) {
    QG_BEGIN
    if (g_dev.initialized) {
        if (device_id >= 0 && device_id != g_dev.dev)
            fail(QG_ERR_RUNTIME, "already initialized on device %d.", g_dev.dev);
        g_dev.arena.limit = memory_limit;
    } else {
        device_init(device_id, memory_limit);
    }
    QG_END
}

int qg_devices_clear(void) {
    QG_BEGIN
    if (g_dev.initialized) {
        QG_CUDA(cudaSetDevice(g_dev.dev));
        cudaStreamSynchronize(g_dev.stream);
        drop_traces(g_dev);
        g_dev.arena.trim();
        if (g_dev.h_batch) cudaFreeHost(g_dev.h_batch);
        g_dev.h_batch = nullptr;
        g_dev.h_batch_bytes = 0;
    }
    QG_END
}

int qg_arena_stats(int64_t *in_use, int64_t *cached) {
    QG_BEGIN
    *in_use = (int64_t)g_dev.arena.in_use;
    *cached = (int64_t)g_dev.arena.cached;
    QG_END
}

int qg_qubit_states_new(int prec, qg_handle *out) {
    QG_BEGIN
    check_prec(prec);
    States *s = new States();
    s->prec = prec;
    g_dev.states.insert(s);
    *out = (qg_handle)s;
    QG_END
}

int qg_qubit_states_delete(qg_handle h) {
    QG_BEGIN
    States *s = get_states(h);
    s->pending.clear();
    drop_contents(s);  // the buffer goes back to the arena unless a lazy object reads it
    g_dev.states.erase(s);
    delete s;
    QG_END
}

int qg_qubit_states_deallocate(qg_handle h) {
    QG_BEGIN
    States *s = get_states(h);
    s->pending.clear();
    drop_contents(s);
    s->n_lanes = -1;
    QG_END
}

int qg_qubit_states_get_n_lanes(qg_handle h, int *n) {
    QG_BEGIN
    *n = get_states(h)->n_lanes;
    QG_END
}

int qg_qubit_processor_new(int prec, qg_handle *out) {
    QG_BEGIN
    check_prec(prec);
    Processor *p = new Processor{prec};
    g_dev.procs.insert(p);
    *out = (qg_handle)p;
    QG_END
}

int qg_qubit_processor_delete(qg_handle h) {
    QG_BEGIN
    Processor *p = lookup(g_dev.procs, h, "processor");
    g_dev.procs.erase(p);
    delete p;
    QG_END
}

int qg_qubit_processor_synchronize(qg_handle h) {
    QG_BEGIN
    lookup(g_dev.procs, h, "processor");
    Device &d = dev();
    flush_all();
    QG_CUDA(cudaStreamSynchronize(d.stream));
    QG_END
}

int qg_qubit_processor_reset(qg_handle h) {
    QG_BEGIN
    lookup(g_dev.procs, h, "processor");
    QG_END
}

int qg_qubit_processor_initialize_qubit_states(qg_handle hp, qg_handle hs, int n_lanes) {
    QG_BEGIN
    Processor *p = lookup(g_dev.procs, hp, "processor");
    States *s = get_states(hs);
    if (p->prec != s->prec) fail(QG_ERR_VALUE, "precision mismatch.");
    if (n_lanes < 0 || n_lanes > 40) fail(QG_ERR_VALUE, "n_lanes %d out of range.", n_lanes);
    Device &d = dev();
    s->pending.clear();
    const size_t bytes = ((size_t)1 << n_lanes) * complex_size(s->prec);
    if (d.arena.limit >= 0 && (long long)Arena::size_class(bytes) > d.arena.limit)
        fail(QG_ERR_NOMEM, "Out of device memory. (arena limit %lld bytes, requested %zu)",
             d.arena.limit, bytes);
    // |0...0> without a buffer: allocated when first read or written
    s->n_lanes = n_lanes;
    set_basis(s, 0);
    QG_END
}

int qg_qubit_processor_reset_qubit_states(qg_handle hp, qg_handle hs) {
    QG_BEGIN
    lookup(g_dev.procs, hp, "processor");
    States *s = get_alloc_states(hs);
    s->pending.clear();
    // |0...0> is left lazy, so that gates reaching the basis state first can
    // still be folded into it; a live state's buffer goes back to the arena
    // and its free list normally hands the same block back when the state is
    // next formed.
    set_basis(s, 0);
    QG_END
}

int qg_qubit_processor_calc_probability(qg_handle hp, qg_handle hs, int lane, double *prob) {
    QG_BEGIN
    lookup(g_dev.procs, hp, "processor");
    States *s = get_alloc_states(hs);
    check_lane(s, lane);
    Device &d = dev();
    flush(s);
    PairIdx pi = pair_pattern({lane}, 0, 0);
    double *d_out = d.d_partials + reduce_partials();
    timed(d, "prob", [&] {
        launch_prob(s->prec, s->d, (idx_t)1 << (s->n_lanes - 1), pi, d.d_partials, d_out, d.stream);
    });
    *prob = read_result(d, d_out);
    QG_END
}

int qg_qubit_processor_join(qg_handle hp, qg_handle hs, const qg_handle *list, int n_list,
                            int n_new_lanes) {
    QG_BEGIN
    lookup(g_dev.procs, hp, "processor");
    States *dst = get_alloc_states(hs);
    Device &d = dev();
    if (n_list < 1) fail(QG_ERR_VALUE, "join needs at least one source.");
    if (n_new_lanes < 0) fail(QG_ERR_VALUE, "join: negative count of new lanes.");
    std::vector<States *> srcs(n_list);
    int total = 0;
    for (int i = 0; i < n_list; ++i) {
        States *s = get_alloc_states(list[i]);
        if (s == dst) fail(QG_ERR_VALUE, "join destination is also a source.");
        if (s->prec != dst->prec) fail(QG_ERR_VALUE, "precision mismatch.");
        srcs[i] = s;
        total += s->n_lanes;
    }
    if (total + n_new_lanes != dst->n_lanes)
        fail(QG_ERR_VALUE, "join: %d + %d lanes != %d.", total, n_new_lanes, dst->n_lanes);
    d.g_joins += 1;
    // The joined state is the kron product of the sources (the last source
    // at the lowest lanes, the new lanes |0> above them all), each source's
    // pending gates moved up by the lanes below it; nothing runs until the
    // product is read.  The sources keep their amplitudes and gates.
    std::vector<Factor> fs;
    std::vector<PendingGate> moved;
    if (n_new_lanes > 0) {
        Factor f;
        f.n_lanes = n_new_lanes;
        fs.push_back(f);
    }
    int offset = total;
    for (States *s : srcs) {
        offset -= s->n_lanes;
        if (s->lazy == States::kView) materialize(d, s);
        if (s->lazy == States::kProduct) {
            fs.insert(fs.end(), s->factors.begin(), s->factors.end());
        } else {
            Factor f;
            f.buf = s->buf;
            f.n_lanes = s->n_lanes;
            fs.push_back(f);
        }
        for (const PendingGate &g : s->pending) {
            PendingGate m = g;
            m.target += offset;
            for (int &c : m.controls) c += offset;
            moved.push_back(m);
        }
    }
    coalesce_factors(fs);
    drop_contents(dst);
    dst->lazy = States::kProduct;
    dst->factors.swap(fs);
    dst->pending.swap(moved);
    dst->streamed = false;
    QG_END
}

int qg_qubit_processor_decohere(qg_handle hp, int value, double prob, qg_handle hs, int lane) {
    QG_BEGIN
    lookup(g_dev.procs, hp, "processor");
    States *s = get_alloc_states(hs);
    check_lane(s, lane);
    if (value != 0 && value != 1) fail(QG_ERR_VALUE, "value must be 0 or 1.");
    Device &d = dev();
    flush(s);
    prepare_write(d, s);
    double norm = value == 0 ? 1. / std::sqrt(prob) : 1. / std::sqrt(1. - prob);
    PairIdx pi = pair_pattern({lane}, 0, 1ULL << lane);
    timed(d, "measure", [&] {
        launch_decohere(s->prec, s->d, (idx_t)1 << (s->n_lanes - 1), pi, value, norm, d.stream);
    });
    QG_END
}

int qg_qubit_processor_decohere_and_separate(qg_handle hp, int value, double prob,
                                             qg_handle h0, qg_handle h1, qg_handle hs,
                                             int lane) {
    QG_BEGIN
    lookup(g_dev.procs, hp, "processor");
    States *s = get_alloc_states(hs);
    States *s0 = get_alloc_states(h0);
    States *s1 = get_alloc_states(h1);
    check_lane(s, lane);
    if (value != 0 && value != 1) fail(QG_ERR_VALUE, "value must be 0 or 1.");
    if (s0->n_lanes != s->n_lanes - 1 || s1->n_lanes != 1)
        fail(QG_ERR_VALUE, "decohere_and_separate: wrong destination sizes.");
    if (s0->prec != s->prec || s1->prec != s->prec) fail(QG_ERR_VALUE, "precision mismatch.");
    if (s0 == s || s1 == s || s0 == s1)
        fail(QG_ERR_VALUE, "decohere_and_separate: the three states objects must differ.");
    Device &d = dev();
    flush(s);
    d.g_separates += 1;
    const double norm = value == 0 ? 1. / std::sqrt(prob) : 1. / std::sqrt(1. - prob);
    // qstates0: a view of the source's buffer with the lane removed (formed
    // when read: in place if the source is gone by then); qstates1 = |value>
    s0->pending.clear();
    s0->streamed = false;
    drop_contents(s0);
    s0->lazy = States::kView;
    s0->parent = s->buf;
    s0->sep_lane = lane;
    s0->sep_value = value;
    s0->sep_norm = norm;
    s1->pending.clear();
    s1->streamed = false;
    set_basis(s1, value);
    QG_END
}

int qg_qubit_processor_apply_reset(qg_handle hp, qg_handle hs, int lane) {
    QG_BEGIN
    lookup(g_dev.procs, hp, "processor");
    States *s = get_alloc_states(hs);
    check_lane(s, lane);
    Device &d = dev();
    flush(s);
    prepare_write(d, s);
    PairIdx pi = pair_pattern({lane}, 0, 1ULL << lane);
    timed(d, "measure", [&] { launch_reset(s->prec, s->d, (idx_t)1 << (s->n_lanes - 1), pi, d.stream); });
    QG_END
}

static void enqueue_gate(qg_handle hp, const double *mat, qg_handle hs, const int *ctrl,
                         int n_ctrl, int target) {
    lookup(g_dev.procs, hp, "processor");
    States *s = get_alloc_states(hs);
    check_lane(s, target);
    PendingGate g;
    g.target = target;
    unsigned long long seen = 1ULL << target;
    for (int i = 0; i < n_ctrl; ++i) {
        check_lane(s, ctrl[i]);
        if (seen & (1ULL << ctrl[i])) fail(QG_ERR_RUNTIME, "control and operand overlapped.");
        seen |= 1ULL << ctrl[i];
        g.controls.push_back(ctrl[i]);
    }
    memcpy(g.m.v, mat, sizeof(g.m.v));
    g.diag = is_diag(g.m);
    s->pending.push_back(g);
    g_dev.n_gates += 1;
    stream_flush(s);
}

int qg_qubit_processor_apply_gate(qg_handle hp, const double *mat, qg_handle hs, int lane) {
    QG_BEGIN
    enqueue_gate(hp, mat, hs, nullptr, 0, lane);
    QG_END
}

int qg_qubit_processor_apply_controlled_gate(qg_handle hp, const double *mat, qg_handle hs,
                                             const int *ctrl, int n_ctrl, int target) {
    QG_BEGIN
    enqueue_gate(hp, mat, hs, ctrl, n_ctrl, target);
    QG_END
}

// ------------------------------------------------------------ compiled circuits

int qg_set_batch_one_launch(int on) {
    QG_BEGIN
    g_dev.batch_one_launch = on != 0;
    QG_END
}

int qg_set_trace_replay(int on) {
    QG_BEGIN
    flush_all();
    g_dev.trace_replay = on != 0;
    if (!on) drop_traces(g_dev);
    QG_END
}

int qg_trace_stats(int64_t *hits, int64_t *captures, int reset) {
    QG_BEGIN
    *hits = g_dev.trace_hits;
    *captures = g_dev.trace_captures;
    if (reset) g_dev.trace_hits = g_dev.trace_captures = 0;
    QG_END
}

int qg_circuit_new(int prec, int n_gates, const int *targets, const int *ctrl_offsets,
                   const int *ctrl_lanes, const double *matrices, qg_handle *out) {
    QG_BEGIN
    check_prec(prec);
    if (n_gates < 0) fail(QG_ERR_VALUE, "negative gate count.");
    if (n_gates > 0 && (!targets || !ctrl_offsets || !matrices))
        fail(QG_ERR_VALUE, "null gate arrays.");
    Circuit *c = new Circuit();
    c->prec = prec;
    try {
        c->gates.reserve(n_gates);
        for (int i = 0; i < n_gates; ++i) {
            PendingGate g;
            g.target = targets[i];
            if (g.target < 0 || g.target >= kMaxLanes)
                fail(QG_ERR_VALUE, "gate %d: target lane %d out of range.", i, g.target);
            unsigned long long seen = 1ULL << g.target;
            c->min_lanes = std::max(c->min_lanes, g.target + 1);
            if (ctrl_offsets[i + 1] < ctrl_offsets[i] || (ctrl_offsets[i + 1] > ctrl_offsets[i] && !ctrl_lanes))
                fail(QG_ERR_VALUE, "gate %d: bad control offsets.", i);
            for (int k = ctrl_offsets[i]; k < ctrl_offsets[i + 1]; ++k) {
                const int cl = ctrl_lanes[k];
                if (cl < 0 || cl >= kMaxLanes)
                    fail(QG_ERR_VALUE, "gate %d: control lane %d out of range.", i, cl);
                if (seen & (1ULL << cl)) fail(QG_ERR_RUNTIME, "control and operand overlapped.");
                seen |= 1ULL << cl;
                g.controls.push_back(cl);
                c->min_lanes = std::max(c->min_lanes, cl + 1);
            }
            memcpy(g.m.v, matrices + 8 * (size_t)i, sizeof(g.m.v));
            g.diag = is_diag(g.m);
            c->gates.push_back(std::move(g));
        }
    } catch (...) {
        delete c;
        throw;
    }
    g_dev.circuits.insert(c);
    *out = (qg_handle)c;
    QG_END
}

int qg_circuit_set_graph(qg_handle hc, int on) {
    QG_BEGIN
    Circuit *c = lookup(g_dev.circuits, hc, "circuit");
    if (!on && (c->exec || !c->chunks.empty())) drop_graph(dev(), c);
    c->graph = on != 0;
    QG_END
}

int qg_circuit_run(qg_handle hc, qg_handle hs) {
    QG_BEGIN
    Circuit *c = lookup(g_dev.circuits, hc, "circuit");
    States *s = get_alloc_states(hs);
    if (s->prec != c->prec) fail(QG_ERR_VALUE, "precision mismatch between circuit and states.");
    if (s->n_lanes < c->min_lanes)
        fail(QG_ERR_VALUE, "circuit uses %d lanes, the states object has %d.", c->min_lanes,
             s->n_lanes);
    Device &d = dev();
    if (c->gates.empty()) {
        t_last_error.clear();
        return QG_OK;
    }
    if (!c->graph) {
        for (const auto &g : c->gates) {
            s->pending.push_back(g);
            stream_flush(s);
        }
        d.n_gates += (long long)c->gates.size();
    } else {
        flush(s);  // earlier gates of this states object run first
        prepare_write(d, s);
        if (c->exec && (c->state != s->d || c->n_lanes != s->n_lanes ||
                        c->version != d.settings_version))
            drop_graph(d, c);
        if (!c->exec) capture_circuit(d, c, s);
        QG_CUDA(cudaGraphLaunch(c->exec, d.stream));
        d.n_gates += (long long)c->gates.size();
        d.n_passes += c->passes;
        d.n_bytes += c->bytes;
    }
    QG_END
}

int qg_circuit_stats(qg_handle hc, int *captured, int64_t *passes) {
    QG_BEGIN
    Circuit *c = lookup(g_dev.circuits, hc, "circuit");
    *captured = c->exec != nullptr;
    *passes = c->passes;
    QG_END
}

int qg_circuit_delete(qg_handle hc) {
    QG_BEGIN
    Circuit *c = lookup(g_dev.circuits, hc, "circuit");
    if (c->exec || !c->chunks.empty()) drop_graph(dev(), c);  // no device work otherwise
    g_dev.circuits.erase(c);
    delete c;
    QG_END
}

int qg_qubit_processor_apply_multi(qg_handle hp, const double *mat, qg_handle hs,
                                   const int *targets, int n_targets, const int *ctrl,
                                   int n_ctrl) {
    QG_BEGIN
    lookup(g_dev.procs, hp, "processor");
    States *s = get_alloc_states(hs);
    if (n_targets < 1 || n_targets > 5) fail(QG_ERR_VALUE, "1..5 targets supported.");
    MultiDesc md;
    memset(&md, 0, sizeof(md));
    md.k = n_targets;
    unsigned long long seen = 0;
    std::vector<int> pos;
    for (int i = 0; i < n_targets; ++i) {
        check_lane(s, targets[i]);
        if (seen & (1ULL << targets[i])) fail(QG_ERR_VALUE, "duplicate target lane.");
        seen |= 1ULL << targets[i];
        md.tpos[i] = targets[i];
        pos.push_back(targets[i]);
    }
    for (int i = 0; i < n_ctrl; ++i) {
        check_lane(s, ctrl[i]);
        if (seen & (1ULL << ctrl[i])) fail(QG_ERR_RUNTIME, "control and operand overlapped.");
        seen |= 1ULL << ctrl[i];
        md.cmask |= 1ULL << ctrl[i];
        pos.push_back(ctrl[i]);
    }
    std::sort(pos.begin(), pos.end());
    md.npos = (int)pos.size();
    for (int i = 0; i < md.npos; ++i) md.pos[i] = pos[i];
    Device &d = dev();
    flush(s);
    prepare_write(d, s);
    size_t dim = (size_t)1 << n_targets;
    size_t bytes = dim * dim * 2 * sizeof(double);
    void *dmat = d.arena.alloc(bytes);
    QG_CUDA(cudaMemcpyAsync(dmat, mat, bytes, cudaMemcpyHostToDevice, d.stream));
    idx_t n_items = (idx_t)1 << (s->n_lanes - md.npos);
    timed(d, "multi", [&] { launch_apply_multi(s->prec, s->d, n_items, md, dmat, d.stream); });
    // The host matrix may be reused by the caller as soon as we return.
    QG_CUDA(cudaStreamSynchronize(d.stream));
    d.arena.release(dmat);
    d.n_gates += 1;
    d.n_passes += 1;
    d.n_bytes += 2 * ((long long)n_items << n_targets) * (long long)complex_size(s->prec);
    QG_END
}

int qg_qubit_processor_calc_pauli_expectation(qg_handle hp, qg_handle hs, uint64_t x_mask,
                                              uint64_t z_mask, double *out) {
    QG_BEGIN
    lookup(g_dev.procs, hp, "processor");
    States *s = get_alloc_states(hs);
    unsigned long long all = s->n_lanes >= 64 ? ~0ULL : ((1ULL << s->n_lanes) - 1);
    if ((x_mask | z_mask) & ~all) fail(QG_ERR_VALUE, "Pauli mask outside the state's lanes.");
    Device &d = dev();
    flush(s);
    double *d_out = d.d_partials + reduce_partials();
    timed(d, "pauli", [&] {
        launch_pauli(s->prec, s->d, s->n_lanes, x_mask, z_mask, d.d_partials, d_out, d.stream);
    });
    *out = read_result(d, d_out);
    QG_END
}

int qg_qubit_processor_calc_norm(qg_handle hp, qg_handle hs, double *out) {
    QG_BEGIN
    lookup(g_dev.procs, hp, "processor");
    States *s = get_alloc_states(hs);
    Device &d = dev();
    flush(s);
    double *d_out = d.d_partials + reduce_partials();
    launch_pauli(s->prec, s->d, s->n_lanes, 0, 0, d.d_partials, d_out, d.stream);
    *out = read_result(d, d_out);
    QG_END
}

int qg_set_fusion(int max_tile_lanes) {
    QG_BEGIN
    if (max_tile_lanes < 0 || max_tile_lanes > kMaxTileLanes)
        fail(QG_ERR_VALUE, "max_tile_lanes must be in [0, %d].", kMaxTileLanes);
    flush_all();
    g_dev.settings_version += 1;  // compiled circuits re-plan
    if (max_tile_lanes == 0) {
        g_dev.tile_lanes[kFP32] = 12;
        g_dev.tile_lanes[kFP64] = 12;
        g_dev.reg_lanes[kFP32] = 4;
        g_dev.reg_lanes[kFP64] = 3;
        g_dev.cost_budget[kFP32] = 0;
        g_dev.cost_budget[kFP64] = 0;
        g_dev.tensor_blocks = true;
        g_dev.pipelined = false;
    } else {
        g_dev.tile_lanes[kFP32] = max_tile_lanes;
        g_dev.tile_lanes[kFP64] = std::min(max_tile_lanes, 13);
    }
    QG_END
}

int qg_set_fusion_params(int prec, int tile_lanes, int reg_lanes, int cost_budget) {
    QG_BEGIN
    check_prec(prec);
    if (tile_lanes < 1 || tile_lanes > kMaxTileLanes) fail(QG_ERR_VALUE, "tile_lanes out of range.");
    if (reg_lanes < 3 || reg_lanes > kMaxRegLanes) fail(QG_ERR_VALUE, "reg_lanes must be in [3, 5].");
    if (cost_budget < 0) fail(QG_ERR_VALUE, "cost_budget must be >= 0.");
    flush_all();
    g_dev.settings_version += 1;  // compiled circuits re-plan
    g_dev.tile_lanes[prec] = tile_lanes;
    g_dev.reg_lanes[prec] = reg_lanes;
    g_dev.cost_budget[prec] = cost_budget;
    QG_END
}

int qg_set_tensor_blocks(int on) {
    QG_BEGIN
    flush_all();
    g_dev.settings_version += 1;  // compiled circuits re-plan
    g_dev.tensor_blocks = on != 0;
    QG_END
}

int qg_tensor_stage_status(int reset, int *status) {
    QG_BEGIN
    Device &d = dev();
    flush_all();
    QG_CUDA(cudaStreamSynchronize(d.stream));
    *status = tstage_status(reset != 0);
    QG_END
}

int qg_set_pool_guide_index_shift(int k) {
    QG_BEGIN
    if (k < -1 || k > 8) fail(QG_ERR_VALUE, "guide index shift must be in [-1, 8].");
    dev().guide_index_shift = k;
    QG_END
}

int qg_set_pageable_copy(int on) {
    QG_BEGIN
    Device &d = dev();
    if (on && !d.host_direct_supported)
        fail(QG_ERR_VALUE, "this device does not access pageable host memory.");
    d.pageable_copy = on != 0;
    QG_END
}

int qg_set_host_direct(int on) {
    QG_BEGIN
    Device &d = dev();
    if (on && !d.host_direct_supported)
        fail(QG_ERR_VALUE, "this device does not access pageable host memory.");
    d.host_direct = on != 0;
    QG_END
}

int qg_set_stage_pipelining(int on) {
    QG_BEGIN
    flush_all();
    g_dev.settings_version += 1;  // compiled circuits re-plan
    g_dev.pipelined = on != 0;
    QG_END
}

int qg_gate_stats(int64_t *gates, int64_t *passes, int64_t *bytes, int reset) {
    QG_BEGIN
    *gates = g_dev.n_gates;
    *passes = g_dev.n_passes;
    *bytes = g_dev.n_bytes;
    if (reset) g_dev.n_gates = g_dev.n_passes = g_dev.n_bytes = 0;
    QG_END
}

int qg_grouping_stats(int64_t *out, int n, int reset) {
    QG_BEGIN
    const long long v[7] = {g_dev.g_joins,     g_dev.g_krons,   g_dev.g_allocs, g_dev.g_separates,
                            g_dev.g_inplace, g_dev.g_copies, g_dev.g_cow};
    for (int i = 0; i < n && i < 7; ++i) out[i] = v[i];
    if (reset)
        g_dev.g_joins = g_dev.g_krons = g_dev.g_allocs = g_dev.g_separates = g_dev.g_inplace =
            g_dev.g_copies = g_dev.g_cow = 0;
    QG_END
}

int qg_qubit_states_get_raw(qg_handle hs, void *host, int64_t n) {
    QG_BEGIN
    States *s = get_alloc_states(hs);
    if (n != ((int64_t)1 << s->n_lanes)) fail(QG_ERR_VALUE, "size mismatch.");
    Device &d = dev();
    flush(s);
    size_t cs = complex_size(s->prec);
    staged_d2h(
        d, host, n, cs,
        [&](idx_t begin, idx_t cnt, void *dbuf) {
            QG_CUDA(cudaMemcpyAsync(dbuf, (char *)s->d + begin * cs, cnt * cs,
                                    cudaMemcpyDeviceToDevice, d.stream));
        },
        false);
    QG_END
}

int qg_qubit_states_set_raw(qg_handle hs, const void *host, int64_t n) {
    QG_BEGIN
    States *s = get_alloc_states(hs);
    if (n != ((int64_t)1 << s->n_lanes)) fail(QG_ERR_VALUE, "size mismatch.");
    Device &d = dev();
    s->pending.clear();
    if (s->lazy != States::kDense || !s->buf || s->buf.use_count() > 1) {
        // overwritten whole: a buffer of its own, nothing to copy
        drop_contents(s);
        set_buffer(s, new_buffer(d, s->prec, s->n_lanes));
    }
    QG_CUDA(cudaMemcpyAsync(s->d, host, n * complex_size(s->prec), cudaMemcpyHostToDevice,
                            d.stream));
    QG_CUDA(cudaStreamSynchronize(d.stream));
    QG_END
}

int qg_timing_enable(int on) {
    QG_BEGIN
    Device &d = dev();
    if (!on) settle_timers(d);
    d.timing = on != 0;
    QG_END
}

int qg_timing_read(const char *kernel_class, int64_t *launches, double *total_ms, int reset) {
    QG_BEGIN
    Device &d = dev();
    settle_timers(d);
    auto it = d.timers.find(kernel_class ? kernel_class : "");
    *launches = it == d.timers.end() ? 0 : it->second.launches;
    *total_ms = it == d.timers.end() ? 0. : it->second.ms;
    if (reset) d.timers.clear();
    QG_END
}

int qg_device_info(int64_t *info, int n) {
    QG_BEGIN
    Device &d = dev();
    const cudaDeviceAttr attrs[] = {cudaDevAttrMultiProcessorCount,
                                    cudaDevAttrMaxSharedMemoryPerBlockOptin,
                                    cudaDevAttrL2CacheSize,
                                    cudaDevAttrPageableMemoryAccess,
                                    cudaDevAttrPageableMemoryAccessUsesHostPageTables,
                                    cudaDevAttrConcurrentManagedAccess,
                                    cudaDevAttrComputeCapabilityMajor,
                                    cudaDevAttrComputeCapabilityMinor,
                                    cudaDevAttrClockRate,
                                    cudaDevAttrMemoryClockRate};
    const int na = (int)(sizeof(attrs) / sizeof(attrs[0]));
    for (int i = 0; i < n && i < na; ++i) {
        int v = 0;
        QG_CUDA(cudaDeviceGetAttribute(&v, attrs[i], d.dev));
        info[i] = v;
    }
    size_t fr = 0, tot = 0;
    QG_CUDA(cudaMemGetInfo(&fr, &tot));
    if (n > na) info[na] = (int64_t)fr;
    if (n > na + 1) info[na + 1] = (int64_t)tot;
    QG_END
}

int qg_get_stream(uint64_t *stream) {
    QG_BEGIN
    *stream = (uint64_t)(uintptr_t)dev().stream;
    QG_END
}

// Greedy stage packing of a gate list (the gate queue's planner, reusable).
static std::vector<std::pair<unsigned long long, std::vector<const PendingGate *>>>
plan_gate_stages(const std::vector<PendingGate> &gates, int n, int M, int low) {
    std::vector<std::pair<unsigned long long, std::vector<const PendingGate *>>> out;
    // (gate index, lane mask) of the gates not yet in a stage, in order
    std::vector<std::pair<int, unsigned long long>> remaining, deferred;
    remaining.reserve(gates.size());
    for (size_t i = 0; i < gates.size(); ++i) remaining.emplace_back((int)i, gate_qmask(gates[i]));
    const unsigned long long all = n >= 64 ? ~0ULL : ((1ULL << n) - 1);
    if (n <= M) M = n;
    const unsigned long long base = (n <= M) ? all : ((1ULL << low) - 1);
    while (!remaining.empty()) {
        unsigned long long S = base, blocked = 0;
        std::vector<const PendingGate *> chosen;
        deferred.clear();
        for (const auto &gq : remaining) {
            const unsigned long long q = gq.second;
            if ((q & blocked) || (int)chosen.size() >= kMaxStageGates ||
                __builtin_popcountll(S | q) > M) {
                deferred.push_back(gq);
                blocked |= q;
                continue;
            }
            S |= q;
            chosen.push_back(&gates[gq.first]);
        }
        if (chosen.empty()) fail(QG_ERR_VALUE, "gate wider than a tile.");
        for (int q = 0; q < n && __builtin_popcountll(S) < M; ++q) S |= 1ULL << q;
        out.emplace_back(S, std::move(chosen));
        remaining.swap(deferred);
    }
    return out;
}

// Slot tables of a batch's register sets.  make_set_slots is a pure
// function of (lanes, rl, m) and a batch reuses few distinct sets, so each
// thread keeps the tables it has made (keyed by the lanes, 4 bits each).
static void append_sets(const std::vector<std::vector<int>> &sets, int m, int rl,
                        std::vector<SetSlots> &sets_all) {
    static thread_local std::unordered_map<unsigned long long, SetSlots> memo;
    if (memo.size() > (1u << 16)) memo.clear();
    for (auto &st : sets) {
        unsigned long long key = ((unsigned long long)m << 32) | ((unsigned long long)rl << 28);
        bool keyed = rl <= 7 && (int)st.size() >= rl;
        for (int k = 0; keyed && k < rl; ++k) {
            keyed = st[k] >= 0 && st[k] < 16;
            key |= (unsigned long long)(st[k] & 15) << (4 * k);
        }
        if (!keyed) {
            sets_all.push_back(make_set_slots(st.data(), rl, m, kFP32));
            continue;
        }
        auto it = memo.find(key);
        if (it == memo.end()) it = memo.emplace(key, make_set_slots(st.data(), rl, m, kFP32)).first;
        sets_all.push_back(it->second);
    }
}

// k with a 0 bit inserted at each of pos[0..npos) in turn (the host copy of
// the kernels' tile-index to amplitude-index map).
static unsigned long long host_insert_zeros(unsigned long long k, const int *pos, int npos) {
    for (int i = 0; i < npos; ++i) {
        const unsigned long long low = k & ((1ULL << pos[i]) - 1);
        k = ((k ^ low) << 1) | low;
    }
    return k;
}

// The bits of k placed, in order, at the set bits of mask.
static unsigned host_deposit(unsigned k, unsigned mask) {
    unsigned r = 0;
    for (unsigned b = 1; mask; b <<= 1) {
        const unsigned low = mask & (0u - mask);
        if (k & b) r |= low;
        mask ^= low;
    }
    return r;
}

// Tiles of one stage per work item (a power of two, so it divides the tile
// count of every large circuit): one wait and one completion count per item.
constexpr int kBatchTilesPerItem = 8;

struct BatchStagePart {
    BatchStage hdr;  // ops_off / sets_off local to the circuit
    // Tile-index bits that can be 1 in a tile with a nonzero amplitude:
    // the run starts from |0...0>, so before this stage every amplitude
    // whose lanes outside the earlier stages' tiles are not all 0 is
    // still 0 (a stage mixes amplitudes only within its tiles).
    unsigned live;
};
struct BatchPlan {
    int n = 0, rl = 0;
    bool resident = false;
    std::vector<RegOp<float>> ops;
    std::vector<SetSlots> sets;
    std::vector<BatchStagePart> stages;
    std::string error;
};

// Plans every circuit of a batch independently (in parallel): circuits of
// at most `resident_max` qubits as one register program over the whole
// state, larger ones as 12-lane stages with their tile headers; a planning
// error is recorded in the circuit's plan.
static void plan_batch(int n_circuits, const int *n_qubits, const int64_t *gate_offsets,
                       const qg_circuit_op *gates, int resident_max,
                       std::vector<BatchPlan> &plans) {
    plans.assign(n_circuits, BatchPlan());
#pragma omp parallel for schedule(dynamic, 8)
    for (int c = 0; c < n_circuits; ++c) {
        BatchPlan &P = plans[c];
        try {
            const int n = n_qubits[c];
            P.n = n;
            if (n < 8 || n > 30) fail(QG_ERR_VALUE, "circuit %d: 8..30 qubits supported.", c);
            std::vector<PendingGate> gl;
            gl.reserve((size_t)(gate_offsets[c + 1] - gate_offsets[c]));
            for (int64_t gi = gate_offsets[c]; gi < gate_offsets[c + 1]; ++gi) {
                const qg_circuit_op &op = gates[gi];
                if (op.kind != 0) fail(QG_ERR_VALUE, "circuit %d: fixed gates only.", c);
                if (op.target < 0 || op.target >= n || op.n_controls < 0 || op.n_controls > 4)
                    fail(QG_ERR_VALUE, "circuit %d: bad gate.", c);
                PendingGate g;
                g.target = op.target;
                unsigned long long seen = 1ULL << op.target;
                for (int k = 0; k < op.n_controls; ++k) {
                    int q = op.controls[k];
                    if (q < 0 || q >= n || (seen & (1ULL << q)))
                        fail(QG_ERR_VALUE, "circuit %d: bad control.", c);
                    seen |= 1ULL << q;
                    g.controls.push_back(q);
                }
                memcpy(g.m.v, op.mat, sizeof(g.m.v));
                g.diag = is_diag(g.m);
                gl.push_back(std::move(g));
            }
            merge_runs(gl);
            std::vector<RegOp<float>> prog;
            std::vector<std::vector<int>> sets;
            if (n <= resident_max) {
                P.resident = true;
                P.rl = n <= 9 ? 3 : (n <= 12 ? 4 : 5);
                std::vector<const PendingGate *> ptrs;
                for (auto &g : gl) ptrs.push_back(&g);
                TileLanes tl = tile_lanes_of((1ULL << n) - 1, n);
                build_program<float>(ptrs, tl, P.rl, prog, sets);
                if (sets.size() > 255) fail(QG_ERR_RUNTIME, "circuit %d: program too long.", c);
                P.ops.swap(prog);
                append_sets(sets, n, P.rl, P.sets);
            } else {
                P.rl = 4;
                auto plan = plan_gate_stages(gl, n, 12, 4);
                // a circuit without gates still takes one (empty) pass, which
                // writes its |0...0> state
                if (plan.empty()) plan.emplace_back((1ULL << 12) - 1, std::vector<const PendingGate *>{});
                unsigned long long support = 0;  // lanes of the stages so far
                for (size_t r = 0; r < plan.size(); ++r) {
                    TileLanes tl = tile_lanes_of(plan[r].first, n);
                    build_program<float>(plan[r].second, tl, 4, prog, sets);
                    if (sets.size() > 255) fail(QG_ERR_RUNTIME, "circuit %d: stage too long.", c);
                    BatchStagePart sp;
                    memset(&sp.hdr, 0, sizeof(sp.hdr));
                    sp.hdr.n = n;
                    sp.hdr.m = 12;
                    sp.hdr.rl = 4;
                    fill_tile_header(tl, n, 4, sp.hdr.lowrun, sp.hdr.nhi, sp.hdr.hi_pos,
                                     sp.hdr.nins, sp.hdr.ins_pos, sp.hdr.dep_hi);
                    sp.hdr.nops = (int)prog.size();
                    sp.hdr.nsets = (int)sets.size();
                    sp.hdr.ops_off = (long long)P.ops.size();
                    sp.hdr.sets_off = (int)P.sets.size();
                    sp.live = 0;
                    for (int i = 0; i < n - 12; ++i)
                        if (host_insert_zeros(1ULL << i, sp.hdr.ins_pos, sp.hdr.nins) & support)
                            sp.live |= 1u << i;
                    support |= plan[r].first;
                    P.ops.insert(P.ops.end(), prog.begin(), prog.end());
                    append_sets(sets, 12, 4, P.sets);
                    P.stages.push_back(sp);
                }
            }
        } catch (const Error &e) {
            P.error = e.msg.empty() ? "planning failed" : e.msg;
        } catch (...) {
            P.error = "planning failed";
        }
    }
}

int qg_batch_sum_z(int prec, int n_circuits, const int *n_qubits, const int64_t *gate_offsets,
                   const qg_circuit_op *gates, double *out) {
    QG_BEGIN
    if (prec != kFP32) fail(QG_ERR_VALUE, "batched circuits run in complex64.");
    if (n_circuits < 1) fail(QG_ERR_VALUE, "no circuits.");
    Device &d = dev();
    // Plan every circuit independently (in parallel), then concatenate.
    std::vector<BatchPlan> plans;
    plan_batch(n_circuits, n_qubits, gate_offsets, gates, d.batch_one_launch ? 12 : 13, plans);
    for (auto &P : plans)
        if (!P.error.empty()) fail(QG_ERR_VALUE, "%s", P.error.c_str());

    // The circuits' programs in one buffer (offsets first, then the copies
    // in parallel).
    std::vector<long long> ops_at(n_circuits + 1, 0), sets_at(n_circuits + 1, 0);
    for (int c = 0; c < n_circuits; ++c) {
        ops_at[c + 1] = ops_at[c] + (long long)plans[c].ops.size();
        sets_at[c + 1] = sets_at[c] + (long long)plans[c].sets.size();
    }
    if (sets_at[n_circuits] > INT32_MAX) fail(QG_ERR_VALUE, "too many register sets in one batch.");
    // straight into pinned memory, so that their upload is one DMA each
    const size_t ops_bytes = (size_t)ops_at[n_circuits] * sizeof(RegOp<float>);
    const size_t sets_bytes = (size_t)sets_at[n_circuits] * sizeof(SetSlots);
    const size_t stage_bytes = ((ops_bytes + 255) & ~(size_t)255) + sets_bytes;
    if (d.h_batch_bytes < stage_bytes) {
        if (d.h_batch) QG_CUDA(cudaFreeHost(d.h_batch));
        d.h_batch = nullptr;
        d.h_batch_bytes = 0;
        QG_CUDA(cudaMallocHost(&d.h_batch, stage_bytes));
        d.h_batch_bytes = stage_bytes;
    }
    RegOp<float> *ops_all = (RegOp<float> *)d.h_batch;
    SetSlots *sets_all = (SetSlots *)(d.h_batch + ((ops_bytes + 255) & ~(size_t)255));
#pragma omp parallel for schedule(dynamic, 64)
    for (int c = 0; c < n_circuits; ++c) {
        std::copy(plans[c].ops.begin(), plans[c].ops.end(), ops_all + ops_at[c]);
        std::copy(plans[c].sets.begin(), plans[c].sets.end(), sets_all + sets_at[c]);
    }
    std::vector<ResidentCircuit> res[14];
    std::vector<BatchStage> stages;
    std::vector<unsigned> stage_live;
    // per round, the (stage, tile) items of the per-round form (the
    // one-launch form needs only the count of rounds)
    std::vector<std::vector<int2>> rounds;
    const bool per_round = !d.batch_one_launch;
    std::vector<long long> big_off;
    std::vector<int> big_n, big_idx;
    long long arena_elems = 0;
    for (int c = 0; c < n_circuits; ++c) {
        BatchPlan &P = plans[c];
        const long long ops_base = ops_at[c];
        const int sets_base = (int)sets_at[c];
        if (P.resident) {
            ResidentCircuit rc;
            rc.ops_off = ops_base;
            rc.nops = (int)P.ops.size();
            rc.sets_off = sets_base;
            rc.out_index = c;
            rc.n = P.n;
            rc.rl = P.rl;
            rc.pad = 0;
            res[P.n].push_back(rc);
        } else {
            const long long off = arena_elems;
            arena_elems += ((1LL << P.n) + 31) & ~31LL;
            big_off.push_back(off);
            big_n.push_back(P.n);
            big_idx.push_back(c);
            for (size_t r = 0; r < P.stages.size(); ++r) {
                BatchStage st = P.stages[r].hdr;
                st.state_off = off;
                st.ops_off += ops_base;
                st.sets_off += sets_base;
                int sidx = (int)stages.size();
                stages.push_back(st);
                stage_live.push_back(P.stages[r].live);
                if (rounds.size() <= r) rounds.resize(r + 1);
                if (!per_round) continue;
                // the per-round form starts from a zeroed arena: only the
                // tiles that can hold a nonzero amplitude run
                const unsigned live = P.stages[r].live;
                for (unsigned k = 0; k < (1u << __builtin_popcount(live)); ++k)
                    rounds[r].push_back(make_int2(sidx, (int)host_deposit(k, live)));
            }
        }
    }
    std::vector<void *> owned;
    auto up = [&](const void *src, size_t bytes) -> void * {
        void *p = d.arena.alloc(std::max<size_t>(bytes, 16));
        owned.push_back(p);
        if (bytes) QG_CUDA(cudaMemcpyAsync(p, src, bytes, cudaMemcpyHostToDevice, d.stream));
        return p;
    };
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    try {
        auto *d_ops = (RegOp<float> *)up(ops_all, ops_bytes);
        auto *d_sets = (SetSlots *)up(sets_all, sets_bytes);
        ResidentCircuit *d_res[14];
        for (int n = 8; n <= 13; ++n)
            d_res[n] = (ResidentCircuit *)up(res[n].data(), res[n].size() * sizeof(ResidentCircuit));
        auto *d_stages = (BatchStage *)up(stages.data(), stages.size() * sizeof(BatchStage));
        std::vector<int2> items_all;
        std::vector<size_t> round_off;
        for (auto &rd : rounds) {
            round_off.push_back(items_all.size());
            items_all.insert(items_all.end(), rd.begin(), rd.end());
        }
        auto *d_items = (int2 *)up(items_all.data(), items_all.size() * sizeof(int2));
        auto *d_off = (long long *)up(big_off.data(), big_off.size() * sizeof(long long));
        auto *d_n = (int *)up(big_n.data(), big_n.size() * sizeof(int));
        auto *d_idx = (int *)up(big_idx.data(), big_idx.size() * sizeof(int));
        const int nbig = (int)big_off.size();
        double *d_part = (double *)d.arena.alloc(sizeof(double) * std::max<size_t>(batch_sumz_partials(nbig), 1));
        owned.push_back(d_part);
        double *d_out = (double *)d.arena.alloc(sizeof(double) * n_circuits);
        owned.push_back(d_out);
        float2 *arena = (float2 *)d.arena.alloc(std::max<long long>(arena_elems, 1) * sizeof(float2));
        owned.push_back(arena);
        // The one-launch form: a work queue of every resident circuit, every
        // (stage, tile) of the large circuits round by round, and the chunks
        // of their final sums, for one persistent launch.
        std::vector<BatchItem> items;
        std::vector<ResidentCircuit> res_all;
        std::vector<BigCircuit> bigs;
        int *d_counters = nullptr;
        unsigned *d_status = nullptr;
        BatchItem *d_bitems = nullptr;
        ResidentCircuit *d_res_all = nullptr;
        BigCircuit *d_big = nullptr;
        int ctas = 0;
        if (d.batch_one_launch) {
            for (int n = 8; n <= 13; ++n) res_all.insert(res_all.end(), res[n].begin(), res[n].end());
            std::vector<int> big_rounds(nbig, 0), big_tiles(nbig, 0);
            for (int b = 0; b < nbig; ++b) {
                BigCircuit bc;
                bc.off = big_off[b];
                bc.n = big_n[b];
                bc.out_index = big_idx[b];
                bigs.push_back(bc);
                big_tiles[b] = 1 << (big_n[b] - 12);
            }
            std::vector<int> stage_big(stages.size());
            {
                int b = -1;
                long long last_off = -1;
                for (size_t si = 0; si < stages.size(); ++si) {
                    if (stages[si].state_off != last_off) {
                        ++b;
                        last_off = stages[si].state_off;
                    }
                    stage_big[si] = b;
                    big_rounds[b] += 1;
                }
            }
            // Queue order: round by round over all large circuits (a round's
            // items wait only on the previous round of their own circuit,
            // which is a whole round of every circuit earlier in the queue,
            // so they rarely wait at all); the resident circuits are spread
            // over the round boundaries, and a circuit's final sums follow
            // the round after its last one.
            std::vector<std::vector<int>> big_stage_list(nbig);
            for (size_t si = 0; si < stages.size(); ++si)
                big_stage_list[stage_big[si]].push_back((int)si);
            // Tiles each stage runs: round 0 writes every tile (the arena is
            // not cleared; tiles other than tile 0 just store zeros), later
            // rounds only the tiles that can hold a nonzero amplitude.
            // done[] of a circuit counts run tiles; before round r it must
            // reach the sum over its earlier rounds.
            std::vector<std::vector<int>> big_need(nbig);
            for (int b = 0; b < nbig; ++b) {
                int acc = 0;
                for (size_t r = 0; r < big_stage_list[b].size(); ++r) {
                    big_need[b].push_back(acc);
                    acc += r == 0 ? big_tiles[b]
                                  : 1 << __builtin_popcount(stage_live[big_stage_list[b][r]]);
                }
                big_need[b].push_back(acc);
            }
            const size_t nrounds = rounds.size();
            const size_t res_per = nrounds ? (res_all.size() + nrounds - 1) / nrounds
                                           : res_all.size();
            size_t next_res = 0;
            auto push_residents = [&](size_t count) {
                for (size_t k = 0; k < count && next_res < res_all.size(); ++k, ++next_res) {
                    BatchItem it;
                    memset(&it, 0, sizeof(it));
                    it.kind = 0;
                    it.index = (int)next_res;
                    it.dep = -1;
                    items.push_back(it);
                }
            };
            auto push_sums = [&](int b) {
                for (int k = 0; k < (int)batch_sumz_partials(1); ++k) {
                    BatchItem it;
                    memset(&it, 0, sizeof(it));
                    it.kind = 2;
                    it.index = b;
                    it.tile = k;
                    it.dep = b;
                    it.need = big_need[b][big_rounds[b]];
                    items.push_back(it);
                }
            };
            for (size_t r = 0; r <= nrounds; ++r) {
                for (int b = 0; b < nbig; ++b) {
                    if ((int)r < big_rounds[b]) {
                        const int si = big_stage_list[b][r];
                        const unsigned live = r == 0 ? (unsigned)big_tiles[b] - 1u : stage_live[si];
                        const int count = 1 << __builtin_popcount(live);
                        const int per = std::min(count, kBatchTilesPerItem);
                        for (int t = 0; t < count; t += per) {
                            BatchItem it;
                            memset(&it, 0, sizeof(it));
                            it.kind = 1;
                            it.index = si;
                            it.tile = t;
                            it.ntiles = per;
                            it.live = live;
                            it.round = (int)r;
                            it.dep = r > 0 ? b : -1;
                            it.need = big_need[b][r];
                            it.dep_done = b;
                            items.push_back(it);
                        }
                    } else if (r == std::min((size_t)big_rounds[b] + 1, nrounds)) {
                        push_sums(b);
                    }
                }
                push_residents(res_per);
            }
            push_residents(res_all.size());
            d_bitems = (BatchItem *)up(items.data(), items.size() * sizeof(BatchItem));
            d_res_all = (ResidentCircuit *)up(res_all.data(), res_all.size() * sizeof(ResidentCircuit));
            d_big = (BigCircuit *)up(bigs.data(), bigs.size() * sizeof(BigCircuit));
            d_counters = (int *)d.arena.alloc(sizeof(int) * (1 + 2 * (size_t)nbig) + 16);
            owned.push_back(d_counters);
            d_status = (unsigned *)d.arena.alloc(16);
            owned.push_back(d_status);
            ctas = batch_persistent_ctas();
        }
        batch_prepare();
        QG_CUDA(cudaStreamSynchronize(d.stream));

        // Record the whole batch as one CUDA graph, then launch it.
        QG_CUDA(cudaStreamBeginCapture(d.stream, cudaStreamCaptureModeThreadLocal));
        try {
            if (d.batch_one_launch) {
                QG_CUDA(cudaMemsetAsync(d_counters, 0, sizeof(int) * (1 + 2 * (size_t)nbig),
                                        d.stream));
                QG_CUDA(cudaMemsetAsync(d_status, 0, sizeof(unsigned), d.stream));
                launch_batch_persistent(d_bitems, (int)items.size(), d_counters, nbig, d_status,
                                        d_res_all, d_stages, d_ops, d_sets, arena, d_big, d_part,
                                        d_out, ctas, d.stream);
            } else {
            if (arena_elems)
                QG_CUDA(cudaMemsetAsync(arena, 0, arena_elems * sizeof(float2), d.stream));
            launch_batch_init(arena, d_off, nbig, d.stream);
            for (int n = 8; n <= 13; ++n)
                launch_batch_resident(n, n <= 9 ? 3 : (n <= 12 ? 4 : 5), d_res[n],
                                      (int)res[n].size(), d_ops, d_sets, d_out, d.stream);
            for (size_t r = 0; r < rounds.size(); ++r)
                launch_batch_stage(d_stages, d_items + round_off[r], (int)rounds[r].size(), d_ops,
                                   d_sets, arena, d.stream);
            launch_batch_sumz(arena, d_off, d_n, d_idx, nbig, d_part, d_out, d.stream);
            }
        } catch (...) {
            cudaStreamEndCapture(d.stream, &graph);
            throw;
        }
        QG_CUDA(cudaStreamEndCapture(d.stream, &graph));
        QG_CUDA(cudaGraphInstantiate(&exec, graph, 0));
        timed(d, "batch", [&] { QG_CUDA(cudaGraphLaunch(exec, d.stream)); });
        // stage passes of the large circuits (each a read and a write of the
        // state, through L2 where it fits) for the caller's statistics
        for (size_t si = 0; si < stages.size(); ++si) {
            const long long tile_bytes = (long long)sizeof(float2) << 12;
            const long long run = 1LL << __builtin_popcount(stage_live[si]);
            d.n_passes += 1;
            d.n_bytes += 2 * run * tile_bytes;
            // round 0 of the one-launch form also stores the zero tiles
            if (d.batch_one_launch && stage_live[si] == 0)
                d.n_bytes += (((long long)1 << (stages[si].n - 12)) - 1) * tile_bytes;
        }
        QG_CUDA(cudaMemcpyAsync(out, d_out, sizeof(double) * n_circuits, cudaMemcpyDeviceToHost,
                                d.stream));
        unsigned status = 0;
        if (d_status)
            QG_CUDA(cudaMemcpyAsync(&status, d_status, sizeof(status), cudaMemcpyDeviceToHost,
                                    d.stream));
        QG_CUDA(cudaStreamSynchronize(d.stream));
        if (status) fail(QG_ERR_TIMEOUT, "batch: a bounded wait of the persistent launch gave up.");
    } catch (...) {
        cudaStreamSynchronize(d.stream);
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
        for (void *p : owned) d.arena.release(p);
        throw;
    }
    cudaGraphExecDestroy(exec);
    cudaGraphDestroy(graph);
    for (void *p : owned) d.arena.release(p);
    QG_END
}

int qg_gate_matrix(const char *name, const double *args, int n_args, int adjoint, double *mat) {
    QG_BEGIN
    if (!name) fail(QG_ERR_VALUE, "null gate name.");
    gate_matrix(name, args, n_args, mat);
    if (adjoint) adjoint2(mat);
    QG_END
}

int qg_qubits_states_getter_new(int prec, qg_handle *out) {
    QG_BEGIN
    check_prec(prec);
    Getter *g = new Getter{prec};
    g_dev.getters.insert(g);
    *out = (qg_handle)g;
    QG_END
}

int qg_qubits_states_getter_delete(qg_handle h) {
    QG_BEGIN
    Getter *g = lookup(g_dev.getters, h, "getter");
    g_dev.getters.erase(g);
    delete g;
    QG_END
}

int qg_qubits_states_getter_get_states(qg_handle hg, void *values, int64_t array_offset,
                                       int mathop, const int *lane_tables,
                                       const int *lane_counts, const qg_handle *qstates_list,
                                       int n_qstates, uint64_t empty_lane_mask, int n_qregs,
                                       int64_t n_states, int64_t start, int64_t step) {
    QG_BEGIN
    Getter *g = lookup(g_dev.getters, hg, "getter");
    if (mathop != QG_MATHOP_NULL && mathop != QG_MATHOP_PROB) fail(QG_ERR_RUNTIME, "Unknown math op.");
    if (n_qregs < 0 || n_qregs > kMaxLanes) fail(QG_ERR_VALUE, "value out of range");
    long long size = 1LL << n_qregs;
    if (n_states <= 0) {
        t_last_error.clear();
        return QG_OK;
    }
    if (start < 0 || size <= start) fail(QG_ERR_VALUE, "value out of range");
    long long end = start + step * (n_states - 1);
    if (end < 0 || size <= end) fail(QG_ERR_VALUE, "value out of range");
    size_t rs = g->prec == kFP64 ? 8 : 4;
    size_t item = mathop == QG_MATHOP_NULL ? 2 * rs : rs;
    char *dst = (char *)values + array_offset * item;
    if (n_qstates == 0) {
        // no states: |0...0> of the empty lanes (qgate/simulator/src/glue.cpp:480-495)
        memset(dst, 0, n_states * item);
        if (start == 0) {
            if (rs == 4)
                *(float *)dst = 1.f;
            else
                *(double *)dst = 1.;
        }
        t_last_error.clear();
        return QG_OK;
    }
    GatherDesc gd = make_gather(lane_tables, lane_counts, qstates_list, n_qstates, g->prec);
    Device &d = dev();
    staged_d2h(d, dst, n_states, item, [&](idx_t begin, idx_t cnt, void *dbuf) {
        timed(d, "gather", [&] {
            launch_gather(g->prec, mathop, dbuf, cnt, start + step * begin, step, empty_lane_mask,
                          gd, d.stream);
        });
    });
    QG_END
}

static double *marginal_to_device(Device &d, Getter *g, const int *lane_tables,
                                  const int *lane_counts, const qg_handle *qstates_list,
                                  int n_qstates, int n_lanes, int n_hidden) {
    if (n_lanes < 0 || n_hidden < 0 || n_lanes + n_hidden > kMaxLanes)
        fail(QG_ERR_VALUE, "lane counts out of range.");
    GatherDesc gd = make_gather(lane_tables, lane_counts, qstates_list, n_qstates, g->prec);
    int total = gd.lane_begin[n_qstates];
    if (total != n_lanes + n_hidden) fail(QG_ERR_VALUE, "lane tables do not cover all lanes.");
    idx_t n_out = (idx_t)1 << n_lanes;
    double *prob = (double *)d.arena.alloc(n_out * sizeof(double));
    size_t sc = marginal_scratch_doubles(n_lanes, n_hidden);
    double *scratch = sc ? (double *)d.arena.alloc(sc * sizeof(double)) : nullptr;
    timed(d, "marginal",
          [&] { launch_marginal(g->prec, prob, n_lanes, n_hidden, gd, scratch, sc, d.stream); });
    if (scratch) d.arena.release(scratch);  // stream-ordered reuse is safe
    return prob;
}

int qg_qubits_states_getter_prepare_prob_array(qg_handle hg, void *prob, const int *lane_tables,
                                               const int *lane_counts,
                                               const qg_handle *qstates_list, int n_qstates,
                                               int n_lanes, int n_hidden_lanes) {
    QG_BEGIN
    Getter *g = lookup(g_dev.getters, hg, "getter");
    Device &d = dev();
    double *dprob = marginal_to_device(d, g, lane_tables, lane_counts, qstates_list, n_qstates,
                                       n_lanes, n_hidden_lanes);
    idx_t n_out = (idx_t)1 << n_lanes;
    size_t rs = g->prec == kFP64 ? 8 : 4;
    try {
        staged_d2h(d, prob, n_out, rs, [&](idx_t begin, idx_t cnt, void *dbuf) {
            launch_convert_f64(g->prec, dbuf, dprob + begin, cnt, d.stream);
        });
    } catch (...) {
        d.arena.release(dprob);
        throw;
    }
    d.arena.release(dprob);
    QG_END
}

int qg_qubits_states_getter_create_sampling_pool(qg_handle hg, const int *lane_tables,
                                                 const int *lane_counts,
                                                 const qg_handle *qstates_list, int n_qstates,
                                                 int n_lanes, int n_hidden_lanes,
                                                 const int *empty_lanes, int n_empty,
                                                 qg_handle *out) {
    QG_BEGIN
    Getter *g = lookup(g_dev.getters, hg, "getter");
    Device &d = dev();
    if (n_empty < 0 || n_lanes + n_empty > kMaxLanes) fail(QG_ERR_VALUE, "too many empty lanes.");
    if (n_lanes < 0 || n_hidden_lanes < 0 || n_lanes + n_hidden_lanes > kMaxLanes)
        fail(QG_ERR_VALUE, "lane counts out of range.");
    idx_t n = (idx_t)1 << n_lanes;
    // One state in its own lane order with nothing summed out: the CDF is
    // scanned straight from its amplitudes; otherwise from the FP64 marginal.
    bool direct = n_qstates == 1 && n_hidden_lanes == 0 && lane_counts[0] == n_lanes;
    for (int l = 0; direct && l < n_lanes; ++l) direct = lane_tables[l] == l;
    unsigned long long *cdf = nullptr, *scratch = nullptr;
    const void *src = nullptr;
    if (direct) {
        GatherDesc gd = make_gather(lane_tables, lane_counts, qstates_list, n_qstates, g->prec);
        src = gd.ptr[0];
        cdf = (unsigned long long *)d.arena.alloc(n * sizeof(unsigned long long));
    } else {
        cdf = (unsigned long long *)marginal_to_device(d, g, lane_tables, lane_counts,
                                                       qstates_list, n_qstates, n_lanes,
                                                       n_hidden_lanes);
    }
    unsigned long long total = 0;
    // Guide table: buckets of 2^(64 - n_lanes) CDF units, about 16 items each
    // for a normalised state (64 above 2^32 items, whose entries then hold
    // the item index shifted right to fit 32 bits); entries cover totals up
    // to (1 + 1/16) * 2^60, beyond the norm check's 1.05.
    PoolGuide guide{};
    void *guide_aux = nullptr;
    const unsigned kLongCap = 1u << 16;
    try {
        if (n_lanes >= 12 && n_lanes <= 34) {
            // 32-bit entries need index >> (lanes - 32) at least
            const int ks = std::max(d.guide_index_shift, std::max(0, n_lanes - 32));
            guide.shift = ks == 0 ? 64 - n_lanes : 66 - n_lanes;
            guide.index_shift = ks;
            guide.nb = (((1ull << 60) + (1ull << 56)) >> guide.shift) + 2;
            guide.g = (unsigned *)d.arena.alloc(guide.nb * sizeof(unsigned));
            guide_aux = d.arena.alloc(16 + (size_t)kLongCap * sizeof(uint4));
            guide.long_count = (unsigned *)guide_aux;
            guide.long_list = (uint4 *)((char *)guide_aux + 16);
            guide.long_cap = kLongCap;
            QG_CUDA(cudaMemsetAsync(guide.long_count, 0, sizeof(unsigned), d.stream));
        }
        scratch = (unsigned long long *)d.arena.alloc(pool_scratch_words(n) * 8);
        const unsigned long long *d_total = nullptr;
        timed(d, "scan", [&] {
            d_total = direct ? launch_pool_cdf_state(g->prec, src, n, cdf, scratch, guide,
                                                     d.stream)
                             : launch_pool_cdf_prob((const double *)cdf, n, cdf, scratch, guide,
                                                    d.stream);
        });
        QG_CUDA(cudaMemcpyAsync(d.h_result, d_total, 8, cudaMemcpyDeviceToHost, d.stream));
        if (guide.g)
            QG_CUDA(cudaMemcpyAsync(d.h_result + 1, guide.long_count, sizeof(unsigned),
                                    cudaMemcpyDeviceToHost, d.stream));
        QG_CUDA(cudaStreamSynchronize(d.stream));
        memcpy(&total, d.h_result, 8);
        if (guide.g) {
            unsigned long_count = 0;
            memcpy(&long_count, d.h_result + 1, sizeof(unsigned));
            d.arena.release(guide_aux);
            guide_aux = nullptr;
            if (long_count > kLongCap) {  // too many long runs: search without the table
                d.arena.release(guide.g);
                guide.g = nullptr;
            }
        }
        if (pool_status(true))
            fail(QG_ERR_RUNTIME, "sampling-pool scan: a bounded wait for a bulk copy gave up.");
        // qgate/simulator/src/CPUSamplingPool.cpp:31-32
        double sum = std::ldexp((double)total, -60);
        if (!(std::fabs(sum - 1.) <= 0.05))
            fail(QG_ERR_RUNTIME, "error in probability sum is beyond 0.05., %g.", sum);
    } catch (...) {
        if (scratch) d.arena.release(scratch);
        if (guide_aux) d.arena.release(guide_aux);
        if (guide.g) d.arena.release(guide.g);
        d.arena.release(cdf);
        throw;
    }
    d.arena.release(scratch);
    Pool *p = new Pool();
    p->cdf = cdf;
    p->total = total;
    p->guide = guide.g;
    p->guide_shift = guide.shift;
    p->guide_index_shift = guide.index_shift;
    p->n = n;
    for (int i = 0; i < n_empty; ++i) p->empty_pos.push_back(empty_lanes[i]);
    std::sort(p->empty_pos.begin(), p->empty_pos.end());
    g_dev.pools.insert(p);
    *out = (qg_handle)p;
    QG_END
}

int qg_sampling_pool_sample(qg_handle hp, int64_t *obs, int64_t n_samples,
                            const double *randnum) {
    QG_BEGIN
    Pool *p = lookup(g_dev.pools, hp, "sampling pool");
    if (n_samples < 0) fail(QG_ERR_VALUE, "negative sample count.");
    if (n_samples == 0) {
        t_last_error.clear();
        return QG_OK;
    }
    Device &d = dev();
    const size_t bytes = (size_t)n_samples * 8;
    if (d.pageable_copy && bytes >= ((size_t)64 << 20) && bytes <= ((size_t)8 << 30)) {
        // One copy each way between the caller's pageable arrays and device
        // buffers (Grace + NVLink-C2C); the index array's pages are touched
        // by all host threads while the uniforms go up and the search runs.
        double *du = (double *)d.arena.alloc(bytes);
        long long *dobs = (long long *)d.arena.alloc(bytes);
        try {
            QG_CUDA(cudaMemcpyAsync(du, randnum, bytes, cudaMemcpyHostToDevice, d.stream));
            timed(d, "search", [&] {
                launch_search(p->cdf, p->n, p->total, p->guide, p->guide_shift,
                              p->guide_index_shift, du, dobs,
                              n_samples, p->empty_pos.data(),
                              (int)p->empty_pos.size(), d.stream);
            });
            char *h = (char *)obs;
            const size_t kPage = host_page_bytes();
#pragma omp parallel for schedule(static)
            for (long long i = 0; i < (long long)((bytes + kPage - 1) / kPage); ++i)
                ((volatile char *)h)[(size_t)i * kPage] = 0;
            QG_CUDA(cudaMemcpyAsync(obs, dobs, bytes, cudaMemcpyDeviceToHost, d.stream));
            QG_CUDA(cudaStreamSynchronize(d.stream));
        } catch (...) {
            cudaStreamSynchronize(d.stream);
            d.arena.release(du);
            d.arena.release(dobs);
            throw;
        }
        d.arena.release(du);
        d.arena.release(dobs);
        t_last_error.clear();
        return QG_OK;
    }
    // Uniforms go up through staging buffer 0, indices come back through 1.
    idx_t chunk = (idx_t)(Device::kStageBytes / 8);
    double *du = (double *)d.arena.alloc(chunk * 8);
    long long *dobs = (long long *)d.arena.alloc(chunk * 8);
    try {
        for (idx_t b = 0; b < n_samples; b += chunk) {
            idx_t cnt = std::min(chunk, (idx_t)n_samples - b);
            host_copy(d.h_stage[0], randnum + b, cnt * 8);
            QG_CUDA(cudaMemcpyAsync(du, d.h_stage[0], cnt * 8, cudaMemcpyHostToDevice, d.stream));
            timed(d, "search", [&] {
                launch_search(p->cdf, p->n, p->total, p->guide, p->guide_shift,
                              p->guide_index_shift, du, dobs, cnt,
                              p->empty_pos.data(),
                              (int)p->empty_pos.size(), d.stream);
            });
            QG_CUDA(cudaMemcpyAsync(d.h_stage[1], dobs, cnt * 8, cudaMemcpyDeviceToHost, d.stream));
            QG_CUDA(cudaStreamSynchronize(d.stream));
            host_copy(obs + b, d.h_stage[1], cnt * 8);
        }
    } catch (...) {
        d.arena.release(du);
        d.arena.release(dobs);
        throw;
    }
    d.arena.release(du);
    d.arena.release(dobs);
    QG_END
}

int qg_sampling_pool_delete(qg_handle hp) {
    QG_BEGIN
    Pool *p = lookup(g_dev.pools, hp, "sampling pool");
    g_dev.arena.release(p->cdf);
    if (p->guide) g_dev.arena.release(p->guide);
    g_dev.pools.erase(p);
    delete p;
    QG_END
}

}  // extern "C"
