// Allocation-free probability entry point.
//
// qg_calc_probability_noalloc() computes Pr(lane == 0) like
// qg_qubit_processor_calc_probability(), but for callers that cannot let the
// library allocate: code that manages every byte of device memory in its own
// pre-sized pool (so a cudaMalloc would fail or steal from that pool), or
// latency-sensitive loops that must not hit the implicit device-wide
// synchronisation a cudaMalloc / cudaFree can cause.  The caller owns the
// state and the output; the per-block partial sums live in a fixed
// file-scope device array instead of engine-owned scratch, and the engine's
// device context (which allocates a stream, pinned buffers and scratch on
// first use) is never touched.
#include <mutex>

#include "qg_device.cuh"
#include "../../include/qgate_gb300.h"

namespace qg {

namespace {

// Per-block FP64 partials of the probability reduction.  The reduction
// launches at most reduce_partials() (1216) blocks whatever the state size, so
// 2048 doubles (16 KiB per GPU, held from module load until process exit)
// always suffice; the entry point still checks the bound.
constexpr int kNoAllocPartials = 2048;
static __device__ __align__(256) double g_noalloc_partials[kNoAllocPartials];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mu;
double *g_partials_addr[kMaxDevices] = {nullptr};

// Host code cannot use g_noalloc_partials directly (on the host it names a
// shadow, not device memory): the device address is looked up once per
// device, with that device current.
int partials_for_current_device(double **out) {
    int dev = -1;
    cudaError_t err = cudaGetDevice(&dev);
    if (err != cudaSuccess) {
        set_last_error(std::string("cudaGetDevice failed: ") + cudaGetErrorString(err));
        return QG_ERR_CUDA;
    }
    if (dev < 0 || dev >= kMaxDevices) {
        set_last_error("device ordinal out of range");
        return QG_ERR_CUDA;
    }
    std::lock_guard<std::mutex> lk(g_setup_mu);
    if (!g_partials_addr[dev]) {
        void *p = nullptr;
        err = cudaGetSymbolAddress(&p, g_noalloc_partials);
        if (err != cudaSuccess || !p) {
            set_last_error(std::string("cudaGetSymbolAddress failed: ") +
                           cudaGetErrorString(err));
            return QG_ERR_CUDA;
        }
        g_partials_addr[dev] = (double *)p;
    }
    *out = g_partials_addr[dev];
    return QG_OK;
}

}  // namespace

}  // namespace qg

using namespace qg;

extern "C" int qg_calc_probability_noalloc(int prec, const void *d_state, int n_lanes,
                                           int local_lane, double *d_prob, uint64_t stream) {
    if (prec != kFP64 && prec != kFP32) {
        set_last_error("prec must be QG_PREC_FP64 or QG_PREC_FP32");
        return QG_ERR_VALUE;
    }
    if (!d_state || !d_prob) {
        set_last_error("null state or output pointer");
        return QG_ERR_VALUE;
    }
    // The reduction reads the state as 16-byte vectors (two complex64 or one
    // complex128 amplitude) and writes one double: a misaligned pointer would
    // fault inside the kernel, so it is refused here, before any launch.
    if (((uintptr_t)d_state & 15u) != 0u) {
        set_last_error("d_state must be 16-byte aligned");
        return QG_ERR_VALUE;
    }
    if (((uintptr_t)d_prob & 7u) != 0u) {
        set_last_error("d_prob must be 8-byte aligned");
        return QG_ERR_VALUE;
    }
    if (n_lanes < 1 || n_lanes > 40) {
        set_last_error("n_lanes must be in [1, 40]");
        return QG_ERR_VALUE;
    }
    if (local_lane < 0 || local_lane >= n_lanes) {
        set_last_error("local_lane out of range");
        return QG_ERR_VALUE;
    }
    if (reduce_partials() > kNoAllocPartials) {
        set_last_error("reduction needs more partials than the fixed scratch array holds");
        return QG_ERR_VALUE;
    }
    double *partials = nullptr;
    int rc = partials_for_current_device(&partials);
    if (rc != QG_OK) return rc;
    PairIdx pi;
    pi.npos = 1;
    pi.pos[0] = local_lane;
    pi.set_mask = 0;
    pi.partner = 0;
    try {
        // Every partial the final sum reads is written by this launch, so the
        // array needs no clearing between calls.
        launch_prob(prec, d_state, (idx_t)1 << (n_lanes - 1), pi, partials, d_prob,
                    (cudaStream_t)(uintptr_t)stream);
    } catch (const Error &e) {
        set_last_error(e.msg);
        return e.code;
    }
    set_last_error("");
    return QG_OK;
}
