/*
 * qgate_gb300 — C ABI of the GB300 (sm_103a) state-vector engine.
 *
 * Every entry point returns an int status (QG_OK on success) and never throws
 * or aborts across the boundary; the message of the last failure on the
 * calling thread is returned by qg_last_error().  Handles are opaque 64-bit
 * values owned by the caller and released with the matching *_delete call.
 *
 * The set of entry points mirrors the reference's CPython glue for its native
 * runtimes (qgate/simulator/src/glue.cpp:605-631 and
 * qgate/simulator/src/cudaext.cpp:127-136), with Python objects replaced by
 * plain pointers and sizes.  Each declaration names the reference entry point
 * it replaces.  Entries marked "extension" have no counterpart in the
 * reference and implement capabilities the reference lacks.
 *
 * Precision codes follow the reference's `enum Precision`
 * (qgate/simulator/src/Types.h:49-53): QG_PREC_FP64 = complex128 states,
 * QG_PREC_FP32 = complex64 states.  Math ops follow `enum MathOp`
 * (qgate/simulator/src/Types.h:55-58).
 *
 * Gate matrices are 2x2 complex128, row-major, passed as 8 doubles
 * {re00, im00, re01, im01, re10, im10, re11, im11} — the layout of the
 * reference's Matrix2x2C64 (qgate/simulator/src/Types.h:22-46).
 */
#ifndef QGATE_GB300_H
#define QGATE_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef uint64_t qg_handle;

enum {
    QG_OK = 0,
    QG_ERR_VALUE = 1,    /* invalid argument (reference raises ValueError) */
    QG_ERR_RUNTIME = 2,  /* invalid state / semantic error (RuntimeError) */
    QG_ERR_CUDA = 3,     /* CUDA runtime failure */
    QG_ERR_NOMEM = 4,    /* "Out of device memory." */
    QG_ERR_TIMEOUT = 5   /* a bounded device-side wait gave up */
};

enum { QG_PREC_FP64 = 1, QG_PREC_FP32 = 2 };
enum { QG_MATHOP_NULL = 0, QG_MATHOP_PROB = 1 };

/* Message of the last failure on this thread ("" if none). */
const char *qg_last_error(void);

/* ---- device / module --------------------------------------------------- */

/* Replaces cudaext.devices_initialize (qgate/simulator/src/cudaext.cpp:32-58).
 * One GPU only: device_id selects it (-1 = current device).  memory_limit
 * caps the arena in bytes (-1 = no cap beyond device memory). */
int qg_devices_initialize(int device_id, int64_t memory_limit);

/* Replaces cudaext.devices_clear / module_finalize
 * (qgate/simulator/src/cudaext.cpp:23-29, 60-67).  Frees the arena cache. */
int qg_devices_clear(void);

/* Bytes currently handed out by / cached in the device arena (diagnostics;
 * the reference reports leaks at finalize,
 * qgate/simulator/src/MultiDeviceMemoryStore.cpp:33-43). */
int qg_arena_stats(int64_t *in_use, int64_t *cached);

/* ---- qubit states (qgate/simulator/src/Interfaces.h:7-20) -------------- */

/* Replaces cudaext.qubit_states_new (qgate/simulator/src/cudaext.cpp:70-87). */
int qg_qubit_states_new(int prec, qg_handle *out);
/* Replaces glue.qubit_states_delete (qgate/simulator/src/glue.cpp:193-205). */
int qg_qubit_states_delete(qg_handle qstates);
/* Replaces glue.qubit_states_deallocate (qgate/simulator/src/glue.cpp:180-190). */
int qg_qubit_states_deallocate(qg_handle qstates);
/* Replaces glue.qubit_states_get_n_lanes (qgate/simulator/src/glue.cpp:237-246). */
int qg_qubit_states_get_n_lanes(qg_handle qstates, int *n_lanes);

/* ---- qubit processor (qgate/simulator/src/Interfaces.h:22-52) ---------- */

/* Replaces cudaext.qubit_processor_new (qgate/simulator/src/cudaext.cpp:90-106). */
int qg_qubit_processor_new(int prec, qg_handle *out);
/* Replaces glue.qubit_processor_delete (qgate/simulator/src/glue.cpp:208-219). */
int qg_qubit_processor_delete(qg_handle proc);
/* Replaces glue.qubit_processor_synchronize (qgate/simulator/src/glue.cpp:251-260). */
int qg_qubit_processor_synchronize(qg_handle proc);
/* Replaces glue.qubit_processor_reset (qgate/simulator/src/glue.cpp:263-272). */
int qg_qubit_processor_reset(qg_handle proc);
/* Replaces glue.qubit_processor_initialize_qubit_states (qgate/simulator/src/glue.cpp:275-286). */
int qg_qubit_processor_initialize_qubit_states(qg_handle proc, qg_handle qstates, int n_lanes);
/* Replaces glue.qubit_processor_reset_qubit_states (qgate/simulator/src/glue.cpp:289-299). */
int qg_qubit_processor_reset_qubit_states(qg_handle proc, qg_handle qstates);
/* Replaces glue.qubit_processor_calc_probability (qgate/simulator/src/glue.cpp:302-311).
 * Pr(lane == 0), accumulated in FP64 for both precisions. */
int qg_qubit_processor_calc_probability(qg_handle proc, qg_handle qstates, int local_lane,
                                        double *prob);
/* Replaces glue.qubit_processor_join (qgate/simulator/src/glue.cpp:314-334).  Kronecker product
 * of the listed states (the last one in the lowest lanes), followed by
 * n_new_lanes |0> lanes in the highest positions. */
int qg_qubit_processor_join(qg_handle proc, qg_handle qstates, const qg_handle *qstates_list,
                            int n_list, int n_new_lanes);
/* Replaces glue.qubit_processor_decohere (qgate/simulator/src/glue.cpp:337-348). */
int qg_qubit_processor_decohere(qg_handle proc, int value, double prob, qg_handle qstates,
                                int local_lane);
/* Replaces glue.qubit_processor_decohere_and_separate (qgate/simulator/src/glue.cpp:351-365). */
int qg_qubit_processor_decohere_and_separate(qg_handle proc, int value, double prob,
                                             qg_handle qstates0, qg_handle qstates1,
                                             qg_handle qstates, int local_lane);
/* Replaces glue.qubit_processor_apply_reset (qgate/simulator/src/glue.cpp:368-379). */
int qg_qubit_processor_apply_reset(qg_handle proc, qg_handle qstates, int local_lane);
/* Replaces glue.qubit_processor_apply_gate (qgate/simulator/src/glue.cpp:383-405); the matrix is
 * built by the caller (qg_gate_matrix) instead of a Python factory object. */
int qg_qubit_processor_apply_gate(qg_handle proc, const double *mat, qg_handle qstates,
                                  int local_lane);
/* Replaces glue.qubit_processor_apply_controlled_gate (qgate/simulator/src/glue.cpp:409-432). */
int qg_qubit_processor_apply_controlled_gate(qg_handle proc, const double *mat,
                                             qg_handle qstates, const int *local_control_lanes,
                                             int n_controls, int local_target_lane);

/* Extension: compiled circuits.  The reference front-end hands a circuit to
 * the runtime one gate per call (qgate/simulator/rop_executor.py:28-34 via
 * qgate/simulator/model_executor.py:151-166); a compiled circuit takes the
 * whole gate list once and applies it in one call.
 *   qg_circuit_new: n_gates gates; gate i has target lane targets[i], control
 *   lanes ctrl_lanes[ctrl_offsets[i] .. ctrl_offsets[i+1]) (ctrl_offsets has
 *   n_gates + 1 entries) and the 2x2 complex128 matrix matrices[8i .. 8i+8)
 *   (row-major, interleaved re/im; adjoints already applied).  Lanes are
 *   checked as apply_controlled_gate checks them (range, no overlap).
 *   qg_circuit_run: applies the gates to qstates (same precision, at least as
 *   many lanes as the circuit uses) exactly as the same sequence of
 *   apply_gate / apply_controlled_gate calls would.
 *   qg_circuit_set_graph: 1 = graph replay: the first run on a states buffer
 *   plans the stages and captures their launches into a CUDA graph, later
 *   runs on the same buffer (same lane count, unchanged fusion settings)
 *   replay it without host planning; a different buffer, lane count or any
 *   qg_set_fusion* / tensor / pipelining change re-captures.  The circuit
 *   owns the graph and the tensor stages' operands (a few MB).
 *   qg_circuit_stats: whether a graph is captured and its HBM passes. */
int qg_circuit_new(int prec, int n_gates, const int *targets, const int *ctrl_offsets,
                   const int *ctrl_lanes, const double *matrices, qg_handle *out);
int qg_circuit_set_graph(qg_handle circuit, int on);
int qg_circuit_run(qg_handle circuit, qg_handle qstates);
int qg_circuit_stats(qg_handle circuit, int *captured, int64_t *passes);
int qg_circuit_delete(qg_handle circuit);

/* Extension: trace replay for the per-gate path.  The reference front-end
 * applies a circuit one apply_gate / apply_controlled_gate call at a time
 * (qgate/simulator/rop_executor.py:28-34) and every run is planned anew.  With
 * trace replay on (default), a run of queued gates flushed at an observation
 * is remembered (the last 8 distinct runs of >= 8 gates); when the same run
 * (same gates, lanes, matrices, precision and lane count) is flushed again,
 * the second time its stages are captured into a CUDA graph and from then on
 * the graph is replayed with no host planning, giving the same state as
 * planning would.  Runs partly launched while still being enqueued (>= 640
 * pending gates) are planned as usual.  qg_set_trace_replay(0) turns it off
 * and frees the remembered runs; qg_trace_stats reports graph replays and
 * captures (reset: clear the counters). */
int qg_set_trace_replay(int on);
int qg_trace_stats(int64_t *hits, int64_t *captures, int reset);

/* Extension: dense 2^k x 2^k complex128 matrix (row-major, interleaved re/im)
 * on k target lanes (targets[0] = least significant matrix bit), optionally
 * controlled.  k <= 6.  Replaces the reference's expansions of multi-qubit
 * gates into CX chains (qgate/model/expand.py:14-16). */
int qg_qubit_processor_apply_multi(qg_handle proc, const double *mat, qg_handle qstates,
                                   const int *targets, int n_targets,
                                   const int *local_control_lanes, int n_controls);

/* Extension: <psi|P|psi> for one Pauli string, FP64 accumulation.
 * x_mask = lanes carrying X or Y, z_mask = lanes carrying Z or Y.  Replaces
 * the reference's diagonalise -> Prob -> undo chain
 * (qgate/model/pauli_gates_diagonalizer.py:96-135, qgate/model/expand.py:66-77):
 * Pr(+1) of that chain equals (1 + <P>) / 2. */
int qg_qubit_processor_calc_pauli_expectation(qg_handle proc, qg_handle qstates,
                                              uint64_t x_mask, uint64_t z_mask, double *out);

/* Extension: sum |psi|^2 in FP64. */
int qg_qubit_processor_calc_norm(qg_handle proc, qg_handle qstates, double *out);

/* Extension: gate fusion control.  max_tile_lanes = lanes staged per tile in
 * shared memory by the fused stage kernel (0 = the defaults: 12-lane tiles,
 * 4 register lanes, no cost budget, tensor-core blocks on, pipelining off;
 * 1 = off: every gate is its own pass).  Pending gates are flushed at every
 * observation, join, measure or synchronize. */
int qg_set_fusion(int max_tile_lanes);
/* Extension: fusion parameters for one precision: lanes per shared-memory
 * tile (1..14; complex128 at most 13), lanes held in each thread's registers
 * by the register-resident stage kernel (3..5; complex128 at most 4), and a
 * per-amplitude instruction budget that closes a stage early (0 = none). */
int qg_set_fusion_params(int prec, int tile_lanes, int reg_lanes, int cost_budget);
/* Extension: 1 runs large fused stages with the persistent, double-buffered
 * stage kernel (and 12-lane tensor-core stages with two threads per tile
 * row); 0 (default) with one CTA per tile (tensor-core stages: one thread
 * per row), which keeps more warps resident per SM for the CUDA-core stage
 * and fewer, busier threads for the tensor-core stage. */
int qg_set_stage_pipelining(int on);
/* Extension: 1 (default) runs complex64 stages of 12- or 13-lane tiles as
 * fused 5-lane blocks (32x32 complex matrices) on the tensor cores, 0 on the
 * register-resident CUDA-core stage kernel.  No reference counterpart: the
 * reference applies one gate per pass
 * (qgate/simulator/src/CUDAQubitProcessor.cpp:271, applyGate). */
int qg_set_tensor_blocks(int on);
/* Extension: 1 lets the getter kernels (gathered states, probability arrays)
 * write straight into the caller's host buffers, allowed only when the
 * device accesses pageable host memory through the host page tables (Grace +
 * NVLink-C2C); faster into buffers the caller reuses, much slower into fresh
 * ones (first touch by GPU page faults).  0 (default) stages every transfer
 * through pinned buffers.  The reference copies through its own pinned buffers
 * (qgate/simulator/src/DeviceGetStates.cu:115-119,
 * qgate/simulator/src/CUDADevice.cpp:37). */
int qg_set_host_direct(int on);
/* Extension: 1 (default where the device accesses pageable host memory)
 * returns large results (64 MiB .. 16 GiB) through one device buffer and one
 * copy into the caller's buffer, after touching its pages with all host
 * threads; 0 stages them through pinned buffers in 64 MiB pieces. */
int qg_set_pageable_copy(int on);
/* Extension: layout of the sampling pools' guide tables created from now on.
 * -1 (default): entries hold the exact item index and buckets span ~16 items
 * up to 2^32 items; above that (33-34 lanes) entries hold index >> (lanes -
 * 32) and buckets span ~64 items.  k in [0, 8] forces entries of index >> k
 * (buckets of ~64 items when k > 0) at any size, which exercises the large-
 * pool layout on small states.  Samples are identical either way. */
int qg_set_pool_guide_index_shift(int k);
/* Extension: status word of the tensor-core stage kernels after a
 * synchronize: 0 = every bounded wait completed; nonzero = a wait gave up
 * (that stage's tiles were left unchanged).  reset != 0 clears it. */
int qg_tensor_stage_status(int reset, int *status);
/* Extension: counters of the gate path since the last reset
 * {gates, passes, bytes_moved}. */
int qg_gate_stats(int64_t *gates, int64_t *passes, int64_t *bytes, int reset);

/* Extension: per-kernel-class launch timing with CUDA events recorded on the
 * engine's stream around each launch (classes: stage, gate, multi, init,
 * prob, pauli, measure, join, gather, marginal, scan, search, batch). */
int qg_timing_enable(int on);
int qg_timing_read(const char *kernel_class, int64_t *launches, double *total_ms, int reset);
/* Extension: device facts {SMs, max opt-in shared memory per block, L2 bytes,
 * pageable memory access, ... uses host page tables, concurrent managed
 * access, CC major, CC minor, SM clock kHz, memory clock kHz, free bytes,
 * total bytes} (first n entries). */
int qg_device_info(int64_t *info, int n);
/* Extension: the engine's CUDA stream (cudaStream_t) for interop. */
int qg_get_stream(uint64_t *stream);

/* Extension: copy raw amplitudes between a states object and host memory
 * (2^n_lanes complex values in the state's precision). */
int qg_qubit_states_get_raw(qg_handle qstates, void *host, int64_t n);
int qg_qubit_states_set_raw(qg_handle qstates, const void *host, int64_t n);

/* ---- adjoint differentiation (extension) -------------------------------- */

/* One gate of a parametrised circuit.  kind 0: fixed 2x2 gate `mat`;
 * kind 1: rotation exp(-i coef theta G) with G = X/Y/Z (axis 1/2/3) on
 * `target` and theta = params[param] (Rx/Ry/Rz: coef 1/2; ExpiZ: coef -1).
 * Up to 4 controls. */
typedef struct {
    int kind;
    int target;
    int n_controls;
    int controls[4];
    int axis;
    int param;
    double coef;
    double mat[8];
} qg_circuit_op;

/* One term coef * P of a Pauli-sum observable: X or Y on x_mask lanes, Z or Y
 * on z_mask lanes (Y where both are set). */
typedef struct {
    double coef;
    uint64_t x_mask;
    uint64_t z_mask;
} qg_pauli_term;

/* Extension (the reference has no differentiation path).  For each of
 * `batch` parameter vectors (params: batch x n_params, row-major) runs the
 * circuit from |0...0> and returns E_b = <psi|H|psi> (FP64 accumulation) and,
 * if gradients != NULL, dE_b/dparams (batch x n_params) by the adjoint
 * method: one forward sweep, then a reverse sweep that un-applies every gate
 * from psi and lambda = H psi while accumulating 2 coef Im<lambda|G|psi> per
 * rotation.  With checkpoint_every = K > 0, psi is stored after every K gates
 * on the way forward and restored there on the way back, which bounds the
 * rounding drift of the un-applied complex64 state.  Blocking. */
int qg_adjoint_expectation(int prec, int n_qubits, const qg_circuit_op *ops, int n_ops,
                           const double *params, int n_params, int batch,
                           const qg_pauli_term *terms, int n_terms, int checkpoint_every,
                           double *expectations, double *gradients);

/* Extension (the reference runs one circuit at a time).  Runs n_circuits
 * independent circuits from |0...0> in complex64 and writes
 * out[c] = sum_i <Z_i> (FP64) of each.  Circuit c has n_qubits[c] lanes
 * (8..30) and the fixed gates (kind 0) gates[gate_offsets[c] ..
 * gate_offsets[c+1]).  Circuits of up to 13 qubits run entirely inside one
 * CTA's shared memory; larger ones advance one fused stage per round over a
 * packed arena; the whole batch is recorded and launched as one CUDA graph.
 * Blocking. */
int qg_batch_sum_z(int prec, int n_circuits, const int *n_qubits, const int64_t *gate_offsets,
                   const qg_circuit_op *gates, double *out);

/* Extension: how qg_batch_sum_z runs a batch: 1 (default) as one persistent
 * launch over a device-side queue of work items (whole circuits of <= 12
 * qubits, tiles of the larger circuits' stages round by round, chunks of
 * their final sums), items that need earlier ones waiting on per-circuit
 * counters; 0 as one launch per round of stages (circuits of <= 13 qubits
 * resident per CTA).  No reference counterpart. */
int qg_set_batch_one_launch(int on);

/* Extension: counters of the qubit-grouping policy, in this order: join
 * calls, kron passes, state buffers allocated, decohere_and_separate calls,
 * separations formed in place, separations formed by copy, copies of a
 * buffer still read by a lazy states object before a write.  Writes the
 * first min(n, 7); reset != 0 zeroes them.  No reference counterpart. */
int qg_grouping_stats(int64_t *out, int n, int reset);

/* ---- allocation-free variant ------------------------------------------- */

/* No counterpart in the reference.  Pr(local_lane == 0) of a state held in
 * caller-owned device memory (2^n_lanes complex64 for QG_PREC_FP32,
 * complex128 for QG_PREC_FP64), written as one double to caller-owned device
 * memory d_prob, enqueued on `stream` (a cudaStream_t; 0 = legacy default
 * stream) and returning before it completes.  For callers that cannot let
 * the library allocate: code that keeps all device memory in its own
 * pre-sized pool, or loops that must not take the device-wide
 * synchronisation a cudaMalloc / cudaFree can imply.  It allocates nothing
 * and never touches the engine's own context: the reduction's per-block
 * partials go to a fixed 2048-double (16 KiB) device array that each GPU
 * holds from library load until process exit.  The reduction uses at most
 * 1216 of those partials for any state size; n_lanes must be in [1, 40] and
 * anything else is rejected with QG_ERR_VALUE, as are a d_state that is not
 * 16-byte aligned and a d_prob that is not 8-byte aligned (the kernel reads
 * the state as 16-byte vectors).  The first call on a device looks up the
 * array's device address (cudaGetSymbolAddress) with that device current and
 * keeps it for the life of the process, so make that first call before any
 * stream capture; a cudaDeviceReset() on that device invalidates the kept
 * address, and the entry point must not be called on that device after one.
 * All calls share the one array: calls whose work overlaps on the GPU
 * (different streams, no ordering between them) race on it and give wrong
 * results. */
int qg_calc_probability_noalloc(int prec, const void *d_state, int n_lanes, int local_lane,
                                double *d_prob, uint64_t stream);

/* ---- gate matrices (qgate/simulator/src/GateMatrix.cpp:13-158) --------- */

/* Replaces glue.register_matrix_factory + the MatFactory call in
 * glue.qubit_processor_apply_gate (qgate/simulator/src/glue.cpp:93-134, 389-395).
 * name: U, U2, U1, ID, X, Y, Z, H, S, T, RX, RY, RZ, ExpiI, ExpiZ, SH. */
int qg_gate_matrix(const char *name, const double *args, int n_args, int adjoint, double *mat);

/* ---- states getter (qgate/simulator/src/Interfaces.h:55-72) ------------ */

/* Replaces cudaext.qubits_states_getter_new (qgate/simulator/src/cudaext.cpp:109-125). */
int qg_qubits_states_getter_new(int prec, qg_handle *out);
/* Replaces glue.qubits_states_getter_delete (qgate/simulator/src/glue.cpp:222-233). */
int qg_qubits_states_getter_delete(qg_handle getter);

/* Replaces glue.qubits_states_getter_get_states (qgate/simulator/src/glue.cpp:448-506).
 * lane_tables holds, for each of the n_qstates states, its
 * local-lane -> external-lane table (lane_counts[i] entries each,
 * concatenated).  values is a host array of n_states elements of
 * complex (mathop NULL) or real (mathop PROB) in the getter's precision,
 * written from values[array_offset].  Element i is taken at external index
 * start + step * i (step may be negative). */
int qg_qubits_states_getter_get_states(qg_handle getter, void *values, int64_t array_offset,
                                       int mathop, const int *lane_tables,
                                       const int *lane_counts, const qg_handle *qstates_list,
                                       int n_qstates, uint64_t empty_lane_mask, int n_qregs,
                                       int64_t n_states, int64_t start, int64_t step);

/* Replaces glue.qubits_states_getter_prepare_prob_array (qgate/simulator/src/glue.cpp:509-536).
 * Writes 2^n_lanes marginal probabilities (hidden lanes summed out) to the
 * host array prob in the getter's precision; accumulation is FP64. */
int qg_qubits_states_getter_prepare_prob_array(qg_handle getter, void *prob,
                                               const int *lane_tables, const int *lane_counts,
                                               const qg_handle *qstates_list, int n_qstates,
                                               int n_lanes, int n_hidden_lanes);

/* Replaces glue.qubits_states_getter_create_sampling_pool (qgate/simulator/src/glue.cpp:539-559).
 * The pool keeps an FP64 cumulative distribution in device memory. */
int qg_qubits_states_getter_create_sampling_pool(qg_handle getter, const int *lane_tables,
                                                 const int *lane_counts,
                                                 const qg_handle *qstates_list, int n_qstates,
                                                 int n_lanes, int n_hidden_lanes,
                                                 const int *empty_lanes, int n_empty_lanes,
                                                 qg_handle *out);

/* ---- sampling pool (qgate/simulator/src/Interfaces.h:75-80) ------------ */

/* Replaces glue.sampling_pool_sample (qgate/simulator/src/glue.cpp:562-589): obs[i] =
 * upper_bound(cdf, randnum[i]) with empty-lane zero bits inserted. */
int qg_sampling_pool_sample(qg_handle pool, int64_t *obs, int64_t n_samples,
                            const double *randnum);
/* Replaces glue.sampling_pool_delete (qgate/simulator/src/glue.cpp:592-603). */
int qg_sampling_pool_delete(qg_handle pool);

#ifdef __cplusplus
}
#endif

#endif /* QGATE_GB300_H */
