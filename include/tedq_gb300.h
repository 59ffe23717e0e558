/*
 * tedq_gb300.h -- C ABI of the GB300 (sm_103a) execution backend for TeD-Q's
 * compiled-circuit state-vector path.
 *
 * Boundary.  The reference executes a recorded circuit in
 * ``PyTorchBackend.__call__`` / ``execute`` (tedq/backends/pytorch_backend.py
 * :124-165, :228-391) after ``CompiledCircuit.__init__`` turned the circuit
 * into per-gate tensordot axes and permutations
 * (tedq/backends/compiled_circuit.py:48-202).  This library replaces that
 * pair: ``tedq_program_create`` is the compile step, ``tedq_run`` the
 * state-vector forward with its measurement reductions
 * (pytorch_backend.py:358-498) and ``tedq_run_adjoint`` the backward that the
 * reference obtains from torch autograd (``back_prop``, :142-144) or from
 * parameter-shift re-execution (``TorchExecute``, :1191-1223).
 *
 * Conventions (identical to the reference):
 *   - qubit q is bit (n-1-q) of the flat amplitude index (qubit 0 is the most
 *     significant axis of the ``[2]*n`` state, pytorch_backend.py:513-522);
 *   - a k-qubit gate matrix is indexed with qubits[0] as its most significant
 *     bit (pytorch_backend.py:741-750);
 *   - parameters are bound positionally: slot s of a circuit is the s-th
 *     trainable parameter walking the gates in order
 *     (compiled_circuit.py:492-547).  Slots are given per gate in
 *     ``tedq_gate_t.param_slot``.
 *
 * All device buffers are owned by the caller and passed as raw device
 * pointers; streams are ``cudaStream_t`` values passed as ``void*``.  No C++
 * exception crosses this boundary: every entry point returns a
 * ``tedq_status`` and ``tedq_last_error`` returns the message of the last
 * failure on the calling thread.
 */
#ifndef TEDQ_GB300_H
#define TEDQ_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define TEDQ_ABI_VERSION 1

typedef enum tedq_status {
  TEDQ_OK = 0,
  TEDQ_ERR_ARG = 1,         /* bad argument: sizes, qubit indices, null pointers   */
  TEDQ_ERR_OOM = 2,         /* host allocation failed or a size exceeds a limit    */
  TEDQ_ERR_CUDA = 3,        /* a CUDA runtime call failed                          */
  TEDQ_ERR_TIMEOUT = 4,     /* a bounded wait expired                              */
  TEDQ_ERR_UNSUPPORTED = 5, /* gate/observable form this backend does not execute  */
  TEDQ_ERR_STATE = 6        /* call made in the wrong state (e.g. stopped server)  */
} tedq_status;

/* Gate opcodes: the reference's gate set (tedq/QInterpreter/operators/qubit.py
 * ``ops``, :1803-1834).  TEDQ_OP_MATRIX carries a fixed matrix (the
 * reference's path for gates without trainable parameters,
 * compiled_circuit.py:432-435, and for ``.inv`` gates). */
enum {
  TEDQ_OP_I = 0, TEDQ_OP_H = 1, TEDQ_OP_X = 2, TEDQ_OP_Y = 3, TEDQ_OP_Z = 4,
  TEDQ_OP_S = 5, TEDQ_OP_T = 6, TEDQ_OP_SX = 7,
  TEDQ_OP_CNOT = 8, TEDQ_OP_CZ = 9, TEDQ_OP_CY = 10, TEDQ_OP_SWAP = 11,
  TEDQ_OP_CSWAP = 12, TEDQ_OP_TOFFOLI = 13,
  TEDQ_OP_RX = 14, TEDQ_OP_RY = 15, TEDQ_OP_RZ = 16, TEDQ_OP_ROT = 17,
  TEDQ_OP_PHASESHIFT = 18, TEDQ_OP_CPHASE = 19,
  TEDQ_OP_CRX = 20, TEDQ_OP_CRY = 21, TEDQ_OP_CRZ = 22,
  TEDQ_OP_MATRIX = 23
};

/* One gate of a recorded circuit (one ``GateBase`` instance,
 * tedq/QInterpreter/operators/ops_abc.py:227-340). */
typedef struct tedq_gate {
  int32_t op;             /* TEDQ_OP_*                                             */
  int32_t n_qubits;       /* 1..3                                                  */
  int32_t qubits[3];      /* qubits[0] is the control / most significant factor     */
  int32_t param_slot[3];  /* parameter slot per gate parameter, -1 = fixed          */
  double fixed[3];        /* value of each parameter whose slot is -1               */
  const double* matrix;   /* TEDQ_OP_MATRIX: 2^k x 2^k row-major (re, im) pairs     */
} tedq_gate_t;

/* Observable factor codes for expectation values
 * (measurement.py ``expval``, :106-155). */
enum { TEDQ_OBS_I = 0, TEDQ_OBS_X = 1, TEDQ_OBS_Y = 2, TEDQ_OBS_Z = 3, TEDQ_OBS_H = 4,
       TEDQ_OBS_MATRIX = 5 };

typedef struct tedq_obs_factor {
  int32_t obs;            /* TEDQ_OBS_*                                            */
  int32_t n_qubits;       /* 1..3 (only TEDQ_OBS_MATRIX may exceed 1)              */
  int32_t qubits[3];
  const double* matrix;   /* TEDQ_OBS_MATRIX: 2^k x 2^k (re, im) pairs              */
} tedq_obs_factor_t;

/* Measurement kinds (measurement.py ``MeasurementReturnTypes``, :240-266). */
enum { TEDQ_MEAS_EXPVAL = 0, TEDQ_MEAS_PROBS = 1, TEDQ_MEAS_STATE = 2 };

typedef struct tedq_meas {
  int32_t kind;                      /* TEDQ_MEAS_*                                 */
  int32_t n_factors;                 /* EXPVAL: factors of the tensor product,      */
  const tedq_obs_factor_t* factors;  /*   applied in list order (pytorch_backend.py:402-424) */
  int32_t n_qubits;                  /* PROBS: measured qubits, 0 = all             */
  const int32_t* qubits;
} tedq_meas_t;

enum { TEDQ_PREC_C64 = 0, TEDQ_PREC_C128 = 1 };

typedef struct tedq_options {
  int32_t precision;   /* TEDQ_PREC_C64 (complex64 state, float32 params/outputs)
                          or TEDQ_PREC_C128 (complex128 state, float64)            */
  int32_t fuse;        /* 1: fused multi-gate passes; 0: one pass per gate (plain) */
  int32_t tile_qubits; /* 0 = default tile size (2^13 amplitudes for c64)          */
  int32_t jit;         /* specialised per-circuit pass kernels compiled with NVRTC:
                          0 = auto (on for states of >= 14 qubits), 1 = on, -1 = off,
                          2 = on in the background (generic kernels until compiled);
                          the environment variable TEDQ_GB300_JIT=0 turns it off   */
  int32_t exact_phase; /* 0: uncontrolled diagonal gates (RZ, Z, S, T, ...) drop their
                          global phase unless the program measures the state (every
                          output of expval / probs is phase-free, and the adjoint
                          sweep moves both of its states by the same phase);
                          1: the final state keeps the exact global phase         */
  int32_t reserved[3];
} tedq_options_t;

typedef struct tedq_program tedq_program_t;

typedef struct tedq_program_info {
  int32_t n_qubits;          /* logical qubits                                     */
  int32_t state_qubits;      /* qubits of the device state (>= n_qubits; small
                                circuits are padded with idle low-order qubits)    */
  int32_t n_params;          /* parameter slots per circuit                        */
  int32_t n_real_outputs;    /* floats per circuit written to out_real             */
  int32_t n_terms;           /* distinct Pauli strings measured                    */
  int32_t n_fwd_passes;      /* HBM passes of the forward schedule                 */
  int32_t n_bwd_passes;      /* HBM passes of the adjoint schedule                 */
  int32_t n_fwd_phases;      /* register phases of the forward schedule            */
  int32_t n_bwd_phases;
  int32_t n_fused_gates;     /* gates after fusion (forward)                       */
  int32_t n_elem_gates;      /* elementary gates (adjoint)                         */
  int32_t precision;
  int64_t workspace_per_circuit; /* bytes of workspace per circuit of a batch      */
  int32_t jit_state;         /* 0 off, 1 compiling, 2 compiled, 3 loaded, -1 failed  */
  int32_t pad;
  int64_t jit_modules_loaded; /* specialised-kernel modules loaded, all devices    */
  int64_t reserved[2];
} tedq_program_info_t;

/* ---- library ------------------------------------------------------------ */
int32_t tedq_abi_version(void);
/* Message of the last failed call on this thread; returns its length. */
int32_t tedq_last_error(char* buf, size_t len);

/* ---- program: compile a recorded circuit --------------------------------
 * Replaces CompiledCircuit.__init__ (compiled_circuit.py:48-202): classifies
 * gates (diagonal / permutation / controlled / dense), fuses runs of
 * one-qubit gates, schedules the gate list into HBM passes over 2^m-amplitude
 * tiles and register phases inside each tile, and decomposes observables into
 * Pauli strings.  ``opts`` may be NULL (defaults). */
int32_t tedq_program_create(const tedq_gate_t* gates, int32_t n_gates, int32_t n_qubits,
                            const tedq_meas_t* meas, int32_t n_meas,
                            const tedq_options_t* opts, tedq_program_t** out);
int32_t tedq_program_destroy(tedq_program_t* prog);
int32_t tedq_program_info(const tedq_program_t* prog, tedq_program_info_t* info);
/* Waits for the program's specialised kernels to be compiled (host only, no
 * GPU needed).  TEDQ_OK when they are ready, TEDQ_ERR_UNSUPPORTED when they are
 * off or could not be built (reason in tedq_last_error); the generic pass
 * kernels are used then. */
int32_t tedq_program_jit_wait(tedq_program_t* prog);
/* Device workspace (bytes) that tedq_run / tedq_run_adjoint need for a batch. */
int64_t tedq_program_workspace_bytes(const tedq_program_t* prog, int64_t batch);
/* Schedule export for inspection: writes a JSON description of the passes
 * and phases (forward when ``adjoint`` == 0) into ``buf``; returns the
 * length needed including the terminating zero. */
int64_t tedq_program_describe(const tedq_program_t* prog, int32_t adjoint, char* buf, int64_t len);

/* ---- forward: PyTorchBackend.execute, state-vector branch ---------------
 * params    [batch][n_params]          float (c64) / double (c128), device
 * psi       [batch][2^state_qubits]    complex, device; receives final states
 * out_real  [batch][n_real_outputs]    float / double, device; expvals then
 *                                      probs, in measurement order (may be NULL
 *                                      when the program has no real outputs)
 * init      [2^n_qubits] complex initial state shared by the batch, or NULL
 *           for |0...0> (pytorch_backend.py:500-522)
 * workspace >= tedq_program_workspace_bytes(batch) bytes, device, 256-byte
 *           aligned (Pauli-term, probability and gradient accumulators) */
int32_t tedq_run(tedq_program_t* prog, const void* params, int64_t batch, void* psi,
                 void* out_real, const void* init, void* workspace, size_t workspace_bytes,
                 void* stream);

/* ---- forward without allocation -----------------------------------------
 * No counterpart in the reference.  Same as tedq_run, but the workspace is a
 * 1 MiB static device array of this library instead of a caller buffer, for
 * callers that cannot allocate device memory where they run circuits (inside
 * stream capture, allocator callbacks, real-time loops, embedders whose device
 * memory belongs to another runtime).  The 1 MiB bounds the forward
 * accumulators: 8 bytes per measured Pauli string and per probability bin of
 * each circuit, each of the two regions rounded up to 256 bytes; larger
 * batches are rejected (TEDQ_ERR_ARG).  The first call on a device looks up
 * the array's address and should come before any stream capture.  The
 * program's specialised pass kernels are used only if an earlier tedq_run /
 * tedq_run_adjoint loaded them on this device, otherwise the generic ones run:
 * this call never waits for a compile and never loads a module.  Calls that
 * overlap on the GPU share the array and race. */
int32_t tedq_run_noalloc(tedq_program_t* prog, const void* params, int64_t batch, void* psi,
                         void* out_real, const void* init, void* stream);

/* ---- adjoint backward ----------------------------------------------------
 * Vector-Jacobian product of tedq_run: grad[b][s] = d/dparam[b][s] of
 *   sum_k dy_real[b][k] * out_real[b][k] + Re sum_x conj(dy_state[b][x]) psi[b][x]
 * psi       final states from tedq_run; overwritten (uncomputed to the
 *           initial state)
 * lambda_   [batch][2^state_qubits] complex device scratch
 * dy_real   [batch][n_real_outputs] or NULL; dy_state [batch][2^state_qubits]
 *           complex or NULL
 * grad      [batch][n_params] float / double, device, written */
int32_t tedq_run_adjoint(tedq_program_t* prog, const void* params, int64_t batch,
                         const void* dy_real, const void* dy_state, void* psi, void* lambda_,
                         void* grad, void* workspace, size_t workspace_bytes, void* stream);

/* ---- serving: continuous batching of circuit evaluations ----------------
 * No counterpart in the reference (it evaluates one circuit per call; its
 * QUDIO backend wraps torch.nn.DataParallel over a dataset,
 * tedq/backends/qudio_backend.py:45-124).  A server owns one device-memory
 * arena (the admission budget), a worker thread and a few streams.  Requests
 * (program, parameters on the host, optional gradient) are queued; the worker
 * groups queued requests of the same program into batches as capacity frees
 * up, runs forward (+ adjoint) on its own streams while other batches are in
 * flight, and completes each request when its batch's results are back on the
 * host.  Requests that arrive while others run are admitted as soon as memory
 * and stream slots allow. */
typedef struct tedq_server tedq_server_t;

typedef struct tedq_server_options {
  int32_t device;              /* CUDA device index                                  */
  int32_t n_streams;           /* concurrent batches (default 4)                     */
  int32_t max_batch;           /* circuits per batch (default 256)                   */
  int32_t max_wait_us;         /* batching window for a partially filled batch       */
  int64_t memory_budget_bytes; /* device arena for states and buffers                */
  int32_t paused;              /* 1: queue requests but launch nothing until
                                  tedq_server_resume (deterministic batching)       */
  int32_t lane_qubits;         /* size-class lanes: states of at most this many
                                  qubits form the small lane (own high-priority
                                  streams, half of n_streams, and a reserved 1/8 of
                                  the budget, at most 8 GiB); 0 = 16, < 0 = one lane */
  int64_t reserved[3];
} tedq_server_options_t;

typedef struct tedq_request_result {
  int32_t status;      /* TEDQ_OK or the failure status of the request             */
  int32_t batch_size;  /* circuits in the batch that carried the request           */
  double queue_us;     /* submit -> batch launch                                   */
  double total_us;     /* submit -> results on the host                            */
} tedq_request_result_t;

typedef struct tedq_server_stats {
  int64_t submitted, completed, failed, cancelled, batches;
  int64_t in_flight_bytes, peak_in_flight_bytes;
  int64_t reserved[4];
} tedq_server_stats_t;

int32_t tedq_server_create(const tedq_server_options_t* opts, tedq_server_t** out);
/* Stops the worker after the batches in flight; queued requests fail with
 * TEDQ_ERR_STATE. */
int32_t tedq_server_destroy(tedq_server_t* server);
/* params: host array of the program's n_params values (float for c64 programs,
 * double for c128), copied at submission.  dy: host array of n_real_outputs
 * cotangents or NULL for all ones; with_grad = 0 skips the adjoint. */
int32_t tedq_server_submit(tedq_server_t* server, tedq_program_t* prog, const void* params,
                           const void* dy, int32_t with_grad, int64_t* ticket);
/* Waits at most timeout_us (< 0: no limit) for a request; copies its outputs
 * (n_real_outputs) and gradient (n_params) into host arrays (either may be
 * NULL).  TEDQ_ERR_TIMEOUT when the wait expires (the request stays valid);
 * otherwise the request is released. */
int32_t tedq_server_wait(tedq_server_t* server, int64_t ticket, int64_t timeout_us, void* out_real,
                         void* grad, tedq_request_result_t* result);
/* Cancels a request that has not been launched yet (TEDQ_ERR_STATE otherwise). */
int32_t tedq_server_cancel(tedq_server_t* server, int64_t ticket);
int32_t tedq_server_stats(tedq_server_t* server, tedq_server_stats_t* out);
int32_t tedq_server_resume(tedq_server_t* server);

/* ---- profiling -----------------------------------------------------------
 * When enabled, tedq_run / tedq_run_adjoint record a CUDA event pair on the
 * launch stream around every kernel launch of the program; tedq_profile_read
 * synchronises those events, returns the accumulated device time per kernel
 * family and clears the record.  No reference counterpart (the reference has
 * no tracing, only ad-hoc wall clocks in its examples). */
typedef struct tedq_profile {
  int64_t fwd_launches;   double fwd_ms;    /* forward pass kernels              */
  int64_t bwd_launches;   double bwd_ms;    /* adjoint pass kernels              */
  int64_t meas_launches;  double meas_ms;   /* expval / probs / finalize kernels */
  int64_t lam_launches;   double lam_ms;    /* lambda init, weights, grad finalize */
  int64_t fwd_amp_passes; /* sum over forward launches of batch * 2^state_qubits */
  int64_t bwd_amp_passes; /* same for adjoint launches                           */
  int64_t reserved[4];
} tedq_profile_t;

int32_t tedq_profile_enable(tedq_program_t* prog, int32_t on);
int32_t tedq_profile_read(tedq_program_t* prog, tedq_profile_t* out);

/* ---- tensor-network mode --------------------------------------------------
 * Replaces the TN branch of PyTorchBackend.execute (pytorch_backend.py:242-356):
 * the sandwich network of gen_tensor_networks (tensor_network.py:850-1099),
 * the external path optimiser (OEWrapper, oe_wrapper.py:24-65; JDOptTN,
 * compiled_circuit.py:388-393) and torch einsum.  One network per
 * measurement, reduced to the backward light cone of its observable, ordered
 * by randomised greedy search and sliced until every intermediate fits
 * 2^max_rank entries.  Small pairwise contractions run in level launches
 * that read their operands in place; each large one as two bit-permutation
 * gathers into planar real operands and one real GEMM on the tensor cores
 * (4M decomposition: [Re A; Im A] x [Re B, Im B]), batched over the circuits
 * of a call.  Expectation values of tensor products of observable factors
 * (the Python layer builds probs(qubits=...) from projector products; a
 * state measurement runs on the state-vector passes). */
typedef struct tedq_tn_plan tedq_tn_plan_t;

/* GEMM arithmetic of the complex64 mode (complex128 uses FP64 FMA GEMMs).
 * All GEMMs are kernels of this library: tcgen05 tensor-core MMAs (TF32
 * operands staged by TMA, FP32 accumulators in tensor memory) or FMA. */
enum {
  TEDQ_TN_GEMM_FP32 = 0,    /* FP32 FMA                                       */
  TEDQ_TN_GEMM_TC32 = 1,    /* FP32 accuracy on the tensor cores: each operand
                               split into two TF32 parts, three products
                               (hi*hi + hi*lo + lo*hi)                        */
  TEDQ_TN_GEMM_TF32 = 2,    /* one TF32 product per term (~1e-3 relative)     */
  TEDQ_TN_GEMM_AUTO = 3     /* TC32 for the contractions of at least 2^16
                               flops per circuit whose shape fills the
                               tensor-core tiles, FP32 FMA for the rest       */
};

typedef struct tedq_tn_options {
  int32_t precision;   /* TEDQ_PREC_C64 / TEDQ_PREC_C128                       */
  int32_t gemm;        /* TEDQ_TN_GEMM_* (complex64 only)                      */
  int32_t max_rank;    /* 0 = 27; at most 28                                   */
  int32_t repeats;     /* randomised greedy trials, 0 = 64                     */
  uint64_t seed;       /* 0 = 1                                                */
  int32_t graphs;      /* 1: replay each call's launches as a CUDA graph       */
  int32_t reserved[3];
} tedq_tn_options_t;

typedef struct tedq_tn_info {
  int32_t n_qubits;
  int32_t n_params;
  int32_t n_meas;
  int32_t n_steps;          /* pairwise contractions, all measurements         */
  int32_t max_rank;         /* largest intermediate: 2^max_rank entries         */
  int32_t n_sliced;         /* sliced indices (largest over measurements)      */
  int32_t gates_kept;       /* circuit gates inside the light cones (sum)      */
  int32_t precision;
  double log2_flops;        /* log2 of real flops per circuit (8 per complex MAC) */
  int64_t workspace_per_circuit;
  int64_t workspace_fixed;  /* bytes independent of the batch                  */
  int64_t reserved[4];
} tedq_tn_info_t;

int32_t tedq_tn_plan_create(const tedq_gate_t* gates, int32_t n_gates, int32_t n_qubits,
                            const tedq_meas_t* meas, int32_t n_meas, const tedq_tn_options_t* opts,
                            tedq_tn_plan_t** out);
int32_t tedq_tn_plan_destroy(tedq_tn_plan_t* plan);
int32_t tedq_tn_plan_info(const tedq_tn_plan_t* plan, tedq_tn_info_t* info);
/* JSON export of the networks, orders, gather tables and layouts; returns the
 * length needed including the terminating zero (-1 on error). */
int64_t tedq_tn_plan_describe(const tedq_tn_plan_t* plan, char* buf, int64_t len);
/* Device workspace (bytes) of tedq_tn_contract for a batch (-1 on error). */
int64_t tedq_tn_workspace_bytes(const tedq_tn_plan_t* plan, int64_t batch);
/* params    [batch][n_params] float (c64) / double (c128), device
 * out       [batch][n_meas]   float / double, device
 * workspace >= tedq_tn_workspace_bytes(batch) bytes, device, 256-byte aligned
 * The first call with a new batch size uploads the plan's table of small
 * contractions for that size (synchronising the device): make one call with
 * a batch size before capturing calls with it in a CUDA graph.  A circuit
 * with a non-finite parameter returns NaN. */
int32_t tedq_tn_contract(tedq_tn_plan_t* plan, const void* params, int64_t batch, void* out,
                         void* workspace, size_t workspace_bytes, void* stream);

/* Kernel timing of tedq_tn_contract (no counterpart in the reference): while
 * enabled, calls run without graphs and record CUDA events around every launch
 * on the launch stream; read sums the durations per launch family since the
 * last read, with the algorithmic work of the launches (gather bytes: source
 * read + planar operand write; contraction flops: 2 per real multiply-add).
 * gemm_* covers every contraction launch (level launches, FMA and tensor-core
 * GEMMs), tc_* the tensor-core GEMMs alone.  gemm_error is the device error
 * word of the tensor-core GEMMs: nonzero when one gave up a bounded wait (the
 * read then returns TEDQ_ERR_TIMEOUT and the calls' results are NaN). */
typedef struct tedq_tn_profile {
  int64_t leaf_launches;
  double leaf_ms;
  int64_t gather_launches;
  double gather_ms;
  double gather_bytes;
  int64_t gemm_launches;
  double gemm_ms;
  double gemm_flops;
  int64_t root_launches;
  double root_ms;
  int64_t tc_launches;
  double tc_ms;
  double tc_flops;
  int32_t gemm_error;
  int32_t pad;
} tedq_tn_profile_t;

int32_t tedq_tn_profile_enable(tedq_tn_plan_t* plan, int32_t on);
int32_t tedq_tn_profile_read(tedq_tn_plan_t* plan, tedq_tn_profile_t* out);

/* The batched real GEMM that tedq_tn_contract runs for each large pairwise
 * contraction, on caller buffers (no counterpart in the reference, whose
 * contractions are torch einsum calls; exposed for testing and for callers
 * with operands of their own):
 *   C[b](i, j) = sum_k A[b](i, k) B[b](j, k),   b < nbatch (<= 65535),
 * A [mr][kr] and B [nr][kr] row-major (K contiguous), C column-major (C[j*mr+i]);
 * sa, sb, sc: elements between batch entries (0: operand shared by all).
 * precision TEDQ_PREC_C64: float data, mode TEDQ_TN_GEMM_* (TC32 / TF32
 * return TEDQ_ERR_UNSUPPORTED where the tensor-core kernel does not apply:
 * kr a multiple of 4, the larger of mr, nr >= 32, the smaller >= 8,
 * 16-byte aligned A and B; AUTO then uses FMA); TEDQ_PREC_C128: double data,
 * FP64 FMA.  err_word: a device int32 that the tensor-core kernel sets when
 * one of its bounded waits gives up (required for TC32 / TF32 / AUTO). */
int32_t tedq_tn_gemm(int32_t precision, int32_t gemm, const void* a, const void* b, void* c, int64_t mr, int64_t nr,
                     int64_t kr, int64_t sa, int64_t sb, int64_t sc, int64_t nbatch, int32_t* err_word, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* TEDQ_GB300_H */
