/*
 * pyramaterised_gb300 -- C ABI of the GB300 statevector engine.
 *
 * The reference (rmdocherty/pyramaterised) has no FFI: its hot path is the
 * Python object API that `Measurements` consumes, with all arithmetic done
 * by QuTiP 4.7.2 sparse matrices.  Each entry point below replaces one of
 * those Python calls; the comment on each cites the reference code it
 * stands in for.  Host code (the Python mirror in `pyramaterised_gb300/`)
 * binds these with ctypes.
 *
 * Conventions
 *   - States are complex128, interleaved (re, im) doubles, row-major
 *     [batch, 2^n_qubits].  Qubit q lives in bit (n_qubits-1-q) of the basis
 *     index (QuTiP `tensor` order: qubit 0 most significant).
 *   - All pointers to arrays are DEVICE pointers unless stated otherwise;
 *     `stream` is a cudaStream_t (NULL = legacy default stream).
 *   - Every call is asynchronous on `stream`, returns 0 on success or a
 *     negative pqc_status, never aborts, and records a message readable
 *     with pqc_last_error() (thread-local).
 *   - Entry points that need scratch memory take (workspace, workspace_bytes)
 *     owned by the caller; the matching *_workspace_size() says how much.
 *   - The library allocates device memory for a program's tables only, all
 *     released by pqc_program_destroy: the op tables and sweep plans in
 *     pqc_program_create, and the derivative / adjoint plans of a generator
 *     list on the first pqc_derivative_states(_from) / pqc_energy_grad call
 *     with that list (cudaMalloc plus a synchronous upload; make that first
 *     call outside stream capture).  Later calls with the same list allocate
 *     nothing.  pqc_run_static allocates nothing at all.
 */
#ifndef PYRAMATERISED_GB300_H
#define PYRAMATERISED_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PQC_ABI_VERSION 2

typedef enum pqc_status {
  PQC_OK = 0,
  PQC_ERR_INVALID = -1,     /* bad argument / malformed program */
  PQC_ERR_UNSUPPORTED = -2, /* gate or size not supported */
  PQC_ERR_CUDA = -3,        /* a CUDA call failed (message has the CUDA error) */
  PQC_ERR_WORKSPACE = -4,   /* workspace missing or too small */
  PQC_ERR_NOMEM = -5
} pqc_status;

/* Primitive operations a circuit is lowered to (gates.py classes -> ops). */
typedef enum pqc_op_kind {
  PQC_OP_RX = 1,        /* exp(-i a X/2) on q0                gates.py:159-162 */
  PQC_OP_RY = 2,        /* exp(-i a Y/2) on q0                gates.py:165-168 */
  PQC_OP_RZ = 3,        /* exp(-i a Z/2) on q0                gates.py:171-174, 180-205 */
  PQC_OP_MAT1 = 4,      /* fixed 2x2 in m[0..7]               H/X/S/T gates.py:211-300 */
  PQC_OP_CNOT = 5,      /* control q0, target q1              gates.py:327-330 */
  PQC_OP_CZ = 6,        /* diag(1,1,1,-1) on (q0,q1)          gates.py:333-349 */
  PQC_OP_RXX = 7,       /* cos(a/2) I - i sin(a/2) XX          gates.py:538-543 */
  PQC_OP_RYY = 8,       /*                     ... YY          gates.py:546-551 */
  PQC_OP_RZZ = 9,       /*                     ... ZZ          gates.py:530-535 */
  PQC_OP_MAT2 = 10,     /* fixed 4x4 in m[0..31], q0 = first tensor factor (sqrtiSWAP gates.py:340-343) */
  PQC_OP_FSIM = 11,     /* fsim(a, b), a from param, b from param2    gates.py:588-606 */
  PQC_OP_FIXED_FSIM = 12, /* fixed_fsim(a)                           gates.py:700-716 */
  PQC_OP_PAULI = 13,    /* (m[0] + i m[1]) * P, P a Pauli string on q0[,q1] given by `pauli` */
  PQC_OP_FSIM_DTHETA = 14, /* gates.py:609-627 matrix (a, b) */
  PQC_OP_FSIM_DPHI = 15,   /* gates.py:630-648 matrix (a, b) */
  PQC_OP_FIXED_FSIM_DTHETA = 16 /* gates.py:719-737 matrix (a) */
} pqc_op_kind;

/* Pauli letters for PQC_OP_PAULI: pauli = letter(q0) | letter(q1) << 8. */
#define PQC_PAULI_I 0
#define PQC_PAULI_X 1
#define PQC_PAULI_Y 2
#define PQC_PAULI_Z 3

typedef struct pqc_op {
  int32_t kind;    /* pqc_op_kind */
  int32_t q0, q1;  /* qubits; q1 = -1 for one-qubit ops */
  int32_t param;   /* theta column of the first angle, -1 = fixed */
  int32_t param2;  /* theta column of the second angle (fSim phi), -1 = none */
  int32_t sel;     /* -1: applied to every batch row; r >= 0: only to row r */
  int32_t pauli;   /* PQC_OP_PAULI letters */
  int32_t pad;
  double scale, offset;   /* angle  = scale  * theta[param]  + offset  (param < 0: offset) */
  double scale2, offset2; /* angle2 = scale2 * theta[param2] + offset2 */
  double m[32];           /* MAT1: 2x2, MAT2: 4x4, row-major (re, im) pairs; PAULI: m[0]+i m[1] */
} pqc_op;

typedef struct pqc_pauli_term {
  uint64_t xmask; /* basis-index bits flipped (X or Y on that qubit) */
  uint64_t zmask; /* basis-index bits with a Z or Y */
  double coef;    /* real coefficient */
  int32_t n_y;    /* number of Y letters (phase i^n_y) */
  int32_t pad;
} pqc_pauli_term;

typedef struct pqc_program pqc_program;

/* ------------------------------------------------------------------ misc */
int pqc_abi_version(void);
const char* pqc_last_error(void);
/* Kernels launched by this library since it was loaded (all threads). */
long long pqc_launch_count(void);

/* ------------------------------------------------------------- programs
 * Replaces `PQC.set_gates` (circuit.py:53-72) + the per-gate operator
 * construction of gates.py (`get_op`, rebuilt on every `set_theta`,
 * gates.py:122-131): the gate list is lowered once to `ops` and planned into
 * shared-memory sweeps of 2^tile_qubits amplitudes (tile_qubits <= 0: auto).
 */
int pqc_program_create(const pqc_op* ops, int32_t n_ops, int32_t n_qubits, int32_t n_params,
                       int32_t tile_qubits, pqc_program** out);
void pqc_program_destroy(pqc_program* prog);
/* Host-only planning (no device needed): the order in which the sweep plan
 * applies the ops (order[i] = op index) and each position's sweep index. */
int pqc_plan_order(const pqc_op* ops, int32_t n_ops, int32_t n_qubits, int32_t tile_qubits, int32_t* order,
                   int32_t* sweep_of, int32_t* n_sweeps);
/* Host-only planning of derivative runs (no device needed): the order in which
 * the derivative plan of pqc_derivative_states applies the forward ops and the
 * generators (order[i] = op index, or -(r + 1) for generator r; n_ops + n_gens
 * entries).  The planner may reorder commuting ops and move each generator
 * later past ops it commutes with, so every run's state equals the reference's
 * `take_derivative` (circuit.py:149-172); this call exposes the order for tests. */
int pqc_derivative_plan_order(const pqc_op* ops, int32_t n_ops, const pqc_op* gens, const int32_t* gen_after,
                              int32_t n_gens, int32_t n_qubits, int32_t tile_qubits, int32_t* order,
                              int32_t* n_sweeps);
/* Number of sweeps (HBM passes) in the plan and the tile size used. */
int pqc_program_info(const pqc_program* prog, int32_t* n_sweeps, int32_t* tile_qubits);
/* Launch shape of the program's sweeps below 2^13-amplitude tiles: 3 (the
 * default, 0) or 2 resident CTAs per SM.  No counterpart in the reference: a
 * tuning knob, set by the autotuner (pyramaterised_gb300.engine.autotune). */
int pqc_program_set_occupancy(pqc_program* prog, int32_t ctas_per_sm);
/* The same with the CTA size: threads 128 or 256 with 3 CTAs per SM, 0 (default) to choose by grid size. */
int pqc_program_set_launch(pqc_program* prog, int32_t ctas_per_sm, int32_t threads);
/* 1 when `limit` is a valid per-row op limit for pqc_run_limited / pqc_energy_grad on this
 * program, 0 when it falls inside a CNOT-RZ-CNOT triple that the forward plan applies as one
 * diagonal ZZ rotation (limits at gate or layer boundaries of the ansatze are always valid). */
int pqc_program_limit_ok(const pqc_program* prog, int32_t limit);

/* Status bits the program's kernels raised since the last call, then cleared (synchronises the device).
 * PQC_STATUS_LOAD_TIMEOUT: a sweep's bulk tile load did not complete within its wait limit (about a
 * second); that tile's results are not valid.  0 after every correct run. */
#define PQC_STATUS_LOAD_TIMEOUT 1
int pqc_program_status(pqc_program* prog, int32_t* flags);

/* --------------------------------------------------------------- forward
 * Replaces `PQC.run` (circuit.py:118-125): psi[b] = G_last ... G_1 psi0 for
 * each parameter row theta[b * theta_stride + j] (theta_stride = 0 shares one
 * row across the batch).  psi0: a device state [2^n] or NULL to start from the
 * basis state `psi0_index`.  Computed in double-float (~48-bit) arithmetic on
 * the FP32 pipes; output complex128.
 */
size_t pqc_run_workspace_size(const pqc_program* prog, int64_t batch);
int pqc_run(const pqc_program* prog, const double* theta, int64_t theta_stride, int64_t batch,
            const void* psi0, int64_t psi0_index, void* psi, void* workspace, size_t workspace_bytes,
            void* stream);
/* pqc_run where row b applies only the ops whose index in `ops` is below
 * row_limit[b] (device int32 [batch]): one launch evaluates circuits of one
 * family at different depths (a depth-d circuit is a prefix of the deepest). */
int pqc_run_limited(const pqc_program* prog, const double* theta, int64_t theta_stride, int64_t batch,
                    const void* psi0, int64_t psi0_index, const int32_t* row_limit, void* psi, void* workspace,
                    size_t workspace_bytes, void* stream);
/* Same results computed in native FP64 (complex128) arithmetic on the FP64
 * pipe, the reference's own precision: the measured comparison arm of the
 * double-float default (GB300 runs FP64 at 1/64 of the FP32 rate).  Same
 * workspace as pqc_run. */
int pqc_run_fp64(const pqc_program* prog, const double* theta, int64_t theta_stride, int64_t batch,
                 const void* psi0, int64_t psi0_index, void* psi, void* workspace, size_t workspace_bytes,
                 void* stream);
/* Same, complex64 output computed in FP32 (the sampling mode). */
int pqc_run_c64(const pqc_program* prog, const double* theta, int64_t theta_stride, int64_t batch,
                const void* psi0, int64_t psi0_index, void* psi_c64, void* workspace,
                size_t workspace_bytes, void* stream);
/* The plain path: one FP64 kernel launch per op (the per-gate structure of
 * circuit.py:123-124), for comparison and as a second implementation. */
int pqc_run_plain(const pqc_program* prog, const double* theta, int64_t theta_stride, int64_t batch,
                  const void* psi0, int64_t psi0_index, void* psi, void* workspace, size_t workspace_bytes,
                  void* stream);  /* workspace: pqc_run_workspace_size bytes */

/* ------------------------------------------------- multi-program forward
 * Replaces one `PQC.run` call per circuit (circuit.py:118-125) for a mix of
 * circuits: item i is pqc_run_limited(items[i].prog, items[i].theta, ...) --
 * programs of any qubit counts, depths and gate lists -- and every item's
 * states equal that call's, bit for bit.  The items share the launches: one
 * coefficient launch and one conversion launch for all of them, then one
 * sweep launch per sweep index over every item that has that sweep (a mix of
 * circuits of up to 13 qubits is three launches).  row_limit: device int32
 * [batch] or NULL (see pqc_run_limited).  All programs must live on the
 * current device.  No counterpart in the reference: a batching entry point
 * for serving loops whose requests are many small circuits. */
typedef struct pqc_run_item {
  const pqc_program* prog;
  const double* theta;      /* device [batch, theta_stride] */
  int64_t theta_stride;
  int64_t batch;
  const void* psi0;         /* device state [2^n] or NULL: basis state psi0_index */
  int64_t psi0_index;
  const int32_t* row_limit; /* device int32 [batch] or NULL */
  void* psi;                /* device complex128 [batch, 2^n] */
} pqc_run_item;
size_t pqc_run_multi_workspace_size(const pqc_run_item* items, int32_t n_items);
int pqc_run_multi(const pqc_run_item* items, int32_t n_items, void* workspace, size_t workspace_bytes,
                  void* stream);

/* ------------------------------------------------- allocation-free forward
 * No counterpart in the reference.  pqc_run without a workspace, for callers
 * that cannot allocate device memory: a host framework that owns all device
 * memory and forbids the libraries it loads from calling cudaMalloc, or a
 * latency-critical loop that must never risk an allocation failing or stalling.
 * Same results as pqc_run.  The scratch is an array compiled into the library,
 * pqc_run_static_capacity() bytes (16 MiB), held on every GPU that loads the
 * library until the process exits; a call needing more returns
 * PQC_ERR_UNSUPPORTED.  The first call on each device looks up the array's
 * address (make that call before any stream capture).  Every call shares the
 * array, so calls that overlap on the GPU race: serialise them. */
size_t pqc_run_static_capacity(void);
int pqc_run_static(const pqc_program* prog, const double* theta, int64_t theta_stride, int64_t batch,
                   const void* psi0, int64_t psi0_index, void* psi, void* stream);

/* --------------------------------------------------------------- measures */
/* <a[ia[k]] | b[ib[k]]> for k < n (Qobj.overlap, measure.py:52,58,135; circuit.py:141).
 * out: complex128 [n].  ia/ib: device int64 row indices. */
size_t pqc_overlaps_workspace_size(int64_t n, int32_t n_qubits);
int pqc_overlaps(const void* a, const void* b, const int64_t* ia, const int64_t* ib, int64_t n,
                 int32_t n_qubits, void* out, void* workspace, size_t workspace_bytes, void* stream);
/* All-pairs fidelities |<psi_a|psi_b>|^2, a < b in itertools.combinations order
 * (measure.py:123-137, 409-419), binned exactly like np.histogram(range=(0,1))
 * with the given nbins+1 edges (measure.py:153-155).  F (optional, may be
 * NULL) receives the S(S-1)/2 fidelities; counts (int64 [nbins]) the histogram. */
size_t pqc_fidelity_hist_workspace_size(int64_t S, int32_t n_qubits);
int pqc_fidelity_hist(const void* psi, int64_t S, int32_t n_qubits, int32_t nbins, const double* edges,
                      double* F, int64_t* counts, void* workspace, size_t workspace_bytes, void* stream);
/* The Gram G[a][b] = <psi_a|psi_b> of S <= 256 states of n_qubits >= 13 on the
 * tensor cores (TF32 products, FP32 accumulation per amplitude slice, FP64 sum
 * of the slices): each component is within *delta_factor ||a|| ||b|| of the
 * exact value.  The low-precision first stage of the counts-only histogram
 * (the Qobj.overlap pairs of measure.py:123-137); pqc_fidelity_hist certifies
 * every pair's bin against that bound.  G: complex128 [S, S], written in full
 * (NaN everywhere if a tile load or MMA wait timed out).  PQC_ERR_UNSUPPORTED
 * where the tensor-core path does not apply (other sizes, a GPU other than
 * sm_103). */
size_t pqc_gram_tf32_workspace_size(int64_t S, int32_t n_qubits);
int pqc_gram_tf32(const void* psi, int64_t S, int32_t n_qubits, void* G, double* delta_factor, void* workspace,
                  size_t workspace_bytes, void* stream);
/* np.histogram(F, bins=nbins, range=(edges[0], edges[nbins])) of M samples
 * (measure.py:153-155) with the same index rule as pqc_fidelity_hist. */
int pqc_histogram(const double* F, int64_t M, int32_t nbins, const double* edges, int64_t* counts, void* stream);
/* KL divergence of a histogram against the Haar fidelity density
 * (d-1)(1-F)^(d-2) at the bin midpoints (measure.py:161-180).  out: double[1]. */
int pqc_expr_kl(const int64_t* counts, int32_t nbins, const double* edges, double d, double* out,
                void* stream);
/* Meyer-Wallach Q = 2(1 - mean_k tr rho_k^2) per state (measure.py:226-237). */
size_t pqc_mw_workspace_size(int64_t batch, int32_t n_qubits);
int pqc_mw(const void* psi, int64_t batch, int32_t n_qubits, double* Q, void* workspace,
           size_t workspace_bytes, void* stream);
/* <psi_b|H|psi_b> for a Pauli sum H (qt.expect in circuit.py:132-137); terms: DEVICE array. */
size_t pqc_expect_workspace_size(int64_t batch, int32_t n_qubits, int32_t n_terms);
int pqc_expect(const void* psi, int64_t batch, int32_t n_qubits, const pqc_pauli_term* terms,
               int32_t n_terms, double* E, void* workspace, size_t workspace_bytes, void* stream);
/* Renyi-alpha stabiliser entropy (measure.py:318-349; alpha = 1/2 gives the
 * GKP input of measure.py:361-368), via a Walsh-Hadamard transform. */
size_t pqc_magic_workspace_size(int64_t batch, int32_t n_qubits);
int pqc_magic(const void* psi, int64_t batch, int32_t n_qubits, double alpha, double* M, void* workspace,
              size_t workspace_bytes, void* stream);  /* n_qubits <= 13 */
/* QFIM F_pq = 4 Re(<d_p|d_q> - <d_p|s><s|d_q>) (measure.py:33-71) from P
 * derivative states dpsi [P, 2^n] and the reference state `state`. */
size_t pqc_qfim_workspace_size(int64_t P, int32_t n_qubits);
int pqc_qfim(const void* state, const void* dpsi, int64_t P, int32_t n_qubits, double* F,
             void* workspace, size_t workspace_bytes, void* stream);
/* The same QFIM with the Gram in native FP64 (the double-float Gram of
 * pqc_qfim is within ~1e-14 relative; a rank decision at numpy's tolerance
 * max(P, P) eps sigma_max needs FP64).  Same workspace as pqc_qfim. */
int pqc_qfim_fp64(const void* state, const void* dpsi, int64_t P, int32_t n_qubits, double* F,
                  void* workspace, size_t workspace_bytes, void* stream);

/* ---------------------------------------------------------- derivatives
 * Derivative states (circuit.py:149-192, `take_derivative`/`get_gradients`):
 * run r inserts the generator op gens[r] (a PQC_OP_PAULI / PQC_OP_FSIM_D* /
 * PQC_OP_FIXED_FSIM_DTHETA op; host array) right after forward op
 * gen_after[r] (-1: before the first op), exactly as the reference replaces
 * gate g by `deriv * g` and re-runs the circuit.  Output row
 * gens[r].sel receives the SUM of the runs that name it (a generator that is
 * a sum of Pauli terms, measure/gates.py:451-457, is one run per term).
 * theta: one parameter row (device).  dpsi: complex128 [n_rows, 2^n]. */
size_t pqc_derivative_states_workspace_size(const pqc_program* prog, int32_t n_runs, int32_t n_rows);
int pqc_derivative_states(const pqc_program* prog, const double* theta, const void* psi0, int64_t psi0_index,
                          const pqc_op* gens, const int32_t* gen_after, int32_t n_runs, int32_t n_rows,
                          const int32_t* row_limit, void* dpsi, void* workspace, size_t workspace_bytes,
                          void* stream);  /* row_limit: device int32 [n_runs] or NULL (see pqc_run_limited) */

/* Layer checkpointing for the derivative states of pqc_derivative_states: run r
 * starts from the stored state psi0_rows[run_psi0[r]] (complex128 [K, 2^N],
 * device), which must equal the circuit's first run_start[r] ops applied to
 * the initial state, and applies only the ops from index run_start[r] on
 * (its generator must sit after an op >= run_start[r] - 1).  The runs skip the
 * arithmetic of their prefix and every middle sweep that holds only prefix
 * ops.  run_psi0 / run_start: device int32 [n_runs].  Same workspace as
 * pqc_derivative_states.  No counterpart in the reference (it re-runs every
 * derivative circuit from the start, circuit.py:149-192). */
int pqc_derivative_states_from(const pqc_program* prog, const double* theta, const void* psi0_rows,
                               const int32_t* run_psi0, const int32_t* run_start, const pqc_op* gens,
                               const int32_t* gen_after, int32_t n_runs, int32_t n_rows, void* dpsi, void* workspace,
                               size_t workspace_bytes, void* stream);

/* Adjoint energy gradient: E_b = <psi_b|H|psi_b> and
 * grad[b, j] = 2 Re <psi_b|H|d_j psi_b> (measure.py:461-471) for j < n_cols,
 * with the derivative of column j given by the generator ops whose `sel` is
 * j (host arrays gens/gen_after as above).  psi is uncomputed with U^dagger
 * of every op instead of re-running the circuit per parameter
 * (circuit.py:174-192).  terms: DEVICE array of n_terms Pauli terms.
 * When every generator is a PQC_OP_PAULI term the reverse pass runs as
 * double-float sweeps over psi and H psi together; otherwise one FP64 kernel
 * per op.  row_limit: device int32 [batch] or NULL; row b then evaluates only
 * the ops with index < row_limit[b] and the generators placed after them
 * (Pauli generators only). */
size_t pqc_energy_grad_workspace_size(const pqc_program* prog, int64_t batch, int32_t n_gens, int32_t n_cols);
int pqc_energy_grad(const pqc_program* prog, const double* theta, int64_t theta_stride, int64_t batch,
                    const void* psi0, int64_t psi0_index, const pqc_pauli_term* terms, int32_t n_terms,
                    const pqc_op* gens, const int32_t* gen_after, int32_t n_gens, int32_t n_cols, double* E,
                    double* grad, const int32_t* row_limit, void* workspace, size_t workspace_bytes,
                    void* stream);

/* Cross Gram G[a][b] = <a_a|b_b> (complex128 [na, nb]) of two state sets,
 * double-float accumulation.  The building block of the blocked QFIM, whose
 * entries 4 Re(<d_p|d_q> - <d_p|psi><psi|d_q>) (measure.py:33-71) are then
 * assembled block by block when P derivative states do not fit in HBM. */
size_t pqc_gram_cross_workspace_size(int64_t na, int64_t nb, int32_t n_qubits);
int pqc_gram_cross(const void* a, int64_t na, const void* b, int64_t nb, int32_t n_qubits, void* G, void* workspace,
                   size_t workspace_bytes, void* stream);

/* Plain baselines: one FP64 kernel per op (no sweeps, no double-float).
 * pqc_energy_grad_plain takes the arguments of pqc_energy_grad without row_limit
 * and always runs the op-by-op path; pqc_derivative_states_plain computes run r
 * (gens[r].sel must equal r) into dpsi[r] op by op with a workspace of
 * pqc_derivative_states_plain_workspace_size bytes.  They replace the same
 * reference calls as their fused counterparts and exist for comparison. */
int pqc_energy_grad_plain(const pqc_program* prog, const double* theta, int64_t theta_stride, int64_t batch,
                          const void* psi0, int64_t psi0_index, const pqc_pauli_term* terms, int32_t n_terms,
                          const pqc_op* gens, const int32_t* gen_after, int32_t n_gens, int32_t n_cols, double* E,
                          double* grad, void* workspace, size_t workspace_bytes, void* stream);
size_t pqc_derivative_states_plain_workspace_size(const pqc_program* prog, int32_t n_runs);
int pqc_derivative_states_plain(const pqc_program* prog, const double* theta, const void* psi0, int64_t psi0_index,
                                const pqc_op* gens, const int32_t* gen_after, int32_t n_runs, void* dpsi,
                                void* workspace, size_t workspace_bytes, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* PYRAMATERISED_GB300_H */
