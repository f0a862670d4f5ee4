// Internal structures shared by the engine's translation units.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/pyramaterised_gb300.h"

namespace pqc {

constexpr int kMaxQubits = 34;  // 2^34 c128 = 256 GiB: the HBM limit of one GB300

// Internal op kinds after host-side classification of pqc_op.
enum DKind : int32_t {
  K_REAL2 = 1,  // real 2x2 [[a,b],[c,d]]           (RY, fixed RY, H)
  K_RX = 2,     // [[c,-is],[-is,c]]
  K_DIAG1 = 3,  // diag(p0, p1)                      (RZ, S, T, fixed RZ)
  K_GEN1 = 4,   // general complex 2x2
  K_CNOT = 5,
  K_CZ = 6,
  K_RZZ = 7,    // phase e^{-i a/2} on even parity, e^{+i a/2} on odd
  K_RXX = 8,    // c x_j - i s x_{j^m}
  K_RYY = 9,    // c x_j + i s sigma_j x_{j^m}
  K_MIX2 = 10,  // (01,10) block [[c,-is],[-is,c]], |11> times p11  (fSim family, sqrtiSWAP)
  K_GEN2 = 11,  // general complex 4x4
  K_PAULI = 12, // coef * Pauli string on <= 2 positions
  K_X = 13,     // swap pair (X gate)
  K_RY = 14,    // [[c,-s],[s,c]]
  K_RZ = 15,    // diag(c - is, c + is)
  K_PHASEBLK = 16,  // marker: the next `aux` ops are diagonal; apply them as one phase-table pass.  The
                    // members are ordered tile-constant | low half | high half | both halves of the local
                    // bits, with the four counts in the marker's c0, c1, r0, r1 and the low half's bit
                    // count in its q0
  K_MEASURE = 17,   // adjoint: accumulate <lambda|coef P|psi> over the tile (Pauli letters in aux)
  K_ROT2 = 18,      // marker: the next 2 ops are real/RX rotations on two different local bits; apply
                    // both in one pass over amplitude quads
  K_MEASZ = 19,     // adjoint marker: the next `aux` (<= 4) ops are Z-type measures, reduced in one pass
  K_MEASG = 20,     // adjoint marker: the next `aux` (<= 4) ops are measures of any Pauli type, one pass
  K_OFFSET = 21     // relabelled sweeps: XOR c0 into the tile's index offset (aux 1: only when the fixed bit at
                    // position p0 is set) -- an X, or a CNOT whose control is not in the tile
};

// One op as the kernels see it.
struct DOp {
  int32_t kind;
  int32_t sel;   // -1 all rows; else only batch row `sel`
  int32_t p0;    // global bit position of the first qubit (q0)
  int32_t p1;    // global bit position of the second qubit (-1 if none)
  int32_t slot;  // >= 0: per-row coefficient slot; < 0: constant table offset -(slot+1) (in doubles)
  int32_t aux;   // K_PAULI: letters(q0) | letters(q1) << 8
  int32_t gidx;  // position in the caller's op list (rows with row_limit <= gidx skip the op)
  // Relabelled sweeps (SweepDesc::lazy): the CNOTs of the sweep are not applied to the data; the tile
  // keeps logical index l at physical slot A l ^ b (A linear over GF(2), b a per-tile offset), and each
  // op carries the masks of its logical bits under the A in force where it runs:
  int16_t c0 = 0, c1 = 0;  // physical masks A e_j of the op's local bits j0, j1
  int16_t r0 = 0, r1 = 0;  // parity masks: logical bit j of physical slot p is parity((p ^ b) & r_j)
  int8_t q0 = 0, q1 = 0;   // pivot bits enumerating the op's pairs (q0) or quads (q0, q1)
  int16_t pad2 = 0;
};

// A row coefficient slot: 4 doubles (c, s, x, y) computed from theta by the
// coefficient kernel for each param op.
struct RowCoefSpec {
  int32_t kind;  // pqc_op_kind of the source op
  int32_t param, param2;
  int32_t pad;
  double scale, offset, scale2, offset2;
};

constexpr int kMaxSweepOps = 768;

// The sweep kernels stage a sweep's ops in shared memory kOpChunk at a time, each with the first four
// coefficients of its row (GEN1/GEN2 read the rest from global memory); the planner keeps every fused block
// (a marker and its members) within kOpChunk ops, so a block is always staged whole.
constexpr int kOpChunk = 64;

// One shared-memory sweep (one HBM pass).
struct SweepDesc {
  int32_t k;          // tile qubits (active bits)
  int32_t c;          // contiguous low positions 0..c-1 (all active)
  int32_t op_begin;   // into the program's DOp array
  int32_t n_ops;
  int64_t offs_begin; // into the offset table: 2^(k-c) int64 offsets of the high local bits
  int32_t n_free;     // number of non-active positions
  int8_t free_pos[kMaxQubits];  // non-active positions, ascending
  int8_t local_of[kMaxQubits];  // position -> local bit, -1 when not active
  int32_t first, last;          // first / last sweep of the plan
  int32_t max_gidx;             // largest op index among the sweep's ops (finalize_plan)
  int32_t lazy;                 // 1: CNOTs relabel the tile instead of moving data (see DOp::c0)
  int32_t out_rec;              // lazy: record of the final A (columns) in Plan::lazy_cols, for the write-out
  // smallest / largest index of the sweep's ops that every row applies (sel < 0), counting the CNOTs that a
  // relabelled sweep folds into its index map; INT32_MAX / -1 when it has none.  A row whose start is at most
  // min_fwd and whose limit is above max_fwd applies all of them, and may take a relabelled twin of the sweep.
  int32_t min_fwd, max_fwd;
};

// Relabelled sweeps keep 16-entry records of column masks (uint16) in Plan::lazy_cols.
constexpr int kLazyRec = 16;

// Per-row controls of a sweep launch (device arrays indexed by row, each may be NULL):
//   limit:    row applies only ops with index < limit[row] (generators: placed after an op < limit)
//   start:    row applies only ops with index >= start[row] (generators: placed after an op >= start - 1),
//             starting from a stored state that already holds the ops before start
//   psi0_row: row starts from psi0 + psi0_row[row] * 2^N instead of the one broadcast psi0
struct RowCtl {
  const int32_t* limit = nullptr;
  const int32_t* start = nullptr;
  const int32_t* psi0_row = nullptr;
};

struct Plan {
  std::vector<SweepDesc> sweeps;
  std::vector<DOp> ops;             // ops in sweep order
  std::vector<int64_t> offs;        // concatenated offset tables
  DOp* d_ops = nullptr;
  int64_t* d_offs = nullptr;
  std::vector<uint16_t> lazy_cols;  // records of kLazyRec column masks (relabelled sweeps)
  uint16_t* d_lazy_cols = nullptr;
  SweepDesc* d_sweeps = nullptr;    // device copy of `sweeps`
};

// Lowered ops with their coefficient sources, on host and device.
struct OpTable {
  std::vector<DOp> dops;              // program order
  std::vector<RowCoefSpec> specs;     // per-row coefficient slots
  std::vector<double> consts;         // constant coefficients (doubles)
  RowCoefSpec* d_specs = nullptr;
  double* d_consts = nullptr;
  DOp* d_dops = nullptr;
};

}  // namespace pqc

struct pqc_program {
  int32_t n_qubits = 0;
  int32_t n_params = 0;
  int32_t tile_qubits = 0;
  int32_t ctas_per_sm = 0;    // sweep kernels below 2^13-amplitude tiles: 3 (default) or 2 resident CTAs per SM
  int32_t sweep_threads = 0;  // with 3 CTAs per SM: 128 or 256 threads per CTA (0: by grid size)
  std::vector<pqc_op> ops;  // the forward ops as given
  std::vector<int32_t> fused_interior;  // op limits that would cut a fused CNOT-RZ-CNOT triple (sorted)
  pqc::OpTable fwd_t;       // lowered forward ops
  pqc::Plan fwd;            // forward sweep plan (CNOTs relabel the tile where possible)
  pqc::Plan fwd_lim;        // the same without relabelled sweeps: the twin that rows with op limits or starts
                            // take for the sweeps they cut (alone outside the double-float dual kernels)
  bool fwd_lazy = false;    // fwd holds relabelled sweeps (else fwd_lim is not built)
  // derivative-run cache (keyed by the generator list)
  std::vector<pqc_op> d_gens;
  std::vector<int32_t> d_after;
  pqc::OpTable deriv_t;     // forward ops followed by the generators
  pqc::Plan deriv_plan;     // generator-inserted sweep plan
  pqc::Plan deriv_lazy;     // its twin with relabelled sweeps, for the rows that apply every op of a sweep
  bool deriv_lazy_ok = false;  // deriv_lazy holds a relabelled sweep (else it is empty)
  pqc::OpTable gen_t;       // the generators alone (adjoint)
  int32_t* d_run_row = nullptr;  // [n_gens] output row of each derivative run (gens[r].sel)
  int32_t* d_status = nullptr;   // device word: PQC_STATUS_* bits raised by the kernels (pqc_program_status)
  bool deriv_valid = false;
  // adjoint-gradient cache (keyed by the generator list): the inverse program
  // in reverse order with K_MEASURE ops at the generator points
  std::vector<pqc_op> adj_gens;
  std::vector<int32_t> adj_after;
  int32_t adj_ncols = 0;
  pqc::OpTable adj_t;
  pqc::Plan adj_plan;      // relabelled where possible
  pqc::Plan adj_plan_lim;  // without relabelling: runs with per-row op limits (empty when adj_plan has none)
  bool adj_lazy = false;
  int32_t* d_adj_cols = nullptr;   // measure indices grouped by gradient column
  int32_t* d_adj_start = nullptr;  // [n_cols + 1] offsets into d_adj_cols
  bool adj_valid = false;
  int device = -1;
};

namespace pqc {

// number of kernels this library has launched (monotonic; read by pqc_launch_count)
void count_launch();

// thread-local last error
void set_error(const std::string& msg);
int fail(int code, const std::string& msg);
int cuda_fail(cudaError_t e, const char* what);

#define PQC_CUDA(call)                                 \
  do {                                                 \
    cudaError_t _e = (call);                           \
    if (_e != cudaSuccess) return cuda_fail(_e, #call); \
  } while (0)

// program.cu
int lower_ops(const pqc_op* ops, int n_ops, int n_qubits, OpTable& t);
int upload_table(OpTable& t);
void free_table(OpTable& t);
int build_plan(const std::vector<DOp>& dops, int n_qubits, int k, int cmin, Plan& plan);
int upload_plan(Plan& plan);
void fuse_diagonal_runs(Plan& plan);
void fuse_rotation_pairs(Plan& plan);
// after fuse_diagonal_runs, before fuse_rotation_pairs; measures: the plan may hold adjoint measures
void relabel_cnots(Plan& plan, bool measures = false, bool gens = false);
void copy_sweep_ranges(Plan& lazy, const Plan& plain);
void finalize_plan(Plan& plan);  // per-sweep max op index; call after the fusion passes
void free_plan(Plan& plan);
int ensure_deriv(pqc_program* prog, const pqc_op* gens, const int32_t* after, int n_gens);
// coef[row * n_slots + slot] (4 doubles each) from theta rows
int launch_row_coefs(const OpTable& t, const double* theta, int64_t theta_stride, int64_t rows, double* coef,
                     cudaStream_t stream);
int launch_to_df(const double* in, float2* out, int64_t n, cudaStream_t stream);

// sweep.cu: run a plan.  coef_stride = slots per row of rowcoef (0 = shared row); twin: the unrelabelled twin
// of a relabelled plan (same sweeps), for rows whose start or limit falls inside a sweep
int run_plan_df(const pqc_program* prog, const Plan& plan, int coef_stride, const float2* rowcoef,
                const float2* consts, int64_t rows, const void* psi0, int64_t psi0_index, void* psi,
                cudaStream_t stream, const int32_t* row_limit = nullptr, const RowCtl* ctl = nullptr,
                const Plan* twin = nullptr);


// adjoint.cu: ψ and λ tiles of 2^kAdjTileQubits amplitudes each share one CTA's shared memory
// gram_tc.cu: the counts-only fidelity Gram on the tensor cores (S <= 256, n_qubits >= 13); G (double2
// [256][256], in ws) is within delta_factor ||a|| ||b|| per component; a CTA that timed out sets *fallback
bool gram_tc_usable(int64_t S, int n_qubits);
size_t gram_tc_ws(int64_t S, int n_qubits);
int launch_gram_tc(const double2* psi, int64_t S, int n_qubits, float* planes, void* ws, double2** G,
                   double* delta_factor, int* fallback, cudaStream_t stream);

constexpr int kAdjTileQubits = 11;
int ensure_adjoint(pqc_program* p, const pqc_op* gens, const int32_t* after, int n_gens, int n_cols);
void free_adjoint(pqc_program* p);
// tiles per row of every adjoint sweep
int64_t adjoint_tiles(const pqc_program* p);
int run_adjoint_sweeps(const pqc_program* prog, const float2* rowcoef, const float2* consts, int64_t rows, void* psi,
                       void* lam, const int32_t* row_limit, double* mpart, cudaStream_t stream);
int launch_adj_final(const pqc_program* prog, const double* mpart, int64_t rows, double* grad, cudaStream_t stream);

// program.cu: one program's share of a multi-program coefficient launch (pqc_run_multi): the FP64 coefficients
// of rows x n_slots slots of `specs` from theta into coef, then coef and the program's constants into
// double-float (coef_df, consts_df)
struct CoefJob {
  const RowCoefSpec* specs;
  int n_slots;
  int n_consts;
  const double* theta;
  int64_t theta_stride;
  int64_t rows;
  double* coef;
  float2* coef_df;
  const double* consts;
  float2* consts_df;
};
constexpr int kMultiMax = 64;  // programs per multi-program launch (their records travel as kernel parameters)
int launch_coefs_multi(const CoefJob* jobs, int n_jobs, cudaStream_t stream);

// sweep.cu: bytes of dynamic shared memory of a sweep launch; the forward plan of a run
size_t sweep_smem_bytes(const SweepDesc& sd, size_t amp_bytes);
const Plan& run_plan_for(const pqc_program* prog, bool row_controls);

// plain.cu
int launch_plain_op(const DOp& op, double2* psi, int n_qubits, int64_t rows, const double* rowcoef, int n_slots,
                    const double* consts, int inv, cudaStream_t stream, const int32_t* row_limit = nullptr);
int init_rows(double2* psi, const void* psi0, int64_t idx, int n_qubits, int64_t rows, cudaStream_t stream);

inline size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

}  // namespace pqc
