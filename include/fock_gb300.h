/*
 * fock_gb300.h -- C ABI of the GB300 Fock-basis circuit simulator.
 *
 * Plain C: device pointers are `void*` / `double*` into GPU memory, host
 * pointers are marked "host", streams are `cudaStream_t` passed as `void*`
 * (NULL = legacy default stream).  Every entry point returns FOCK_OK (0) or a
 * negative status; `fock_last_error` returns the message of the last failure
 * on the calling thread.  No entry point allocates device memory: callers pass
 * every state buffer and workspace (sizes from the *_bytes queries).
 *
 * States (layout of strawberryfields/backends/fockbackend/backend.py:50-56):
 * a pure n-mode state is a C-order tensor [D]^n (mode 0 slowest); a mixed
 * state is [D]^(2n) with interleaved (ket, bra) axes.  dtype FOCK_C64 stores
 * interleaved float pairs (complex64), FOCK_C128 double pairs (complex128).
 * Gate matrices are always built on the device in FP64.
 *
 * Each entry point cites the reference interface it replaces (paths relative
 * to the Strawberry Fields source tree).
 */
#ifndef FOCK_GB300_H
#define FOCK_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define FOCK_OK 0
#define FOCK_ERR_INVALID (-1)     /* bad argument (Python: ValueError) */
#define FOCK_ERR_CUDA (-2)        /* CUDA runtime error */
#define FOCK_ERR_UNSUPPORTED (-3) /* valid request this build does not implement (NotImplementedError) */

/* state precision */
#define FOCK_C64 0
#define FOCK_C128 1

/* gate kinds (names follow strawberryfields/backends/base.py) */
#define FOCK_ROTATION 1          /* R(phi) = exp(i phi n)            base.py:301  */
#define FOCK_KERR 2              /* K(kappa) = exp(i kappa n^2)       base.py:583  */
#define FOCK_DISPLACEMENT 3      /* D(r e^{i phi})                    base.py:310  */
#define FOCK_SQUEEZE 4           /* S(r e^{i phi})                    base.py:320  */
#define FOCK_BEAMSPLITTER 5      /* BS(theta, phi)                    base.py:330  */
#define FOCK_TWO_MODE_SQUEEZE 6  /* S2(r e^{i phi})                   base.py:602  */
#define FOCK_MZGATE 7            /* MZ(phi_in, phi_ex)                base.py:341  */
#define FOCK_CROSS_KERR 8        /* CK(kappa) = exp(i kappa n1 n2)    base.py:592  */
#define FOCK_LOSS 9              /* loss channel N(T) (mixed states)  base.py:352  */

/* One gate of a circuit.  Parameters live in a device array `params`;
 * p0 = params[pidx], p1 = params[pidx + 1] (two-parameter gates). */
typedef struct fock_gate {
  int32_t kind;
  int32_t mode1;
  int32_t mode2; /* -1 for single-mode gates */
  int32_t pidx;
} fock_gate;

/* ---------------------------------------------------------------- errors */
int fock_last_error(char* buf, size_t len);
int fock_version(void);

/* ------------------------------------------------------- gate matrices (G1-G5)
 * Number of complex entries of the matrix `fock_gate_matrix` writes:
 * D*D for single-mode kinds, D(2D^2+1)/3 (photon-number blocks) for two-mode
 * kinds, 0 for unknown kinds.  Replaces the builders of
 * strawberryfields/backends/fockbackend/ops.py: displacement :219,
 * squeezing :238, two_mode_squeeze :257, kerr :274, cross_kerr :284,
 * phase :309, beamsplitter :318, mzgate :332, lossChannel :471. */
int64_t fock_gate_matrix_entries(int kind, int cutoff);
/* Device workspace (bytes) the builder needs for one gate. */
int64_t fock_gate_workspace_bytes(int kind, int cutoff);
/* Build one gate matrix in FP64 on the device: `out` (device, complex128,
 * fock_gate_matrix_entries entries) and, when `dout` is non-NULL, the
 * derivative with respect to p0 (r or theta).  Single-mode kinds are
 * row-major [out][in]; two-mode kinds are stored as photon-number blocks
 * (see fock_expand_blocks).  Loss stores the superoperator on a (ket, bra)
 * axis pair in difference-conserving blocks. */
int fock_gate_matrix(int kind, double p0, double p1, int cutoff, void* out, void* dout,
                     void* workspace, void* stream);
/* Expand block storage to a dense [out1][in1][out2][in2] tensor of D^4
 * complex128 entries (the index order of fockbackend/ops.py:329). */
int fock_expand_blocks(int kind, int cutoff, const void* blocks, void* dense, void* stream);

/* ------------------------------------------------------- state updates (K1-K6)
 * Apply one gate to `in`, writing `out` (in != out).  Mixed states need
 * `tmp` (a third state-sized buffer; NULL for pure states).
 * `workspace`: fock_gate_workspace_bytes(kind, cutoff) bytes.
 * `pre` (host, 4 doubles {theta1, kappa1, theta2, kappa2}, or NULL) are
 * rotation angles and Kerr strengths applied to mode1/mode2 BEFORE the gate,
 * i.e. exp(i (theta n + kappa n^2)): pending rotation/Kerr gates are folded
 * into the next gate on the same mode this way.  Rotation, Kerr and
 * cross-Kerr kinds run as one diagonal phase pass.
 * Replaces Circuit.apply_gate_BLAS (fockbackend/circuit.py:118),
 * apply_twomode_gate (:219), _apply_two_mode_passive (:307), _apply_S2 (:338)
 * and _apply_channel for the loss channel (:65). */
int fock_apply_gate(int kind, double p0, double p1, int mode1, int mode2,
                    int num_modes, int cutoff, int pure, int dtype, const double* pre,
                    const void* in, void* out, void* tmp, void* workspace, void* stream);
/* Apply a caller-built single-mode matrix (device, complex128, D*D row-major)
 * to one mode (e.g. cubic phase, fockbackend/circuit.py:590). */
int fock_apply_matrix1(const void* mat, int mode, int num_modes, int cutoff, int pure, int dtype,
                       const void* in, void* out, void* tmp, void* stream);
/* Fock matrix of an m-mode Gaussian unitary (m = 1..3) from its Choi
 * parameters -- the TF backend's Ggate (strawberryfields/backends/tfbackend/
 * ops.py:457-572: choi_trick, then the renormalised multidimensional Hermite
 * polynomials of the third-party thewalrus).  R: 2m x 2m complex, y: 2m
 * complex, C: one complex, all host arrays of (re, im) doubles; mat: device
 * complex128 [D]^(2m) in C order over (out_1..out_m, in_1..in_m), i.e. the
 * D^m x D^m matrix from input to output multi-index.  FP64. */
int fock_gaussian_gate_matrix(int num_gate_modes, int cutoff, const double* R, const double* y,
                              const double* C, void* mat, void* stream);
/* Apply a dense D^k x D^k matrix (device complex128, rows the output
 * multi-index over modes[0..k-1] in C order) to k modes (any order, any
 * positions): n_mode_gate of tfbackend/ops.py.  Mixed states: M on the ket
 * axes, conj(M) on the bra axes (tmp: a state-sized buffer).  workspace:
 * fock_apply_modes_workspace_bytes(k, cutoff, dtype); at most 4096
 * amplitudes per column (D^k). */
int64_t fock_apply_modes_workspace_bytes(int k, int cutoff, int dtype);
int fock_apply_modes(int num_modes, int cutoff, int pure, int dtype, int k, const int* modes, const void* mat,
                     const void* in, void* out, void* tmp, void* workspace, void* stream);
/* Diagonal phases: multiply every amplitude by
 * exp(i (sum_m angles[m*D + n_m] + sum_k ck_kappa[k] n_{a_k} n_{b_k}))
 * (bra side conjugated for mixed states).  `angles` device (num_modes*D) or
 * NULL; ck_modes/ck_kappa host arrays of n_ck <= 32 pairs.  Rotation,
 * Kerr and cross-Kerr of fockbackend/circuit.py:155-177 (diagonal path). */
int fock_apply_phases(int num_modes, int cutoff, int pure, int dtype, const double* angles,
                      int n_ck, const int* ck_modes, const double* ck_kappa,
                      const void* in, void* out, void* stream);
/* rho = |psi><psi| with interleaved axes (fockbackend/ops.py:110 mix). */
int fock_mix(int num_modes, int cutoff, int dtype, const void* ket, void* dm, void* stream);
/* Vacuum state (fockbackend/ops.py:363,373). */
int fock_vacuum(int num_modes, int cutoff, int pure, int dtype, void* state, void* stream);
/* Replace the modes in `modes` (host, n_sub entries, any order) of a mixed
 * state by the mixed state `sub` (device, complex128 [D]^(2 n_sub),
 * interleaved): out = tr_modes(in) (x) sub, re-ordered so sub's k-th mode
 * lands on modes[k] (fockbackend/circuit.py:393 prepare_multimode). */
int fock_prepare_modes(int num_modes, int cutoff, int dtype, int n_sub, const int* modes,
                       const void* sub, const void* in, void* out, void* workspace, void* stream);
int64_t fock_prepare_workspace_bytes(int num_modes, int cutoff, int dtype, int n_sub);
/* out = in (x) |0...0> with `n_new` vacuum modes appended after the
 * `num_modes` modes of `in` (pure: [D]^(num_modes + n_new); mixed:
 * interleaved [D]^(2 (num_modes + n_new))); Circuit.alloc,
 * fockbackend/circuit.py:373-382 (BaseBackend.add_mode, base.py:175). */
int fock_append_vacuum(int num_modes, int n_new, int cutoff, int pure, int dtype, const void* in, void* out,
                       void* stream);
/* out = Tr_modes(rho) for a mixed state: the `n_traced` modes listed in
 * `modes` (host, distinct, fewer than num_modes) are traced out, the others
 * keep their order with interleaved axes; FP64 sums.  Circuit.dealloc via
 * ops.partial_trace, fockbackend/circuit.py:384-391 and ops.py:144
 * (BaseBackend.del_mode, base.py:186). */
int fock_partial_trace(int num_modes, int cutoff, int dtype, int n_traced, const int* modes, const void* rho,
                       void* out, void* stream);

/* ------------------------------------------------------------ readouts (R1-R3)
 * probs: |psi|^2 (pure) or diag(rho) (mixed), D^n doubles
 * (states.py:580 all_fock_probs). */
int fock_probs(int num_modes, int cutoff, int pure, int dtype, const void* state, double* probs,
               void* stream);
/* Photon-number distribution of every mode: out[m*D + k] = P(n_m = k), from
 * one pass over the state (states.py:657 mean_photon without forming the full
 * density matrix).  `workspace`: fock_marginals_workspace_bytes bytes. */
int fock_marginals(int num_modes, int cutoff, int pure, int dtype, const void* state,
                   double* out, void* workspace, void* stream);
int64_t fock_marginals_workspace_bytes(int num_modes, int cutoff, int pure, int dtype);
/* Single-mode reduced density matrix (complex128 D*D) of `mode`
 * (states.py:613 reduced_dm, fockbackend/backend.py:209 state(modes)). */
int fock_reduced_dm1(int num_modes, int cutoff, int pure, int dtype, int mode, const void* state,
                     void* out, void* workspace, void* stream);
int64_t fock_reduced_dm1_workspace_bytes(int num_modes, int cutoff, int pure, int dtype);

/* Same result as fock_reduced_dm1, for callers that cannot allocate device
 * memory (no workspace argument).  No counterpart in the reference.  The
 * reduction's partial sums live in a fixed 512 KiB array in device global
 * memory owned by the library (held by every GPU that loads it until exit),
 * which bounds the cutoff to <= FOCK_NOALLOC_MAX_CUTOFF; larger cutoffs are
 * rejected with FOCK_ERR_INVALID.  Each call outside stream capture looks up
 * that array's device address (cudaGetSymbolAddress) with the device current;
 * a call made while `stream` is capturing uses the address found by the last
 * uncaptured call on the device, so make one call before any stream capture
 * (and again after a cudaDeviceReset before capturing).  All calls share the
 * array, so calls that overlap on the GPU (different streams, or concurrent
 * host threads) race; serialise them.  Allocates nothing: no
 * cudaMalloc/cudaFree. */
#define FOCK_NOALLOC_MAX_CUTOFF 60
int fock_reduced_dm1_noalloc(int num_modes, int cutoff, int pure, int dtype, int mode, const void* state,
                             void* out, void* stream);

/* ---------------------------------------------- compiled circuits + adjoint (A1-A3)
 * A plan is a gate list compiled on the host: rotation/Kerr/cross-Kerr gates
 * are fused into the neighbouring non-diagonal gate, so the state crosses HBM
 * once per remaining op.  pure = 0 compiles for density matrices [D]^(2n)
 * with interleaved (ket, bra) axes: every unitary op is applied as M on its
 * ket axes and conj(M) on its bra axes (one matrix build, two ops), and
 * FOCK_LOSS gates (parameter T) become the loss superoperator on the mode's
 * (ket, bra) pair -- fockbackend/circuit.py:186-217 and :65-87; phases next
 * to a loss are carried by it (+p on the ket, -p on the bra).  A plan's ops
 * (fock_plan_op) are these applications.
 * Forward: op k maps the previous state to its output; `store_every` = k
 * decides which outputs are kept in `states` (slots of batch * D^n entries):
 * 0 -> two ping-pong slots (final state in slot (n_ops-1) & 1); 1 -> every
 * output (slot j, n_ops slots); k > 1 -> checkpoints: the output of op j goes
 * to slot (j+1)/k - 1 when (j+1) % k == 0, the last op's output to slot
 * ceil(n_ops/k) - 1, the rest through two scratch slots after them
 * (ceil(n_ops/k) + 2 slots).
 * Backward: the adjoint sweep of the gradient contract of
 * strawberryfields/backends/tfbackend/ops.py:190-454 (custom gradients) and
 * :688-854 (state contractions): given grad_state = dL/dpsi of the final state
 * (torch convention dL/dRe + i dL/dIm), write dL/dparams and leave dL/dpsi_in
 * in grad_state.  With store_every = k > 1 each segment of k ops is first
 * recomputed from its checkpoint into `seg` (k - 1 slots), so memory is
 * ceil(n_ops/k) + k + 1 states instead of n_ops. */
typedef struct fock_plan fock_plan;
typedef struct fock_plan_info {
  int32_t n_ops;            /* fused ops */
  int32_t n_gates;          /* gates in the list */
  int64_t state_elems;      /* complex entries per state */
  int64_t state_bytes;
  int64_t workspace_bytes;  /* for forward and backward */
  int64_t flops_fwd;        /* real flops of one forward */
  int64_t bytes_fwd;        /* algorithmic HBM bytes of one forward (2 S per op, whole batch) */
  int32_t batch;            /* circuits per call */
} fock_plan_info;

int fock_plan_create(int num_modes, int cutoff, int pure, int dtype, const fock_gate* gates,
                     int n_gates, int n_params, fock_plan** out);
/* A batch of `batch` circuits with this gate list, each with its own
 * parameters -- the batch axis of the reference's TF backend
 * (tfbackend/circuit.py:129-185).  params: [batch][n_params]; state_in:
 * [batch][D^n]; states: [n_ops or 2][batch][D^n]; gradients likewise. */
int fock_plan_create_batch(int num_modes, int cutoff, int pure, int dtype, const fock_gate* gates,
                           int n_gates, int n_params, int batch, fock_plan** out);
void fock_plan_destroy(fock_plan* plan);
int fock_plan_get_info(const fock_plan* plan, fock_plan_info* info);
/* Fused op k: kind code (1 dense single-mode, 2 number-sum block, 3
 * number-difference block), modes, number of gates fused into it. */
int fock_plan_op(const fock_plan* plan, int k, int* kind, int* mode1, int* mode2, int* n_fused);
/* Fused tile group of op k: its index (-1 when the op runs on its own), the
 * group's first op and its number of ops.  A complex64 pure-state plan with
 * cutoff <= 16 and enough columns groups consecutive ops whose modes lie in
 * one set of three modes; each group runs as one launch over tiles held in
 * shared memory, when FOCK_GB300_TILE_GROUPS=1 at plan creation (off by
 * default: measured slower than per-op launches on GB300).
 * Ops are reordered only where they commute (no shared mode), so every
 * mode's ops keep their order.  No reference counterpart (the reference
 * applies every gate as its own pass over the state). */
int fock_plan_op_group(const fock_plan* plan, int k, int* group, int* first, int* count);
int fock_plan_forward(fock_plan* plan, const double* params, const void* state_in, void* states,
                      int store_every, void* workspace, void* stream);
int fock_plan_backward(fock_plan* plan, const double* params, const void* state_in,
                       const void* states, int store_every, void* seg, void* grad_state, void* grad_tmp,
                       double* grad_params, void* workspace, void* stream);
/* As fock_plan_backward, with `seg` holding only `seg_slots` states (at least
 * 3 when seg_slots < store_every - 1): each checkpoint segment is then
 * recomputed recursively -- chunk boundaries into seg slots through two
 * scratch slots, every chunk processed the same way, last chunk first -- so
 * the adjoint of a long segment (a density matrix of many GB between
 * checkpoints) runs in bounded memory at the cost of extra forward passes. */
#define FOCK_BACKWARD_REUSE_BUILD 1 /* flags: `workspace` holds the matrices (and derivatives)
                                     built by the last forward sweep with these `params`; skip the
                                     rebuild */
int fock_plan_backward_recompute(fock_plan* plan, const double* params, const void* state_in,
                                 const void* states, int store_every, void* seg, int seg_slots,
                                 void* grad_state, void* grad_tmp, double* grad_params, int flags,
                                 void* workspace, void* stream);

/* Per-op device timing of plan sweeps (CUDA events recorded between the op
 * launches on the sweep's stream).  After enabling, every forward/backward
 * call records; fock_plan_op_times reads the last sweep of each direction
 * (milliseconds per op, op order) once the stream has completed. */
int fock_plan_enable_timing(fock_plan* plan, int enable);
int fock_plan_op_times(fock_plan* plan, float* fwd_ms, float* bwd_ms);

/* Wigner function of one mode on a grid: BaseFockState.wigner
 * (strawberryfields/backends/states.py:730-785).  rho: the mode's D x D
 * reduced density matrix, complex128 on the device (fock_reduced_dm1);
 * xvec[nx], pvec[np]: device float64 grids; out: device float64 [np][nx],
 * out[i][j] = W(xvec[j], pvec[i]) (the reference's meshgrid order), for the
 * quadratures x = sqrt(hbar/2)(a + a^dagger).  FP64 throughout. */
int fock_wigner(int cutoff, const void* rho, const double* xvec, int nx, const double* pvec, int np,
                double hbar, double* out, void* stream);

/* Per-op kernel selection, the knobs of the autotuner
 * (CompiledCircuit.autotune times each candidate with fock_plan_op_times and
 * keeps the fastest per op).  family: 0 block kernels (one column per
 * thread), 1 plane-tile kernels (two-mode ops whose plane geometry exists:
 * `plane_ok`), -1 unchanged; adj_ctas_per_sm: CTAs per SM of the block
 * adjoint launch (1..64; 0 unchanged; default 8); plane_tile_columns:
 * columns per plane tile of a two-mode op (8..32; 0 unchanged; default 32;
 * op_config reports the dense ops' fixed tile).  Changes the partial-sum
 * layout and so workspace_bytes (read fock_plan_get_info again and
 * reallocate the workspace) and any captured graph of the plan.  Call with no
 * sweep of the plan in flight.  No reference counterpart (the reference has
 * one einsum per gate, tfbackend/ops.py:688-854). */
int fock_plan_tune(fock_plan* plan, int op, int family, int adj_ctas_per_sm, int plane_tile_columns);
int fock_plan_op_config(const fock_plan* plan, int op, int* family, int* adj_ctas_per_sm, int* plane_ok,
                        int* plane_tile_columns);

/* Persistent sweeps.  A single-circuit complex64 plan whose state is at most
 * FOCK_GB300_SWEEP_MAX_BYTES bytes (read at plan creation; default 0 = off,
 * since per-op launches measured faster on GB300) runs a forward
 * sweep with store_every 0 or 1, and a backward sweep with store_every 1, as
 * one cooperative launch that walks every op with a grid barrier between ops
 * (no per-op launch).  Per-op timing and checkpointed sweeps use the per-op
 * launches.  `grids` (2 ints, or null) receives the CTAs of the persistent
 * forward and backward launches (0 when the plan uses per-op launches); `error` is
 * nonzero when a grid barrier of the last persistent sweep on `workspace`
 * gave up waiting (the outputs are then invalid).  A barrier gives up after
 * FOCK_GB300_SWEEP_SPIN_LIMIT polls of its generation word (read at plan
 * creation; default 2^24, about a second); the launch then returns.
 * Synchronous: call after the sweep's stream has been synchronised.  No reference counterpart (the
 * reference applies one gate per Python call, fockbackend/circuit.py). */
int fock_plan_sweep_status(const fock_plan* plan, const void* workspace, int* grids, int* error);

#ifdef __cplusplus
}
#endif
#endif /* FOCK_GB300_H */
