/*
 * pl_gb300.h — C ABI of the GB300 (sm_103a) state-vector backend.
 *
 * This is the drop-in boundary for lightning.qubit's hot path: the entry
 * points are what the reference's Python binding module
 * (`lightning_qubit_ops`, built from
 *  pennylane_lightning/core/bindings/Bindings.hpp and
 *  pennylane_lightning/core/simulators/lightning_qubit/bindings/LQubitBindings.hpp)
 * binds, flattened to plain pointers and sizes.  The reference paths cited
 * below are relative to the reference project root.
 *
 * Conventions
 *   - Every function returns PLGB_OK (0) or a non-zero status; the message of
 *     the last failure on the calling thread is returned by plgb_last_error().
 *     (Reference: PL_ABORT -> LightningException, core/utils/Error.hpp:23-65.)
 *   - precision is 64 (complex64, float pairs) or 128 (complex128).
 *   - Host state buffers are interleaved (re, im) arrays in the handle's
 *     precision; matrices, coefficients and parameters are passed as
 *     interleaved complex128 / double and converted to the handle's precision
 *     (as the reference's binding converts numpy arrays to PrecisionT).
 *   - Wire w is bit (n-1-w) of the amplitude index; within a k-wire matrix the
 *     first listed wire is the most significant bit of the local index.
 *   - Gate application is asynchronous on the state vector's CUDA stream;
 *     every call that returns data to the host synchronizes first.
 *   - There is no CPU fallback: when no CUDA device is present, creating a
 *     state vector fails with PLGB_ERR_CUDA.
 */
#ifndef PL_GB300_H
#define PL_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PLGB_OK 0
#define PLGB_ERR_INVALID 1    /* bad argument (wires, sizes, names) */
#define PLGB_ERR_CUDA 2       /* CUDA runtime failure or no device */
#define PLGB_ERR_UNSUPPORTED 3
#define PLGB_ERR_INTERNAL 4

typedef struct plgb_sv plgb_sv;   /* StateVectorLQubitManaged<T> counterpart */
typedef struct plgb_obs plgb_obs; /* Observable<SV> counterpart */
typedef struct plgb_ops plgb_ops; /* OpsData<SV> counterpart */

/* ---- module level (Bindings.hpp:284-367, LQubitBindings.hpp:464-475) ---- */
const char *plgb_last_error(void);
/* JSON text: {"NAME": "lightning.gb300", ...}; backend_info() */
int plgb_backend_info(char *buf, size_t len);
/* JSON text with CUDA device / compile details; compile_info(), runtime_info() */
int plgb_runtime_info(char *buf, size_t len);
int plgb_device_count(int *out);
/* number of kernels this library has launched in the process (monotonic) */
int plgb_kernel_launches(uint64_t *out);
/* number of device-memory requests this library has made in the process
 * (monotonic; every request, whether cudaMalloc or a reuse-pool hit): a
 * diagnostic with no counterpart in the reference */
int plgb_device_allocations(uint64_t *out);

/* ---- state vector (StateVectorLQubitManaged.hpp:52-188,
 *      StateVectorLQubit.hpp:359-1036, Bindings.hpp:870-922,
 *      LQubitBindings.hpp:178-243) ---- */
/* StateVectorC64/C128.__init__(num_qubits): |0...0> */
int plgb_sv_create(int num_qubits, int precision, plgb_sv **out);
/* StateVectorLQubitRaw counterpart: wraps caller-owned DEVICE memory of
 * 2^num_qubits amplitudes (not freed by plgb_sv_destroy) */
int plgb_sv_create_raw(void *device_data, int num_qubits, int precision, plgb_sv **out);
/* deep copy (StateVectorLQubitManaged copy constructor) */
int plgb_sv_clone(const plgb_sv *src, plgb_sv **out);
int plgb_sv_destroy(plgb_sv *sv);
int plgb_sv_num_qubits(const plgb_sv *sv, int *out);
int plgb_sv_precision(const plgb_sv *sv, int *out);
/* __len__ / size */
int plgb_sv_length(const plgb_sv *sv, uint64_t *out);
int plgb_sv_device_ptr(plgb_sv *sv, void **out);
int plgb_sv_synchronize(plgb_sv *sv);
/* the CUDA stream (cudaStream_t) the state vector's kernels run on, so a
 * caller can time them with CUDA events or order its own work after them */
int plgb_sv_stream(plgb_sv *sv, void **out);
/* resetStateVector (StateVectorLQubit.hpp:959-963) */
int plgb_sv_reset(plgb_sv *sv);
/* setBasisState(state, wires) (StateVectorLQubit.hpp:939-957) */
int plgb_sv_set_basis_state(plgb_sv *sv, const int64_t *bits, const int64_t *wires, int nw);
/* setStateVector(state, wires) (StateVectorLQubit.hpp:971-1036); len = 2^nw */
int plgb_sv_set_state_vector(plgb_sv *sv, const void *host_state, uint64_t len, const int64_t *wires, int nw);
/* updateData(ndarray) (LQubitBindings.hpp:183-196) */
int plgb_sv_update_data(plgb_sv *sv, const void *host_data, uint64_t len);
/* getState(out_ndarray) (LQubitBindings.hpp:227-243) */
int plgb_sv_get_state(const plgb_sv *sv, void *host_out, uint64_t len);
/* per-gate methods: st.<Name>(wires, inverse, params) (Bindings.hpp:223-234,
 * StateVectorLQubit.hpp:378-391) */
int plgb_sv_apply_operation(plgb_sv *sv, const char *name, const int64_t *wires, int nw, int inverse,
                            const double *params, int np);
/* controlled per-gate methods: st.<Name>(cwires, cvals, wires, inverse, params)
 * (Bindings.hpp:256-276, StateVectorLQubit.hpp:404-424) */
int plgb_sv_apply_controlled_operation(plgb_sv *sv, const char *name, const int64_t *cwires, const uint8_t *cvals,
                                       int ncw, const int64_t *wires, int nw, int inverse, const double *params,
                                       int np);
/* applyMatrix(matrix, wires, inverse) (Bindings.hpp:153-165,
 * StateVectorLQubit.hpp:674-710); matrix: 4^nw interleaved complex128 */
int plgb_sv_apply_matrix(plgb_sv *sv, const double *matrix, const int64_t *wires, int nw, int inverse);
/* applyControlledMatrix (Bindings.hpp:177-200, StateVectorLQubit.hpp:571-622) */
int plgb_sv_apply_controlled_matrix(plgb_sv *sv, const double *matrix, const int64_t *cwires, const uint8_t *cvals,
                                    int ncw, const int64_t *wires, int nw, int inverse);
/* applySparseMatrix / applyControlledSparseMatrix (LQubitBindings.hpp:150-175,
 * StateVectorLQubit.hpp:724-870); local CSR operator on `wires` */
int plgb_sv_apply_sparse_matrix(plgb_sv *sv, const int64_t *indptr, const int64_t *indices, const double *data,
                                int64_t nnz, const int64_t *cwires, const uint8_t *cvals, int ncw,
                                const int64_t *wires, int nw);
/* applyPauliRot(wires, inverse, params, word) (LQubitBindings.hpp:198-207,
 * GateImplementationsLM.hpp:577-629) */
int plgb_sv_apply_pauli_rot(plgb_sv *sv, const int64_t *wires, int nw, int inverse, double angle, const char *word);
/* applyGenerator, plain and controlled (StateVectorLQubit.hpp:527-560);
 * writes the generator's scaling factor */
int plgb_sv_apply_generator(plgb_sv *sv, const char *name, const int64_t *cwires, const uint8_t *cvals, int ncw,
                            const int64_t *wires, int nw, int adj, double *scale_out);
/* collapse(wire, branch) / normalize() (StateVectorLQubit.hpp:881-921) */
int plgb_sv_collapse(plgb_sv *sv, int64_t wire, int branch);
int plgb_sv_normalize(plgb_sv *sv);

/* ---- measurements (MeasurementsLQubit.hpp:73-768, Bindings.hpp:651-688,
 *      LQubitBindings.hpp:262-349) ---- */
/* probs() (nw < 0) / probs(wires); out holds 2^nw (or 2^n) doubles */
int plgb_meas_probs(plgb_sv *sv, const int64_t *wires, int nw, double *out);
/* expval(name, wires) */
int plgb_meas_expval_named(plgb_sv *sv, const char *name, const int64_t *wires, int nw, double *out);
/* expval(matrix, wires) */
int plgb_meas_expval_matrix(plgb_sv *sv, const double *matrix, const int64_t *wires, int nw, double *out);
/* expval(row_map, col_idx, values) over the full register */
int plgb_meas_expval_sparse(plgb_sv *sv, const int64_t *indptr, int64_t nptr, const int64_t *indices,
                            const double *data, int64_t nnz, double *out);
/* expval(obs) / var(obs) */
int plgb_meas_expval_obs(plgb_sv *sv, const plgb_obs *obs, double *out);
int plgb_meas_var_obs(plgb_sv *sv, const plgb_obs *obs, double *out);
/* var(name, wires), var(matrix, wires), var(row_map, col_idx, values) */
int plgb_meas_var_named(plgb_sv *sv, const char *name, const int64_t *wires, int nw, double *out);
int plgb_meas_var_matrix(plgb_sv *sv, const double *matrix, const int64_t *wires, int nw, double *out);
int plgb_meas_var_sparse(plgb_sv *sv, const int64_t *indptr, int64_t nptr, const int64_t *indices,
                         const double *data, int64_t nnz, double *out);
/* generate_samples(wires, shots) / generate_samples(num_wires, shots) (nw < 0)
 * with set_random_seed(seed) (MeasurementsLQubit.hpp:646-679,
 * MeasurementsBase.hpp:77-93); out holds shots * nw int64 bits, last wire
 * fastest */
int plgb_meas_generate_samples(plgb_sv *sv, const int64_t *wires, int nw, int64_t shots, uint64_t seed,
                               int64_t *out);
/* generate_mcmc_samples(num_wires, kernelname, num_burnin, num_shots) with
 * set_random_seed(seed) (LQubitBindings.hpp:340-349 ->
 * MeasurementsLQubit.hpp:551-594 generate_samples_metropolis,
 * TransitionKernels.hpp:37-163); out holds num_shots * num_qubits int64 bits */
int plgb_meas_generate_mcmc_samples(plgb_sv *sv, const char *kernelname, int64_t num_burnin, int64_t num_shots,
                                    uint64_t seed, int64_t *out);

/* ---- observables (Bindings.hpp:467-591, LQubitBindings.hpp:358-407) ---- */
/* NamedObsC*(name, wires) */
int plgb_obs_named(const char *name, const int64_t *wires, int nw, plgb_obs **out);
/* HermitianObsC*(matrix, wires); matrix: 4^nw interleaved complex128 */
int plgb_obs_hermitian(const double *matrix, const int64_t *wires, int nw, plgb_obs **out);
/* TensorProdObsC*(list) */
int plgb_obs_tensor_prod(plgb_obs *const *obs, int n, plgb_obs **out);
/* HamiltonianC*(coeffs, list) */
int plgb_obs_hamiltonian(const double *coeffs, plgb_obs *const *obs, int n, plgb_obs **out);
/* SparseHamiltonianC*(data, indices, indptr, wires) */
int plgb_obs_sparse_hamiltonian(const double *data, const int64_t *indices, int64_t nnz, const int64_t *indptr,
                                int64_t nptr, const int64_t *wires, int nw, plgb_obs **out);
int plgb_obs_destroy(plgb_obs *obs);
/* get_wires(): writes up to cap wires, *nw = total */
int plgb_obs_wires(const plgb_obs *obs, int64_t *wires, int cap, int *nw);
/* __repr__ */
int plgb_obs_repr(const plgb_obs *obs, char *buf, size_t len);

/* ---- algorithms (Bindings.hpp:704-851, JacobianData.hpp:39-393,
 *      AdjointJacobianLQubit.hpp:347-491) ---- */
/* OpsStructC*(names, params, wires, inverses, matrices, cwires, cvals) /
 * create_ops_listC*: flattened with per-op counts; mat_sizes[k] = number of
 * complex entries of op k's matrix (0 when none) */
int plgb_ops_create(int nops, const char *const *names, const double *params, const int *nparams,
                    const int64_t *wires, const int *nwires, const uint8_t *inverses, const double *mats,
                    const int64_t *mat_sizes, const int64_t *cwires, const int *ncwires, const uint8_t *cvals,
                    plgb_ops **out);
int plgb_ops_destroy(plgb_ops *ops);
int plgb_ops_num_par_ops(const plgb_ops *ops, int *out);
/* StateVectorBase::applyOperations (core/simulators/base/StateVectorBase.hpp:
 * 127-175): apply every operation of `ops` (each with its own inverse flag).
 * tile_bits = 0 launches one kernel per gate; tile_bits = t > 0 fuses the
 * list into shared-memory tile passes of up to 2^t amplitudes (the compiled
 * passes are cached on `ops` per register size, precision and t); complex64
 * registers of 22 qubits and more instead run it as dense blocks of up to six
 * wires (as plgb_sv_apply_operations_blocks with 6) while the tensor cores are
 * on (plgb_set_tc_dense).  *passes_out (optional) receives the number of
 * kernel passes (or blocks) per call. */
int plgb_sv_apply_operations(plgb_sv *sv, plgb_ops *ops, int tile_bits, int *passes_out);
/* Dense-block fusion (no counterpart in the reference): the operations of
 * `ops` merged, in order, into dense blocks on at most block_wires (1..6)
 * wires, each applied as one dense kernel, i.e. one pass over the state.
 * complex64 blocks on four to six wires run on the tensor cores (tcgen05,
 * widened to six wires); the others on the CUDA cores.  The block list is
 * cached on `ops` per register size, precision and width.  *blocks_out
 * (optional) receives the number of kernels per call. */
int plgb_sv_apply_operations_blocks(plgb_sv *sv, plgb_ops *ops, int block_wires, int *blocks_out);
/* The block list of plgb_sv_apply_operations_blocks as JSON, computed on the
 * host without a GPU: per block its kind (0 = one-wire pair, 2 = 4x4, 3 =
 * dense 2^k) and targets (first = most significant local bit), and with
 * with_matrices its row-major matrix as [re, im] pairs (no counterpart in
 * the reference). */
int plgb_ops_block_plan(const plgb_ops *ops, int num_qubits, int precision, int block_wires, int with_matrices,
                        char *buf, size_t len);
/* Arithmetic of complex128 fused passes, batched passes and the fused
 * adjoint sweep (no counterpart in the reference): on = 1 (default) runs
 * them in FP64, like the reference's kernels; on = 0 opts into double-float
 * arithmetic on the FP32 pipe (about 48 significant bits, FP32 exponent
 * range: |amplitude| < 2^127, magnitudes below 2^-126 flush to zero; GB300
 * executes FP64 at 1/64 of its FP32 rate).  Process-wide; returns the
 * previous setting. */
int plgb_set_c128_fp64_passes(int on);
/* Dense complex64 gates on six wires without controls (applyMatrix and the
 * unfused path) on the tensor cores (tcgen05, split-TF32 operands: about
 * 2^-21 relative accuracy per gate) when on = 1 (default), or on the CUDA
 * cores.  No counterpart in the reference.  Process-wide; returns the
 * previous setting. */
int plgb_set_tc_dense(int on);
/* Register-tile kernel variant for a precision (64 or 128): occ = 0 lets a
 * thread use up to 255 registers, occ = 1 caps it at 128 (twice the
 * resident warps, some spills).  Returns the previous setting, or -1 for a
 * bad precision (no counterpart in the reference). */
int plgb_set_tile_variant(int precision, int occ);
/* Lazy fusion of per-gate calls (no counterpart in the reference; on by
 * default): on a lazy handle the gate calls (plgb_sv_apply_operation,
 * _controlled_operation, _matrix, _controlled_matrix) validate their
 * arguments and queue the gate; the next call that reads or rewrites the
 * state first runs the queue as fused tile passes.  Results are those of
 * the gates applied one by one within the precision's tolerance.
 * plgb_set_lazy_fusion sets the default for handles created afterwards and
 * returns the previous default; plgb_sv_set_lazy switches one handle (its
 * queue runs first).  Handles on fewer than plgb_set_lazy_min_qubits qubits
 * (default 17) apply each gate at its call; the setter returns the previous
 * value, or -1 for q < 1. */
int plgb_set_lazy_fusion(int on);
int plgb_sv_set_lazy(plgb_sv *sv, int on);
int plgb_set_lazy_min_qubits(int q);
/* Plan introspection (no device needed): the tile passes plgb_sv_apply_operations
 * would run for `ops` on num_qubits at precision / tile_bits, as a JSON array
 * with one object per pass (tile size, op counts, execution stages). */
int plgb_ops_fusion_plan(const plgb_ops *ops, int num_qubits, int precision, int tile_bits, char *buf, size_t len);
/* AdjointJacobianC*.__call__(sv, observables, ops, trainable_params):
 * jac_out holds nobs * ntp doubles, row-major [obs][param].  With apply_ops
 * the operations are first applied to a copy of the state. */
int plgb_adjoint_jacobian(plgb_sv *sv, plgb_obs *const *obs, int nobs, const plgb_ops *ops, const int64_t *trainable,
                          int ntp, int apply_ops, double *jac_out);
/* VectorJacobianProductC*.__call__(sv, ops, dy, trainable_params)
 * (LQubitBindings.hpp:412-457, VectorJacobianProduct.hpp:79-160): sv holds
 * the final state, dy the cotangent (2^n complex, interleaved re/im);
 * out receives ntp complex values <dy | d psi / d theta_j> (interleaved). */
int plgb_vjp(plgb_sv *sv, const plgb_ops *ops, const double *dy, const int64_t *trainable, int ntp, double *out);
/* The same Jacobian with apply_ops = 0, computed in place: sv holds the
 * final state and is overwritten by the backward sweep (left holding the
 * initial state up to rounding).  Registers held: 1 + nobs for Pauli-sum
 * observables and Pauli-word generators, instead of 2 + nobs plus
 * temporaries; this is what lets a 32-qubit complex128 adjoint fit on one
 * GPU.  No counterpart in the reference (AdjointJacobianLQubit.hpp:225-491
 * always copies the state). */
int plgb_adjoint_jacobian_inplace(plgb_sv *sv, plgb_obs *const *obs, int nobs, const plgb_ops *ops,
                                  const int64_t *trainable, int ntp, double *jac_out);

/* ---- batch engine (no counterpart in the reference: lightning.qubit runs
 *      circuits one at a time, one Python -> C++ call per gate,
 *      pennylane_lightning/lightning_qubit/_state_vector.py:220-299) ----
 * Many independent circuits, each from |0...0> on its own register, run
 * together: pass k of every circuit's fused program is one persistent launch
 * over all their tiles; Pauli-sum expectation values are reduced in one
 * batched launch.  A circuit's results do not depend on what else is in the
 * batch (bit-identical). */
typedef struct plgb_batch plgb_batch;
int plgb_batch_create(int precision, plgb_batch **out);
int plgb_batch_destroy(plgb_batch *b);
/* tile_bits 0 = autotuned per register size (measured once per size);
 * wave_bytes 0 = 8 GiB of registers per wave; threads 0 = all host cores */
int plgb_batch_configure(plgb_batch *b, int tile_bits, int64_t wave_bytes, int threads);
/* Circuits in packed arrays: circuit c has num_qubits[c] wires and ops
 * [op_offsets[c], op_offsets[c+1]); op o is gate plgb_gate_name(op_codes[o])
 * on wires op_wires[4o..4o+3] (-1 = unused), parameters op_params[3o..3o+2]
 * (unused ones ignored), adjoint if op_inverse[o] (op_inverse may be NULL).
 * Circuit c's observables are [obs_offsets[c], obs_offsets[c+1]); observable
 * k is sum over terms [term_offsets[k], term_offsets[k+1]) of
 * term_coeffs[t] * (X on wires term_x[t]) (Y on term_y[t]) (Z on term_z[t]),
 * the masks holding bit w for wire w.  out receives one value per
 * observable. */
int plgb_batch_run(plgb_batch *b, int ncirc, const int32_t *num_qubits, const int64_t *op_offsets,
                   const int32_t *op_codes, const int32_t *op_wires, const double *op_params, const uint8_t *op_inverse,
                   const int64_t *obs_offsets, const int64_t *term_offsets, const double *term_coeffs,
                   const uint64_t *term_x, const uint64_t *term_y, const uint64_t *term_z, double *out);
/* Adjoint requests in the same packed layout: for each circuit, <O> of each
 * of its observables into values (one per observable) and the Jacobian of
 * each <O> with respect to the parameter of every parametric gate of the
 * circuit (the in-place adjoint sweep; AdjointJacobianLQubit.hpp:225-491)
 * into jac: circuit after circuit, per circuit one row per observable of
 * (number of parametric gates) entries.  Circuits run concurrently on host
 * threads, each on its own stream, three registers each within the
 * engine's memory budget. */
int plgb_batch_adjoint(plgb_batch *b, int ncirc, const int32_t *num_qubits, const int64_t *op_offsets,
                       const int32_t *op_codes, const int32_t *op_wires, const double *op_params,
                       const uint8_t *op_inverse, const int64_t *obs_offsets, const int64_t *term_offsets,
                       const double *term_coeffs, const uint64_t *term_x, const uint64_t *term_y,
                       const uint64_t *term_z, double *values, double *jac);
/* JSON of the last run: waves, launches, tile sizes, compile and device ms,
 * completion time of each wave and the wave of each circuit */
int plgb_batch_stats(const plgb_batch *b, char *buf, size_t len);
/* gate-name code table of plgb_batch_run: name of code, NULL past the end */
const char *plgb_gate_name(int code);

/* expval(matrix, wires) for at most 5 wires without any device allocation.
 * No counterpart in the reference: plgb_meas_expval_matrix may grow device
 * scratch with cudaMalloc (after a cudaFree, which waits for the device);
 * this variant uses one fixed device array per device instead, for callers
 * that have filled the device up to a memory budget.  Same result as
 * plgb_meas_expval_matrix.  nw > 5 returns PLGB_ERR_INVALID, and so does a
 * lazy handle with gates still queued (running them would compile and
 * upload a fused program, which allocates; plgb_sv_synchronize runs them).
 * The first call on a device resolves the array's address.  Every call
 * copies the matrix in and synchronises the state vector's stream, so it
 * must not be called while any stream is being captured.  Overlapping calls
 * on one device race on the shared array: serialise them. */
int plgb_meas_expval_matrix_noalloc(plgb_sv *sv, const double *matrix, const int64_t *wires, int nw, double *out);

#ifdef __cplusplus
}
#endif
#endif /* PL_GB300_H */
