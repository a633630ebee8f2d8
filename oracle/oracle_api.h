/*
 * Test-infrastructure C API shared by the two CPU oracles:
 *   - liboracle.so   : this repository's restatement of lightning.qubit's LM
 *                      algorithms (oracle/lm_oracle.hpp), prefix "orc_";
 *   - _ref/libplref.so: a shim over the reference's own C++ headers, compiled
 *                      from the reference sources in place, prefix "ref_".
 *
 * Only tests, the smoke check and the CPU-baseline leg of the benchmark load
 * these libraries, and only as checkers / baselines.  The GPU product path
 * never links or calls them.
 *
 * Conventions (identical for both prefixes):
 *   - a state vector handle is created for a precision: is_double=1 gives
 *     complex128 amplitudes, 0 gives complex64;
 *   - state buffers passed in/out are in the handle's precision, interleaved
 *     (re, im);
 *   - gate parameters, matrices and coefficients are always passed in double
 *     precision and converted to the handle's precision first (as the Python
 *     binding does when it converts numpy arrays);
 *   - every int-returning call returns 0 on success and non-zero on error,
 *     with the message available from <prefix>last_error().
 *
 * Observable specs are whitespace separated token streams:
 *   named <Name> <wire>
 *   herm  <k> <w_1..w_k> <off>             matrix = cdata[off : off + 4^k]
 *   prod  <m> <obs_1> ... <obs_m>
 *   ham   <m> <coeff_1> <obs_1> ... <coeff_m> <obs_m>
 *   sparse <k> <w_1..w_k> <nnz> <off_data> <off_indices> <off_indptr>
 *                                          data = cdata[off_data : +nnz],
 *                                          indices = idata[off_indices : +nnz],
 *                                          indptr = idata[off_indptr : +2^k+1]
 */
#ifndef PL_GB300_ORACLE_API_H
#define PL_GB300_ORACLE_API_H
#include <stdint.h>

#ifndef ORC_PREFIX
#define ORC_PREFIX orc_
#endif
#define ORC_CAT2(a, b) a##b
#define ORC_CAT(a, b) ORC_CAT2(a, b)
#define ORC_FN(name) ORC_CAT(ORC_PREFIX, name)

#ifdef __cplusplus
extern "C" {
#endif

const char *ORC_FN(last_error)(void);
void *ORC_FN(sv_new)(int num_qubits, int is_double);
void ORC_FN(sv_free)(void *sv);
int ORC_FN(sv_set_state)(void *sv, const void *data);
int ORC_FN(sv_get_state)(void *sv, void *out);
int ORC_FN(sv_apply)(void *sv, const char *name, const int64_t *cwires,
                     const uint8_t *cvals, int ncw, const int64_t *wires,
                     int nw, int inverse, const double *params, int np);
int ORC_FN(sv_apply_matrix)(void *sv, const double *mat,
                            const int64_t *cwires, const uint8_t *cvals,
                            int ncw, const int64_t *wires, int nw, int inverse);
int ORC_FN(sv_apply_sparse)(void *sv, const int64_t *indptr,
                            const int64_t *indices, const double *data,
                            int64_t nnz, const int64_t *cwires,
                            const uint8_t *cvals, int ncw, const int64_t *wires,
                            int nw);
int ORC_FN(sv_apply_pauli_rot)(void *sv, const int64_t *wires, int nw,
                               int inverse, double angle, const char *word);
int ORC_FN(sv_apply_generator)(void *sv, const char *name,
                               const int64_t *cwires, const uint8_t *cvals,
                               int ncw, const int64_t *wires, int nw, int adj,
                               double *scale_out);
int ORC_FN(sv_collapse)(void *sv, int64_t wire, int branch);
int ORC_FN(sv_normalize)(void *sv);
int ORC_FN(sv_set_basis_state)(void *sv, const int64_t *bits,
                               const int64_t *wires, int nw);
int ORC_FN(probs)(void *sv, const int64_t *wires, int nw, double *out);
int ORC_FN(expval_named)(void *sv, const char *name, const int64_t *wires,
                         int nw, double *out);
int ORC_FN(expval_matrix)(void *sv, const double *mat, const int64_t *wires,
                          int nw, double *out);
int ORC_FN(var_named)(void *sv, const char *name, const int64_t *wires,
                      int nw, double *out);
int ORC_FN(var_matrix)(void *sv, const double *mat, const int64_t *wires,
                       int nw, double *out);
int ORC_FN(expval_sparse)(void *sv, const int64_t *indptr, int64_t nptr,
                          const int64_t *indices, const double *data,
                          int64_t nnz, double *out);
int ORC_FN(expval_obs)(void *sv, const char *spec, const double *cdata,
                       const int64_t *idata, double *out);
int ORC_FN(var_obs)(void *sv, const char *spec, const double *cdata,
                    const int64_t *idata, double *out);
int ORC_FN(samples)(void *sv, const int64_t *wires, int nw, int64_t shots,
                    uint64_t seed, int64_t *out);
/* generate_mcmc_samples: shots x num_qubits bits (MeasurementsLQubit.hpp:551) */
int ORC_FN(mcmc_samples)(void *sv, const char *kernel, int64_t burnin,
                         int64_t shots, uint64_t seed, int64_t *out);
int ORC_FN(adjoint)(void *sv, int nops, const char **names,
                    const double *params, const int *nparams,
                    const int64_t *wires, const int *nwires,
                    const uint8_t *inverses, const double *mats,
                    const int64_t *mat_sizes, const int64_t *cwires,
                    const int *ncwires, const uint8_t *cvals, int nobs,
                    const char **obs_specs, const double *cdata,
                    const int64_t *idata, const int64_t *trainable, int ntp,
                    int apply_ops, double *jac_out);
/* VectorJacobianProduct (lightning_qubit/algorithms/VectorJacobianProduct.hpp:79):
 * w_j = <dy| d psi / d theta_j> for the trainable parameters, complex
 * (re, im) pairs in out; dy is 2^n interleaved (re, im) doubles. */
int ORC_FN(vjp)(void *sv, int nops, const char **names, const double *params,
                const int *nparams, const int64_t *wires, const int *nwires,
                const uint8_t *inverses, const double *mats,
                const int64_t *mat_sizes, const int64_t *cwires,
                const int *ncwires, const uint8_t *cvals, const double *dy,
                const int64_t *trainable, int ntp, int apply_ops,
                double *out);
int ORC_FN(num_threads)(void);

#ifdef __cplusplus
}
#endif
#endif
