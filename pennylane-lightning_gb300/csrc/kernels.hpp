// Internal launch interface between the C++ host layer and the CUDA kernels.
// Everything here takes plain device pointers, sizes and small POD
// descriptors; nothing is allocated by the launchers.
#pragma once

#include "plgb_common.cuh"

namespace plgb {

enum Mode1 : int {
    M1_DENSE = 0,  // general complex 2x2
    M1_REAL = 1,   // real 2x2 (RY, Hadamard)
    M1_RXF = 2,    // [[c, i s], [i s, c]] (RX family)
    M1_DIAG = 3,   // diag(d0, d1)
    M1_PHASE1 = 4, // diag(1, d1): only the |1> half is touched
    M1_SWAP = 5,   // X: amplitude swap, no arithmetic
    M1_ANTI = 6,   // [[0, b], [c, 0]]
    M1_NEG1 = 7,   // diag(1, -1): sign flip of the |1> half
};

template <class T> struct Mat1 {
    cx<T> m[4];
};
template <class T> struct Mat2 {
    cx<T> m[16];
};
struct LocalOffsets {
    u64 off[32];
};
struct TBits {
    int b[16];
};

template <class T>
void launch_1q(cudaStream_t s, cx<T> *sv, const GroupGeom &g, u64 o0, u64 o1, int mode, const Mat1<T> &m);
template <class T>
void launch_2q(cudaStream_t s, cx<T> *sv, const GroupGeom &g, int bit_hi_local, int bit_lo_local, bool diag,
               const Mat2<T> &m);
template <class T>
void launch_kq(cudaStream_t s, cx<T> *sv, const GroupGeom &g, int k, const LocalOffsets &lo, const cx<T> *dmat,
               const u64 *dloc);
template <class T>
void launch_diag(cudaStream_t s, cx<T> *sv, u64 N, u64 cmask, u64 cval, int k, const TBits &tb, const cx<T> *dd);
template <class T>
void launch_parity(cudaStream_t s, cx<T> *sv, u64 N, u64 pmask, u64 cmask, u64 cval, cx<T> s0, cx<T> s1,
                   bool zero_outside);
template <class T> void launch_pauli_rot(cudaStream_t s, cx<T> *sv, int n, u64 mxy, u64 my, u64 mz, T c, cx<T> sn);
template <class T> void launch_zero_outside(cudaStream_t s, cx<T> *sv, u64 N, u64 cmask, u64 cval);
template <class T> void launch_scale(cudaStream_t s, cx<T> *sv, u64 N, cx<T> f, u64 cmask, u64 cval);
template <class T> void launch_axpy(cudaStream_t s, cx<T> *y, const cx<T> *x, u64 N, cx<T> f);
template <class T> void launch_scatter_sub(cudaStream_t s, cx<T> *sv, const cx<T> *sub, u64 D, const u64 *loc);
template <class T>
void launch_sparse_local(cudaStream_t s, cx<T> *sv, const GroupGeom &g, const LocalOffsets &lo, int k,
                         const long long *indptr, const long long *indices, const cx<T> *vals);

// ---------------------------------------------------------------------------
// Reductions.  Every reduction writes per-block partial sums (double) into
// `partials` (at least kReduceBlocks * nout doubles) and a final kernel sums
// them in a fixed order into `out` (nout doubles, device memory), so results
// are deterministic for a given size.
// ---------------------------------------------------------------------------
constexpr int kReduceBlocks = 152 * 4;
constexpr int kReduceThreads = 256;

// One Pauli word: P|k> = i^ny * (-1)^popcount(k & yz) |k ^ x>.
struct PauliTerm {
    double coeff;
    u64 yz;
    int ny4; // ny mod 4
    int pad;
};
constexpr int kMaxTermsPerGroup = 64;
struct PauliGroup {
    u64 x;      // common flip mask
    int hb;     // highest set bit of x (unused when x == 0)
    int nterms; // <= kMaxTermsPerGroup
    PauliTerm t[kMaxTermsPerGroup];
};

template <class T> void reduce_norm2(cudaStream_t s, const cx<T> *sv, u64 N, double *partials, double *out);
template <class T>
void reduce_inner(cudaStream_t s, const cx<T> *a, const cx<T> *b, u64 N, double *partials, double *out);
// named one-wire expval: kind 0=X 1=Y 2=Z 3=H
template <class T>
void reduce_expval1(cudaStream_t s, const cx<T> *sv, u64 N, int tbit, int kind, double *partials, double *out);
// Re <psi| sum_t c_t P_t |psi> over one flip-mask group
template <class T>
void reduce_pauli_group(cudaStream_t s, const cx<T> *sv, u64 N, const PauliGroup &g, double *partials, double *out);
// Im / Re of <a| P |b> restricted to indices (j & pmask) == pval; out[0]=Re, out[1]=Im
template <class T>
void reduce_pauli_transition(cudaStream_t s, const cx<T> *a, const cx<T> *b, u64 N, u64 x, u64 yz, int ny4,
                             u64 pmask, u64 pval, double *partials, double *out);
// Re sum_groups v^H M v on k wires (Hermitian expval)
template <class T>
void reduce_expval_matrix(cudaStream_t s, const cx<T> *sv, const GroupGeom &g, int k, const LocalOffsets &lo,
                          const cx<T> *dmat, double *partials, double *out);
// Re <psi| A |psi> with A in CSR over the full register
template <class T>
void reduce_expval_csr(cudaStream_t s, const cx<T> *sv, u64 N, const long long *indptr, const long long *indices,
                       const cx<T> *vals, double *partials, double *out);
// out = A psi (CSR SpMV over the full register)
template <class T>
void launch_csr_apply(cudaStream_t s, const cx<T> *sv, cx<T> *out, u64 N, const long long *indptr,
                      const long long *indices, const cx<T> *vals);

// Pauli-sum expectation values by passes (kernels_measure.cu): a pass
// holds up to kPassTerms Pauli words whose flip bits all fit one tile of
// 2^t amplitudes; the tile's local bits are those flip bits and the lowest
// other bits.  One read of the state evaluates every word of the pass: per
// word the kernel sums, over the amplitude pairs (j, j ^ x) of the tile
// (j without x's top bit), (-1)^{|j & yz|} times Re or Im of
// conj(psi_j) psi_{j^x} (the part the word's Y count selects), or for x = 0
// (-1)^{|j & yz|} |psi_j|^2; the host applies each word's coefficient.
constexpr int kPassTerms = 16;
constexpr int kPassMaxTileBits = 12;
struct PauliPassTerm {
    u64 yz;          // Y|Z mask over the full index
    unsigned x;      // flip mask over the local index (0: diagonal word)
    unsigned yzl;    // Y|Z mask over the local index
    int hb;          // highest set bit of x (local)
    int im;          // 1: sum Im conj(psi_j) psi_{j^x}; 0: Re
    // tiles of 2^12 amplitudes, 512 threads: pair k = r * 512 + tid, r < 4,
    // has j = jt(tid) | jr[r] (k with a zero inserted at bit hb); srm bit r =
    // parity of jr[r] & yzl (x = 0: of (r << 9) & yzl, r < 8)
    unsigned short jr[4];
    unsigned srm;
};
struct PauliPass {
    int t;                  // local bits per tile
    int lbit[kPassMaxTileBits];
    int nglob;
    int glob[64];
    u64 ntiles;
    int nterms;             // <= kPassTerms
    PauliPassTerm term[kPassTerms];
};
// per-block partial sums of the pass's words into partials[block * kPassTerms + w];
// returns the grid size (the number of blocks to finalize)
template <class T> int launch_pauli_pass(cudaStream_t s, const cx<T> *sv, const PauliPass &p, double *partials);
void launch_finalize_pass(cudaStream_t s, const double *partials, int nblocks, double *out);

// All flip-mask groups of a Pauli sum in one sweep (kernels_measure.cu):
// out[j] (+)= sum_g sum_{t in g} c_t i^ny_t (-1)^{|k & yz_t|} psi[k], k = j ^ x_g,
// in double-float arithmetic (coefficients split on the host).
struct PauliTermDF {
    u64 yz;
    float chi, clo; // coefficient as a double-float pair
    int ny4, pad;
};
struct PauliGroupHdr {
    u64 x;
    int tbegin, tend; // terms [tbegin, tend) of the term array
};
constexpr int kApplyMaxGroups = 256, kApplyMaxTerms = 1024; // per launch (staged in shared memory)
template <class T>
void launch_pauli_apply(cudaStream_t s, const cx<T> *psi, cx<T> *out, u64 N, const PauliGroupHdr *groups, int ngroups,
                        const PauliTermDF *terms, int nterms, bool first);

// Probabilities: all wires (elementwise), or marginal over `k` wires given by
// their bit positions (wires[0] = MSB of the output index).
template <class T> void launch_probs_all(cudaStream_t s, const cx<T> *sv, u64 N, T *out);

// Metropolis-Hastings sampling (kernels_mcmc.cu)
constexpr u64 kMcmcChunk = 4096; // amplitudes per non-zero counting chunk
template <class T>
void launch_nz_count(cudaStream_t s, const cx<T> *sv, u64 N, T eps, u64 nchunks, unsigned *counts);
template <class T>
void launch_nz_select(cudaStream_t s, const cx<T> *sv, u64 N, T eps, const u64 *prefix, u64 nchunks, const u64 *rank,
                      u64 steps, u64 *tidx, T *tplog);
template <class T>
void launch_mcmc_chain_nz(cudaStream_t s, const cx<T> *sv, const u64 *tidx, const T *tplog, const T *ran, u64 steps,
                          u64 burnin, u64 *out);
template <class T>
void launch_mcmc_chain_local(cudaStream_t s, const cx<T> *sv, const unsigned char *site, const unsigned char *value,
                             const T *ran, u64 steps, u64 burnin, u64 *out);
void launch_index_bits(cudaStream_t s, const u64 *idx, u64 shots, int n, long long *out);
// Marginal probabilities in the reference's summation order (bit-exact): k
// wires at bit positions wb (wb[0] = most significant output bit), cmask =
// the other bits
struct MarginalGeom {
    int k;
    int wb[64];
    u64 cmask;
};
template <class T> void launch_probs_marginal_serial(cudaStream_t s, const cx<T> *sv, const MarginalGeom &g, T *out);

} // namespace plgb
