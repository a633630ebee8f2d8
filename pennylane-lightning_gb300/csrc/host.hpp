// C++ host layer: the GB300 counterparts of lightning.qubit's
// StateVectorLQubitManaged / Measurements / Observables / AdjointJacobian.
// Device memory is owned here (cudaMalloc), kernels are launched on the
// state vector's stream, and results are copied back only by the calls that
// return data to the host.
#pragma once

#include "kernels.hpp"
#include "kernels_tc.hpp"

#include <complex>
#include <cstdint>
#include <memory>
#include <mutex>
#include <random>
#include <string>
#include <vector>
#include <map>
#include <unordered_map>

namespace plgb {

struct PLError : std::runtime_error {
    using std::runtime_error::runtime_error;
};
#define PLGB_REQUIRE(cond, msg)                                                                                   \
    do {                                                                                                          \
        if (!(cond)) {                                                                                            \
            throw ::plgb::PLError(msg);                                                                           \
        }                                                                                                         \
    } while (0)

using cd = std::complex<double>;

// ---------------------------------------------------------------------------
// Observables (precision-agnostic description; converted when applied).
// ---------------------------------------------------------------------------
struct ObsNode {
    enum Kind { Named, Herm, Prod, Ham, Sparse } kind{Named};
    std::string name;
    std::vector<int64_t> wires;
    std::vector<cd> mat;
    std::vector<std::shared_ptr<ObsNode>> children;
    std::vector<double> coeffs;
    std::vector<cd> sp_data;
    std::vector<int64_t> sp_indices, sp_indptr;
    std::vector<int64_t> all_wires() const;
    std::string repr() const;
};
using ObsPtr = std::shared_ptr<ObsNode>;

// One operation of an OpsData list (core/algorithms/JacobianData.hpp:39-253)
struct OpRec {
    std::string name;
    std::vector<double> params;
    std::vector<int64_t> wires;
    bool inverse{false};
    std::vector<cd> matrix;
    std::vector<int64_t> cwires;
    std::vector<bool> cvals;
};
struct OpsList {
    std::vector<OpRec> ops;
    size_t num_par_ops() const;
};

bool is_named_gate(const std::string &name);

// ---------------------------------------------------------------------------
// Device and pinned buffers of the host layer.  Outside a ReuseScope these
// are cudaMalloc / cudaFree (cudaFree waits for the whole device).  Inside
// one, the thread's ReusePool hands out buffers it already holds and takes
// freed ones back without waiting; they become reusable after
// ReusePool::recycle(), which the owner calls once the work that used them
// has completed (the batch engine's adjoint workers: after each request).
// ---------------------------------------------------------------------------
class ReusePool {
  public:
    ReusePool() = default;
    ReusePool(const ReusePool &) = delete;
    ReusePool &operator=(const ReusePool &) = delete;
    ~ReusePool();
    void *take(size_t bytes, bool pinned);
    bool give(void *p); // false: not handed out by this pool
    void recycle();     // pending buffers become reusable (their work is done)
    size_t cap_bytes{size_t{4} << 30}; // held beyond this are released
  private:
    struct Buf {
        size_t cap;
        bool pinned;
    };
    std::unordered_map<void *, Buf> out_;
    std::multimap<size_t, void *> free_[2]; // [pinned]
    std::vector<std::pair<void *, Buf>> pending_;
    size_t held_{0};
};
class ReuseScope {
  public:
    explicit ReuseScope(ReusePool &pool);
    ~ReuseScope();
    ReuseScope(const ReuseScope &) = delete;
    ReuseScope &operator=(const ReuseScope &) = delete;

  private:
    ReusePool *prev_;
};
void *dev_alloc(size_t bytes);
// every request for device memory the library makes (dev_alloc, the batch
// engine's arena) is counted; the count is a diagnostic of the C ABI
void count_device_allocation();
unsigned long long device_allocation_count();
void dev_free(void *p);
void *pinned_alloc(size_t bytes);
void pinned_free(void *p);

// ---------------------------------------------------------------------------
// Device scratch owned by a state vector.
// ---------------------------------------------------------------------------
struct DeviceScratch {
    double *red{nullptr};       // reduction partials + outputs
    double *host_out{nullptr};  // pinned
    void *mat{nullptr};         // matrices / diagonals / offsets
    size_t mat_bytes{0};
    int *flag{nullptr};         // error word of the tensor-core kernel (allocated on first use)
    void ensure_mat(size_t bytes);
    int *ensure_flag();
    // Carve consecutive sub-buffers of the given byte sizes out of `mat`,
    // each starting on a 256-byte boundary (16-byte vector loads of
    // complex128 need at least 16).
    std::vector<char *> carve(std::initializer_list<size_t> sizes);
    ~DeviceScratch();
};
inline size_t align_up(size_t x, size_t a = 256) { return (x + a - 1) / a * a; }

// A gate lowered to one streaming-kernel primitive.  The unfused path
// launches one kernel per primitive; the fusion engine (host_fusion.cpp)
// schedules primitives into shared-memory tile passes.
template <class T> struct Prim {
    enum Kind : int { Pair, Dense2, DenseK, DiagK, Parity, Scale, PauliRot, ZeroOut, Reduce };
    Kind kind{Pair};
    int mode{0};              // Pair: Mode1
    std::vector<int> tbits;   // target bit positions (first = MSB of the local index)
    u64 o0{0}, o1{0};         // Pair: offsets of the two mixed amplitudes
    std::vector<int> cbits;   // control bit positions
    u64 cmask{0}, cval{0};    // control mask / values over the full index
    std::vector<cx<T>> m;     // coefficients (Pair 4, Dense2 16, DenseK 4^k, DiagK 2^k, Parity 2, Scale 1)
    u64 pmask{0}, my{0}, mz{0}; // Parity mask; PauliRot x|y mask, y mask, z mask
    T c{0};                   // PauliRot cosine
    bool zero_outside{false};
    // Reduce (adjoint sweep): Im <H lambda| P G |lambda> into slot rslot, G
    // the Pauli word with flip mask rx, Y|Z mask ryz, ny4 Ys mod 4, P the
    // projector (index & rpm) == rpv
    u64 rx{0}, ryz{0}, rpm{0}, rpv{0};
    int rny4{0}, rslot{-1};
    u64 touched() const;      // every bit the primitive reads or writes
    bool diagonal() const;    // multiplies each amplitude by a factor (no mixing)
};

struct LowerOnly {}; // a register description for lowering gates without device memory

template <class T> class StateVector {
  public:
    using CT = cx<T>;
    explicit StateVector(int num_qubits, cudaStream_t stream = nullptr);
    StateVector(int num_qubits, LowerOnly); // no device memory: only lower_op() may be used
    StateVector(CT *external, int num_qubits, cudaStream_t stream = nullptr); // non-owning
    StateVector(const StateVector &other);                                     // deep copy, same stream
    StateVector &operator=(const StateVector &) = delete;
    ~StateVector();

    int num_qubits() const { return n_; }
    u64 length() const { return N_; }
    CT *data() { return d_; }
    const CT *data() const { return d_; }
    cudaStream_t stream() const { return s_; }
    void synchronize() const;

    // state management (StateVectorLQubit.hpp:881-1036, Managed :169-183)
    void reset();
    void set_basis_state_index(u64 index);
    void set_basis_state(const std::vector<int64_t> &bits, const std::vector<int64_t> &wires);
    void set_state_vector(const std::complex<T> *host_state, u64 len, const std::vector<int64_t> &wires);
    void update_data(const std::complex<T> *host, u64 len);
    void get_state(std::complex<T> *host_out, u64 len) const;
    void copy_from(const StateVector &other);
    void collapse(int64_t wire, bool branch);
    void normalize();

    // gates (StateVectorLQubit.hpp:359-870)
    void apply_operation(const std::string &name, const std::vector<int64_t> &wires, bool inverse,
                         const std::vector<double> &params);
    void apply_controlled_operation(const std::string &name, const std::vector<int64_t> &cwires,
                                    const std::vector<bool> &cvals, const std::vector<int64_t> &wires,
                                    bool inverse, const std::vector<double> &params);
    void apply_matrix(const cd *mat, const std::vector<int64_t> &wires, bool inverse,
                      const std::vector<int64_t> &cwires = {}, const std::vector<bool> &cvals = {});
    void apply_sparse_matrix(const int64_t *indptr, const int64_t *indices, const cd *data, int64_t nnz,
                             const std::vector<int64_t> &wires, const std::vector<int64_t> &cwires = {},
                             const std::vector<bool> &cvals = {});
    void apply_pauli_rot(const std::vector<int64_t> &wires, bool inverse, double angle, const std::string &word);
    double apply_generator(const std::string &name, const std::vector<int64_t> &cwires,
                           const std::vector<bool> &cvals, const std::vector<int64_t> &wires);
    void apply_op(const OpRec &op, bool inverse);

    // primitives used by the dispatcher, the observables and the adjoint
    void prim_pair(const std::vector<int> &ins_bits, u64 o0, u64 o1, const std::vector<int64_t> &cwires,
                   const std::vector<bool> &cvals, int mode, const Mat1<T> &m);
    void prim_1q(int64_t wire, const std::vector<int64_t> &cwires, const std::vector<bool> &cvals, int mode,
                 const Mat1<T> &m);
    void prim_dense(const std::vector<int64_t> &wires, const std::vector<int64_t> &cwires,
                    const std::vector<bool> &cvals, const std::vector<CT> &mat);
    void prim_diag(const std::vector<int64_t> &wires, const std::vector<int64_t> &cwires,
                   const std::vector<bool> &cvals, const std::vector<CT> &diag);
    void prim_zero_outside(const std::vector<int64_t> &cwires, const std::vector<bool> &cvals);
    void scale_add(const StateVector &x, cd factor); // this += factor * x

    // lowering: the primitives an operation expands to, without running them
    std::vector<Prim<T>> lower_op(const OpRec &op, bool inverse);
    // the primitives any gate-applying call f() would run (validated exactly
    // as when it runs), without running them
    template <class F> std::vector<Prim<T>> capture_prims(F &&f) {
        std::vector<Prim<T>> out;
        auto *saved = sink_;
        sink_ = &out;
        try {
            f();
        } catch (...) {
            sink_ = saved;
            throw;
        }
        sink_ = saved;
        return out;
    }
    void run_prim(const Prim<T> &p);
    // fused application of a primitive list in shared-memory tile passes
    // (host_fusion.cpp); tile_bits = log2 of the amplitudes a CTA stages
    void apply_prims_fused(const std::vector<Prim<T>> &prims, int tile_bits);

    // reductions (return to host, synchronizing)
    double norm2() const;
    cd inner(const StateVector &ket) const; // <this|ket>
    double *scratch_red() const { return scratch_.red; }
    double *host_out() const { return scratch_.host_out; }
    DeviceScratch &scratch() const { return scratch_; }
    int bit_of(int64_t wire) const;

  private:
    void alloc_(bool zero);
    void check_wires_(const std::vector<int64_t> &wires, const std::vector<int64_t> &cwires) const;
    GroupGeom geom_(const std::vector<int> &target_bits, const std::vector<int64_t> &cwires,
                    const std::vector<bool> &cvals) const;
    void apply_named_(const std::string &name, std::vector<int64_t> cw, std::vector<bool> cv,
                      std::vector<int64_t> wires, bool inverse, const std::vector<double> &params);
    void global_phase_(const std::vector<int64_t> &cw, const std::vector<bool> &cv, bool inverse, T angle);

    void emit_(Prim<T> &&p);
    std::vector<Prim<T>> *sink_{nullptr};
    int n_{0};
    u64 N_{0};
    CT *d_{nullptr};
    bool owns_{true};
    cudaStream_t s_{nullptr};
    bool owns_stream_{false};
    mutable DeviceScratch scratch_;
};

// ---------------------------------------------------------------------------
// Fusion (host_fusion.cpp): a primitive list compiled into tile passes, with
// its op tables resident in device memory; reusable across calls.
// ---------------------------------------------------------------------------
template <class T> struct FusedProgram;
template <class T>
std::shared_ptr<FusedProgram<T>> compile_fused(int n, const std::vector<Prim<T>> &prims, int tile_bits,
                                               bool upload = true, bool recipes = false);
// Arithmetic of fused complex128 passes (and of the batch engine and the
// fused adjoint sweep): FP64 (default) or, opted into, double-float on the
// FP32 pipe (hi + lo floats: ~48 significant bits, |x| < 2^127, magnitudes
// below 2^-126 flush to zero).
void set_c128_fp64_passes(bool on);
bool c128_fp64_passes();
// JSON description of a compiled program's passes (plan introspection)
template <class T> std::string fused_plan_json(const FusedProgram<T> &prog);
template <class T> void run_fused(StateVector<T> &sv, const FusedProgram<T> &prog);
// An adjoint program (with Reduce primitives) on lambda and H lambda (same
// stream); reductions land in partials[slot * G + CTA].
template <class T>
void run_fused_adjoint(StateVector<T> &lam, StateVector<T> &hlam, const FusedProgram<T> &prog, double *partials,
                       int G);
// Dense-block fusion (host_blocks.cpp): the primitives merged into dense
// blocks on at most kmax bits (Pair / Dense2 / DenseK primitives; others
// pass through)
template <class T> std::vector<Prim<T>> fuse_dense_blocks(const std::vector<Prim<T>> &prims, int n, int kmax);
// A dense-block program prepared for one register size: complex64 blocks on
// six wires carry their tensor-core geometry, and their matrix images are
// uploaded to the device once, so an application launches one kernel per
// block and checks the tensor-core error word once at the end.
template <class T> struct BlockProgram {
    std::vector<Prim<T>> prims;
    std::vector<int> tc;      // per primitive: its tensor-core block, -1 = the CUDA-core kernels
    std::vector<TcGeom> geom; // per tensor-core block
    void *images{nullptr};    // device: one image of tc_a_image_bytes() per tensor-core block
    BlockProgram() = default;
    BlockProgram(const BlockProgram &) = delete;
    BlockProgram &operator=(const BlockProgram &) = delete;
    ~BlockProgram() { dev_free(images); }
};
template <class T> std::shared_ptr<const BlockProgram<T>> prepare_blocks(std::vector<Prim<T>> prims, int n);
template <class T> void run_blocks(StateVector<T> &sv, const BlockProgram<T> &prog);
struct FusedStats {
    size_t passes, unfused, prims;
};
template <class T> FusedStats fused_stats(const FusedProgram<T> &prog);

// ---------------------------------------------------------------------------
// Measurements (MeasurementsLQubit.hpp) and sampling.
// ---------------------------------------------------------------------------
// expval(matrix, wires), at most 5 wires, with fixed device scratch and no
// allocation (noalloc.cu).
template <class T>
double expval_matrix_noalloc(StateVector<T> &sv, const double *matrix, const int64_t *wires, int nw);

template <class T> struct Measure {
    static std::vector<double> probs(StateVector<T> &sv, const std::vector<int64_t> &wires, bool all_wires);
    static double expval_named(StateVector<T> &sv, const std::string &name, const std::vector<int64_t> &wires);
    static double expval_matrix(StateVector<T> &sv, const cd *mat, const std::vector<int64_t> &wires);
    static double expval_sparse(StateVector<T> &sv, const int64_t *indptr, int64_t nptr, const int64_t *indices,
                                const cd *data, int64_t nnz);
    static double var_sparse(StateVector<T> &sv, const int64_t *indptr, int64_t nptr, const int64_t *indices,
                             const cd *data, int64_t nnz);
    static double expval_obs(StateVector<T> &sv, const ObsNode &obs);
    static double var_obs(StateVector<T> &sv, const ObsNode &obs);
    static std::vector<int64_t> samples(StateVector<T> &sv, const std::vector<int64_t> &wires, int64_t shots,
                                        uint64_t seed);
    static std::vector<int64_t> mcmc_samples(StateVector<T> &sv, const std::string &kernel, int64_t burnin,
                                             int64_t shots, uint64_t seed);
    static void apply_obs(StateVector<T> &sv, const ObsNode &obs);
    // dst = obs |src> (dst: same register size, any content); Pauli sums
    // need no temporary register
    static void apply_obs_into(const StateVector<T> &src, StateVector<T> &dst, const ObsNode &obs);
};

// Pauli-sum compilation of an observable tree.
struct PauliSum {
    struct Term {
        double c;
        u64 x, yz;
        int ny4;
    };
    std::vector<Term> terms;
};
bool compile_pauli(const ObsNode &obs, int n, PauliSum &out);
std::vector<PauliGroup> group_pauli(const PauliSum &ps);

// ---------------------------------------------------------------------------
// Adjoint Jacobian (AdjointJacobianLQubit.hpp:225-491).
// ---------------------------------------------------------------------------
template <class T> struct Adjoint {
    // VectorJacobianProduct (VectorJacobianProduct.hpp:79-160): w_j =
    // <dy | d psi / d theta_j> for the trainable parameters, sv = final state
    static std::vector<cd> vjp(StateVector<T> &sv, const OpsList &ops, const std::complex<T> *dy,
                               const std::vector<int64_t> &trainable);
    // consume: sv already holds the final state and may be overwritten; the
    // sweep then runs in place on it (registers needed: 1 + observables for
    // Pauli-sum observables and Pauli-word generators, instead of 2 + 2x)
    // fused_tile_bits > 0: for one observable and Pauli-word generators the
    // backward sweep runs as fused two-register tile passes with the
    // reductions inside (kernels_adjoint.cu); otherwise op by op.
    static std::vector<double> jacobian(StateVector<T> &sv, const std::vector<ObsPtr> &obs, const OpsList &ops,
                                        const std::vector<int64_t> &trainable, bool apply_ops, bool consume = false,
                                        int fused_tile_bits = 11);
};

// ---------------------------------------------------------------------------
// Thread-local error message for the C ABI.
// ---------------------------------------------------------------------------
void set_last_error(const std::string &msg);
const char *last_error();

} // namespace plgb
