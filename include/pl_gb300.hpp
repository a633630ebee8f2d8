/*
 * C++ API of the GB300 state-vector backend: the classes a C++ caller of
 * lightning.qubit uses, with the reference's method names, argument order,
 * defaults and error type, over the C ABI of pl_gb300.h.  Header-only; link
 * against libplgb300.so.
 *
 *   reference (inside the reference project)           here
 *   ------------------------------------------------   -----------------------
 *   StateVectorLQubitManaged<PrecisionT>               StateVectorGB300<PrecisionT>
 *     core/simulators/base/StateVectorBase.hpp:109-204,
 *     LQ/StateVectorLQubit.hpp:378-482,527-710,881-1036,
 *     LQ/StateVectorLQubitManaged.hpp:75-183
 *   Measurements<SV>                                   MeasurementsGB300<SV>
 *     LQ/measurements/MeasurementsLQubit.hpp:73-768,
 *     core/measurements/MeasurementsBase.hpp:56-93
 *   Observable / NamedObs / HermitianObs /             Observable<SV>, NamedObs<SV>, ...
 *   TensorProdObs / Hamiltonian / SparseHamiltonian
 *     core/observables/Observables.hpp:36-520,
 *     LQ/observables/ObservablesLQubit.hpp
 *   OpsData<SV> / JacobianData<SV>                     OpsData<SV> / JacobianData<SV>
 *     core/algorithms/JacobianData.hpp:39-393
 *   AdjointJacobian<SV>::adjointJacobian               AdjointJacobianGB300<SV>::adjointJacobian
 *     LQ/algorithms/AdjointJacobianLQubit.hpp:347-491
 *   LightningException (PL_ABORT)                      LightningException
 *     core/utils/Error.hpp:23-65
 *
 * (LQ = core/simulators/lightning_qubit.)  Differences that follow from the
 * state living in GPU memory: getData() is a device pointer; the host copy
 * is getDataVector() (by value) or CopyGpuDataToHost.  Calls return once
 * their results are on the host; gate calls may still be running on the
 * state vector's stream (or queued for fusion) when they return, and every
 * call that reads the state waits for them.
 */
#ifndef PL_GB300_HPP
#define PL_GB300_HPP

#include <complex>
#include <cstddef>
#include <cstdint>
#include <exception>
#include <memory>
#include <optional>
#include <random>
#include <span>
#include <string>
#include <type_traits>
#include <unordered_set>
#include <utility>
#include <vector>

#include "pl_gb300.h"

namespace Pennylane::LightningGB300 {

/* core/utils/Error.hpp:23-65: the exception PL_ABORT throws. */
class LightningException : public std::exception {
  public:
    explicit LightningException(std::string err_msg) noexcept : err_msg_{std::move(err_msg)} {}
    [[nodiscard]] const char *what() const noexcept override { return err_msg_.c_str(); }

  private:
    std::string err_msg_;
};

namespace detail {
inline void check(int rc) {
    if (rc != PLGB_OK) {
        const char *m = plgb_last_error();
        throw LightningException(m != nullptr && *m != '\0' ? m : "GB300 backend error");
    }
}
inline std::vector<int64_t> wires64(const std::vector<std::size_t> &w) { return {w.begin(), w.end()}; }
inline std::vector<uint8_t> bools8(const std::vector<bool> &v) { return {v.begin(), v.end()}; }
/* matrices cross the C ABI as interleaved complex128 */
template <class T> std::vector<double> to_c128(const std::complex<T> *m, std::size_t count) {
    std::vector<double> out(2 * count);
    for (std::size_t i = 0; i < count; i++) {
        out[2 * i] = static_cast<double>(m[i].real());
        out[2 * i + 1] = static_cast<double>(m[i].imag());
    }
    return out;
}
template <class T> std::vector<double> to_f64(const std::vector<T> &v) { return {v.begin(), v.end()}; }
/* names the dispatcher knows (DynamicDispatcher::hasGateOp) */
inline bool has_gate_op(const std::string &name) {
    static const std::unordered_set<std::string> names = [] {
        std::unordered_set<std::string> s;
        for (int c = 0;; c++) {
            const char *g = plgb_gate_name(c);
            if (g == nullptr) {
                break;
            }
            s.insert(g);
        }
        return s;
    }();
    return names.count(name) != 0;
}
} // namespace detail

/* StateVectorLQubitManaged<PrecisionT>: owns a 2^n complex register in GPU
 * memory (copyable: deep copy). */
template <class PrecisionT> class StateVectorGB300 {
    static_assert(std::is_same_v<PrecisionT, double> || std::is_same_v<PrecisionT, float>,
                  "StateVectorGB300 holds complex64 or complex128 amplitudes");

  public:
    using PrecisionType = PrecisionT;
    using ComplexT = std::complex<PrecisionT>;
    static constexpr int kPrecision = std::is_same_v<PrecisionT, double> ? 128 : 64;

    /* StateVectorLQubitManaged(num_qubits): |0...0> */
    explicit StateVectorGB300(std::size_t num_qubits) {
        plgb_sv *h = nullptr;
        detail::check(plgb_sv_create(static_cast<int>(num_qubits), kPrecision, &h));
        h_ = h;
    }
    /* StateVectorLQubitManaged(other_data, other_size) */
    StateVectorGB300(const ComplexT *other_data, std::size_t other_size)
        : StateVectorGB300(log2_exact(other_size)) {
        updateData(other_data, other_size);
    }
    StateVectorGB300(const StateVectorGB300 &other) {
        plgb_sv *h = nullptr;
        detail::check(plgb_sv_clone(other.h_, &h));
        h_ = h;
    }
    StateVectorGB300(StateVectorGB300 &&other) noexcept : h_{std::exchange(other.h_, nullptr)} {}
    StateVectorGB300 &operator=(const StateVectorGB300 &) = delete;
    StateVectorGB300 &operator=(StateVectorGB300 &&other) noexcept {
        std::swap(h_, other.h_);
        return *this;
    }
    ~StateVectorGB300() {
        if (h_ != nullptr) {
            plgb_sv_destroy(h_);
        }
    }

    [[nodiscard]] std::size_t getNumQubits() const {
        int n = 0;
        detail::check(plgb_sv_num_qubits(h_, &n));
        return static_cast<std::size_t>(n);
    }
    [[nodiscard]] std::size_t getLength() const {
        uint64_t len = 0;
        detail::check(plgb_sv_length(h_, &len));
        return static_cast<std::size_t>(len);
    }
    /* device pointer of the amplitudes (waits for queued gates) */
    [[nodiscard]] ComplexT *getData() {
        void *p = nullptr;
        detail::check(plgb_sv_device_ptr(h_, &p));
        return static_cast<ComplexT *>(p);
    }
    [[nodiscard]] plgb_sv *handle() const { return h_; }

    /* ---- state management (StateVectorLQubit.hpp:881-1036) ---- */
    void resetStateVector() { detail::check(plgb_sv_reset(h_)); }
    void setBasisState(const std::vector<std::size_t> &state, const std::vector<std::size_t> &wires) {
        const auto b = detail::wires64(state), w = detail::wires64(wires);
        detail::check(plgb_sv_set_basis_state(h_, b.data(), w.data(), static_cast<int>(w.size())));
    }
    void setStateVector(const ComplexT *state, const std::vector<std::size_t> &wires) {
        const auto w = detail::wires64(wires);
        detail::check(plgb_sv_set_state_vector(h_, state, uint64_t{1} << wires.size(), w.data(),
                                               static_cast<int>(w.size())));
    }
    void updateData(const ComplexT *new_data, std::size_t new_size) {
        detail::check(plgb_sv_update_data(h_, new_data, new_size));
    }
    void updateData(const std::vector<ComplexT> &new_data) { updateData(new_data.data(), new_data.size()); }
    /* host copy of the amplitudes */
    [[nodiscard]] std::vector<ComplexT> getDataVector() const {
        std::vector<ComplexT> out(getLength());
        CopyGpuDataToHost(out.data(), out.size());
        return out;
    }
    void CopyGpuDataToHost(ComplexT *host, std::size_t length) const {
        detail::check(plgb_sv_get_state(h_, host, length));
    }
    void collapse(std::size_t wire, bool branch) {
        detail::check(plgb_sv_collapse(h_, static_cast<int64_t>(wire), branch ? 1 : 0));
    }
    void normalize() { detail::check(plgb_sv_normalize(h_)); }

    /* ---- gates (StateVectorBase.hpp:109-204, StateVectorLQubit.hpp:378-482) ---- */
    void applyOperation(const std::string &opName, const std::vector<std::size_t> &wires, bool inverse = false,
                        const std::vector<PrecisionT> &params = {}) {
        const auto w = detail::wires64(wires);
        const auto p = detail::to_f64(params);
        detail::check(plgb_sv_apply_operation(h_, opName.c_str(), w.data(), static_cast<int>(w.size()),
                                              inverse ? 1 : 0, p.data(), static_cast<int>(p.size())));
    }
    void applyOperation(const std::string &opName, const std::vector<std::size_t> &controlled_wires,
                        const std::vector<bool> &controlled_values, const std::vector<std::size_t> &wires,
                        bool inverse = false, const std::vector<PrecisionT> &params = {}) {
        const auto cw = detail::wires64(controlled_wires), w = detail::wires64(wires);
        const auto cv = detail::bools8(controlled_values);
        if (controlled_wires.size() != controlled_values.size()) {
            throw LightningException("`controlled_wires` must have the same size as `controlled_values`.");
        }
        const auto p = detail::to_f64(params);
        detail::check(plgb_sv_apply_controlled_operation(h_, opName.c_str(), cw.data(), cv.data(),
                                                         static_cast<int>(cw.size()), w.data(),
                                                         static_cast<int>(w.size()), inverse ? 1 : 0, p.data(),
                                                         static_cast<int>(p.size())));
    }
    /* a named gate, or the matrix when the name is not a gate the backend knows */
    template <class Alloc>
    void applyOperation(const std::string &opName, const std::vector<std::size_t> &wires, bool inverse,
                        const std::vector<PrecisionT> &params, const std::vector<ComplexT, Alloc> &matrix) {
        if (detail::has_gate_op(opName)) {
            applyOperation(opName, wires, inverse, params);
        } else {
            applyMatrix(matrix.data(), wires, inverse);
        }
    }
    template <class Alloc>
    void applyOperation(const std::string &opName, const std::vector<std::size_t> &controlled_wires,
                        const std::vector<bool> &controlled_values, const std::vector<std::size_t> &wires,
                        bool inverse, const std::vector<PrecisionT> &params,
                        const std::vector<ComplexT, Alloc> &matrix) {
        if (!controlled_wires.empty()) {
            if (detail::has_gate_op(opName)) {
                applyOperation(opName, controlled_wires, controlled_values, wires, inverse, params);
            } else {
                applyControlledMatrix(matrix.data(), controlled_wires, controlled_values, wires, inverse);
            }
            return;
        }
        applyOperation(opName, wires, inverse, params, matrix);
    }
    void applyOperations(const std::vector<std::string> &ops, const std::vector<std::vector<std::size_t>> &ops_wires,
                         const std::vector<bool> &ops_adjoint,
                         const std::vector<std::vector<PrecisionT>> &ops_params) {
        if (ops.size() != ops_wires.size() || ops.size() != ops_adjoint.size() || ops.size() != ops_params.size()) {
            throw LightningException("Invalid arguments: number of operations, wires, inverses, and parameters "
                                     "must all be equal");
        }
        for (std::size_t i = 0; i < ops.size(); i++) {
            applyOperation(ops[i], ops_wires[i], ops_adjoint[i], ops_params[i]);
        }
    }
    void applyOperations(const std::vector<std::string> &ops, const std::vector<std::vector<std::size_t>> &ops_wires,
                         const std::vector<bool> &ops_adjoint) {
        if (ops.size() != ops_wires.size() || ops.size() != ops_adjoint.size()) {
            throw LightningException("Invalid arguments: number of operations, wires, and inverses must all be equal");
        }
        for (std::size_t i = 0; i < ops.size(); i++) {
            applyOperation(ops[i], ops_wires[i], ops_adjoint[i], {});
        }
    }
    /* row-major 2^k x 2^k matrix on `wires` (first wire = most significant) */
    void applyMatrix(const ComplexT *matrix, const std::vector<std::size_t> &wires, bool inverse = false) {
        const auto w = detail::wires64(wires);
        const auto m = detail::to_c128(matrix, std::size_t{1} << (2 * wires.size()));
        detail::check(plgb_sv_apply_matrix(h_, m.data(), w.data(), static_cast<int>(w.size()), inverse ? 1 : 0));
    }
    void applyMatrix(const std::vector<ComplexT> &matrix, const std::vector<std::size_t> &wires,
                     bool inverse = false) {
        if (matrix.size() != (std::size_t{1} << (2 * wires.size()))) {
            throw LightningException("The size of matrix does not match with the given number of wires");
        }
        applyMatrix(matrix.data(), wires, inverse);
    }
    void applyControlledMatrix(const ComplexT *matrix, const std::vector<std::size_t> &controlled_wires,
                               const std::vector<bool> &controlled_values, const std::vector<std::size_t> &wires,
                               bool inverse = false) {
        const auto cw = detail::wires64(controlled_wires), w = detail::wires64(wires);
        const auto cv = detail::bools8(controlled_values);
        const auto m = detail::to_c128(matrix, std::size_t{1} << (2 * wires.size()));
        detail::check(plgb_sv_apply_controlled_matrix(h_, m.data(), cw.data(), cv.data(), static_cast<int>(cw.size()),
                                                      w.data(), static_cast<int>(w.size()), inverse ? 1 : 0));
    }
    void applyPauliRot(const std::vector<std::size_t> &wires, bool inverse, const std::vector<PrecisionT> &params,
                       const std::string &word) {
        const auto w = detail::wires64(wires);
        detail::check(plgb_sv_apply_pauli_rot(h_, w.data(), static_cast<int>(w.size()), inverse ? 1 : 0,
                                              static_cast<double>(params.at(0)), word.c_str()));
    }
    /* G|psi> in place; returns the generator's scaling factor */
    [[nodiscard]] PrecisionT applyGenerator(const std::string &opName, const std::vector<std::size_t> &wires,
                                            bool adj = false) {
        return applyGenerator(opName, {}, {}, wires, adj);
    }
    [[nodiscard]] PrecisionT applyGenerator(const std::string &opName,
                                            const std::vector<std::size_t> &controlled_wires,
                                            const std::vector<bool> &controlled_values,
                                            const std::vector<std::size_t> &wires, bool adj = false) {
        const auto cw = detail::wires64(controlled_wires), w = detail::wires64(wires);
        const auto cv = detail::bools8(controlled_values);
        double scale = 0.0;
        detail::check(plgb_sv_apply_generator(h_, opName.c_str(), cw.data(), cv.data(), static_cast<int>(cw.size()),
                                              w.data(), static_cast<int>(w.size()), adj ? 1 : 0, &scale));
        return static_cast<PrecisionT>(scale);
    }

  private:
    static std::size_t log2_exact(std::size_t len) {
        std::size_t n = 0;
        while ((std::size_t{1} << n) < len) {
            n++;
        }
        if ((std::size_t{1} << n) != len) {
            throw LightningException("The size of provided data must be a power of 2.");
        }
        return n;
    }
    plgb_sv *h_{nullptr};
};

/* ---- observables (core/observables/Observables.hpp:36-520) ---- */
template <class StateVectorT> class Observable {
  public:
    using PrecisionT = typename StateVectorT::PrecisionType;
    using ComplexT = typename StateVectorT::ComplexT;
    virtual ~Observable() = default;
    [[nodiscard]] plgb_obs *handle() const { return h_.get(); }
    [[nodiscard]] std::vector<std::size_t> getWires() const {
        int nw = 0;
        detail::check(plgb_obs_wires(h_.get(), nullptr, 0, &nw));
        std::vector<int64_t> w(static_cast<std::size_t>(nw));
        detail::check(plgb_obs_wires(h_.get(), w.data(), nw, &nw));
        return {w.begin(), w.end()};
    }
    [[nodiscard]] std::string getObsName() const {
        std::string buf(4096, '\0');
        detail::check(plgb_obs_repr(h_.get(), buf.data(), buf.size()));
        buf.resize(std::char_traits<char>::length(buf.c_str()));
        return buf;
    }

  protected:
    Observable() = default;
    void adopt(plgb_obs *h) { h_.reset(h, [](plgb_obs *p) { plgb_obs_destroy(p); }); }

  private:
    std::shared_ptr<plgb_obs> h_;
};

template <class StateVectorT> class NamedObs final : public Observable<StateVectorT> {
  public:
    NamedObs(std::string obs_name, std::vector<std::size_t> wires) {
        const auto w = detail::wires64(wires);
        plgb_obs *h = nullptr;
        detail::check(plgb_obs_named(obs_name.c_str(), w.data(), static_cast<int>(w.size()), &h));
        this->adopt(h);
    }
};

template <class StateVectorT> class HermitianObs final : public Observable<StateVectorT> {
  public:
    using ComplexT = typename StateVectorT::ComplexT;
    HermitianObs(std::vector<ComplexT> matrix, std::vector<std::size_t> wires) {
        if (matrix.size() != (std::size_t{1} << (2 * wires.size()))) {
            throw LightningException("The size of matrix does not match with the given number of wires");
        }
        const auto w = detail::wires64(wires);
        const auto m = detail::to_c128(matrix.data(), matrix.size());
        plgb_obs *h = nullptr;
        detail::check(plgb_obs_hermitian(m.data(), w.data(), static_cast<int>(w.size()), &h));
        this->adopt(h);
    }
};

template <class StateVectorT> class TensorProdObs final : public Observable<StateVectorT> {
  public:
    explicit TensorProdObs(std::vector<std::shared_ptr<Observable<StateVectorT>>> obs) {
        std::vector<plgb_obs *> hs;
        for (const auto &o : obs) {
            hs.push_back(o->handle());
        }
        plgb_obs *h = nullptr;
        detail::check(plgb_obs_tensor_prod(hs.data(), static_cast<int>(hs.size()), &h));
        this->adopt(h);
    }
    static auto create(std::initializer_list<std::shared_ptr<Observable<StateVectorT>>> obs)
        -> std::shared_ptr<TensorProdObs<StateVectorT>> {
        return std::make_shared<TensorProdObs<StateVectorT>>(std::vector(obs));
    }
};

template <class StateVectorT> class Hamiltonian final : public Observable<StateVectorT> {
  public:
    using PrecisionT = typename StateVectorT::PrecisionType;
    Hamiltonian(std::vector<PrecisionT> coeffs, std::vector<std::shared_ptr<Observable<StateVectorT>>> obs) {
        if (coeffs.size() != obs.size()) {
            throw LightningException("Hamiltonian: the number of coefficients and observables must match");
        }
        std::vector<plgb_obs *> hs;
        for (const auto &o : obs) {
            hs.push_back(o->handle());
        }
        const auto c = detail::to_f64(coeffs);
        plgb_obs *h = nullptr;
        detail::check(plgb_obs_hamiltonian(c.data(), hs.data(), static_cast<int>(hs.size()), &h));
        this->adopt(h);
    }
    static auto create(std::initializer_list<PrecisionT> coeffs,
                       std::initializer_list<std::shared_ptr<Observable<StateVectorT>>> obs)
        -> std::shared_ptr<Hamiltonian<StateVectorT>> {
        return std::make_shared<Hamiltonian<StateVectorT>>(std::vector(coeffs), std::vector(obs));
    }
};

template <class StateVectorT> class SparseHamiltonian final : public Observable<StateVectorT> {
  public:
    using ComplexT = typename StateVectorT::ComplexT;
    /* CSR over the listed wires: data, column indices, row offsets */
    SparseHamiltonian(std::vector<ComplexT> data, std::vector<std::size_t> indices, std::vector<std::size_t> offsets,
                      std::vector<std::size_t> wires) {
        const auto d = detail::to_c128(data.data(), data.size());
        const auto ix = detail::wires64(indices), off = detail::wires64(offsets), w = detail::wires64(wires);
        plgb_obs *h = nullptr;
        detail::check(plgb_obs_sparse_hamiltonian(d.data(), ix.data(), static_cast<int64_t>(ix.size()), off.data(),
                                                  static_cast<int64_t>(off.size()), w.data(),
                                                  static_cast<int>(w.size()), &h));
        this->adopt(h);
    }
};

/* ---- measurements (MeasurementsLQubit.hpp:73-768) ---- */
template <class StateVectorT> class MeasurementsGB300 {
  public:
    using PrecisionT = typename StateVectorT::PrecisionType;
    using ComplexT = typename StateVectorT::ComplexT;

    explicit MeasurementsGB300(const StateVectorT &statevector) : sv_{statevector.handle()} {}

    /* MeasurementsBase::setSeed: samples drawn after it use this seed */
    void setSeed(std::optional<std::size_t> seed = std::nullopt) { seed_ = seed; }

    auto probs() -> std::vector<PrecisionT> { return probs_(nullptr, -1, num_qubits_()); }
    auto probs(const std::vector<std::size_t> &wires) -> std::vector<PrecisionT> {
        const auto w = detail::wires64(wires);
        return probs_(w.data(), static_cast<int>(w.size()), wires.size());
    }
    auto expval(const Observable<StateVectorT> &obs) -> PrecisionT {
        double out = 0.0;
        detail::check(plgb_meas_expval_obs(sv_, obs.handle(), &out));
        return static_cast<PrecisionT>(out);
    }
    auto expval(const std::string &operation, const std::vector<std::size_t> &wires) -> PrecisionT {
        const auto w = detail::wires64(wires);
        double out = 0.0;
        detail::check(plgb_meas_expval_named(sv_, operation.c_str(), w.data(), static_cast<int>(w.size()), &out));
        return static_cast<PrecisionT>(out);
    }
    auto expval(const std::vector<ComplexT> &matrix, const std::vector<std::size_t> &wires) -> PrecisionT {
        const auto w = detail::wires64(wires);
        const auto m = detail::to_c128(matrix.data(), matrix.size());
        double out = 0.0;
        detail::check(plgb_meas_expval_matrix(sv_, m.data(), w.data(), static_cast<int>(w.size()), &out));
        return static_cast<PrecisionT>(out);
    }
    /* CSR operator over the full register (MeasurementsLQubit.hpp:322-338) */
    template <class IndexT>
    auto expval(const IndexT *row_map_ptr, const IndexT row_map_size, const IndexT *entries_ptr,
                const ComplexT *values, const IndexT numNNZ) -> PrecisionT {
        const std::vector<int64_t> rows(row_map_ptr, row_map_ptr + row_map_size), cols(entries_ptr, entries_ptr + numNNZ);
        const auto v = detail::to_c128(values, static_cast<std::size_t>(numNNZ));
        double out = 0.0;
        detail::check(plgb_meas_expval_sparse(sv_, rows.data(), static_cast<int64_t>(row_map_size), cols.data(),
                                              v.data(), static_cast<int64_t>(numNNZ), &out));
        return static_cast<PrecisionT>(out);
    }
    auto var(const Observable<StateVectorT> &obs) -> PrecisionT {
        double out = 0.0;
        detail::check(plgb_meas_var_obs(sv_, obs.handle(), &out));
        return static_cast<PrecisionT>(out);
    }
    auto var(const std::string &operation, const std::vector<std::size_t> &wires) -> PrecisionT {
        const auto w = detail::wires64(wires);
        double out = 0.0;
        detail::check(plgb_meas_var_named(sv_, operation.c_str(), w.data(), static_cast<int>(w.size()), &out));
        return static_cast<PrecisionT>(out);
    }
    auto var(const std::vector<ComplexT> &matrix, const std::vector<std::size_t> &wires) -> PrecisionT {
        const auto w = detail::wires64(wires);
        const auto m = detail::to_c128(matrix.data(), matrix.size());
        double out = 0.0;
        detail::check(plgb_meas_var_matrix(sv_, m.data(), w.data(), static_cast<int>(w.size()), &out));
        return static_cast<PrecisionT>(out);
    }
    /* alias-method samples with std::mt19937, last wire fastest
     * (MeasurementsLQubit.hpp:646-679): num_samples x wires.size() bits */
    auto generate_samples(const std::vector<std::size_t> &wires, std::size_t num_samples) -> std::vector<std::size_t> {
        const auto w = detail::wires64(wires);
        return samples_(w.data(), static_cast<int>(w.size()), wires.size(), num_samples);
    }
    auto generate_samples(std::size_t num_samples) -> std::vector<std::size_t> {
        return samples_(nullptr, -1, num_qubits_(), num_samples);
    }

  private:
    std::size_t num_qubits_() const {
        int n = 0;
        detail::check(plgb_sv_num_qubits(sv_, &n));
        return static_cast<std::size_t>(n);
    }
    std::vector<PrecisionT> probs_(const int64_t *w, int nw, std::size_t nbits) {
        std::vector<double> out(std::size_t{1} << nbits);
        detail::check(plgb_meas_probs(sv_, w, nw, out.data()));
        return {out.begin(), out.end()};
    }
    std::vector<std::size_t> samples_(const int64_t *w, int nw, std::size_t nbits, std::size_t shots) {
        /* MeasurementsBase::generate_samples without a seed draws one from
         * std::random_device */
        const uint64_t seed = seed_.has_value() ? static_cast<uint64_t>(*seed_) : std::random_device{}();
        std::vector<int64_t> out(shots * nbits);
        detail::check(plgb_meas_generate_samples(sv_, w, nw, static_cast<int64_t>(shots), seed, out.data()));
        return {out.begin(), out.end()};
    }
    plgb_sv *sv_;
    std::optional<std::size_t> seed_;
};

/* ---- algorithms (core/algorithms/JacobianData.hpp:39-393) ---- */
template <class StateVectorT> class OpsData {
  public:
    using PrecisionT = typename StateVectorT::PrecisionType;
    using ComplexT = typename StateVectorT::ComplexT;

    OpsData(std::vector<std::string> ops_name, const std::vector<std::vector<PrecisionT>> &ops_params,
            std::vector<std::vector<std::size_t>> ops_wires, std::vector<bool> ops_inverses,
            std::vector<std::vector<ComplexT>> ops_matrices,
            std::vector<std::vector<std::size_t>> ops_controlled_wires,
            std::vector<std::vector<bool>> ops_controlled_values)
        : name_{std::move(ops_name)}, params_{ops_params}, wires_{std::move(ops_wires)},
          inverses_{std::move(ops_inverses)}, matrices_{std::move(ops_matrices)},
          cwires_{std::move(ops_controlled_wires)}, cvals_{std::move(ops_controlled_values)} {
        build_();
    }
    OpsData(std::vector<std::string> ops_name, const std::vector<std::vector<PrecisionT>> &ops_params,
            std::vector<std::vector<std::size_t>> ops_wires, std::vector<bool> ops_inverses,
            std::vector<std::vector<ComplexT>> ops_matrices)
        : OpsData(ops_name, ops_params, std::move(ops_wires), std::move(ops_inverses), std::move(ops_matrices),
                  std::vector<std::vector<std::size_t>>(ops_name.size()),
                  std::vector<std::vector<bool>>(ops_name.size())) {}
    OpsData(const std::vector<std::string> &ops_name, const std::vector<std::vector<PrecisionT>> &ops_params,
            std::vector<std::vector<std::size_t>> ops_wires, std::vector<bool> ops_inverses)
        : OpsData(ops_name, ops_params, std::move(ops_wires), std::move(ops_inverses),
                  std::vector<std::vector<ComplexT>>(ops_name.size())) {}

    [[nodiscard]] std::size_t getSize() const { return name_.size(); }
    [[nodiscard]] const std::vector<std::string> &getOpsName() const { return name_; }
    [[nodiscard]] const std::vector<std::vector<PrecisionT>> &getOpsParams() const { return params_; }
    [[nodiscard]] const std::vector<std::vector<std::size_t>> &getOpsWires() const { return wires_; }
    [[nodiscard]] const std::vector<std::vector<std::size_t>> &getOpsControlledWires() const { return cwires_; }
    [[nodiscard]] const std::vector<std::vector<bool>> &getOpsControlledValues() const { return cvals_; }
    [[nodiscard]] const std::vector<bool> &getOpsInverses() const { return inverses_; }
    [[nodiscard]] const std::vector<std::vector<ComplexT>> &getOpsMatrices() const { return matrices_; }
    [[nodiscard]] std::size_t getNumParOps() const { return num_par_ops_; }
    [[nodiscard]] std::size_t getNumNonParOps() const { return name_.size() - num_par_ops_; }
    [[nodiscard]] std::size_t getTotalNumParams() const {
        std::size_t t = 0;
        for (const auto &p : params_) {
            t += p.size();
        }
        return t;
    }
    [[nodiscard]] plgb_ops *handle() const { return h_.get(); }

  private:
    void build_() {
        const std::size_t n = name_.size();
        if (params_.size() != n || wires_.size() != n || inverses_.size() != n || matrices_.size() != n ||
            cwires_.size() != n || cvals_.size() != n) {
            throw LightningException("OpsData: every operation field needs one entry per operation");
        }
        std::vector<const char *> names;
        std::vector<double> params, mats;
        std::vector<int> nparams, nwires, ncwires;
        std::vector<int64_t> wires, matsz, cwires;
        std::vector<uint8_t> inv, cvals;
        for (std::size_t k = 0; k < n; k++) {
            names.push_back(name_[k].c_str());
            num_par_ops_ += params_[k].empty() ? 0 : 1;
            nparams.push_back(static_cast<int>(params_[k].size()));
            params.insert(params.end(), params_[k].begin(), params_[k].end());
            nwires.push_back(static_cast<int>(wires_[k].size()));
            wires.insert(wires.end(), wires_[k].begin(), wires_[k].end());
            inv.push_back(inverses_[k] ? 1 : 0);
            matsz.push_back(static_cast<int64_t>(matrices_[k].size()));
            const auto m = detail::to_c128(matrices_[k].data(), matrices_[k].size());
            mats.insert(mats.end(), m.begin(), m.end());
            ncwires.push_back(static_cast<int>(cwires_[k].size()));
            cwires.insert(cwires.end(), cwires_[k].begin(), cwires_[k].end());
            cvals.insert(cvals.end(), cvals_[k].begin(), cvals_[k].end());
        }
        plgb_ops *h = nullptr;
        detail::check(plgb_ops_create(static_cast<int>(n), names.data(), params.data(), nparams.data(), wires.data(),
                                      nwires.data(), inv.data(), mats.data(), matsz.data(), cwires.data(),
                                      ncwires.data(), cvals.data(), &h));
        h_.reset(h, [](plgb_ops *p) { plgb_ops_destroy(p); });
    }
    std::vector<std::string> name_;
    std::vector<std::vector<PrecisionT>> params_;
    std::vector<std::vector<std::size_t>> wires_;
    std::vector<bool> inverses_;
    std::vector<std::vector<ComplexT>> matrices_;
    std::vector<std::vector<std::size_t>> cwires_;
    std::vector<std::vector<bool>> cvals_;
    std::size_t num_par_ops_{0};
    std::shared_ptr<plgb_ops> h_;
};

template <class StateVectorT> class JacobianData {
  public:
    using ComplexT = typename StateVectorT::ComplexT;
    /* psi: host amplitudes of the initial state (num_elem of them), or
     * nullptr to start from the ref_data state passed to adjointJacobian */
    JacobianData(std::size_t num_params, std::size_t num_elem, const ComplexT *sv_ptr,
                 std::vector<std::shared_ptr<Observable<StateVectorT>>> obs, OpsData<StateVectorT> ops,
                 std::vector<std::size_t> trainP)
        : num_parameters_{num_params}, num_elements_{num_elem}, psi_{sv_ptr}, observables_{std::move(obs)},
          operations_{std::move(ops)}, trainable_params_{std::move(trainP)} {}
    [[nodiscard]] std::size_t getNumParams() const { return num_parameters_; }
    [[nodiscard]] std::size_t getSizeStateVec() const { return num_elements_; }
    [[nodiscard]] const ComplexT *getPtrStateVec() const { return psi_; }
    [[nodiscard]] const std::vector<std::shared_ptr<Observable<StateVectorT>>> &getObservables() const {
        return observables_;
    }
    [[nodiscard]] std::size_t getNumObservables() const { return observables_.size(); }
    [[nodiscard]] const OpsData<StateVectorT> &getOperations() const { return operations_; }
    [[nodiscard]] const std::vector<std::size_t> &getTrainableParams() const { return trainable_params_; }
    [[nodiscard]] bool hasTrainableParams() const { return !trainable_params_.empty(); }

  private:
    std::size_t num_parameters_, num_elements_;
    const ComplexT *psi_;
    std::vector<std::shared_ptr<Observable<StateVectorT>>> observables_;
    OpsData<StateVectorT> operations_;
    std::vector<std::size_t> trainable_params_;
};

/* AdjointJacobian<SV>::adjointJacobian (AdjointJacobianLQubit.hpp:347-491):
 * jac is row-major [observable][trainable parameter]. */
template <class StateVectorT> class AdjointJacobianGB300 {
  public:
    using PrecisionT = typename StateVectorT::PrecisionType;

    void adjointJacobian(std::span<PrecisionT> jac, const JacobianData<StateVectorT> &jd,
                         const StateVectorT &ref_data, bool apply_operations = false) {
        const auto &obs = jd.getObservables();
        const auto &tp = jd.getTrainableParams();
        if (jac.size() != obs.size() * tp.size()) {
            throw LightningException("The size of preallocated jacobian must be same as the number of trainable "
                                     "parameters times the number of observables provided.");
        }
        if (tp.empty()) {
            return;
        }
        std::optional<StateVectorT> from_host;
        if (jd.getPtrStateVec() != nullptr) {
            from_host.emplace(jd.getPtrStateVec(), jd.getSizeStateVec());
        }
        const StateVectorT &start = from_host.has_value() ? *from_host : ref_data;
        std::vector<plgb_obs *> hs;
        for (const auto &o : obs) {
            hs.push_back(o->handle());
        }
        const std::vector<int64_t> t(tp.begin(), tp.end());
        std::vector<double> out(jac.size());
        detail::check(plgb_adjoint_jacobian(start.handle(), hs.data(), static_cast<int>(hs.size()),
                                            jd.getOperations().handle(), t.data(), static_cast<int>(t.size()),
                                            apply_operations ? 1 : 0, out.data()));
        for (std::size_t i = 0; i < out.size(); i++) {
            jac[i] = static_cast<PrecisionT>(out[i]);
        }
    }
};

} // namespace Pennylane::LightningGB300

#endif
