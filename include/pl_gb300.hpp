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

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstddef>
#include <cstdint>
#include <exception>
#include <numeric>
#include <memory>
#include <optional>
#include <random>
#include <span>
#include <string>
#include <type_traits>
#include <unordered_map>
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

/* Eigen-decomposition of a Hermitian matrix (row-major, dim x dim) by the
 * cyclic Jacobi method (Golub and Van Loan, Matrix Computations, 4th ed.,
 * section 8.5), carried to complex Hermitian matrices by a phase that makes
 * each pivot real: with a_pq = r e^{i phi}, G = diag(1, e^{-i phi}) J(c, s)
 * zeroes a_pq in G^H A G, (c, s) the real symmetric Jacobi rotation of
 * [[a_pp, r], [r, a_qq]].  Returns the eigenvalues ascending in w and the
 * matching orthonormal eigenvectors as the columns of v (row-major).  Used for
 * the shot-based measurement of Hermitian observables, whose matrices span a
 * few wires. */
inline void hermitian_eigh(std::vector<std::complex<double>> a, std::size_t dim, std::vector<double> &w,
                           std::vector<std::complex<double>> &v) {
    using C = std::complex<double>;
    if (a.size() != dim * dim) {
        throw LightningException("hermitian_eigh: the matrix must be dim x dim");
    }
    std::vector<C> vv(dim * dim, C{0.0, 0.0});
    for (std::size_t i = 0; i < dim; i++) {
        vv[i * dim + i] = 1.0;
    }
    double total = 0.0;
    for (const C &x : a) {
        total += std::norm(x);
    }
    auto off_diagonal = [&] {
        double s = 0.0;
        for (std::size_t i = 0; i < dim; i++) {
            for (std::size_t j = 0; j < dim; j++) {
                s += i != j ? std::norm(a[i * dim + j]) : 0.0;
            }
        }
        return s;
    };
    for (int sweep = 0; sweep < 64 && total > 0.0 && off_diagonal() > 1e-32 * total; sweep++) {
        for (std::size_t p = 0; p + 1 < dim; p++) {
            for (std::size_t q = p + 1; q < dim; q++) {
                const C apq = a[p * dim + q];
                const double r = std::abs(apq);
                if (r <= 1e-300) {
                    continue;
                }
                const C ph = apq / r;
                const double tau = (a[q * dim + q].real() - a[p * dim + p].real()) / (2.0 * r);
                const double t = (tau >= 0.0 ? 1.0 : -1.0) / (std::abs(tau) + std::sqrt(1.0 + tau * tau));
                const double c = 1.0 / std::sqrt(1.0 + t * t), s = t * c;
                const C g_qp = -s * std::conj(ph), g_qq = c * std::conj(ph); // G: (p,p) c, (p,q) s
                for (std::size_t k = 0; k < dim; k++) {                      // A <- A G, V <- V G
                    for (C *m : {a.data(), vv.data()}) {
                        const C xp = m[k * dim + p], xq = m[k * dim + q];
                        m[k * dim + p] = c * xp + g_qp * xq;
                        m[k * dim + q] = s * xp + g_qq * xq;
                    }
                }
                for (std::size_t k = 0; k < dim; k++) { // A <- G^H A
                    const C xp = a[p * dim + k], xq = a[q * dim + k];
                    a[p * dim + k] = c * xp + std::conj(g_qp) * xq;
                    a[q * dim + k] = s * xp + std::conj(g_qq) * xq;
                }
                a[p * dim + q] = a[q * dim + p] = C{0.0, 0.0};
            }
        }
    }
    std::vector<std::size_t> order(dim);
    std::iota(order.begin(), order.end(), std::size_t{0});
    std::stable_sort(order.begin(), order.end(),
                     [&](std::size_t i, std::size_t j) { return a[i * dim + i].real() < a[j * dim + j].real(); });
    w.resize(dim);
    v.assign(dim * dim, C{0.0, 0.0});
    for (std::size_t k = 0; k < dim; k++) {
        w[k] = a[order[k] * dim + order[k]].real();
        for (std::size_t i = 0; i < dim; i++) {
            v[i * dim + k] = vv[i * dim + order[k]];
        }
    }
}

/* kron of eigenvalue lists, first list most significant */
template <class T> std::vector<T> kron_values(const std::vector<std::vector<T>> &lists) {
    std::vector<T> out{T{1}};
    for (const auto &l : lists) {
        std::vector<T> next;
        next.reserve(out.size() * l.size());
        for (const T x : out) {
            for (const T y : l) {
                next.push_back(x * y);
            }
        }
        out.swap(next);
    }
    return out;
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
    /* Observable::applyInPlaceShots (Observables.hpp:76): rotates `sv` into
     * the observable's eigenbasis and returns, per factor, its eigenvalues
     * and the wires to sample (shot-based expval / var / probs) */
    virtual void applyInPlaceShots([[maybe_unused]] StateVectorT &sv,
                                   [[maybe_unused]] std::vector<std::vector<PrecisionT>> &eigenValues,
                                   [[maybe_unused]] std::vector<std::size_t> &ob_wires) const {
        throw LightningException("This observable does not support shot measurement.");
    }
    /* the terms of a tensor product or a Hamiltonian, and a Hamiltonian's
     * coefficients (Observables.hpp:94-104) */
    [[nodiscard]] virtual auto getObs() const -> std::vector<std::shared_ptr<Observable<StateVectorT>>> { return {}; }
    [[nodiscard]] virtual auto getCoeffs() const -> std::vector<PrecisionT> { return {}; }

  protected:
    Observable() = default;
    void adopt(plgb_obs *h) { h_.reset(h, [](plgb_obs *p) { plgb_obs_destroy(p); }); }

  private:
    std::shared_ptr<plgb_obs> h_;
};

template <class StateVectorT> class NamedObs final : public Observable<StateVectorT> {
  public:
    using PrecisionT = typename StateVectorT::PrecisionType;
    NamedObs(std::string obs_name, std::vector<std::size_t> wires) : name_{std::move(obs_name)}, wires_{wires} {
        const auto w = detail::wires64(wires);
        plgb_obs *h = nullptr;
        detail::check(plgb_obs_named(name_.c_str(), w.data(), static_cast<int>(w.size()), &h));
        this->adopt(h);
    }
    /* Observables.hpp:176-202: X by H, Y by Z S H, Hadamard by RY(-pi/4);
     * eigenvalues (1, -1), Identity (1, 1) */
    void applyInPlaceShots(StateVectorT &sv, std::vector<std::vector<PrecisionT>> &eigenValues,
                           std::vector<std::size_t> &ob_wires) const override {
        ob_wires.assign(1, wires_.at(0));
        eigenValues.clear();
        if (name_ == "PauliX") {
            sv.applyOperation("Hadamard", wires_, false);
        } else if (name_ == "PauliY") {
            sv.applyOperations({"PauliZ", "S", "Hadamard"}, {wires_, wires_, wires_}, {false, false, false});
        } else if (name_ == "Hadamard") {
            sv.applyOperation("RY", wires_, false, {static_cast<PrecisionT>(-std::acos(-1.0) / 4.0)});
        } else if (name_ != "PauliZ" && name_ != "Identity") {
            throw LightningException("Provided NamedObs does not support shot measurement.");
        }
        eigenValues.push_back(name_ == "Identity" ? std::vector<PrecisionT>{1, 1} : std::vector<PrecisionT>{1, -1});
    }

  private:
    std::string name_;
    std::vector<std::size_t> wires_;
};

template <class StateVectorT> class HermitianObs final : public Observable<StateVectorT> {
  public:
    using PrecisionT = typename StateVectorT::PrecisionType;
    using ComplexT = typename StateVectorT::ComplexT;
    HermitianObs(std::vector<ComplexT> matrix, std::vector<std::size_t> wires) : matrix_{matrix}, wires_{wires} {
        if (matrix.size() != (std::size_t{1} << (2 * wires.size()))) {
            throw LightningException("The size of matrix does not match with the given number of wires");
        }
        const auto w = detail::wires64(wires);
        const auto m = detail::to_c128(matrix.data(), matrix.size());
        plgb_obs *h = nullptr;
        detail::check(plgb_obs_hermitian(m.data(), w.data(), static_cast<int>(w.size()), &h));
        this->adopt(h);
    }
    /* Observables.hpp:290-302: the matrix's eigenvectors rotated onto the
     * computational basis (U = V^H on the observable's wires), eigenvalues
     * ascending; the decomposition is computed once */
    void applyInPlaceShots(StateVectorT &sv, std::vector<std::vector<PrecisionT>> &eigenValues,
                           std::vector<std::size_t> &ob_wires) const override {
        if (eigen_values_.empty()) {
            const std::size_t dim = std::size_t{1} << wires_.size();
            std::vector<std::complex<double>> a(matrix_.begin(), matrix_.end()), vecs;
            std::vector<double> vals;
            detail::hermitian_eigh(a, dim, vals, vecs);
            unitary_.resize(dim * dim);
            for (std::size_t i = 0; i < dim; i++) {
                for (std::size_t j = 0; j < dim; j++) {
                    unitary_[i * dim + j] = static_cast<ComplexT>(std::conj(vecs[j * dim + i]));
                }
            }
            eigen_values_.assign(vals.begin(), vals.end());
        }
        ob_wires = wires_;
        sv.applyMatrix(unitary_, wires_);
        eigenValues.assign(1, eigen_values_);
    }

  private:
    std::vector<ComplexT> matrix_;
    std::vector<std::size_t> wires_;
    mutable std::vector<PrecisionT> eigen_values_;
    mutable std::vector<ComplexT> unitary_;
};

template <class StateVectorT> class TensorProdObs final : public Observable<StateVectorT> {
  public:
    using PrecisionT = typename StateVectorT::PrecisionType;
    explicit TensorProdObs(std::vector<std::shared_ptr<Observable<StateVectorT>>> obs) : obs_{obs} {
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
    [[nodiscard]] auto getObs() const -> std::vector<std::shared_ptr<Observable<StateVectorT>>> override {
        return obs_;
    }
    /* Observables.hpp:428-448: every factor rotated in turn; a multi-wire
     * Hermitian factor contributes all of its wires and its whole eigenvalue
     * list (the reference keeps its first wire only) */
    void applyInPlaceShots(StateVectorT &sv, std::vector<std::vector<PrecisionT>> &eigenValues,
                           std::vector<std::size_t> &ob_wires) const override {
        eigenValues.clear();
        ob_wires.clear();
        for (const auto &ob : obs_) {
            if (!ob->getCoeffs().empty() || ob->getObsName().find("Hamiltonian") != std::string::npos) {
                throw LightningException("Hamiltonian observables as a term of an TensorProd observable do not "
                                         "support shot measurement.");
            }
        }
        for (const auto &ob : obs_) {
            std::vector<std::vector<PrecisionT>> ev;
            std::vector<std::size_t> w;
            ob->applyInPlaceShots(sv, ev, w);
            ob_wires.insert(ob_wires.end(), w.begin(), w.end());
            eigenValues.push_back(detail::kron_values(ev));
        }
    }

  private:
    std::vector<std::shared_ptr<Observable<StateVectorT>>> obs_;
};

template <class StateVectorT> class Hamiltonian final : public Observable<StateVectorT> {
  public:
    using PrecisionT = typename StateVectorT::PrecisionType;
    Hamiltonian(std::vector<PrecisionT> coeffs, std::vector<std::shared_ptr<Observable<StateVectorT>>> obs)
        : coeffs_{coeffs}, obs_{obs} {
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
    [[nodiscard]] auto getObs() const -> std::vector<std::shared_ptr<Observable<StateVectorT>>> override {
        return obs_;
    }
    [[nodiscard]] auto getCoeffs() const -> std::vector<PrecisionT> override { return coeffs_; }

  private:
    std::vector<PrecisionT> coeffs_;
    std::vector<std::shared_ptr<Observable<StateVectorT>>> obs_;
};

template <class StateVectorT> class SparseHamiltonian final : public Observable<StateVectorT> {
  public:
    using PrecisionT = typename StateVectorT::PrecisionType;
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
    /* MeasurementsBase.hpp:164-167 */
    void applyInPlaceShots([[maybe_unused]] StateVectorT &sv,
                           [[maybe_unused]] std::vector<std::vector<PrecisionT>> &eigenValues,
                           [[maybe_unused]] std::vector<std::size_t> &ob_wires) const override {
        throw LightningException("SparseHamiltonian observables do not support shot measurement.");
    }
};

/* ---- measurements (MeasurementsLQubit.hpp:73-768) ---- */
template <class StateVectorT> class MeasurementsGB300 {
  public:
    using PrecisionT = typename StateVectorT::PrecisionType;
    using ComplexT = typename StateVectorT::ComplexT;

    explicit MeasurementsGB300(const StateVectorT &statevector) : svp_{&statevector}, sv_{statevector.handle()} {}

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
    /* Metropolis-Hastings samples, kernel "Local" or "NonZeroRandom"
     * (MeasurementsLQubit.hpp:551-594): num_samples x num_qubits bits */
    auto generate_samples_metropolis(const std::string &kernelname, std::size_t num_burnin,
                                     std::size_t num_samples) -> std::vector<std::size_t> {
        const uint64_t seed = seed_.has_value() ? static_cast<uint64_t>(*seed_) : std::random_device{}();
        std::vector<int64_t> out(num_samples * num_qubits_());
        detail::check(plgb_meas_generate_mcmc_samples(sv_, kernelname.c_str(), static_cast<int64_t>(num_burnin),
                                                      static_cast<int64_t>(num_samples), seed, out.data()));
        return {out.begin(), out.end()};
    }
    auto sample(const std::size_t &num_shots) -> std::vector<std::size_t> { return generate_samples(num_shots); }

    /* ---- shot-based measurements (MeasurementsBase.hpp:150-420) ---- */
    /* probabilities of the sampled basis states over `wires` */
    auto probs(const std::vector<std::size_t> &wires, std::size_t num_shots) -> std::vector<PrecisionT> {
        const std::size_t n = num_qubits_();
        const auto smp = generate_samples(num_shots);
        std::vector<std::size_t> hits(std::size_t{1} << wires.size(), 0);
        for (std::size_t i = 0; i < num_shots; i++) {
            std::size_t idx = 0;
            for (const std::size_t w : wires) {
                idx = (idx << 1) | smp[i * n + w];
            }
            hits[idx]++;
        }
        std::vector<PrecisionT> out(hits.size());
        for (std::size_t k = 0; k < hits.size(); k++) {
            out[k] = static_cast<PrecisionT>(hits[k]) / static_cast<PrecisionT>(num_shots);
        }
        return out;
    }
    auto probs(std::size_t num_shots) -> std::vector<PrecisionT> {
        std::vector<std::size_t> all(num_qubits_());
        std::iota(all.begin(), all.end(), std::size_t{0});
        return probs(all, num_shots);
    }
    /* eigenvalue of the observable for each sampled shot: the state copied,
     * rotated into the observable's eigenbasis, the whole register sampled
     * with this object's seed (MeasurementsBase.hpp:195-225, 477-518) */
    auto measure_with_samples(const Observable<StateVectorT> &obs, const std::size_t &num_shots,
                              const std::vector<std::size_t> &shot_range) -> std::vector<PrecisionT> {
        StateVectorT rotated(*svp_);
        std::vector<std::vector<PrecisionT>> eigen_values;
        std::vector<std::size_t> obs_wires;
        obs.applyInPlaceShots(rotated, eigen_values, obs_wires);
        MeasurementsGB300<StateVectorT> m(rotated);
        m.setSeed(seed_);
        const std::size_t n = num_qubits_();
        const auto smp = m.generate_samples(num_shots);
        const auto values = detail::kron_values(eigen_values);
        std::vector<std::size_t> shots = shot_range;
        if (shots.empty()) {
            shots.resize(num_shots);
            std::iota(shots.begin(), shots.end(), std::size_t{0});
        }
        std::vector<PrecisionT> out;
        out.reserve(shots.size());
        for (const std::size_t i : shots) {
            if (i >= num_shots) {
                throw LightningException("shot_range holds a shot index beyond num_shots");
            }
            std::size_t idx = 0;
            for (const std::size_t w : obs_wires) {
                idx = (idx << 1) | smp[i * n + w];
            }
            out.push_back(values.at(idx));
        }
        return out;
    }
    /* a Hamiltonian term by term, its terms and other observables by
     * sampling (MeasurementsBase.hpp:159-183) */
    auto expval(const Observable<StateVectorT> &obs, const std::size_t &num_shots,
                const std::vector<std::size_t> &shot_range = {}) -> PrecisionT {
        if (dynamic_cast<const SparseHamiltonian<StateVectorT> *>(&obs) != nullptr) {
            throw LightningException("SparseHamiltonian observables do not support shot measurement.");
        }
        if (const auto *h = dynamic_cast<const Hamiltonian<StateVectorT> *>(&obs)) {
            const auto coeffs = h->getCoeffs();
            const auto terms = h->getObs();
            PrecisionT result{0};
            for (std::size_t k = 0; k < coeffs.size(); k++) {
                result += coeffs[k] * expval(*terms[k], num_shots, shot_range);
            }
            return result;
        }
        const auto v = measure_with_samples(obs, num_shots, shot_range);
        return std::accumulate(v.begin(), v.end(), PrecisionT{0}) / static_cast<PrecisionT>(v.size());
    }
    /* eigenvalues of the observable drawn in num_shots shots
     * (MeasurementsBase.hpp:382-391) */
    auto sample(const Observable<StateVectorT> &obs, const std::size_t &num_shots) -> std::vector<PrecisionT> {
        no_hamiltonian_(obs);
        return measure_with_samples(obs, num_shots, {});
    }
    /* eigenvalue -> occurrences, and basis state -> occurrences
     * (MeasurementsBase.hpp:411-460) */
    auto counts(const Observable<StateVectorT> &obs, const std::size_t &num_shots)
        -> std::unordered_map<PrecisionT, std::size_t> {
        std::unordered_map<PrecisionT, std::size_t> out;
        for (const PrecisionT v : sample(obs, num_shots)) {
            out[v]++;
        }
        return out;
    }
    auto counts(const std::size_t &num_shots) -> std::unordered_map<std::size_t, std::size_t> {
        const std::size_t n = num_qubits_();
        const auto smp = generate_samples(num_shots);
        std::unordered_map<std::size_t, std::size_t> out;
        for (std::size_t s = 0; s < num_shots; s++) {
            std::size_t idx = 0;
            for (std::size_t w = 0; w < n; w++) {
                idx = (idx << 1) | smp[s * n + w];
            }
            out[idx]++;
        }
        return out;
    }
    /* probabilities of the observable's eigenbasis states over its wires,
     * analytic or from num_shots samples (MeasurementsBase.hpp:283-318) */
    auto probs(const Observable<StateVectorT> &obs, std::size_t num_shots = 0) -> std::vector<PrecisionT> {
        no_hamiltonian_(obs);
        StateVectorT rotated(*svp_);
        std::vector<std::vector<PrecisionT>> eigen_values;
        std::vector<std::size_t> obs_wires;
        obs.applyInPlaceShots(rotated, eigen_values, obs_wires);
        MeasurementsGB300<StateVectorT> m(rotated);
        m.setSeed(seed_);
        return num_shots > 0 ? m.probs(obs_wires, num_shots) : m.probs(obs_wires);
    }
    /* a Hamiltonian as sum_k c_k^2 var(term_k), as the reference computes it
     * (MeasurementsBase.hpp:239-268) */
    auto var(const Observable<StateVectorT> &obs, const std::size_t &num_shots) -> PrecisionT {
        if (dynamic_cast<const SparseHamiltonian<StateVectorT> *>(&obs) != nullptr) {
            throw LightningException("SparseHamiltonian observables do not support shot measurement.");
        }
        if (const auto *h = dynamic_cast<const Hamiltonian<StateVectorT> *>(&obs)) {
            const auto coeffs = h->getCoeffs();
            const auto terms = h->getObs();
            PrecisionT result{0};
            for (std::size_t k = 0; k < coeffs.size(); k++) {
                result += coeffs[k] * coeffs[k] * var(*terms[k], num_shots);
            }
            return result;
        }
        const auto v = measure_with_samples(obs, num_shots, {});
        const auto len = static_cast<PrecisionT>(v.size());
        const PrecisionT mean = std::accumulate(v.begin(), v.end(), PrecisionT{0}) / len;
        const PrecisionT mean_sq =
            std::accumulate(v.begin(), v.end(), PrecisionT{0}, [](PrecisionT a, PrecisionT x) { return a + x * x; }) /
            len;
        return mean_sq - mean * mean;
    }

  private:
    static void no_hamiltonian_(const Observable<StateVectorT> &obs) {
        if (dynamic_cast<const Hamiltonian<StateVectorT> *>(&obs) != nullptr ||
            dynamic_cast<const SparseHamiltonian<StateVectorT> *>(&obs) != nullptr) {
            throw LightningException("Hamiltonian and Sparse Hamiltonian do not support samples().");
        }
    }
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
    const StateVectorT *svp_;
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
