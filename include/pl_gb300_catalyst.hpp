/*
 * Catalyst runtime device over the GB300 backend: the simulator Catalyst's
 * runtime drives for a `lightning.qubit` program (qubit allocation and
 * release, gates, mid-circuit measurements, observables, analytic and
 * shot-based measurements, tape recording and the adjoint gradient), with the
 * method names, argument meaning and error messages of
 *
 *   LightningSimulator   core/simulators/lightning_qubit/catalyst/LightningSimulator.hpp:35-197,
 *                        LightningSimulator.cpp:29-975
 *   QubitManager         core/catalyst/LightningQubitManager.hpp:37-196
 *   LightningObsManager  core/simulators/lightning_qubit/catalyst/LightningObsManager.hpp:39-205
 *
 * over the C++ layer of pl_gb300.hpp (the state lives in GPU memory).
 *
 * Catalyst's own runtime headers (QuantumDevice.hpp, DataView.hpp, Types.h,
 * CacheManager.hpp) are not part of the reference's sources, so this device
 * does not derive from Catalyst::Runtime::QuantumDevice: it defines the few
 * runtime types its methods take (qubit and observable ids, the result
 * pointer, the observable id enum and a strided DataView) in its own
 * namespace.  A Catalyst build binds it with a thin subclass of QuantumDevice
 * whose overrides forward to these methods.
 *
 * Header-only; link against libplgb300.so.  Complex128 amplitudes, like the
 * reference's device.
 */
#ifndef PL_GB300_CATALYST_HPP
#define PL_GB300_CATALYST_HPP

#include <cstdint>
#include <iterator>
#include <map>
#include <memory>
#include <optional>
#include <random>
#include <set>
#include <string>
#include <tuple>
#include <unordered_map>
#include <utility>
#include <vector>

#include "pl_gb300.hpp"

namespace Pennylane::LightningGB300::Catalyst {

/* ---- runtime types the device's methods take ---- */
using QubitIdType = intptr_t; // program qubit id
using ObsIdType = intptr_t;   // key of a cached observable
using Result = bool *;        // mid-circuit measurement outcome

/* named observables a program can request */
enum class ObsId : int8_t { Identity = 0, PauliX, PauliY, PauliZ, Hadamard, Hermitian };

/* how an observable was measured while the tape was recording */
enum class MeasurementsT : uint8_t { None = 0, Expval, Var };

/* A rank-R strided view of caller-owned memory (a memref): element
 * (i_0, ..., i_{R-1}) sits at data[offset + sum_k i_k * strides[k]];
 * iteration runs over the elements in row-major order of the indices. */
template <class T, std::size_t R> class DataView {
  public:
    DataView(T *data, std::size_t offset, const std::size_t *sizes, const std::size_t *strides)
        : data_{data}, offset_{offset} {
        for (std::size_t k = 0; k < R; k++) {
            sizes_[k] = sizes[k];
            strides_[k] = strides[k];
        }
    }
    /* a contiguous vector as a rank-1 view */
    explicit DataView(std::vector<T> &buf)
        requires(R == 1)
        : data_{buf.data()}, offset_{0} {
        sizes_[0] = buf.size();
        strides_[0] = 1;
    }
    [[nodiscard]] std::size_t size() const {
        std::size_t n = 1;
        for (std::size_t k = 0; k < R; k++) {
            n *= sizes_[k];
        }
        return n;
    }
    template <class... I> T &operator()(I... idx) {
        static_assert(sizeof...(I) == R, "one index per dimension");
        const std::size_t ix[R] = {static_cast<std::size_t>(idx)...};
        std::size_t at = offset_;
        for (std::size_t k = 0; k < R; k++) {
            at += ix[k] * strides_[k];
        }
        return data_[at];
    }

    class iterator {
      public:
        using iterator_category = std::forward_iterator_tag;
        using value_type = T;
        using difference_type = std::ptrdiff_t;
        using pointer = T *;
        using reference = T &;
        iterator(DataView *view, std::size_t linear) : view_{view}, linear_{linear} {}
        T &operator*() const { return view_->data_[view_->offset_of_(linear_)]; }
        iterator &operator++() {
            linear_++;
            return *this;
        }
        iterator operator++(int) {
            iterator before = *this;
            linear_++;
            return before;
        }
        bool operator==(const iterator &other) const { return linear_ == other.linear_; }
        bool operator!=(const iterator &other) const { return linear_ != other.linear_; }

      private:
        DataView *view_;
        std::size_t linear_;
    };
    iterator begin() { return iterator(this, 0); }
    iterator end() { return iterator(this, size()); }

  private:
    std::size_t offset_of_(std::size_t linear) const {
        std::size_t at = offset_;
        for (std::size_t k = R; k-- > 0;) {
            at += (linear % sizes_[k]) * strides_[k];
            linear /= sizes_[k];
        }
        return at;
    }
    T *data_;
    std::size_t offset_;
    std::size_t sizes_[R];
    std::size_t strides_[R];
};

/* Device keyword arguments: "{'mcmc': True, 'num_burnin': 200}" and
 * the same without braces or quotes, as key -> value strings.  Items are
 * separated by commas outside quotes and parentheses; braces outside quotes
 * are dropped; a key and its value are split at the first colon outside
 * quotes; surrounding quotes are stripped. */
inline std::unordered_map<std::string, std::string> parse_kwargs(const std::string &kwargs) {
    std::vector<std::string> items;
    std::string cur;
    char quote = 0;
    int depth = 0;
    for (const char ch : kwargs) {
        if (quote != 0) {
            if (ch == quote) {
                quote = 0;
            }
            cur.push_back(ch);
            continue;
        }
        if (ch == '\'' || ch == '"') {
            quote = ch;
            cur.push_back(ch);
        } else if (ch == '{' || ch == '}') {
            continue;
        } else if (ch == '(') {
            depth++;
            cur.push_back(ch);
        } else if (ch == ')') {
            depth = depth > 0 ? depth - 1 : 0;
            cur.push_back(ch);
        } else if (ch == ',' && depth == 0) {
            items.push_back(cur);
            cur.clear();
        } else {
            cur.push_back(ch);
        }
    }
    items.push_back(cur);
    auto trim = [](std::string s) {
        const auto b = s.find_first_not_of(" \t\n\r");
        if (b == std::string::npos) {
            return std::string{};
        }
        s = s.substr(b, s.find_last_not_of(" \t\n\r") - b + 1);
        if (s.size() >= 2 && (s.front() == '\'' || s.front() == '"') && s.back() == s.front()) {
            s = s.substr(1, s.size() - 2);
        }
        return s;
    };
    std::unordered_map<std::string, std::string> out;
    for (const auto &item : items) {
        char q = 0;
        std::size_t colon = std::string::npos;
        for (std::size_t i = 0; i < item.size() && colon == std::string::npos; i++) {
            if (q != 0) {
                q = item[i] == q ? 0 : q;
            } else if (item[i] == '\'' || item[i] == '"') {
                q = item[i];
            } else if (item[i] == ':') {
                colon = i;
            }
        }
        if (colon == std::string::npos) {
            continue;
        }
        const std::string key = trim(item.substr(0, colon));
        if (!key.empty()) {
            out[key] = trim(item.substr(colon + 1));
        }
    }
    return out;
}

/* Program qubit ids -> wires of the device register
 * (LightningQubitManager.hpp:37-196): program ids are never reused; the
 * wires of released qubits stay in the register, marked free, until the
 * register is reduced or a new qubit takes one of them (the lowest first). */
class QubitMap {
  public:
    [[nodiscard]] std::size_t size() const { return to_wire_.size(); }
    [[nodiscard]] bool valid(QubitIdType id) const { return to_wire_.count(id) != 0; }
    [[nodiscard]] bool valid(const std::vector<QubitIdType> &ids) const {
        for (const auto id : ids) {
            if (!valid(id)) {
                return false;
            }
        }
        return true;
    }
    [[nodiscard]] std::size_t wire(QubitIdType id) const {
        const auto it = to_wire_.find(id);
        if (it == to_wire_.end()) {
            throw LightningException("Invalid program qubit ID");
        }
        return it->second;
    }
    [[nodiscard]] std::vector<std::size_t> wires(const std::vector<QubitIdType> &ids) const {
        std::vector<std::size_t> out;
        out.reserve(ids.size());
        for (const auto id : ids) {
            out.push_back(wire(id));
        }
        return out;
    }
    QubitIdType allocate(std::size_t device_wire) {
        to_wire_[next_] = device_wire;
        return next_++;
    }
    std::vector<QubitIdType> allocate_range(std::size_t first_wire, std::size_t count) {
        std::vector<QubitIdType> ids;
        for (std::size_t i = 0; i < count; i++) {
            ids.push_back(allocate(first_wire + i));
        }
        return ids;
    }
    void release(QubitIdType id) {
        const auto it = to_wire_.find(id);
        if (it == to_wire_.end()) {
            throw LightningException("Cannot release qubit, the given ID is invalid");
        }
        free_.insert(it->second);
        to_wire_.erase(it);
    }
    void release_all() {
        to_wire_.clear();
        free_.clear();
    }
    std::optional<std::size_t> pop_free() {
        if (free_.empty()) {
            return std::nullopt;
        }
        const std::size_t w = *free_.begin();
        free_.erase(free_.begin());
        return w;
    }
    [[nodiscard]] const std::set<std::size_t> &free_wires() const { return free_; }
    void clear_free() { free_.clear(); }
    /* (wire, program id) of the live qubits, by wire */
    [[nodiscard]] std::vector<std::pair<std::size_t, QubitIdType>> live_by_wire() const {
        std::vector<std::pair<std::size_t, QubitIdType>> out;
        for (const auto &[id, w] : to_wire_) {
            out.emplace_back(w, id);
        }
        std::sort(out.begin(), out.end());
        return out;
    }
    void remap(const std::map<std::size_t, std::size_t> &old_to_new) {
        for (auto &[id, w] : to_wire_) {
            const auto it = old_to_new.find(w);
            if (it != old_to_new.end()) {
                w = it->second;
            }
        }
    }

  private:
    std::map<QubitIdType, std::size_t> to_wire_;
    std::set<std::size_t> free_;
    QubitIdType next_{0};
};

/* Purity Tr(rho_S^2) of the reduced state of the wires in `subset` of a
 * (possibly unnormalised) register held on the host: rho_S = sum over the
 * other wires' basis states e of |psi_e><psi_e| / <psi|psi>, accumulated in
 * one pass over the amplitudes (dim(S) operations per amplitude).  A pure
 * state's two parts have the same purity, so the smaller part is used. */
inline double subsystem_purity(const std::vector<std::complex<double>> &psi, std::size_t num_qubits,
                               std::vector<std::size_t> subset) {
    if (2 * subset.size() > num_qubits) {
        std::vector<std::size_t> other;
        for (std::size_t w = 0; w < num_qubits; w++) {
            if (std::find(subset.begin(), subset.end(), w) == subset.end()) {
                other.push_back(w);
            }
        }
        subset.swap(other);
    }
    const std::size_t k = subset.size(), dim = std::size_t{1} << k;
    std::vector<std::size_t> bit(k);
    std::size_t mask = 0;
    for (std::size_t i = 0; i < k; i++) {
        bit[i] = num_qubits - 1 - subset[i];
        mask |= std::size_t{1} << bit[i];
    }
    std::vector<std::complex<double>> rho(dim * dim);
    double norm2 = 0.0;
    for (std::size_t rest = 0; rest < psi.size(); rest++) {
        if ((rest & mask) != 0) {
            continue;
        }
        for (std::size_t r1 = 0; r1 < dim; r1++) {
            std::size_t i1 = rest;
            for (std::size_t i = 0; i < k; i++) {
                i1 |= ((r1 >> (k - 1 - i)) & 1U) << bit[i];
            }
            const std::complex<double> a1 = psi[i1];
            norm2 += std::norm(a1);
            for (std::size_t r2 = 0; r2 < dim; r2++) {
                std::size_t i2 = rest;
                for (std::size_t i = 0; i < k; i++) {
                    i2 |= ((r2 >> (k - 1 - i)) & 1U) << bit[i];
                }
                rho[r1 * dim + r2] += a1 * std::conj(psi[i2]);
            }
        }
    }
    if (norm2 <= 0.0) {
        return 0.0;
    }
    double p = 0.0;
    for (const auto &x : rho) {
        p += std::norm(x);
    }
    return p / (norm2 * norm2);
}

/* The Catalyst device (LightningSimulator.hpp:35-197) on one GB300. */
class LightningGB300Simulator {
  public:
    using StateVectorT = StateVectorGB300<double>;
    using MeasurementsT_ = ::Pennylane::LightningGB300::MeasurementsGB300<StateVectorT>;
    using ObservableT = ::Pennylane::LightningGB300::Observable<StateVectorT>;

    /* kwargs: mcmc (True / False), num_burnin, kernel_name
     * (LightningSimulator.hpp:118-129) */
    explicit LightningGB300Simulator(const std::string &kwargs = "{}") {
        auto args = parse_kwargs(kwargs);
        mcmc_ = args.count("mcmc") != 0 && args["mcmc"] == "True";
        num_burnin_ = args.count("num_burnin") != 0 ? static_cast<std::size_t>(std::stoll(args["num_burnin"])) : 100;
        kernel_name_ = args.count("kernel_name") != 0 ? args["kernel_name"] : "Local";
    }
    LightningGB300Simulator(const LightningGB300Simulator &) = delete;
    LightningGB300Simulator &operator=(const LightningGB300Simulator &) = delete;
    LightningGB300Simulator(LightningGB300Simulator &&) = delete;
    LightningGB300Simulator &operator=(LightningGB300Simulator &&) = delete;
    ~LightningGB300Simulator() = default;

    /* ---- qubits (LightningSimulator.cpp:29-138) ---- */
    auto AllocateQubit() -> QubitIdType {
        if (qubits_.size() == 0) {
            fresh_register_(1);
            return qubits_.allocate(0);
        }
        const auto candidate = qubits_.pop_free();
        if (!candidate.has_value()) {
            // |psi> (x) |0>: the new qubit is the register's last wire
            const std::size_t n = sv_->getNumQubits();
            const auto host = sv_->getDataVector();
            auto grown = std::make_unique<StateVectorT>(n + 1);
            std::vector<std::size_t> old_wires(n);
            std::iota(old_wires.begin(), old_wires.end(), std::size_t{0});
            grown->setStateVector(host.data(), old_wires);
            sv_ = std::move(grown);
            return qubits_.allocate(n);
        }
        // reuse a released wire: it must be disentangled, then reset to |0>
        if (std::abs(subsystem_purity(sv_->getDataVector(), sv_->getNumQubits(), {*candidate}) - 1.0) >= 1e-6) {
            throw LightningException("Cannot reuse qubit: qubit is entangled with remaining qubits. Release qubits "
                                     "must be disentangled.");
        }
        const QubitIdType id = qubits_.allocate(*candidate);
        if (*Measure(id)) {
            NamedOperation("PauliX", {}, {id});
        }
        return id;
    }
    auto AllocateQubits(std::size_t num_qubits) -> std::vector<QubitIdType> {
        if (num_qubits == 0) {
            return {};
        }
        if (qubits_.size() == 0) {
            fresh_register_(num_qubits);
            return qubits_.allocate_range(0, num_qubits);
        }
        std::vector<QubitIdType> ids;
        for (std::size_t i = 0; i < num_qubits; i++) {
            ids.push_back(AllocateQubit());
        }
        return ids;
    }
    void ReleaseQubit(QubitIdType q) {
        if (!qubits_.valid(q)) {
            throw LightningException("Invalid qubit to release");
        }
        qubits_.release(q);
        needs_reduction_ = true;
    }
    void ReleaseQubits(const std::vector<QubitIdType> &ids) {
        if (ids.size() == qubits_.size() && qubits_.valid(ids) &&
            std::set<QubitIdType>(ids.begin(), ids.end()).size() == ids.size()) {
            fresh_register_(0);
            return;
        }
        for (const auto id : ids) {
            ReleaseQubit(id);
        }
    }
    [[nodiscard]] auto GetNumQubits() const -> std::size_t { return qubits_.size(); }

    /* ---- device settings ---- */
    void StartTapeRecording() {
        if (recording_) {
            throw LightningException("Cannot re-activate the cache manager");
        }
        recording_ = true;
        tape_ = Tape{};
    }
    void StopTapeRecording() {
        if (!recording_) {
            throw LightningException("Cannot stop an already stopped cache manager");
        }
        recording_ = false;
    }
    void SetDeviceShots(std::size_t shots) { shots_ = shots; }
    [[nodiscard]] auto GetDeviceShots() const -> std::size_t { return shots_; }
    void SetDevicePRNG(std::mt19937 *gen) { gen_ = gen; }

    /* ---- state preparation (LightningSimulator.cpp:427-437) ---- */
    void SetState(DataView<std::complex<double>, 1> &state, std::vector<QubitIdType> &wires) {
        const std::vector<std::complex<double>> data(state.begin(), state.end());
        if (data.size() != (std::size_t{1} << wires.size())) {
            throw LightningException("Inconsistent state and wires dimensions.");
        }
        sv_->setStateVector(data.data(), qubits_.wires(wires));
    }
    void SetBasisState(DataView<int8_t, 1> &n, std::vector<QubitIdType> &wires) {
        std::vector<std::size_t> bits;
        for (auto it = n.begin(); it != n.end(); ++it) {
            bits.push_back(static_cast<std::size_t>(*it));
        }
        sv_->setBasisState(bits, qubits_.wires(wires));
    }

    /* ---- gates (LightningSimulator.cpp:439-541) ---- */
    void NamedOperation(const std::string &name, const std::vector<double> &params,
                        const std::vector<QubitIdType> &wires, bool inverse = false,
                        const std::vector<QubitIdType> &controlled_wires = {},
                        const std::vector<bool> &controlled_values = {},
                        const std::vector<std::string> &optional_params = {}) {
        check_operation_wires_(wires, controlled_wires, controlled_values);
        const auto dev_wires = qubits_.wires(wires);
        const auto dev_cwires = qubits_.wires(controlled_wires);
        if (name == "PauliRot") {
            if (optional_params.size() != 1) {
                throw LightningException("PauliRot operation requires one string parameter for the Pauli word");
            }
            if (!controlled_wires.empty()) {
                throw LightningException("Controlled PauliRot is not supported");
            }
            if (recording_) {
                throw LightningException("PauliRot operation is not supported when tape recording is active");
            }
            const std::string &word = optional_params[0];
            if (word.size() != dev_wires.size()) {
                throw LightningException("PauliRot word and wires must have the same length");
            }
            std::string kept;
            std::vector<std::size_t> kept_wires;
            for (std::size_t i = 0; i < word.size(); i++) {
                if (word[i] != 'I') {
                    kept.push_back(word[i]);
                    kept_wires.push_back(dev_wires[i]);
                }
            }
            if (!kept.empty()) { // an all-identity word is a global phase
                sv_->applyPauliRot(kept_wires, inverse, params, kept);
            }
            return;
        }
        if (controlled_wires.empty()) {
            sv_->applyOperation(name, dev_wires, inverse, params);
        } else {
            sv_->applyOperation(name, dev_cwires, controlled_values, dev_wires, inverse, params);
        }
        if (recording_) {
            tape_.add(name, params, dev_wires, inverse, {}, dev_cwires, controlled_values);
        }
    }
    void MatrixOperation(const std::vector<std::complex<double>> &matrix, const std::vector<QubitIdType> &wires,
                         bool inverse = false, const std::vector<QubitIdType> &controlled_wires = {},
                         const std::vector<bool> &controlled_values = {}) {
        check_operation_wires_(wires, controlled_wires, controlled_values);
        const auto dev_wires = qubits_.wires(wires);
        const auto dev_cwires = qubits_.wires(controlled_wires);
        if (matrix.size() != (std::size_t{1} << (2 * dev_wires.size()))) {
            throw LightningException("The size of matrix does not match with the given number of wires");
        }
        if (controlled_wires.empty()) {
            sv_->applyMatrix(matrix.data(), dev_wires, inverse);
        } else {
            sv_->applyControlledMatrix(matrix.data(), dev_cwires, controlled_values, dev_wires, inverse);
        }
        if (recording_) {
            tape_.add("QubitUnitary", {}, dev_wires, inverse, matrix, dev_cwires, controlled_values);
        }
    }

    /* ---- observables (LightningSimulator.cpp:543-571,
     *      LightningObsManager.hpp:39-205) ---- */
    auto Observable(ObsId id, const std::vector<std::complex<double>> &matrix, const std::vector<QubitIdType> &wires)
        -> ObsIdType {
        if (wires.size() > GetNumQubits()) {
            throw LightningException("Invalid number of wires");
        }
        if (!qubits_.valid(wires)) {
            throw LightningException("Invalid given wires");
        }
        const auto dev_wires = qubits_.wires(wires);
        if (id == ObsId::Hermitian) {
            return cache_obs_(std::make_shared<HermitianObs<StateVectorT>>(matrix, dev_wires));
        }
        return cache_obs_(std::make_shared<NamedObs<StateVectorT>>(named_obs_(id), dev_wires));
    }
    auto TensorObservable(const std::vector<ObsIdType> &obs) -> ObsIdType {
        return cache_obs_(std::make_shared<TensorProdObs<StateVectorT>>(cached_(obs)));
    }
    auto HamiltonianObservable(const std::vector<double> &coeffs, const std::vector<ObsIdType> &obs) -> ObsIdType {
        if (coeffs.size() != obs.size()) {
            throw LightningException("Incompatible list of observables and coefficients; Number of observables and "
                                     "number of coefficients must be equal");
        }
        return cache_obs_(std::make_shared<Hamiltonian<StateVectorT>>(coeffs, cached_(obs)));
    }

    /* ---- measurements (LightningSimulator.cpp:573-832) ---- */
    auto Expval(ObsIdType obsKey) -> double {
        const auto obs = observable_(obsKey);
        if (recording_) {
            tape_.observe(obsKey, MeasurementsT::Expval);
        }
        auto m = measurements_();
        return shots_ != 0 ? m.expval(*obs, shots_, {}) : m.expval(*obs);
    }
    auto Var(ObsIdType obsKey) -> double {
        const auto obs = observable_(obsKey);
        if (recording_) {
            tape_.observe(obsKey, MeasurementsT::Var);
        }
        auto m = measurements_();
        return shots_ != 0 ? m.var(*obs, shots_) : m.var(*obs);
    }
    void State(DataView<std::complex<double>, 1> &state) {
        reduce_();
        const auto data = sv_->getDataVector();
        if (state.size() != data.size()) {
            throw LightningException("Invalid size for the pre-allocated state vector");
        }
        std::copy(data.begin(), data.end(), state.begin());
    }
    void Probs(DataView<double, 1> &probs) {
        auto m = measurements_();
        const auto p = shots_ != 0 ? m.probs(shots_) : m.probs();
        if (probs.size() != p.size()) {
            throw LightningException("Invalid size for the pre-allocated probabilities");
        }
        std::copy(p.begin(), p.end(), probs.begin());
    }
    void PartialProbs(DataView<double, 1> &probs, const std::vector<QubitIdType> &wires) {
        check_measured_wires_(wires);
        auto m = measurements_();
        const auto dev_wires = qubits_.wires(wires);
        std::vector<double> p;
        if (shots_ != 0) {
            p = m.probs(dev_wires, shots_);
        } else if (dev_wires.empty()) {
            const auto all = m.probs();
            p = {std::accumulate(all.begin(), all.end(), 0.0)};
        } else {
            p = m.probs(dev_wires);
        }
        if (probs.size() != p.size()) {
            throw LightningException("Invalid size for the pre-allocated partial-probabilities");
        }
        std::copy(p.begin(), p.end(), probs.begin());
    }
    void Sample(DataView<double, 2> &samples) {
        const auto bits = GenerateSamples(shots_);
        if (samples.size() != bits.size()) {
            throw LightningException("Invalid size for the pre-allocated samples");
        }
        std::copy(bits.begin(), bits.end(), samples.begin()); // shots x qubits, row-major
    }
    void PartialSample(DataView<double, 2> &samples, const std::vector<QubitIdType> &wires) {
        check_measured_wires_(wires);
        if (samples.size() != shots_ * wires.size()) {
            throw LightningException("Invalid size for the pre-allocated partial-samples");
        }
        const auto bits = GenerateSamples(shots_);
        const std::size_t n = GetNumQubits();
        const auto dev_wires = qubits_.wires(wires);
        auto out = samples.begin();
        for (std::size_t s = 0; s < shots_; s++) {
            for (const std::size_t w : dev_wires) {
                *out = static_cast<double>(bits[s * n + w]);
                ++out;
            }
        }
    }
    void Counts(DataView<double, 1> &eigvals, DataView<int64_t, 1> &counts) {
        const std::size_t n = GetNumQubits();
        const std::size_t num_elements = std::size_t{1} << n;
        if (eigvals.size() != num_elements || counts.size() != num_elements) {
            throw LightningException("Invalid size for the pre-allocated counts");
        }
        const auto bits = GenerateSamples(shots_);
        std::vector<std::size_t> all(qubits_.size());
        std::iota(all.begin(), all.end(), std::size_t{0});
        fill_counts_(bits, n, all, eigvals, counts);
    }
    void PartialCounts(DataView<double, 1> &eigvals, DataView<int64_t, 1> &counts,
                       const std::vector<QubitIdType> &wires) {
        check_measured_wires_(wires);
        const std::size_t num_elements = std::size_t{1} << wires.size();
        if (eigvals.size() != num_elements || counts.size() != num_elements) {
            throw LightningException("Invalid size for the pre-allocated partial-counts");
        }
        const auto bits = GenerateSamples(shots_);
        fill_counts_(bits, GetNumQubits(), qubits_.wires(wires), eigvals, counts);
    }
    /* mid-circuit measurement: draw the outcome from the wire's probability,
     * then collapse onto it (LightningSimulator.cpp:834-856) */
    auto Measure(QubitIdType wire, std::optional<int32_t> postselect = std::nullopt) -> Result {
        std::vector<double> p(2);
        DataView<double, 1> view(p);
        const std::size_t shots = shots_;
        shots_ = 0;
        try {
            PartialProbs(view, {wire});
        } catch (...) {
            shots_ = shots;
            throw;
        }
        shots_ = shots;
        const bool outcome = draw_outcome_(p, postselect);
        sv_->collapse(qubits_.wire(wire), outcome);
        return outcome ? &kTrue : &kFalse;
    }
    /* a Pauli-word measurement: basis change, parity onto the first wire by
     * CNOTs, measure it, undo (LightningSimulator.cpp:858-927) */
    auto PauliMeasure(const std::string &pauli_word, const std::vector<QubitIdType> &wires) -> Result {
        if (pauli_word.size() != wires.size()) {
            throw LightningException("Pauli word length must match number of wires");
        }
        for (const char p : pauli_word) {
            if (p != 'I' && p != 'X' && p != 'Y' && p != 'Z') {
                throw LightningException("Invalid character in Pauli word");
            }
        }
        for (std::size_t i = 0; i < pauli_word.size(); i++) {
            if (pauli_word[i] == 'X') {
                NamedOperation("Hadamard", {}, {wires[i]});
            } else if (pauli_word[i] == 'Y') {
                NamedOperation("S", {}, {wires[i]}, true);
                NamedOperation("Hadamard", {}, {wires[i]});
            }
        }
        for (std::size_t i = 1; i < wires.size(); i++) {
            NamedOperation("CNOT", {}, {wires[i], wires[0]});
        }
        const bool outcome = *Measure(wires[0]);
        for (std::size_t i = 1; i < wires.size(); i++) {
            NamedOperation("CNOT", {}, {wires[i], wires[0]});
        }
        for (std::size_t i = 0; i < pauli_word.size(); i++) {
            if (pauli_word[i] == 'X') {
                NamedOperation("Hadamard", {}, {wires[i]});
            } else if (pauli_word[i] == 'Y') {
                NamedOperation("Hadamard", {}, {wires[i]});
                NamedOperation("S", {}, {wires[i]});
            }
        }
        return outcome ? &kTrue : &kFalse;
    }

    /* ---- gradient of the recorded tape by the adjoint method
     *      (LightningSimulator.cpp:944-975) ---- */
    void Gradient(std::vector<DataView<double, 1>> &gradients, const std::vector<std::size_t> &trainParams) {
        const std::size_t num_obs = tape_.obs_keys.size();
        const std::size_t num_params = tape_.num_params;
        const std::size_t num_train = trainParams.empty() ? num_params : trainParams.size();
        if (num_train * num_obs == 0) {
            return;
        }
        if (gradients.size() != num_obs) {
            throw LightningException("Invalid number of pre-allocated gradients");
        }
        for (const auto kind : tape_.obs_kinds) {
            if (kind != MeasurementsT::Expval) {
                throw LightningException("Unsupported measurements to compute gradient; Adjoint differentiation "
                                         "method only supports expectation return type");
            }
        }
        OpsData<StateVectorT> ops(tape_.names, tape_.params, tape_.wires, tape_.inverses, tape_.matrices,
                                  tape_.cwires, tape_.cvals);
        std::vector<std::shared_ptr<ObservableT>> obs;
        for (const auto key : tape_.obs_keys) {
            obs.push_back(observable_(key));
        }
        std::vector<std::size_t> tp = trainParams;
        if (tp.empty()) {
            tp.resize(num_params);
            std::iota(tp.begin(), tp.end(), std::size_t{0});
        }
        JacobianData<StateVectorT> jd(num_params, sv_->getLength(), nullptr, obs, ops, tp);
        std::vector<double> jac(num_obs * num_train);
        AdjointJacobianGB300<StateVectorT>().adjointJacobian(std::span<double>(jac), jd, *sv_, false);
        for (std::size_t o = 0; o < num_obs; o++) {
            if (gradients[o].size() < num_train) {
                throw LightningException("Invalid size for the pre-allocated gradient");
            }
            std::copy(jac.begin() + static_cast<std::ptrdiff_t>(o * num_train),
                      jac.begin() + static_cast<std::ptrdiff_t>((o + 1) * num_train), gradients[o].begin());
        }
    }

    /* recorded tape: operations, observables, parameters, operation names,
     * observable keys (LightningSimulator.cpp:399-406) */
    auto CacheManagerInfo() -> std::tuple<std::size_t, std::size_t, std::size_t, std::vector<std::string>,
                                          std::vector<ObsIdType>> {
        return {tape_.names.size(), tape_.obs_keys.size(), tape_.num_params, tape_.names, tape_.obs_keys};
    }

    /* samples of the whole register: the alias method, or Metropolis-Hastings
     * with the device's kernel and burn-in (LightningSimulator.cpp:626-671) */
    auto GenerateSamples(std::size_t shots) -> std::vector<std::size_t> {
        auto m = measurements_();
        return m.generate_samples(shots);
    }
    auto GenerateSamplesMetropolis(std::size_t shots) -> std::vector<std::size_t> {
        auto m = measurements_();
        return m.generate_samples_metropolis(kernel_name_, num_burnin_, shots);
    }
    [[nodiscard]] bool mcmc() const { return mcmc_; }
    [[nodiscard]] std::size_t num_burnin() const { return num_burnin_; }
    [[nodiscard]] const std::string &kernel_name() const { return kernel_name_; }

  private:
    struct Tape {
        std::vector<std::string> names;
        std::vector<std::vector<double>> params;
        std::vector<std::vector<std::size_t>> wires;
        std::vector<bool> inverses;
        std::vector<std::vector<std::complex<double>>> matrices;
        std::vector<std::vector<std::size_t>> cwires;
        std::vector<std::vector<bool>> cvals;
        std::vector<ObsIdType> obs_keys;
        std::vector<MeasurementsT> obs_kinds;
        std::size_t num_params{0};
        void add(const std::string &name, const std::vector<double> &p, const std::vector<std::size_t> &w, bool inv,
                 const std::vector<std::complex<double>> &m, const std::vector<std::size_t> &cw,
                 const std::vector<bool> &cv) {
            names.push_back(name);
            params.push_back(p);
            wires.push_back(w);
            inverses.push_back(inv);
            matrices.push_back(m);
            cwires.push_back(cw);
            cvals.push_back(cv);
            num_params += p.size();
        }
        void observe(ObsIdType key, MeasurementsT kind) {
            obs_keys.push_back(key);
            obs_kinds.push_back(kind);
        }
    };

    static inline bool kTrue = true;
    static inline bool kFalse = false;

    void fresh_register_(std::size_t n) {
        qubits_.release_all();
        sv_ = std::make_unique<StateVectorT>(n);
        needs_reduction_ = false;
    }
    void check_operation_wires_(const std::vector<QubitIdType> &wires, const std::vector<QubitIdType> &cwires,
                                const std::vector<bool> &cvals) const {
        if (cwires.size() != cvals.size()) {
            throw LightningException("Controlled wires/values size mismatch");
        }
        if (!qubits_.valid(wires)) {
            throw LightningException("Given wires do not refer to qubits");
        }
        if (!qubits_.valid(cwires)) {
            throw LightningException("Given controlled wires do not refer to qubits");
        }
    }
    void check_measured_wires_(const std::vector<QubitIdType> &wires) const {
        if (wires.size() > GetNumQubits()) {
            throw LightningException("Invalid number of wires");
        }
        if (!qubits_.valid(wires)) {
            throw LightningException("Invalid given wires to measure");
        }
    }
    static std::string named_obs_(ObsId id) {
        switch (id) {
        case ObsId::Identity:
            return "Identity";
        case ObsId::PauliX:
            return "PauliX";
        case ObsId::PauliY:
            return "PauliY";
        case ObsId::PauliZ:
            return "PauliZ";
        case ObsId::Hadamard:
            return "Hadamard";
        default:
            throw LightningException("The given observable is not supported by the simulator");
        }
    }
    ObsIdType cache_obs_(std::shared_ptr<ObservableT> obs) {
        observables_.push_back(std::move(obs));
        return static_cast<ObsIdType>(observables_.size() - 1);
    }
    std::vector<std::shared_ptr<ObservableT>> cached_(const std::vector<ObsIdType> &keys) const {
        std::vector<std::shared_ptr<ObservableT>> out;
        for (const auto key : keys) {
            if (key < 0 || static_cast<std::size_t>(key) >= observables_.size()) {
                throw LightningException("Invalid observable key");
            }
            out.push_back(observables_[static_cast<std::size_t>(key)]);
        }
        return out;
    }
    std::shared_ptr<ObservableT> observable_(ObsIdType key) const {
        if (key < 0 || static_cast<std::size_t>(key) >= observables_.size()) {
            throw LightningException("Invalid key for cached observables");
        }
        return observables_[static_cast<std::size_t>(key)];
    }
    MeasurementsT_ measurements_() {
        reduce_();
        MeasurementsT_ m(*sv_);
        if (gen_ != nullptr) {
            m.setSeed(static_cast<std::size_t>((*gen_)()));
        }
        return m;
    }
    /* outcome 1 with the wire's probability of 1: a uniform draw u in [0, 1)
     * from the device's generator (a fresh one without it) gives 1 when
     * u >= P(0); a postselected outcome is taken as given */
    bool draw_outcome_(const std::vector<double> &p, std::optional<int32_t> postselect) {
        if (postselect.has_value()) {
            if (*postselect != 0 && *postselect != 1) {
                throw LightningException("Invalid postselect value");
            }
            if (p[static_cast<std::size_t>(*postselect)] <= 0.0) {
                throw LightningException("Invalid postselect value: the outcome has probability zero");
            }
            return *postselect == 1;
        }
        std::uniform_real_distribution<double> u(0.0, 1.0);
        if (gen_ != nullptr) {
            return u(*gen_) >= p[0];
        }
        std::mt19937 local(std::random_device{}());
        return u(local) >= p[0];
    }
    template <class W>
    void fill_counts_(const std::vector<std::size_t> &bits, std::size_t n, const W &dev_wires,
                      DataView<double, 1> &eigvals, DataView<int64_t, 1> &counts) {
        std::size_t k = 0;
        for (auto it = eigvals.begin(); it != eigvals.end(); ++it) {
            *it = static_cast<double>(k++);
        }
        for (auto it = counts.begin(); it != counts.end(); ++it) {
            *it = 0;
        }
        for (std::size_t s = 0; s < shots_; s++) {
            std::size_t idx = 0;
            for (const std::size_t w : dev_wires) {
                idx = (idx << 1) | bits[s * n + w];
            }
            counts(idx) += 1;
        }
    }
    /* drop the wires of released qubits from the register
     * (LightningSimulator.cpp:147-259): they must be disentangled from the
     * live ones; the live wires' slice through the first amplitude of
     * magnitude above 1e-15 is normalised and becomes the new register, the
     * live qubits keep their order */
    void reduce_() {
        if (!needs_reduction_) {
            return;
        }
        const auto &freed = qubits_.free_wires();
        if (freed.empty()) { // the released wires were all taken again
            needs_reduction_ = false;
            return;
        }
        const std::size_t n = sv_->getNumQubits();
        const auto host = sv_->getDataVector();
        const auto live = qubits_.live_by_wire();
        if (!live.empty()) {
            const double purity =
                subsystem_purity(host, n, std::vector<std::size_t>(freed.begin(), freed.end()));
            if (!std::isfinite(purity) || std::abs(purity - 1.0) > 1e-6) {
                throw LightningException("Cannot release qubits: released qubits are entangled with remaining "
                                         "qubits (purity = " +
                                         std::to_string(purity) + ")");
            }
        }
        std::size_t ref = 0;
        for (std::size_t i = 0; i < host.size(); i++) {
            if (std::abs(host[i]) > 1e-15) {
                ref = i;
                break;
            }
        }
        const std::size_t m = live.size();
        std::vector<std::complex<double>> reduced(std::size_t{1} << m);
        for (std::size_t j = 0; j < reduced.size(); j++) {
            std::size_t idx = ref;
            for (std::size_t i = 0; i < m; i++) {
                const std::size_t b = n - 1 - live[i].first;
                if ((j >> (m - 1 - i)) & 1U) {
                    idx |= std::size_t{1} << b;
                } else {
                    idx &= ~(std::size_t{1} << b);
                }
            }
            reduced[j] = host[idx];
        }
        auto next = std::make_unique<StateVectorT>(m);
        next->updateData(reduced);
        next->normalize();
        sv_ = std::move(next);
        std::map<std::size_t, std::size_t> old_to_new;
        for (std::size_t i = 0; i < m; i++) {
            old_to_new[live[i].first] = i;
        }
        qubits_.remap(old_to_new);
        qubits_.clear_free();
        needs_reduction_ = false;
    }

    QubitMap qubits_;
    std::unique_ptr<StateVectorT> sv_ = std::make_unique<StateVectorT>(0);
    std::vector<std::shared_ptr<ObservableT>> observables_;
    Tape tape_;
    bool recording_{false};
    std::size_t shots_{0};
    std::mt19937 *gen_{nullptr};
    bool mcmc_{false};
    std::size_t num_burnin_{100};
    std::string kernel_name_{"Local"};
    bool needs_reduction_{false};
};

} // namespace Pennylane::LightningGB300::Catalyst

#endif
