// ORACLE — test infrastructure only, never part of the product path.
//
// A CPU restatement of lightning.qubit's "LM" state-vector algorithms
// (pennylane_lightning/core/simulators/lightning_qubit/...), written for this
// repository.  It is used (a) as the parity checker of the GPU kernels on
// inputs the CPU finishes in seconds and (b) as the timed CPU baseline on the
// GPU host (OpenMP over the outer group index, as PL_LQ_KERNEL_OMP does).
//
// Parity of this restatement is pinned against the reference itself: the shim
// in ref_shim.cpp compiles the reference's own headers, and tests compare the
// two on random circuits, every gate and the reference's known-answer values.
//
// Conventions kept from the reference (they decide parity):
//   * wire w is bit (n-1-w) of the amplitude index (StateVectorLQubit.hpp:950);
//   * within a k-wire group the local index has wires[0] as its most
//     significant bit (GateIndices.cpp generateBitPatterns);
//   * gate coefficients are formed in the working precision T with the same
//     formulas as GateImplementationsLM.hpp (cited per gate below).
#pragma once

#include <algorithm>
#include <bit>
#include <cmath>
#include <complex>
#include <cstdint>
#include <functional>
#include <limits>
#include <memory>
#include <numeric>
#include <random>
#include <stack>
#include <stdexcept>
#include <string>
#include <unordered_map>
#include <utility>
#include <vector>

namespace orc {

using std::size_t;
template <class T> using C = std::complex<T>;

struct OracleError : std::runtime_error {
    using std::runtime_error::runtime_error;
};
#define ORC_CHECK(cond, msg)                                                   \
    do {                                                                       \
        if (!(cond)) {                                                         \
            throw ::orc::OracleError(msg);                                     \
        }                                                                      \
    } while (0)

// ---------------------------------------------------------------------------
// Index helpers (core/utils/BitUtil.hpp:95-123 revWireParity,
// GateImplementationsLM.hpp parity_2_offset).
// ---------------------------------------------------------------------------
inline size_t trailing_ones(size_t n) {
    return n == 0 ? 0 : (~size_t{0}) >> (64 - n);
}
inline size_t leading_ones(size_t n) { return ~trailing_ones(n); }

// Masks that spread a compact counter k over all bits except `bits`.
inline std::vector<size_t> spread_masks(std::vector<size_t> bits) {
    std::sort(bits.begin(), bits.end());
    std::vector<size_t> m(bits.size() + 1);
    if (bits.empty()) {
        m[0] = ~size_t{0};
        return m;
    }
    m[0] = trailing_ones(bits[0]);
    for (size_t i = 1; i < bits.size(); i++) {
        m[i] = leading_ones(bits[i - 1] + 1) & trailing_ones(bits[i]);
    }
    m[bits.size()] = leading_ones(bits.back() + 1);
    return m;
}
inline size_t spread(const std::vector<size_t> &m, size_t k) {
    size_t r = 0;
    for (size_t i = 0; i < m.size(); i++) {
        r |= (k << i) & m[i];
    }
    return r;
}

// All groups of a gate on `wires` controlled on (`cwires` == `cvals`):
// offset(k) for k < count spreads k over the free bits, and local[j] is the
// target pattern j (wires[0] = MSB of j) with the control values or'ed in.
struct Groups {
    std::vector<size_t> masks;
    std::vector<size_t> local;
    size_t count{0};
    size_t offset(size_t k) const { return spread(masks, k); }
};
inline Groups make_groups(size_t n, const std::vector<size_t> &wires,
                          const std::vector<size_t> &cwires,
                          const std::vector<bool> &cvals) {
    Groups g;
    std::vector<size_t> bits;
    for (auto w : wires) {
        bits.push_back(n - 1 - w);
    }
    for (auto w : cwires) {
        bits.push_back(n - 1 - w);
    }
    g.masks = spread_masks(bits);
    size_t cbits = 0;
    for (size_t i = 0; i < cwires.size(); i++) {
        if (cvals[i]) {
            cbits |= size_t{1} << (n - 1 - cwires[i]);
        }
    }
    const size_t k = wires.size();
    g.local.resize(size_t{1} << k);
    for (size_t j = 0; j < g.local.size(); j++) {
        size_t idx = cbits;
        for (size_t m = 0; m < k; m++) {
            if ((j >> (k - 1 - m)) & 1U) {
                idx |= size_t{1} << (n - 1 - wires[m]);
            }
        }
        g.local[j] = idx;
    }
    g.count = size_t{1} << (n - wires.size() - cwires.size());
    return g;
}

inline void check_wires(size_t n, const std::vector<size_t> &wires,
                        const std::vector<size_t> &cwires) {
    std::vector<size_t> all(wires);
    all.insert(all.end(), cwires.begin(), cwires.end());
    for (auto w : all) {
        ORC_CHECK(w < n, "wire index out of range");
    }
    std::vector<size_t> s(all);
    std::sort(s.begin(), s.end());
    ORC_CHECK(std::adjacent_find(s.begin(), s.end()) == s.end(),
              "`controlled_wires` and `target wires` must be disjoint.");
}

// Apply `core(arr, local_indices_with_offset)` over every group.  The 1-wire
// uncontrolled case uses the two-mask form of applyNC1 (LM:653-703).
template <class T, class Core>
void for_groups(C<T> *arr, size_t n, const std::vector<size_t> &wires,
                const std::vector<size_t> &cwires,
                const std::vector<bool> &cvals, Core &&core) {
    check_wires(n, wires, cwires);
    const Groups g = make_groups(n, wires, cwires, cvals);
    const size_t nloc = g.local.size();
    const long long count = static_cast<long long>(g.count);
#pragma omp parallel for schedule(static)
    for (long long k = 0; k < count; k++) {
        const size_t off = g.offset(static_cast<size_t>(k));
        size_t idx[64];
        for (size_t j = 0; j < nloc && j < 64; j++) {
            idx[j] = g.local[j] + off;
        }
        core(arr, idx);
    }
}

template <class T> inline C<T> IMAG() { return {0, 1}; }
template <class T> constexpr T INVSQRT2() {
    return static_cast<T>(0.7071067811865475244008443621048490392848359376884740L);
}

// ---------------------------------------------------------------------------
// Gate matrices (core/gates/Gates.hpp), used for Rot/CRot (LM:1276-1301).
// ---------------------------------------------------------------------------
template <class T> std::vector<C<T>> rot_matrix(T phi, T theta, T omega) {
    // Gates.hpp:389-399 getRot
    const T c = std::cos(theta / 2);
    const T s = std::sin(theta / 2);
    const T p{phi + omega};
    const T m{phi - omega};
    return {C<T>{std::cos(p / 2) * c, -std::sin(p / 2) * c},
            C<T>{-std::cos(m / 2) * s, -std::sin(m / 2) * s},
            C<T>{std::cos(m / 2) * s, -std::sin(m / 2) * s},
            C<T>{std::cos(p / 2) * c, std::sin(p / 2) * c}};
}

template <class T>
std::vector<C<T>> dagger(const std::vector<C<T>> &m, size_t dim) {
    std::vector<C<T>> r(m.size());
    for (size_t i = 0; i < dim; i++) {
        for (size_t j = 0; j < dim; j++) {
            r[j * dim + i] = std::conj(m[i * dim + j]);
        }
    }
    return r;
}

// Dense (controlled) k-wire matrix: applyNC{Single,Two,Multi}QubitOp (LM:278-498)
template <class T>
void apply_matrix(C<T> *arr, size_t n, const std::vector<C<T>> &matrix,
                  const std::vector<size_t> &cwires,
                  const std::vector<bool> &cvals,
                  const std::vector<size_t> &wires, bool inverse) {
    ORC_CHECK(!wires.empty(), "Number of wires must be larger than 0");
    const size_t dim = size_t{1} << wires.size();
    ORC_CHECK(matrix.size() == dim * dim,
              "The size of matrix does not match with the given number of "
              "wires");
    const std::vector<C<T>> mat = inverse ? dagger(matrix, dim) : matrix;
    if (dim == 2) {
        for_groups<T>(arr, n, wires, cwires, cvals,
                      [&mat](C<T> *a, const size_t *ix) {
                          const C<T> v0 = a[ix[0]];
                          const C<T> v1 = a[ix[1]];
                          a[ix[0]] = mat[0] * v0 + mat[1] * v1;
                          a[ix[1]] = mat[2] * v0 + mat[3] * v1;
                      });
        return;
    }
    if (dim == 4) {
        for_groups<T>(arr, n, wires, cwires, cvals,
                      [&mat](C<T> *a, const size_t *ix) {
                          const C<T> v0 = a[ix[0]], v1 = a[ix[1]],
                                     v2 = a[ix[2]], v3 = a[ix[3]];
                          for (size_t r = 0; r < 4; r++) {
                              a[ix[r]] = mat[4 * r] * v0 + mat[4 * r + 1] * v1 +
                                         mat[4 * r + 2] * v2 +
                                         mat[4 * r + 3] * v3;
                          }
                      });
        return;
    }
    ORC_CHECK(wires.size() <= 6, "oracle supports dense matrices on <= 6 wires");
    for_groups<T>(arr, n, wires, cwires, cvals,
                  [&mat, dim](C<T> *a, const size_t *ix) {
                      C<T> v[64];
                      for (size_t i = 0; i < dim; i++) {
                          v[i] = a[ix[i]];
                      }
                      for (size_t i = 0; i < dim; i++) {
                          C<T> acc = 0.0;
                          for (size_t j = 0; j < dim; j++) {
                              acc += mat[i * dim + j] * v[j];
                          }
                          a[ix[i]] = acc;
                      }
                  });
}

// Sparse CSR local operator: applyNCMultiQubitSparseOp (LM:505-560)
template <class T>
void apply_sparse(C<T> *arr, size_t n, const std::vector<size_t> &indptr,
                  const std::vector<size_t> &indices,
                  const std::vector<C<T>> &values,
                  const std::vector<size_t> &cwires,
                  const std::vector<bool> &cvals,
                  const std::vector<size_t> &wires) {
    ORC_CHECK(!wires.empty(), "Number of wires must be larger than 0");
    const size_t dim = size_t{1} << wires.size();
    ORC_CHECK(indptr.size() == dim + 1,
              "The size of matrix does not match with the given number of "
              "wires");
    ORC_CHECK(wires.size() <= 6, "oracle supports sparse matrices on <= 6 wires");
    for_groups<T>(arr, n, wires, cwires, cvals,
                  [&](C<T> *a, const size_t *ix) {
                      C<T> v[64];
                      for (size_t i = 0; i < dim; i++) {
                          v[i] = a[ix[i]];
                      }
                      for (size_t i = 0; i < dim; i++) {
                          C<T> acc = 0.0;
                          for (size_t p = indptr[i]; p < indptr[i + 1]; p++) {
                              acc += values[p] * v[indices[p]];
                          }
                          a[ix[i]] = acc;
                      }
                  });
}

// PauliRot (LM:577-629)
template <class T>
void apply_pauli_rot(C<T> *arr, size_t n, const std::vector<size_t> &wires,
                     bool inverse, T angle, const std::string &word);

template <class T>
void apply_multirz(C<T> *arr, size_t n, const std::vector<size_t> &cwires,
                   const std::vector<bool> &cvals,
                   const std::vector<size_t> &wires, bool inverse, T angle) {
    // LM:1989-2043 applyMultiRZ / applyNCMultiRZ
    const C<T> first{std::cos(angle / 2), -std::sin(angle / 2)};
    const C<T> second{std::cos(angle / 2), std::sin(angle / 2)};
    const C<T> shifts[2] = {inverse ? std::conj(first) : first,
                            inverse ? std::conj(second) : second};
    size_t parity = 0;
    for (auto w : wires) {
        parity |= size_t{1} << (n - 1 - w);
    }
    if (cwires.empty()) {
        const long long N = static_cast<long long>(size_t{1} << n);
#pragma omp parallel for schedule(static)
        for (long long k = 0; k < N; k++) {
            arr[k] *= shifts[std::popcount(static_cast<size_t>(k) & parity) % 2];
        }
        return;
    }
    const size_t nloc = size_t{1} << wires.size();
    for_groups<T>(arr, n, wires, cwires, cvals,
                  [&](C<T> *a, const size_t *ix) {
                      for (size_t j = 0; j < nloc; j++) {
                          a[ix[j]] *= shifts[std::popcount(ix[j] & parity) % 2];
                      }
                  });
}

template <class T>
void apply_phase_shift(C<T> *arr, size_t n, const std::vector<size_t> &cwires,
                       const std::vector<bool> &cvals,
                       const std::vector<size_t> &wires, bool inverse,
                       T angle) {
    // LM:1001-1031 applyNCPhaseShift
    const C<T> s = inverse ? std::exp(-C<T>(0, angle)) : std::exp(C<T>(0, angle));
    for_groups<T>(arr, n, wires, cwires, cvals,
                  [&s](C<T> *a, const size_t *ix) { a[ix[1]] *= s; });
}

template <class T>
void apply_global_phase(C<T> *arr, size_t n, const std::vector<size_t> &cwires,
                        const std::vector<bool> &cvals, bool inverse,
                        T angle) {
    // LM:2046-2111 applyNCGlobalPhase
    const C<T> phase = std::exp(C<T>(0, inverse ? angle : -angle));
    if (n == 0) {
        arr[0] *= phase;
        return;
    }
    if (cwires.size() == 1 && cvals[0]) {
        apply_phase_shift<T>(arr, n, {}, {}, cwires, inverse, -angle);
        return;
    }
    if (n == 1 && cwires.size() == 1 && !cvals[0]) {
        apply_phase_shift<T>(arr, n, {}, {}, cwires, inverse, angle);
        apply_global_phase<T>(arr, n, {}, {}, inverse, angle);
        return;
    }
    size_t target = 0;
    if (!cwires.empty()) {
        for (size_t i = 0; i < n; i++) {
            if (std::find(cwires.begin(), cwires.end(), i) == cwires.end()) {
                target = i;
                break;
            }
        }
    }
    for_groups<T>(arr, n, {target}, cwires, cvals,
                  [&phase](C<T> *a, const size_t *ix) {
                      a[ix[0]] *= phase;
                      a[ix[1]] *= phase;
                  });
}

// ---------------------------------------------------------------------------
// Named gates: GateImplementationsLM.hpp, one core per gate.
// ---------------------------------------------------------------------------
template <class T>
void apply_named(C<T> *arr, size_t n, const std::string &name,
                 std::vector<size_t> cw, std::vector<bool> cv,
                 std::vector<size_t> wires, bool inverse,
                 const std::vector<T> &params) {
    ORC_CHECK(cw.size() == cv.size(),
              "`controlled_wires` must have the same size as "
              "`controlled_values`.");
    auto P = [&](size_t i) -> T {
        ORC_CHECK(params.size() > i, "missing gate parameter");
        return params[i];
    };
    auto need = [&](size_t k) {
        ORC_CHECK(wires.size() == k, "wrong number of wires for gate " + name);
    };
    // The uncontrolled two/three-wire gates below are the controlled one-wire
    // gates of LM (CNOT = applyNC2 core on (i10,i11), Toffoli = NCPauliX ...).
    auto lift = [&](size_t ncontrols) {
        for (size_t i = 0; i < ncontrols; i++) {
            cw.push_back(wires[i]);
            cv.push_back(true);
        }
        wires.erase(wires.begin(), wires.begin() + static_cast<long>(ncontrols));
    };
    if (name == "Identity") {
        return;
    }
    if (name == "CNOT" || name == "CY" || name == "CZ" || name == "CRX" ||
        name == "CRY" || name == "CRZ" || name == "CRot" ||
        name == "ControlledPhaseShift" || name == "CSWAP") {
        need(name == "CSWAP" ? 3 : 2);
        ORC_CHECK(cw.empty(), "gate " + name + " takes no extra controls");
        lift(1);
    } else if (name == "Toffoli") {
        need(3);
        ORC_CHECK(cw.empty(), "gate Toffoli takes no extra controls");
        lift(2);
    }
    const std::string base =
        name == "CNOT"                   ? "PauliX"
        : name == "Toffoli"              ? "PauliX"
        : name == "CY"                   ? "PauliY"
        : name == "CZ"                   ? "PauliZ"
        : name == "CRX"                  ? "RX"
        : name == "CRY"                  ? "RY"
        : name == "CRZ"                  ? "RZ"
        : name == "CRot"                 ? "Rot"
        : name == "ControlledPhaseShift" ? "PhaseShift"
        : name == "CSWAP"                ? "SWAP"
                                         : name;
    const bool uncontrolled_form = (base == name);

    if (base == "PauliX") { // LM:705-734
        need(1);
        for_groups<T>(arr, n, wires, cw, cv, [](C<T> *a, const size_t *ix) {
            std::swap(a[ix[0]], a[ix[1]]);
        });
    } else if (base == "PauliY") { // LM:762-800
        need(1);
        for_groups<T>(arr, n, wires, cw, cv, [](C<T> *a, const size_t *ix) {
            const auto v0 = a[ix[0]];
            const auto v1 = a[ix[1]];
            a[ix[0]] = {std::imag(v1), -std::real(v1)};
            a[ix[1]] = {-std::imag(v0), std::real(v0)};
        });
    } else if (base == "PauliZ") { // LM:820-855
        need(1);
        for_groups<T>(arr, n, wires, cw, cv,
                      [](C<T> *a, const size_t *ix) { a[ix[1]] *= -1; });
    } else if (base == "Hadamard") { // LM:857-890
        need(1);
        const T isqrt2 = INVSQRT2<T>();
        for_groups<T>(arr, n, wires, cw, cv, [isqrt2](C<T> *a, const size_t *ix) {
            const C<T> v0 = a[ix[0]];
            const C<T> v1 = a[ix[1]];
            a[ix[0]] = isqrt2 * v0 + isqrt2 * v1;
            a[ix[1]] = isqrt2 * v0 - isqrt2 * v1;
        });
    } else if (base == "S") { // LM:892-925
        need(1);
        const C<T> shift = inverse ? -IMAG<T>() : IMAG<T>();
        for_groups<T>(arr, n, wires, cw, cv,
                      [shift](C<T> *a, const size_t *ix) { a[ix[1]] *= shift; });
    } else if (base == "T") { // LM:927-958
        need(1);
        const T isqrt2 = INVSQRT2<T>();
        const C<T> shift = {isqrt2, inverse ? -isqrt2 : isqrt2};
        for_groups<T>(arr, n, wires, cw, cv,
                      [shift](C<T> *a, const size_t *ix) { a[ix[1]] *= shift; });
    } else if (base == "SX") { // LM:960-1000
        need(1);
        const T shift = inverse ? T(-1.0) : T(1.0);
        for_groups<T>(arr, n, wires, cw, cv, [shift](C<T> *a, const size_t *ix) {
            const C<T> v0 = a[ix[0]];
            const C<T> v1 = a[ix[1]];
            const T vr_plus = v0.real() + v1.real();
            const T vi_plus = v0.imag() + v1.imag();
            const T vr_minus = (v0.real() - v1.real()) * shift;
            const T vi_minus = (-v0.imag() + v1.imag()) * shift;
            a[ix[0]] = C<T>(vr_plus + vi_minus, vi_plus + vr_minus) * T(0.5);
            a[ix[1]] = C<T>(vr_plus - vi_minus, vi_plus - vr_minus) * T(0.5);
        });
    } else if (base == "PhaseShift") { // LM:1001-1031
        need(1);
        apply_phase_shift<T>(arr, n, cw, cv, wires, inverse, P(0));
    } else if (base == "RX") { // LM:1063-1095
        need(1);
        const T angle = P(0);
        const T c = std::cos(angle / 2);
        const T js = inverse ? -std::sin(-angle / 2) : std::sin(-angle / 2);
        for_groups<T>(arr, n, wires, cw, cv, [c, js](C<T> *a, const size_t *ix) {
            const C<T> v0 = a[ix[0]];
            const C<T> v1 = a[ix[1]];
            a[ix[0]] = c * v0 + C<T>{-std::imag(v1) * js, std::real(v1) * js};
            a[ix[1]] = C<T>{-std::imag(v0) * js, std::real(v0) * js} + c * v1;
        });
    } else if (base == "RY") { // LM:1126-1158
        need(1);
        const T angle = P(0);
        const T c = std::cos(angle / 2);
        const T s = inverse ? -std::sin(angle / 2) : std::sin(angle / 2);
        for_groups<T>(arr, n, wires, cw, cv, [c, s](C<T> *a, const size_t *ix) {
            const C<T> v0 = a[ix[0]];
            const C<T> v1 = a[ix[1]];
            a[ix[0]] = C<T>{c * std::real(v0) - s * std::real(v1),
                            c * std::imag(v0) - s * std::imag(v1)};
            a[ix[1]] = C<T>{s * std::real(v0) + c * std::real(v1),
                            s * std::imag(v0) + c * std::imag(v1)};
        });
    } else if (base == "RZ") { // LM:1190-1220
        need(1);
        const T angle = P(0);
        const C<T> first{std::cos(angle / 2), -std::sin(angle / 2)};
        const C<T> second{std::cos(angle / 2), std::sin(angle / 2)};
        const C<T> s0 = inverse ? std::conj(first) : first;
        const C<T> s1 = inverse ? std::conj(second) : second;
        for_groups<T>(arr, n, wires, cw, cv, [s0, s1](C<T> *a, const size_t *ix) {
            a[ix[0]] *= s0;
            a[ix[1]] *= s1;
        });
    } else if (base == "Rot") { // LM:1262-1301
        need(1);
        if (uncontrolled_form && cw.empty()) {
            const auto m = inverse ? rot_matrix<T>(-P(2), -P(1), -P(0))
                                   : rot_matrix<T>(P(0), P(1), P(2));
            apply_matrix<T>(arr, n, m, {}, {}, wires, false);
        } else if (uncontrolled_form) {
            apply_matrix<T>(arr, n, rot_matrix<T>(P(0), P(1), P(2)), cw, cv,
                            wires, inverse);
        } else { // CRot: LM applyCRot uses the Rot rule for the inverse
            const auto m = inverse ? rot_matrix<T>(-P(2), -P(1), -P(0))
                                   : rot_matrix<T>(P(0), P(1), P(2));
            apply_matrix<T>(arr, n, m, cw, cv, wires, false);
        }
    } else if (base == "SWAP") { // LM:1388-1426
        need(2);
        for_groups<T>(arr, n, wires, cw, cv, [](C<T> *a, const size_t *ix) {
            std::swap(a[ix[2]], a[ix[1]]);
        });
    } else if (base == "IsingXX") { // LM:1429-1467
        need(2);
        const T angle = P(0);
        const T cr = std::cos(angle / 2);
        const T sj = inverse ? -std::sin(angle / 2) : std::sin(angle / 2);
        for_groups<T>(arr, n, wires, cw, cv, [cr, sj](C<T> *a, const size_t *ix) {
            const C<T> v00 = a[ix[0]], v01 = a[ix[1]], v10 = a[ix[2]],
                       v11 = a[ix[3]];
            a[ix[0]] = C<T>{cr * v00.real() + sj * v11.imag(),
                            cr * v00.imag() - sj * v11.real()};
            a[ix[1]] = C<T>{cr * v01.real() + sj * v10.imag(),
                            cr * v01.imag() - sj * v10.real()};
            a[ix[2]] = C<T>{cr * v10.real() + sj * v01.imag(),
                            cr * v10.imag() - sj * v01.real()};
            a[ix[3]] = C<T>{cr * v11.real() + sj * v00.imag(),
                            cr * v11.imag() - sj * v00.real()};
        });
    } else if (base == "IsingXY") { // LM:1469-1505
        need(2);
        const T angle = P(0);
        const T cr = std::cos(angle / 2);
        const T sj = inverse ? -std::sin(angle / 2) : std::sin(angle / 2);
        for_groups<T>(arr, n, wires, cw, cv, [cr, sj](C<T> *a, const size_t *ix) {
            const C<T> v01 = a[ix[1]], v10 = a[ix[2]];
            a[ix[1]] = C<T>{cr * v01.real() - sj * v10.imag(),
                            cr * v01.imag() + sj * v10.real()};
            a[ix[2]] = C<T>{cr * v10.real() - sj * v01.imag(),
                            cr * v10.imag() + sj * v01.real()};
        });
    } else if (base == "IsingYY") { // LM:1507-1545
        need(2);
        const T angle = P(0);
        const T cr = std::cos(angle / 2);
        const T sj = inverse ? -std::sin(angle / 2) : std::sin(angle / 2);
        for_groups<T>(arr, n, wires, cw, cv, [cr, sj](C<T> *a, const size_t *ix) {
            const C<T> v00 = a[ix[0]], v01 = a[ix[1]], v10 = a[ix[2]],
                       v11 = a[ix[3]];
            a[ix[0]] = C<T>{cr * v00.real() - sj * v11.imag(),
                            cr * v00.imag() + sj * v11.real()};
            a[ix[1]] = C<T>{cr * v01.real() + sj * v10.imag(),
                            cr * v01.imag() - sj * v10.real()};
            a[ix[2]] = C<T>{cr * v10.real() + sj * v01.imag(),
                            cr * v10.imag() - sj * v01.real()};
            a[ix[3]] = C<T>{cr * v11.real() - sj * v00.imag(),
                            cr * v11.imag() + sj * v00.real()};
        });
    } else if (base == "IsingZZ") { // LM:1547-1575
        need(2);
        const T angle = P(0);
        const C<T> first{std::cos(angle / 2), -std::sin(angle / 2)};
        const C<T> second{std::cos(angle / 2), std::sin(angle / 2)};
        const C<T> s0 = inverse ? std::conj(first) : first;
        const C<T> s1 = inverse ? std::conj(second) : second;
        for_groups<T>(arr, n, wires, cw, cv, [s0, s1](C<T> *a, const size_t *ix) {
            a[ix[0]] *= s0;
            a[ix[1]] *= s1;
            a[ix[2]] *= s1;
            a[ix[3]] *= s0;
        });
    } else if (base == "SingleExcitation" || base == "SingleExcitationMinus" ||
               base == "SingleExcitationPlus") { // LM:1613-1710
        need(2);
        const T angle = P(0);
        const T c = std::cos(angle / 2);
        const T s = inverse ? -std::sin(angle / 2) : std::sin(angle / 2);
        const bool minus = base == "SingleExcitationMinus";
        const bool plus = base == "SingleExcitationPlus";
        C<T> e{1, 0};
        if (minus) {
            e = inverse ? std::exp(C<T>(0, angle / 2))
                        : std::exp(-C<T>(0, angle / 2));
        } else if (plus) {
            e = inverse ? std::exp(-C<T>(0, angle / 2))
                        : std::exp(C<T>(0, angle / 2));
        }
        const bool phase = minus || plus;
        for_groups<T>(arr, n, wires, cw, cv,
                      [c, s, e, phase](C<T> *a, const size_t *ix) {
                          const C<T> v01 = a[ix[1]];
                          const C<T> v10 = a[ix[2]];
                          if (phase) {
                              a[ix[0]] *= e;
                          }
                          a[ix[1]] = c * v01 - s * v10;
                          a[ix[2]] = s * v01 + c * v10;
                          if (phase) {
                              a[ix[3]] *= e;
                          }
                      });
    } else if (base == "PSWAP") { // LM:1742-1770
        need(2);
        const T angle = P(0);
        const C<T> phase = std::exp(C<T>(0, inverse ? -angle : angle));
        for_groups<T>(arr, n, wires, cw, cv, [phase](C<T> *a, const size_t *ix) {
            a[ix[2]] *= phase;
            a[ix[1]] *= phase;
            std::swap(a[ix[2]], a[ix[1]]);
        });
    } else if (base == "DoubleExcitation" || base == "DoubleExcitationMinus" ||
               base == "DoubleExcitationPlus") { // LM:1798-1985
        need(4);
        const T angle = P(0);
        const T cr = std::cos(angle / 2);
        const T sj = inverse ? -std::sin(angle / 2) : std::sin(angle / 2);
        C<T> e{1, 0};
        const bool minus = base == "DoubleExcitationMinus";
        const bool plus = base == "DoubleExcitationPlus";
        if (minus) {
            e = inverse ? std::exp(C<T>{0, angle / 2})
                        : std::exp(C<T>{0, -angle / 2});
        } else if (plus) {
            e = inverse ? std::exp(C<T>{0, -angle / 2})
                        : std::exp(C<T>{0, angle / 2});
        }
        const bool phase = minus || plus;
        for_groups<T>(arr, n, wires, cw, cv,
                      [cr, sj, e, phase](C<T> *a, const size_t *ix) {
                          const C<T> v3 = a[ix[3]];
                          const C<T> v12 = a[ix[12]];
                          if (phase) {
                              for (size_t j = 0; j < 16; j++) {
                                  a[ix[j]] *= e;
                              }
                          }
                          a[ix[3]] = cr * v3 - sj * v12;
                          a[ix[12]] = sj * v3 + cr * v12;
                      });
    } else if (base == "MultiRZ") {
        ORC_CHECK(!wires.empty(), "MultiRZ needs wires");
        apply_multirz<T>(arr, n, cw, cv, wires, inverse, P(0));
    } else if (base == "GlobalPhase") {
        apply_global_phase<T>(arr, n, cw, cv, inverse, P(0));
    } else if (base == "PCPhase") { // LM:2114-2162
        const T angle = P(0);
        const T dim = P(1);
        const auto dim_size = static_cast<size_t>(std::round(dim));
        ORC_CHECK(dim_size <= (size_t{1} << n),
                  "The dimension of the PCPhase gate must be a positive "
                  "integer and less than or equal to statevector size.");
        const T ph = inverse ? -angle : angle;
        const C<T> upper{std::cos(ph), std::sin(ph)};
        const C<T> lower = std::conj(upper);
        const size_t md = size_t{1} << wires.size();
        std::vector<C<T>> m(md * md);
        for (size_t i = 0; i < md; i++) {
            m[i * md + i] = i < dim_size ? upper : lower;
        }
        apply_matrix<T>(arr, n, m, cw, cv, wires, false);
    } else {
        throw OracleError("Gate " + name + " is not supported");
    }
}

// ---------------------------------------------------------------------------
// Generators: LM:2165-2940 and PauliGenerator.hpp:27-57.  Controlled forms
// zero every amplitude outside the control subspace (applyNCGenerator1/2/4).
// ---------------------------------------------------------------------------
template <class T>
void zero_outside_controls(C<T> *arr, size_t n, const std::vector<size_t> &cw,
                           const std::vector<bool> &cv) {
    if (cw.empty()) {
        return;
    }
    size_t mask = 0, val = 0;
    for (size_t i = 0; i < cw.size(); i++) {
        mask |= size_t{1} << (n - 1 - cw[i]);
        if (cv[i]) {
            val |= size_t{1} << (n - 1 - cw[i]);
        }
    }
    const long long N = static_cast<long long>(size_t{1} << n);
#pragma omp parallel for schedule(static)
    for (long long k = 0; k < N; k++) {
        if ((static_cast<size_t>(k) & mask) != val) {
            arr[k] = 0;
        }
    }
}

template <class T>
T apply_generator(C<T> *arr, size_t n, const std::string &name,
                  std::vector<size_t> cw, std::vector<bool> cv,
                  std::vector<size_t> wires) {
    auto need = [&](size_t k) {
        ORC_CHECK(wires.size() == k, "wrong number of wires for generator " + name);
    };
    auto lift = [&]() {
        ORC_CHECK(cw.empty(), "generator " + name + " takes no extra controls");
        cw.push_back(wires[0]);
        cv.push_back(true);
        wires.erase(wires.begin());
    };
    std::string base = name;
    if (name == "CRX" || name == "CRY" || name == "CRZ" ||
        name == "ControlledPhaseShift") {
        need(2);
        lift();
        base = name == "CRX"   ? "RX"
               : name == "CRY" ? "RY"
               : name == "CRZ" ? "RZ"
                               : "PhaseShift";
    }
    check_wires(n, wires, cw);
    if (base == "GlobalPhase") { // LM:2231-2265
        if (!cw.empty()) {
            zero_outside_controls<T>(arr, n, cw, cv);
        }
        return T(-1.0);
    }
    if (base == "MultiRZ") { // LM:2880-2940
        size_t parity = 0;
        for (auto w : wires) {
            parity |= size_t{1} << (n - 1 - w);
        }
        zero_outside_controls<T>(arr, n, cw, cv);
        size_t mask = 0, val = 0;
        for (size_t i = 0; i < cw.size(); i++) {
            mask |= size_t{1} << (n - 1 - cw[i]);
            if (cv[i]) {
                val |= size_t{1} << (n - 1 - cw[i]);
            }
        }
        const long long N = static_cast<long long>(size_t{1} << n);
#pragma omp parallel for schedule(static)
        for (long long k = 0; k < N; k++) {
            if ((static_cast<size_t>(k) & mask) == val) {
                arr[k] *= static_cast<T>(
                    1 - 2 * int(std::popcount(static_cast<size_t>(k) & parity) % 2));
            }
        }
        return -static_cast<T>(0.5);
    }
    zero_outside_controls<T>(arr, n, cw, cv);
    const C<T> I = IMAG<T>();
    if (base == "RX") {
        need(1);
        for_groups<T>(arr, n, wires, cw, cv, [](C<T> *a, const size_t *ix) {
            std::swap(a[ix[0]], a[ix[1]]);
        });
        return -static_cast<T>(0.5);
    }
    if (base == "RY") {
        need(1);
        for_groups<T>(arr, n, wires, cw, cv, [](C<T> *a, const size_t *ix) {
            const auto v0 = a[ix[0]];
            const auto v1 = a[ix[1]];
            a[ix[0]] = {std::imag(v1), -std::real(v1)};
            a[ix[1]] = {-std::imag(v0), std::real(v0)};
        });
        return -static_cast<T>(0.5);
    }
    if (base == "RZ") {
        need(1);
        for_groups<T>(arr, n, wires, cw, cv,
                      [](C<T> *a, const size_t *ix) { a[ix[1]] *= -1; });
        return -static_cast<T>(0.5);
    }
    if (base == "PhaseShift") {
        need(1);
        for_groups<T>(arr, n, wires, cw, cv,
                      [](C<T> *a, const size_t *ix) { a[ix[0]] = C<T>{0.0}; });
        return static_cast<T>(1.0);
    }
    if (base == "IsingXX") {
        need(2);
        for_groups<T>(arr, n, wires, cw, cv, [](C<T> *a, const size_t *ix) {
            std::swap(a[ix[0]], a[ix[3]]);
            std::swap(a[ix[2]], a[ix[1]]);
        });
        return -static_cast<T>(0.5);
    }
    if (base == "IsingXY") {
        need(2);
        for_groups<T>(arr, n, wires, cw, cv, [](C<T> *a, const size_t *ix) {
            std::swap(a[ix[2]], a[ix[1]]);
            a[ix[0]] = C<T>{0.0};
            a[ix[3]] = C<T>{0.0};
        });
        return static_cast<T>(0.5);
    }
    if (base == "IsingYY") {
        need(2);
        for_groups<T>(arr, n, wires, cw, cv, [](C<T> *a, const size_t *ix) {
            const auto v00 = a[ix[0]];
            a[ix[0]] = -a[ix[3]];
            a[ix[3]] = -v00;
            std::swap(a[ix[2]], a[ix[1]]);
        });
        return -static_cast<T>(0.5);
    }
    if (base == "IsingZZ") {
        need(2);
        for_groups<T>(arr, n, wires, cw, cv, [](C<T> *a, const size_t *ix) {
            a[ix[2]] *= -1;
            a[ix[1]] *= -1;
        });
        return -static_cast<T>(0.5);
    }
    if (base == "SingleExcitation") {
        need(2);
        for_groups<T>(arr, n, wires, cw, cv, [I](C<T> *a, const size_t *ix) {
            a[ix[0]] = C<T>{};
            a[ix[1]] *= I;
            a[ix[2]] *= -I;
            a[ix[3]] = C<T>{};
            std::swap(a[ix[2]], a[ix[1]]);
        });
        return -static_cast<T>(0.5);
    }
    if (base == "SingleExcitationMinus") {
        need(2);
        for_groups<T>(arr, n, wires, cw, cv, [I](C<T> *a, const size_t *ix) {
            a[ix[1]] *= I;
            a[ix[2]] *= -I;
            std::swap(a[ix[2]], a[ix[1]]);
        });
        return -static_cast<T>(0.5);
    }
    if (base == "SingleExcitationPlus") {
        need(2);
        for_groups<T>(arr, n, wires, cw, cv, [I](C<T> *a, const size_t *ix) {
            a[ix[0]] *= -1;
            a[ix[1]] *= I;
            a[ix[2]] *= -I;
            a[ix[3]] *= -1;
            std::swap(a[ix[2]], a[ix[1]]);
        });
        return -static_cast<T>(0.5);
    }
    if (base == "PSWAP") {
        need(2);
        for_groups<T>(arr, n, wires, cw, cv, [](C<T> *a, const size_t *ix) {
            a[ix[0]] = C<T>{0.0};
            a[ix[3]] = C<T>{0.0};
            std::swap(a[ix[2]], a[ix[1]]);
        });
        return static_cast<T>(1.0);
    }
    if (base == "DoubleExcitation") {
        need(4);
        for_groups<T>(arr, n, wires, cw, cv, [I](C<T> *a, const size_t *ix) {
            const C<T> v3 = a[ix[3]];
            const C<T> v12 = a[ix[12]];
            for (size_t j = 0; j < 16; j++) {
                a[ix[j]] = C<T>{};
            }
            a[ix[3]] = -v12 * I;
            a[ix[12]] = v3 * I;
        });
        return -static_cast<T>(0.5);
    }
    if (base == "DoubleExcitationMinus") {
        need(4);
        for_groups<T>(arr, n, wires, cw, cv, [I](C<T> *a, const size_t *ix) {
            a[ix[3]] *= I;
            a[ix[12]] *= -I;
            std::swap(a[ix[12]], a[ix[3]]);
        });
        return -static_cast<T>(0.5);
    }
    if (base == "DoubleExcitationPlus") {
        need(4);
        for_groups<T>(arr, n, wires, cw, cv, [I](C<T> *a, const size_t *ix) {
            a[ix[3]] *= -I;
            a[ix[12]] *= I;
            std::swap(a[ix[12]], a[ix[3]]);
        });
        return static_cast<T>(0.5);
    }
    throw OracleError("Generator of " + name + " is not supported");
}

template <class T>
void apply_pauli_rot(C<T> *arr, size_t n, const std::vector<size_t> &wires,
                     bool inverse, T angle, const std::string &word) {
    ORC_CHECK(wires.size() == word.size(),
              "wires and word have incompatible dimensions.");
    if (std::all_of(word.begin(), word.end(), [](char w) { return w == 'Z'; })) {
        apply_multirz<T>(arr, n, {}, {}, wires, inverse, angle);
        return;
    }
    const C<T> I = IMAG<T>();
    const T c = std::cos(angle / 2);
    const C<T> s = (inverse ? I : -I) * std::sin(angle / 2);
    const C<T> sines[4] = {s, I * s, -s, -I * s};
    size_t mask_xy = 0, mask_y = 0, mask_z = 0;
    for (size_t i = 0; i < wires.size(); i++) {
        const size_t bit = size_t{1} << (n - 1 - wires[i]);
        if (word[i] != 'Z') {
            mask_xy |= bit;
        }
        if (word[i] == 'Y') {
            mask_y |= bit;
        }
        if (word[i] == 'Z') {
            mask_z |= bit;
        }
    }
    const int count_mask_y = std::popcount(mask_y);
    const long long N = static_cast<long long>(size_t{1} << n);
#pragma omp parallel for schedule(static)
    for (long long k = 0; k < N; k++) {
        const size_t i0 = static_cast<size_t>(k);
        const size_t i1 = i0 ^ mask_xy;
        if (i0 > i1) {
            continue;
        }
        const int count_y = std::popcount(i0 & mask_y) * 2;
        const int count_z = std::popcount(i0 & mask_z) * 2;
        const int sign_i0 = count_z + count_mask_y * 3 - count_y;
        const int sign_i1 = count_z + count_mask_y + count_y;
        const C<T> v0 = arr[i0];
        const C<T> v1 = arr[i1];
        arr[i0] = c * v0 + sines[sign_i0 % 4] * v1;
        arr[i1] = c * v1 + sines[sign_i1 % 4] * v0;
    }
}

// ---------------------------------------------------------------------------
// Linear algebra: LinearAlgebra.hpp innerProdC (:122-145), scaleAndAdd.
// ---------------------------------------------------------------------------
template <class T> C<T> inner_prod_c(const C<T> *a, const C<T> *b, size_t N) {
    T re = 0, im = 0;
    const long long NN = static_cast<long long>(N);
#pragma omp parallel for reduction(+ : re, im) schedule(static)
    for (long long i = 0; i < NN; i++) {
        const C<T> p = std::conj(a[i]) * b[i];
        re += p.real();
        im += p.imag();
    }
    return {re, im};
}

// ---------------------------------------------------------------------------
// State vector (StateVectorLQubitManaged.hpp + StateVectorLQubit.hpp).
// ---------------------------------------------------------------------------
template <class T> struct StateVec {
    size_t n;
    std::vector<C<T>> data;
    explicit StateVec(size_t nq) : n(nq), data(size_t{1} << nq) {
        data[0] = {1, 0};
    }
    size_t len() const { return data.size(); }
    C<T> *ptr() { return data.data(); }
};

// collapse / normalize (StateVectorLQubit.hpp:881-921)
template <class T> void normalize(StateVec<T> &sv) {
    T sq = 0;
    const long long N = static_cast<long long>(sv.len());
#pragma omp parallel for reduction(+ : sq) schedule(static)
    for (long long k = 0; k < N; k++) {
        sq += std::norm(sv.data[k]);
    }
    const T norm = std::sqrt(sq);
    ORC_CHECK(!(norm < std::numeric_limits<T>::epsilon() * 1e2),
              "Vector has norm close to zero and cannot be normalized");
    const C<T> inv = T(1.) / norm;
#pragma omp parallel for schedule(static)
    for (long long k = 0; k < N; k++) {
        sv.data[k] *= inv;
    }
}
template <class T> void collapse(StateVec<T> &sv, size_t wire, bool branch) {
    ORC_CHECK(wire < sv.n, "wire index out of range");
    const size_t bit = size_t{1} << (sv.n - 1 - wire);
    const long long N = static_cast<long long>(sv.len());
#pragma omp parallel for schedule(static)
    for (long long k = 0; k < N; k++) {
        const bool one = (static_cast<size_t>(k) & bit) != 0;
        if (one != branch) {
            sv.data[k] = {0., 0.};
        }
    }
    normalize(sv);
}

// ---------------------------------------------------------------------------
// Observables (core/observables/Observables.hpp, LQ/observables/...).
// ---------------------------------------------------------------------------
template <class T> struct Obs {
    virtual ~Obs() = default;
    virtual void apply(StateVec<T> &sv) const = 0;
};
template <class T> using ObsPtr = std::shared_ptr<Obs<T>>;

template <class T> struct NamedObs : Obs<T> { // Observables.hpp:172-174
    std::string name;
    std::vector<size_t> wires;
    void apply(StateVec<T> &sv) const override {
        apply_named<T>(sv.ptr(), sv.n, name, {}, {}, wires, false, {});
    }
};
template <class T> struct HermObs : Obs<T> { // Observables.hpp:286-288
    std::vector<C<T>> m;
    std::vector<size_t> wires;
    void apply(StateVec<T> &sv) const override {
        apply_matrix<T>(sv.ptr(), sv.n, m, {}, {}, wires, false);
    }
};
template <class T> struct ProdObs : Obs<T> { // Observables.hpp:414-418
    std::vector<ObsPtr<T>> obs;
    void apply(StateVec<T> &sv) const override {
        for (const auto &o : obs) {
            o->apply(sv);
        }
    }
};
template <class T> struct HamObs : Obs<T> { // ObservablesLQubit.hpp:156-251
    std::vector<T> coeffs;
    std::vector<ObsPtr<T>> obs;
    void apply(StateVec<T> &sv) const override {
        std::vector<C<T>> res(sv.len(), C<T>{0.0, 0.0});
        StateVec<T> tmp(sv.n);
        for (size_t t = 0; t < obs.size(); t++) {
            tmp.data = sv.data;
            obs[t]->apply(tmp);
            const C<T> c{coeffs[t], 0.0};
            const long long N = static_cast<long long>(sv.len());
#pragma omp parallel for schedule(static)
            for (long long k = 0; k < N; k++) {
                res[k] += c * tmp.data[k];
            }
        }
        sv.data.swap(res);
    }
};
template <class T> struct SparseObs : Obs<T> { // ObservablesLQubit.hpp:426-435
    std::vector<C<T>> data;
    std::vector<size_t> indices, indptr, wires;
    void apply(StateVec<T> &sv) const override {
        ORC_CHECK(wires.size() == sv.n,
                  "SparseH wire count does not match state-vector size");
        std::vector<C<T>> out(sv.len());
        const long long N = static_cast<long long>(sv.len());
#pragma omp parallel for schedule(static)
        for (long long r = 0; r < N; r++) {
            C<T> acc = 0;
            for (size_t p = indptr[r]; p < indptr[r + 1]; p++) {
                acc += data[p] * sv.data[indices[p]];
            }
            out[r] = acc;
        }
        sv.data.swap(out);
    }
};

// ---------------------------------------------------------------------------
// Measurements (LQ/measurements/MeasurementsLQubit.hpp).
// ---------------------------------------------------------------------------
template <class T>
std::vector<T> probs(const StateVec<T> &sv, const std::vector<size_t> &wires) {
    // :90-163.  Output index: wires[0] is its most significant bit.
    const size_t n = sv.n;
    if (wires.empty()) {
        return {1.0};
    }
    bool all = wires.size() == n;
    for (size_t k = 0; k < wires.size() && all; k++) {
        all = wires[k] == k;
    }
    if (all) {
        std::vector<T> p(sv.len());
        const long long N = static_cast<long long>(sv.len());
#pragma omp parallel for schedule(static)
        for (long long k = 0; k < N; k++) {
            p[k] = std::norm(sv.data[k]);
        }
        return p;
    }
    check_wires(n, wires, {});
    const Groups g = make_groups(n, wires, {}, {});
    const size_t np = g.local.size();
    std::vector<T> p(np, 0);
    const long long npl = static_cast<long long>(np);
#pragma omp parallel for schedule(static)
    for (long long j = 0; j < npl; j++) {
        T acc = 0;
        for (size_t k = 0; k < g.count; k++) {
            acc += std::norm(sv.data[g.local[j] + g.offset(k)]);
        }
        p[j] = acc;
    }
    return p;
}

template <class T>
T expval_named(const StateVec<T> &sv, const std::string &name,
               const std::vector<size_t> &wires) {
    // :247-305 + ExpValFunc.hpp:69-90 applyExpVal1
    if (name == "Identity") {
        return 1.0;
    }
    ORC_CHECK(wires.size() == 1, "named expval takes one wire");
    check_wires(sv.n, wires, {});
    const size_t bit = size_t{1} << (sv.n - 1 - wires[0]);
    const std::vector<size_t> m = spread_masks({sv.n - 1 - wires[0]});
    const long long half = static_cast<long long>(sv.len() / 2);
    const C<T> *a = sv.data.data();
    int kind = name == "PauliX" ? 0 : name == "PauliY" ? 1 : name == "PauliZ" ? 2
             : name == "Hadamard" ? 3 : -1;
    ORC_CHECK(kind >= 0, "Expval does not exist for named observable " + name);
    T ev = 0;
#pragma omp parallel for reduction(+ : ev) schedule(static)
    for (long long k = 0; k < half; k++) {
        const size_t i0 = spread(m, static_cast<size_t>(k));
        const size_t i1 = i0 | bit;
        switch (kind) {
        case 0:
            ev += (a[i0].real() * a[i1].real() + a[i0].imag() * a[i1].imag()) * 2.0;
            break;
        case 1:
            ev += (a[i0].real() * a[i1].imag() - a[i0].imag() * a[i1].real()) * 2.0;
            break;
        case 2:
            ev += std::norm(a[i0]) - std::norm(a[i1]);
            break;
        default: {
            const C<T> v0 = a[i0], v1 = a[i1];
            ev += static_cast<T>(M_SQRT1_2) *
                  (std::norm(v0) - std::norm(v1) +
                   2.0 * (v0.real() * v1.real() + v0.imag() * v1.imag()));
        }
        }
    }
    return ev;
}

template <class T>
T expval_matrix(const StateVec<T> &sv, const std::vector<C<T>> &mat,
                const std::vector<size_t> &wires) {
    // :213-238 + ExpValFunc.hpp:107-335 applyExpValMatWires*
    const size_t dim = size_t{1} << wires.size();
    ORC_CHECK(mat.size() == dim * dim,
              "The size of matrix does not match with the given number of "
              "wires");
    check_wires(sv.n, wires, {});
    const Groups g = make_groups(sv.n, wires, {}, {});
    const C<T> *a = sv.data.data();
    T ev = 0;
    const long long count = static_cast<long long>(g.count);
#pragma omp parallel for reduction(+ : ev) schedule(static)
    for (long long k = 0; k < count; k++) {
        const size_t off = g.offset(static_cast<size_t>(k));
        for (size_t i = 0; i < dim; i++) {
            C<T> row = 0;
            for (size_t j = 0; j < dim; j++) {
                row += mat[i * dim + j] * a[g.local[j] + off];
            }
            ev += std::real(std::conj(a[g.local[i] + off]) * row);
        }
    }
    return ev;
}

template <class T> T expval_obs(const StateVec<T> &sv, const Obs<T> &obs) {
    // :372-394 (copy, applyInPlace, innerProdC)
    StateVec<T> bra(sv);
    obs.apply(bra);
    return std::real(inner_prod_c(bra.data.data(), sv.data.data(), sv.len()));
}
template <class T> T var_obs(const StateVec<T> &sv, const Obs<T> &obs) {
    // :420-442 calculateObsVar
    StateVec<T> bra(sv);
    obs.apply(bra);
    const T ms = std::real(inner_prod_c(bra.data.data(), bra.data.data(), bra.len()));
    const T sm = std::real(inner_prod_c(bra.data.data(), sv.data.data(), sv.len()));
    return ms - static_cast<T>(std::pow(sm, 2));
}
template <class T>
T expval_sparse(const StateVec<T> &sv, const std::vector<size_t> &indptr,
                const std::vector<size_t> &indices, const std::vector<C<T>> &data) {
    // :322-338
    ORC_CHECK(sv.len() == indptr.size() - 1,
              "Statevector and Hamiltonian have incompatible sizes.");
    SparseObs<T> o;
    o.data = data;
    o.indices = indices;
    o.indptr = indptr;
    o.wires.resize(sv.n);
    std::iota(o.wires.begin(), o.wires.end(), 0);
    StateVec<T> tmp(sv);
    o.apply(tmp);
    return std::real(inner_prod_c(sv.data.data(), tmp.data.data(), sv.len()));
}

// Alias-method sampler: MeasurementKernels.hpp:308-381 DiscreteRandomVariable
template <class T> struct AliasSampler {
    static constexpr size_t none = std::numeric_limits<size_t>::max();
    std::mt19937 &gen;
    size_t n;
    std::vector<std::pair<double, size_t>> buckets;
    mutable std::uniform_real_distribution<T> dist{0.0, 1.0};
    AliasSampler(std::mt19937 &g, const std::vector<T> &p)
        : gen(g), n(p.size()), buckets(p.size(), {0.0, none}) {
        std::stack<size_t> under, over;
        for (size_t i = 0; i < n; i++) {
            buckets[i].first = n * p[i];
            if (buckets[i].first < 1.0) {
                under.push(i);
            } else {
                over.push(i);
            }
        }
        while (!under.empty() && !over.empty()) {
            auto i = over.top();
            over.pop();
            auto j = under.top();
            under.pop();
            buckets[j].second = i;
            buckets[i].first += buckets[j].first - 1.0;
            if (buckets[i].first < 1.0) {
                under.push(i);
            } else {
                over.push(i);
            }
        }
    }
    size_t operator()() const {
        const auto idx = static_cast<size_t>(dist(gen) * n);
        if (dist(gen) >= buckets[idx].first && buckets[idx].second != none) {
            return buckets[idx].second;
        }
        return idx;
    }
};

// MeasurementsLQubit.hpp:646-679 generate_samples(wires, shots)
template <class T>
std::vector<size_t> samples(const StateVec<T> &sv, const std::vector<size_t> &wires,
                            size_t shots, size_t seed) {
    std::mt19937 rng;
    rng.seed(seed);
    const auto p = probs<T>(sv, wires);
    AliasSampler<T> drv{rng, p};
    const size_t nw = wires.size();
    std::vector<size_t> out(shots * nw);
    for (size_t s = 0; s < shots; s++) {
        const size_t idx = drv();
        for (size_t j = 0; j < nw; j++) {
            out[s * nw + (nw - 1 - j)] = (idx >> j) & 1U;
        }
    }
    return out;
}

// MeasurementsLQubit.hpp:551-594 generate_samples_metropolis and :740-770
// metropolis_step, with the transition kernels of TransitionKernels.hpp.
// kernel_factory (TransitionKernels.hpp:150-162) builds the non-zero-random
// kernel for the type Local (any name but "NonZeroRandom") and the local
// bit-flip kernel for NonZeroRandom; restated as the reference behaves.
template <class T>
std::vector<size_t> mcmc_samples(const StateVec<T> &sv, const std::string &kernel, size_t burnin, size_t shots,
                                 size_t seed) {
    std::mt19937 rng;
    rng.seed(seed);
    std::uniform_real_distribution<T> distrib(0.0, 1.0);
    const size_t n = sv.n;
    const bool nonzero_kernel = kernel != "NonZeroRandom";
    std::vector<size_t> nz;
    std::uniform_int_distribution<size_t> d_nz, d_site(0, n - 1), d_bin(0, 1);
    if (nonzero_kernel) {
        for (size_t i = 0; i < sv.len(); i++) {
            if (std::abs(sv.data[i]) > std::numeric_limits<T>::epsilon()) {
                nz.push_back(i);
            }
        }
        if (nz.empty()) {
            throw std::runtime_error("MCMC sampling: the state has no non-zero amplitude");
        }
        d_nz = std::uniform_int_distribution<size_t>(0, nz.size() - 1);
    }
    auto plog = [&](size_t i) { return std::log((sv.data[i] * std::conj(sv.data[i])).real()); };
    auto step = [&](size_t init) {
        const T init_plog = plog(init);
        size_t trans = init;
        if (nonzero_kernel) {
            trans = nz[d_nz(rng)];
        } else {
            const size_t site = d_site(rng);
            const size_t value = d_bin(rng);
            const size_t bit = (static_cast<unsigned>(init) >> static_cast<unsigned>(site)) & 1U;
            if (value != bit) {
                trans = bit == 0 ? init + (size_t{1} << site) : init - (size_t{1} << site);
            }
        }
        const T trans_plog = plog(trans);
        const T alph = std::min<T>(1., T(1) * std::exp(trans_plog - init_plog));
        const T ran = distrib(rng);
        return ran < alph ? trans : init;
    };
    std::vector<size_t> out(shots * n, 0);
    size_t idx = 0;
    for (size_t i = 0; i < burnin; i++) {
        idx = step(idx);
    }
    for (size_t s = 0; s < shots; s++) {
        idx = step(idx);
        for (size_t j = 0; j < n; j++) {
            out[s * n + (n - 1 - j)] = (idx >> j) & 1U;
        }
    }
    return out;
}

// ---------------------------------------------------------------------------
// Adjoint Jacobian (LQ/algorithms/AdjointJacobianLQubit.hpp:225-491,
// core/algorithms/AdjointJacobianBase.hpp, JacobianData.hpp OpsData).
// ---------------------------------------------------------------------------
template <class T> struct Op {
    std::string name;
    std::vector<T> params;
    std::vector<size_t> wires;
    bool inverse{false};
    std::vector<C<T>> matrix;
    std::vector<size_t> cwires;
    std::vector<bool> cvals;
};

inline bool is_named_gate(const std::string &name) {
    static const char *names[] = {
        "Identity", "PauliX", "PauliY", "PauliZ", "Hadamard", "S", "SX", "T",
        "PhaseShift", "RX", "RY", "RZ", "Rot", "CNOT", "CY", "CZ", "SWAP",
        "IsingXX", "IsingXY", "IsingYY", "IsingZZ", "ControlledPhaseShift",
        "CRX", "CRY", "CRZ", "CRot", "SingleExcitation",
        "SingleExcitationMinus", "SingleExcitationPlus", "PSWAP", "Toffoli",
        "CSWAP", "DoubleExcitation", "DoubleExcitationMinus",
        "DoubleExcitationPlus", "MultiRZ", "GlobalPhase", "PCPhase"};
    for (auto *nm : names) {
        if (name == nm) {
            return true;
        }
    }
    return false;
}

// StateVectorLQubit.hpp:431-482: named if known, else the matrix.
template <class T> void apply_op(StateVec<T> &sv, const Op<T> &op, bool inverse) {
    if (!op.cwires.empty()) {
        if (is_named_gate(op.name)) {
            apply_named<T>(sv.ptr(), sv.n, op.name, op.cwires, op.cvals, op.wires,
                           inverse, op.params);
        } else {
            apply_matrix<T>(sv.ptr(), sv.n, op.matrix, op.cwires, op.cvals,
                            op.wires, inverse);
        }
        return;
    }
    if (is_named_gate(op.name)) {
        apply_named<T>(sv.ptr(), sv.n, op.name, {}, {}, op.wires, inverse, op.params);
    } else {
        apply_matrix<T>(sv.ptr(), sv.n, op.matrix, {}, {}, op.wires, inverse);
    }
}

template <class T>
void adjoint_jacobian(std::vector<T> &jac, const StateVec<T> &state,
                      const std::vector<Op<T>> &ops,
                      const std::vector<ObsPtr<T>> &obs,
                      const std::vector<size_t> &tp, bool apply_ops) {
    const size_t nobs = obs.size();
    const size_t ntp = tp.size();
    jac.assign(nobs * ntp, T{0});
    if (ntp == 0) {
        return;
    }
    size_t num_param_ops = 0;
    for (const auto &op : ops) {
        num_param_ops += op.params.empty() ? 0 : 1;
    }
    StateVec<T> lambda(state);
    if (apply_ops) {
        for (const auto &op : ops) {
            apply_op(lambda, op, op.inverse);
        }
    }
    std::vector<StateVec<T>> hl(nobs, StateVec<T>(state.n));
    for (size_t h = 0; h < nobs; h++) {
        hl[h].data = lambda.data;
        obs[h]->apply(hl[h]);
    }
    StateVec<T> mu(state.n);
    size_t tp_num = ntp - 1;
    size_t cur = num_param_ops - 1;
    auto tp_it = tp.rbegin();
    for (long op_idx = static_cast<long>(ops.size()) - 1; op_idx >= 0; op_idx--) {
        const auto &op = ops[static_cast<size_t>(op_idx)];
        ORC_CHECK(op.params.size() <= 1,
                  "The operation is not supported using the adjoint "
                  "differentiation method");
        if (op.name == "StatePrep" || op.name == "BasisState") {
            continue;
        }
        if (tp_it == tp.rend()) {
            break;
        }
        if (!op.params.empty()) {
            if (cur == *tp_it) {
                mu.data = lambda.data;
                const T scale =
                    apply_generator<T>(mu.ptr(), mu.n, op.name, op.cwires,
                                       op.cvals, op.wires) *
                    (op.inverse ? -1 : 1);
                // AdjointJacobianLQubit.hpp:60-77: jac[row + obs] layout,
                // transposed to [obs][param] at the end.
                for (size_t h = 0; h < nobs; h++) {
                    jac[tp_num * nobs + h] =
                        -2 * scale *
                        std::imag(inner_prod_c(hl[h].data.data(), mu.data.data(),
                                               mu.len()));
                }
                tp_num--;
                ++tp_it;
            }
            cur--;
        }
        apply_op(lambda, op, !op.inverse);
        for (size_t h = 0; h < nobs; h++) {
            apply_op(hl[h], op, !op.inverse);
        }
    }
    std::vector<T> t(jac.size());
    for (size_t p = 0; p < ntp; p++) {
        for (size_t h = 0; h < nobs; h++) {
            t[h * ntp + p] = jac[p * nobs + h];
        }
    }
    jac.swap(t);
}

// VectorJacobianProduct.hpp:79-160 (lightning_qubit/algorithms): w_j =
// <dy| d psi / d theta_j>.  The cotangent mu = dy and lambda = psi are swept
// back together (U^dagger on both, last op first); at a trainable
// parameter's op, with G its generator and s its scale (negated for an
// inverse op), w = i s <G mu | lambda>.
template <class T>
void vjp(std::vector<C<T>> &out, const StateVec<T> &state,
         const std::vector<Op<T>> &ops, const std::vector<C<T>> &dy,
         const std::vector<size_t> &tp, bool apply_ops) {
    ORC_CHECK(dy.size() == state.len(), "dy must have the state's length");
    const size_t ntp = tp.size();
    out.assign(ntp, C<T>{0, 0});
    if (ntp == 0) {
        return;
    }
    size_t num_param_ops = 0;
    for (const auto &op : ops) {
        num_param_ops += op.params.empty() ? 0 : 1;
    }
    StateVec<T> lambda(state);
    if (apply_ops) {
        for (const auto &op : ops) {
            apply_op(lambda, op, op.inverse);
        }
    }
    StateVec<T> mu(state.n);
    mu.data = dy;
    StateVec<T> gmu(state.n);
    size_t slot = ntp - 1;
    size_t cur = num_param_ops - 1;
    auto tp_it = tp.rbegin();
    for (long op_idx = static_cast<long>(ops.size()) - 1; op_idx >= 0; op_idx--) {
        const auto &op = ops[static_cast<size_t>(op_idx)];
        ORC_CHECK(op.params.size() <= 1,
                  "The operation is not supported using the adjoint "
                  "differentiation method");
        if (op.name == "StatePrep" || op.name == "BasisState") {
            continue;
        }
        if (tp_it == tp.rend()) {
            break;
        }
        if (!op.params.empty()) {
            if (cur == *tp_it) {
                gmu.data = mu.data;
                const T scale =
                    apply_generator<T>(gmu.ptr(), gmu.n, op.name, op.cwires,
                                       op.cvals, op.wires) *
                    (op.inverse ? -1 : 1);
                out[slot] = C<T>{0, scale} *
                            inner_prod_c(gmu.data.data(), lambda.data.data(),
                                         lambda.len());
                slot--;
                ++tp_it;
            }
            cur--;
        }
        apply_op(lambda, op, !op.inverse);
        apply_op(mu, op, !op.inverse);
    }
}

} // namespace orc
