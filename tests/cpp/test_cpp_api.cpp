// The C++ API (include/pl_gb300.hpp) driven the way a C++ caller of
// lightning.qubit drives StateVectorLQubitManaged / Measurements /
// AdjointJacobian, checked against the CPU oracle's C API (test
// infrastructure, liboracle.so) on the same circuit: state, probs, named and
// Hamiltonian expectation values, var, seeded samples, the adjoint Jacobian
// through JacobianData, and LightningException on a bad call.  Prints
// "PASS" and exits 0 when every check holds.
#include "pl_gb300.hpp"

#include "oracle_api.h"

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <random>
#include <string>
#include <vector>

using namespace Pennylane::LightningGB300;

namespace {
int failures = 0;
void expect(bool ok, const std::string &what) {
    if (!ok) {
        std::printf("FAIL: %s\n", what.c_str());
        failures++;
    }
}
template <class T> bool close_vec(const std::vector<T> &a, const std::vector<T> &b, double tol) {
    if (a.size() != b.size()) {
        return false;
    }
    double num = 0.0, den = 0.0;
    for (size_t i = 0; i < a.size(); i++) {
        num += std::norm(std::complex<double>(a[i]) - std::complex<double>(b[i]));
        den += std::norm(std::complex<double>(b[i]));
    }
    return std::sqrt(num) <= tol * std::sqrt(den);
}
bool close(double a, double b, double tol, double mag) { return std::abs(a - b) <= tol * std::max(std::abs(b), mag); }

template <class P> int run(double tol) {
    using SV = StateVectorGB300<P>;
    using C = std::complex<P>;
    const size_t n = 10;
    const int is_double = std::is_same_v<P, double> ? 1 : 0;
    std::mt19937_64 rng(1234);
    std::uniform_real_distribution<double> ang(0.0, 6.283185307179586);

    // config-0 style ansatz: RX, RY, RZ on every qubit, CNOT ring; plus one
    // controlled gate and one dense matrix
    std::vector<std::string> names;
    std::vector<std::vector<P>> params;
    std::vector<std::vector<size_t>> wires;
    for (int layer = 0; layer < 3; layer++) {
        for (size_t q = 0; q < n; q++) {
            for (const char *g : {"RX", "RY", "RZ"}) {
                names.emplace_back(g);
                params.push_back({static_cast<P>(ang(rng))});
                wires.push_back({q});
            }
        }
        for (size_t q = 0; q < n; q++) {
            names.emplace_back("CNOT");
            params.emplace_back();
            wires.push_back({q, (q + 1) % n});
        }
    }
    SV sv(n);
    sv.applyOperations(names, wires, std::vector<bool>(names.size(), false), params);
    sv.applyOperation("RY", {3, 0}, {true, false}, {7}, false, {static_cast<P>(0.7)});
    const double s = std::sqrt(0.5);
    const std::vector<C> had{C(s), C(s), C(s), C(-s)};
    sv.applyMatrix(had, {5});

    void *o = orc_sv_new(static_cast<int>(n), is_double);
    std::vector<C> zero(size_t{1} << n);
    zero[0] = 1;
    orc_sv_set_state(o, zero.data());
    for (size_t k = 0; k < names.size(); k++) {
        std::vector<int64_t> w(wires[k].begin(), wires[k].end());
        std::vector<double> p(params[k].begin(), params[k].end());
        orc_sv_apply(o, names[k].c_str(), nullptr, nullptr, 0, w.data(), static_cast<int>(w.size()), 0, p.data(),
                     static_cast<int>(p.size()));
    }
    {
        const int64_t cw[2] = {3, 0}, w[1] = {7};
        const uint8_t cv[2] = {1, 0};
        const double p[1] = {static_cast<double>(static_cast<P>(0.7))};
        orc_sv_apply(o, "RY", cw, cv, 2, w, 1, 0, p, 1);
        const double m[8] = {s, 0, s, 0, s, 0, -s, 0};
        const int64_t w5[1] = {5};
        orc_sv_apply_matrix(o, m, nullptr, nullptr, 0, w5, 1, 0);
    }
    std::vector<C> ref(size_t{1} << n);
    orc_sv_get_state(o, ref.data());
    expect(close_vec(sv.getDataVector(), ref, tol), "state vs oracle");

    MeasurementsGB300<SV> m(sv);
    const auto pr = m.probs({4, 1});
    std::vector<double> pref(4);
    const int64_t pw[2] = {4, 1};
    orc_probs(o, pw, 2, pref.data());
    expect(close_vec(std::vector<double>(pr.begin(), pr.end()), pref, tol), "probs({4, 1})");

    double e_ref = 0.0;
    const int64_t w2[1] = {2};
    orc_expval_named(o, "PauliX", w2, 1, &e_ref);
    expect(close(m.expval("PauliX", {2}), e_ref, tol, 1.0), "expval(PauliX, {2})");

    // H = 0.5 Z0 Z1 - 1.25 Y2 + 0.3 X9
    auto z0 = std::make_shared<NamedObs<SV>>("PauliZ", std::vector<size_t>{0});
    auto z1 = std::make_shared<NamedObs<SV>>("PauliZ", std::vector<size_t>{1});
    auto y2 = std::make_shared<NamedObs<SV>>("PauliY", std::vector<size_t>{2});
    auto x9 = std::make_shared<NamedObs<SV>>("PauliX", std::vector<size_t>{9});
    auto zz = TensorProdObs<SV>::create({z0, z1});
    auto H = Hamiltonian<SV>::create({static_cast<P>(0.5), static_cast<P>(-1.25), static_cast<P>(0.3)}, {zz, y2, x9});
    const std::string spec = "ham 3 0.5 prod 2 named PauliZ 0 named PauliZ 1 -1.25 named PauliY 2 0.3 named PauliX 9";
    double h_ref = 0.0, v_ref = 0.0;
    orc_expval_obs(o, spec.c_str(), nullptr, nullptr, &h_ref);
    orc_var_obs(o, spec.c_str(), nullptr, nullptr, &v_ref);
    expect(close(m.expval(*H), h_ref, tol, 2.05), "expval(Hamiltonian)");
    expect(close(m.var(*H), v_ref, tol, 2.05 * 2.05), "var(Hamiltonian)");
    expect(H->getWires().size() == 4, "Hamiltonian wires");

    m.setSeed(37);
    const auto smp = m.generate_samples({7, 0, 2}, 2000);
    std::vector<int64_t> sref(2000 * 3);
    const int64_t sw[3] = {7, 0, 2};
    orc_samples(o, sw, 3, 2000, 37, sref.data());
    bool same = smp.size() == sref.size();
    for (size_t i = 0; same && i < smp.size(); i++) {
        same = static_cast<int64_t>(smp[i]) == sref[i];
    }
    expect(same, "seeded samples equal the oracle's");

    // adjoint Jacobian of <H> over every parameter of the ansatz
    std::vector<std::vector<C>> mats(names.size());
    OpsData<SV> ops(names, params, wires, std::vector<bool>(names.size(), false), mats);
    std::vector<size_t> tp;
    for (size_t k = 0; k < ops.getNumParOps(); k++) {
        tp.push_back(k);
    }
    JacobianData<SV> jd(tp.size(), zero.size(), zero.data(), {H}, ops, tp);
    std::vector<P> jac(tp.size());
    AdjointJacobianGB300<SV>().adjointJacobian(std::span<P>(jac), jd, sv, true);

    std::vector<const char *> cn;
    std::vector<double> cp;
    std::vector<int> np, nw;
    std::vector<int64_t> cwv, msz(names.size(), 0), t64(tp.begin(), tp.end());
    std::vector<uint8_t> inv(names.size(), 0);
    std::vector<int> ncw(names.size(), 0);
    for (size_t k = 0; k < names.size(); k++) {
        cn.push_back(names[k].c_str());
        np.push_back(static_cast<int>(params[k].size()));
        cp.insert(cp.end(), params[k].begin(), params[k].end());
        nw.push_back(static_cast<int>(wires[k].size()));
        cwv.insert(cwv.end(), wires[k].begin(), wires[k].end());
    }
    const char *specs[1] = {spec.c_str()};
    std::vector<double> jref(tp.size());
    void *o2 = orc_sv_new(static_cast<int>(n), is_double);
    orc_sv_set_state(o2, zero.data());
    const int rc = orc_adjoint(o2, static_cast<int>(names.size()), cn.data(), cp.data(), np.data(), cwv.data(),
                               nw.data(), inv.data(), nullptr, msz.data(), nullptr, ncw.data(), nullptr, 1, specs,
                               nullptr, nullptr, t64.data(), static_cast<int>(t64.size()), 1, jref.data());
    expect(rc == 0, "oracle adjoint ran");
    expect(close_vec(std::vector<double>(jac.begin(), jac.end()), jref, tol), "adjoint Jacobian vs oracle");

    // shot-based <H> (MeasurementsBase.hpp:159-183): each term's state copy is
    // rotated into the term's eigenbasis and sampled with the seed, so the
    // complex128 value equals the one formed from the oracle's samples of the
    // same rotated states; complex64 within five standard errors
    {
        const int64_t shots = 4000;
        m.setSeed(41);
        const double e_shots = static_cast<double>(m.expval(*H, static_cast<size_t>(shots)));
        struct Term {
            double c;
            std::vector<std::pair<const char *, int64_t>> factors;
        };
        const Term terms[3] = {{0.5, {{"PauliZ", 0}, {"PauliZ", 1}}}, {-1.25, {{"PauliY", 2}}}, {0.3, {{"PauliX", 9}}}};
        double from_samples = 0.0;
        for (const auto &t : terms) {
            void *r = orc_sv_new(static_cast<int>(n), is_double);
            orc_sv_set_state(r, ref.data());
            for (const auto &[name, w] : t.factors) {
                const int64_t ww[1] = {w};
                const std::string s = name;
                for (const char *g : s == "PauliX"   ? std::vector<const char *>{"Hadamard"}
                                     : s == "PauliY" ? std::vector<const char *>{"PauliZ", "S", "Hadamard"}
                                                     : std::vector<const char *>{}) {
                    orc_sv_apply(r, g, nullptr, nullptr, 0, ww, 1, 0, nullptr, 0);
                }
            }
            std::vector<int64_t> bits(static_cast<size_t>(shots) * n);
            orc_samples(r, nullptr, -1, shots, 41, bits.data());
            double acc = 0.0;
            for (size_t s = 0; s < static_cast<size_t>(shots); s++) {
                double v = 1.0;
                for (const auto &[name, w] : t.factors) {
                    v *= bits[s * n + static_cast<size_t>(w)] != 0 ? -1.0 : 1.0;
                }
                acc += v;
            }
            from_samples += t.c * acc / static_cast<double>(shots);
            orc_sv_free(r);
        }
        if (is_double != 0) {
            expect(std::abs(e_shots - from_samples) <= 1e-12, "shot-based expval(H) from the oracle's samples");
        } else {
            expect(std::abs(e_shots - h_ref) <= 5.0 * (0.5 + 1.25 + 0.3) / std::sqrt(static_cast<double>(shots)),
                   "shot-based expval(H) within five standard errors");
        }
        const auto pz = m.probs({4, 1}, static_cast<size_t>(shots));
        double total = 0.0;
        for (const auto x : pz) {
            total += static_cast<double>(x);
        }
        expect(pz.size() == 4 && std::abs(total - 1.0) < 1e-6 && std::abs(pz[0] - pref[0]) < 0.05,
               "shot-based probs({4, 1})");
        const double v_shots = static_cast<double>(m.var(*x9, static_cast<size_t>(shots)));
        double vx = 0.0;
        const int64_t w9[1] = {9};
        orc_var_named(o, "PauliX", w9, 1, &vx);
        expect(std::abs(v_shots - vx) < 0.1, "shot-based var(X9)");

        // eigenbasis probabilities, eigenvalue counts and basis-state counts
        double ex = 0.0;
        orc_expval_named(o, "PauliX", w9, 1, &ex);
        const auto px = m.probs(*x9);
        expect(px.size() == 2 && close(px[0], (1.0 + ex) / 2, tol, 1.0) && close(px[1], (1.0 - ex) / 2, tol, 1.0),
               "probs(X9) in its eigenbasis");
        const auto cx = m.counts(*x9, static_cast<size_t>(shots));
        size_t counted = 0;
        for (const auto &[value, k] : cx) {
            expect(value == P{1} || value == P{-1}, "X9 samples are eigenvalues");
            counted += k;
        }
        expect(counted == static_cast<size_t>(shots), "counts(X9) adds up to the shots");
        m.setSeed(43);
        const auto basis = m.counts(static_cast<size_t>(shots));
        m.setSeed(43);
        const auto again = m.generate_samples(static_cast<size_t>(shots));
        std::vector<size_t> tally(size_t{1} << n, 0);
        for (size_t s = 0; s < static_cast<size_t>(shots); s++) {
            size_t idx = 0;
            for (size_t w = 0; w < n; w++) {
                idx = (idx << 1) | again[s * n + w];
            }
            tally[idx]++;
        }
        bool same_counts = true;
        for (const auto &[idx, k] : basis) {
            same_counts = same_counts && tally[idx] == k;
        }
        expect(same_counts && !basis.empty(), "counts(shots) tallies the seeded samples");
        bool refused = false;
        try {
            (void)m.probs(*H);
        } catch (const LightningException &e) {
            refused = std::string(e.what()).find("do not support samples()") != std::string::npos;
        }
        expect(refused, "probs(Hamiltonian) is refused");
    }

    bool threw = false;
    try {
        sv.applyOperation("RX", {0}, {true}, {0}, false, {static_cast<P>(0.1)});
    } catch (const LightningException &e) {
        threw = std::string(e.what()).find("disjoint") != std::string::npos;
    }
    expect(threw, "controlled and target wires overlap -> LightningException");

    SV copy(sv);
    copy.applyOperation("PauliX", {0});
    expect(!close_vec(copy.getDataVector(), sv.getDataVector(), tol), "copy is deep");

    orc_sv_free(o);
    orc_sv_free(o2);
    return 0;
}
} // namespace

int main() {
    run<double>(1e-12);
    run<float>(1e-5);
    if (failures != 0) {
        std::printf("%d check(s) failed\n", failures);
        return 1;
    }
    std::printf("PASS\n");
    return 0;
}
