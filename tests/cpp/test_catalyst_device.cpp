// The Catalyst device (include/pl_gb300_catalyst.hpp) driven the way
// Catalyst's runtime drives lightning.qubit's LightningSimulator: qubit
// allocation, release and reuse, gates, state preparation, observables,
// analytic and shot-based measurements, mid-circuit measurements and the
// adjoint gradient of a recorded tape.  Analytic results are checked against
// the CPU oracle's C API (test infrastructure, liboracle.so) on the same
// circuit, seeded shot results against the oracle's samples with the same
// seed, and the rest against the known answers and error messages of the
// reference's device tests
// (core/simulators/lightning_qubit/catalyst/tests/Test_LightningSimulator.cpp,
// Test_LightningMeasures.cpp, Test_LightningGradient.cpp).  Prints "PASS"
// and exits 0 when every check holds.
#include "pl_gb300_catalyst.hpp"

#include "oracle_api.h"

#include <cmath>
#include <cstdio>
#include <functional>
#include <random>
#include <string>
#include <vector>

using namespace Pennylane::LightningGB300;
using namespace Pennylane::LightningGB300::Catalyst;
using cd = std::complex<double>;

namespace {
int failures = 0;
void expect(bool ok, const std::string &what) {
    if (!ok) {
        std::printf("FAIL: %s\n", what.c_str());
        failures++;
    }
}
bool throws_with(const std::function<void()> &f, const std::string &fragment) {
    try {
        f();
    } catch (const LightningException &e) {
        const bool ok = std::string(e.what()).find(fragment) != std::string::npos;
        if (!ok) {
            std::printf("  (message was: %s)\n", e.what());
        }
        return ok;
    }
    return false;
}
bool close(double a, double b, double tol) { return std::abs(a - b) <= tol; }
double rel_err(const std::vector<cd> &a, const std::vector<cd> &b) {
    if (a.size() != b.size()) {
        return 1e300;
    }
    double num = 0.0, den = 0.0;
    for (size_t i = 0; i < a.size(); i++) {
        num += std::norm(a[i] - b[i]);
        den += std::norm(b[i]);
    }
    return std::sqrt(num / den);
}
std::vector<cd> device_state(LightningGB300Simulator &sim) {
    std::vector<cd> s(size_t{1} << sim.GetNumQubits());
    DataView<cd, 1> view(s);
    sim.State(view);
    return s;
}

// The same register on the CPU oracle: every gate the device gets, on the
// same wires (program ids 0..n-1 of a fresh register are wires 0..n-1).
struct Mirror {
    void *o;
    size_t n;
    explicit Mirror(size_t num_qubits) : o{orc_sv_new(static_cast<int>(num_qubits), 1)}, n{num_qubits} {
        std::vector<cd> zero(size_t{1} << n);
        zero[0] = 1.0;
        orc_sv_set_state(o, zero.data());
    }
    ~Mirror() { orc_sv_free(o); }
    Mirror(const Mirror &) = delete;
    Mirror &operator=(const Mirror &) = delete;
    void gate(const std::string &name, const std::vector<double> &params, const std::vector<int64_t> &wires,
              bool inverse = false, const std::vector<int64_t> &cw = {}, const std::vector<bool> &cv = {}) {
        const std::vector<uint8_t> cv8(cv.begin(), cv.end());
        const int rc = orc_sv_apply(o, name.c_str(), cw.data(), cv8.data(), static_cast<int>(cw.size()), wires.data(),
                                    static_cast<int>(wires.size()), inverse ? 1 : 0, params.data(),
                                    static_cast<int>(params.size()));
        expect(rc == 0, "oracle applies " + name);
    }
    void matrix(const std::vector<cd> &m, const std::vector<int64_t> &wires, bool inverse = false,
                const std::vector<int64_t> &cw = {}, const std::vector<bool> &cv = {}) {
        const std::vector<uint8_t> cv8(cv.begin(), cv.end());
        const int rc = orc_sv_apply_matrix(o, reinterpret_cast<const double *>(m.data()), cw.data(), cv8.data(),
                                           static_cast<int>(cw.size()), wires.data(), static_cast<int>(wires.size()),
                                           inverse ? 1 : 0);
        expect(rc == 0, "oracle applies a matrix");
    }
    std::vector<cd> state() const {
        std::vector<cd> s(size_t{1} << n);
        orc_sv_get_state(o, s.data());
        return s;
    }
    std::vector<int64_t> samples(int64_t shots, uint64_t seed) const {
        std::vector<int64_t> out(static_cast<size_t>(shots) * n);
        orc_samples(o, nullptr, -1, shots, seed, out.data());
        return out;
    }
};

// e^{i g} [[a, -conj(b)], [b, conj(a)]] with |a|^2 + |b|^2 = 1
std::vector<cd> random_unitary2(std::mt19937_64 &rng) {
    std::uniform_real_distribution<double> ang(0.0, 6.283185307179586);
    const double t = ang(rng) / 2.0;
    const cd a = std::polar(std::cos(t), ang(rng)), b = std::polar(std::sin(t), ang(rng)), g = std::polar(1.0, ang(rng));
    return {g * a, -g * std::conj(b), g * b, g * std::conj(a)};
}

// ---- qubits and tape (Test_LightningSimulator.cpp:61-116) ----
void qubits_and_tape() {
    LightningGB300Simulator sim;
    expect(sim.GetNumQubits() == 0, "a new device has no qubits");
    expect(sim.AllocateQubits(0).empty() && sim.GetNumQubits() == 0, "AllocateQubits(0)");
    sim.AllocateQubits(2);
    expect(sim.GetNumQubits() == 2, "2 qubits");
    sim.AllocateQubits(2);
    expect(sim.GetNumQubits() == 4, "4 qubits");
    sim.ReleaseQubit(0);
    expect(sim.GetNumQubits() == 3, "release one");
    sim.ReleaseQubits({1, 3});
    expect(sim.GetNumQubits() == 1, "release two");
    sim.ReleaseQubits({2});
    expect(sim.GetNumQubits() == 0, "release the last");
    expect(throws_with([&] { sim.ReleaseQubit(7); }, "Invalid qubit to release"), "release of an unknown id");

    LightningGB300Simulator tape;
    tape.AllocateQubits(1);
    tape.StartTapeRecording();
    expect(throws_with([&] { tape.StartTapeRecording(); }, "Cannot re-activate the cache manager"), "restart tape");
    tape.StopTapeRecording();
    expect(throws_with([&] { tape.StopTapeRecording(); }, "Cannot stop an already stopped cache manager"),
           "stop a stopped tape");

    // released qubits are reused once they are disentangled
    LightningGB300Simulator reuse;
    auto qs = reuse.AllocateQubits(2);
    QubitIdType q = reuse.AllocateQubit();
    reuse.PauliMeasure("XYZ", {qs[0], qs[1], q});
    reuse.PauliMeasure("Z", {q});
    reuse.ReleaseQubit(q);
    q = reuse.AllocateQubit();
    reuse.PauliMeasure("Z", {qs[0]});
    reuse.ReleaseQubit(qs[0]);
    reuse.PauliMeasure("Z", {qs[1]});
    reuse.ReleaseQubit(qs[1]);
    qs = reuse.AllocateQubits(2);
    reuse.NamedOperation("PauliX", {}, {q});
    std::vector<double> p(2);
    DataView<double, 1> pv(p);
    reuse.PartialProbs(pv, {q});
    expect(close(p[0], 0.0, 1e-12) && close(p[1], 1.0, 1e-12), "reused qubit starts in |0>");
    expect(reuse.GetNumQubits() == 3, "three qubits after reuse");

    // an entangled qubit cannot be released and measured around
    LightningGB300Simulator ent;
    auto e = ent.AllocateQubits(2);
    ent.NamedOperation("Hadamard", {}, {e[0]});
    ent.NamedOperation("CNOT", {}, {e[0], e[1]});
    ent.ReleaseQubit(e[1]);
    expect(throws_with([&] { device_state(ent); }, "released qubits are entangled"), "entangled release");

    // a disentangled qubit is dropped from the register on the next read
    LightningGB300Simulator red;
    auto r = red.AllocateQubits(3);
    red.NamedOperation("RY", {0.7}, {r[0]});
    red.NamedOperation("PauliX", {}, {r[1]});
    red.NamedOperation("RX", {1.1}, {r[2]});
    red.ReleaseQubit(r[1]);
    const auto st = device_state(red);
    const double c0 = std::cos(0.35), s0 = std::sin(0.35), c2 = std::cos(0.55), s2 = std::sin(0.55);
    const std::vector<cd> want{c0 * c2, cd(0, -c0 * s2), s0 * c2, cd(0, -s0 * s2)};
    expect(st.size() == 4 && rel_err(st, want) < 1e-12, "register reduced to the live qubits");
}

// ---- gates against the oracle (Test_LightningSimulator.cpp:118-905) ----
void gates() {
    const size_t n = 5;
    LightningGB300Simulator sim;
    const auto q = sim.AllocateQubits(n);
    Mirror m(n);
    std::mt19937_64 rng(2024);
    std::uniform_real_distribution<double> ang(0.0, 6.283185307179586);
    std::uniform_int_distribution<int> wire(0, static_cast<int>(n) - 1);
    auto distinct = [&](size_t k) {
        std::vector<int64_t> w;
        while (w.size() < k) {
            const int64_t x = wire(rng);
            if (std::find(w.begin(), w.end(), x) == w.end()) {
                w.push_back(x);
            }
        }
        return w;
    };
    auto ids = [&](const std::vector<int64_t> &w) {
        std::vector<QubitIdType> out;
        for (const auto x : w) {
            out.push_back(q[static_cast<size_t>(x)]);
        }
        return out;
    };
    struct G {
        const char *name;
        size_t wires, params;
    };
    const G table[] = {{"RX", 1, 1},      {"RY", 1, 1},      {"RZ", 1, 1},       {"Rot", 1, 3},
                       {"PhaseShift", 1, 1}, {"Hadamard", 1, 0}, {"S", 1, 0},        {"T", 1, 0},
                       {"PauliY", 1, 0},  {"CNOT", 2, 0},    {"CZ", 2, 0},       {"SWAP", 2, 0},
                       {"CRX", 2, 1},     {"IsingXX", 2, 1}, {"IsingZZ", 2, 1},  {"Toffoli", 3, 0},
                       {"CSWAP", 3, 0},   {"MultiRZ", 3, 1}, {"SingleExcitation", 2, 1}};
    for (int step = 0; step < 80; step++) {
        const int kind = static_cast<int>(rng() % 23);
        const bool inverse = (rng() & 1U) != 0;
        if (kind < 19) {
            const G &g = table[kind];
            std::vector<double> params;
            for (size_t i = 0; i < g.params; i++) {
                params.push_back(ang(rng));
            }
            const auto w = distinct(g.wires);
            sim.NamedOperation(g.name, params, ids(w), inverse);
            m.gate(g.name, params, w, inverse);
        } else if (kind == 19) { // controlled rotation, mixed control values
            const auto w = distinct(3);
            const std::vector<double> params{ang(rng)};
            const std::vector<bool> cv{true, false};
            sim.NamedOperation("RY", params, ids({w[0]}), inverse, ids({w[1], w[2]}), cv);
            m.gate("RY", params, {w[0]}, inverse, {w[1], w[2]}, cv);
        } else if (kind == 20) { // dense one-wire matrix
            const auto w = distinct(1);
            const auto u = random_unitary2(rng);
            sim.MatrixOperation(u, ids(w), inverse);
            m.matrix(u, w, inverse);
        } else if (kind == 21) { // controlled dense matrix
            const auto w = distinct(2);
            const auto u = random_unitary2(rng);
            sim.MatrixOperation(u, ids({w[0]}), inverse, ids({w[1]}), {true});
            m.matrix(u, {w[0]}, inverse, {w[1]}, {true});
        } else { // Pauli rotation, identity entries stripped
            const auto w = distinct(3);
            const std::vector<double> params{ang(rng)};
            sim.NamedOperation("PauliRot", params, ids(w), inverse, {}, {}, {"XIY"});
            std::vector<int64_t> kept{w[0], w[2]};
            const int rc = orc_sv_apply_pauli_rot(m.o, kept.data(), 2, inverse ? 1 : 0, params[0], "XY");
            expect(rc == 0, "oracle applies PauliRot");
        }
    }
    const double err = rel_err(device_state(sim), m.state());
    std::printf("gates: 80 random operations on 5 qubits, norm-relative %.3e\n", err);
    expect(err < 1e-12, "state after random gates vs oracle");

    // Identity with zero or several wires leaves |0...0>
    LightningGB300Simulator id;
    const auto qi = id.AllocateQubits(4);
    id.NamedOperation("Identity", {}, {});
    id.NamedOperation("Identity", {}, {qi[0], qi[3]});
    const auto s0 = device_state(id);
    expect(s0[0] == cd(1.0, 0.0), "Identity keeps |0...0>");

    // controlled global phase with no target wires (probabilities unchanged)
    LightningGB300Simulator gp;
    const auto qg = gp.AllocateQubits(2);
    gp.NamedOperation("GlobalPhase", {std::acos(-1.0) / 2}, {}, false, {qg[0]}, {true});
    gp.NamedOperation("GlobalPhase", {std::acos(-1.0) / 2}, {}, false, {qg[0]}, {false});
    const auto z = gp.Observable(ObsId::PauliZ, {}, {qg[0]});
    expect(close(gp.Expval(z), 1.0, 1e-12), "controlled GlobalPhase keeps <Z> = 1");

    // PauliRot: identity entries, all-identity words, errors
    LightningGB300Simulator pa, pb;
    const auto qa = pa.AllocateQubits(2), qb = pb.AllocateQubits(2);
    pa.NamedOperation("PauliRot", {0.5}, {qa[0], qa[1]}, false, {}, {}, {"YI"});
    pb.NamedOperation("PauliRot", {0.5}, {qb[0]}, false, {}, {}, {"Y"});
    expect(rel_err(device_state(pa), device_state(pb)) < 1e-14, "PauliRot strips identity entries");
    pb.NamedOperation("PauliRot", {0.5}, {qb[0], qb[1]}, false, {}, {}, {"II"});
    expect(rel_err(device_state(pa), device_state(pb)) < 1e-14, "all-identity PauliRot is a no-op");
    expect(throws_with([&] { pa.NamedOperation("PauliRot", {0.5}, {qa[0]}, false, {}, {}, {"X", "Y"}); },
                       "PauliRot operation requires one string"),
           "PauliRot without one word");
    expect(throws_with([&] { pa.NamedOperation("PauliRot", {0.5}, {qa[0]}, false, {qa[1]}, {false}, {"XY"}); },
                       "Controlled PauliRot is not supported"),
           "controlled PauliRot");
    expect(throws_with([&] { pa.NamedOperation("RX", {0.5}, {5}); }, "Given wires do not refer to qubits"),
           "gate on an unknown qubit");
    expect(throws_with([&] { pa.NamedOperation("CRX", {0.5}, {qa[0]}, false, {qa[1]}, {}); },
                       "Controlled wires/values size mismatch"),
           "controlled values missing");

    // state preparation (Test_LightningSimulator.cpp:779-819)
    LightningGB300Simulator prep;
    const auto qp = prep.AllocateQubits(2);
    std::vector<cd> sub{{0.5, 0.5}, {0.0, 0.0}};
    DataView<cd, 1> subv(sub);
    std::vector<QubitIdType> w1{qp[1]};
    prep.SetState(subv, w1);
    const auto ps = device_state(prep);
    expect(ps[0] == cd(0.5, 0.5) && std::abs(ps[1]) + std::abs(ps[2]) + std::abs(ps[3]) == 0.0,
           "SetState on one wire");
    std::vector<int8_t> bits{1, 0};
    DataView<int8_t, 1> bv(bits);
    std::vector<QubitIdType> w2{qp[0], qp[1]};
    prep.SetBasisState(bv, w2);
    const auto pb2 = device_state(prep);
    expect(pb2[2] == cd(1.0, 0.0) && std::abs(pb2[0]) == 0.0, "SetBasisState |10>");
}

// ---- observables and measurements (Test_LightningMeasures.cpp) ----
void measurements() {
    const size_t n = 4;
    LightningGB300Simulator sim;
    const auto q = sim.AllocateQubits(n);
    Mirror m(n);
    const std::vector<std::pair<const char *, double>> ry{{"RY", 0.4}, {"RY", 1.3}, {"RY", 2.1}, {"RY", 0.9}};
    for (size_t i = 0; i < n; i++) {
        sim.NamedOperation(ry[i].first, {ry[i].second}, {q[i]});
        m.gate(ry[i].first, {ry[i].second}, {static_cast<int64_t>(i)});
    }
    for (size_t i = 0; i + 1 < n; i++) {
        sim.NamedOperation("CNOT", {}, {q[i], q[i + 1]});
        m.gate("CNOT", {}, {static_cast<int64_t>(i), static_cast<int64_t>(i + 1)});
    }
    sim.NamedOperation("RX", {0.6}, {q[2]});
    m.gate("RX", {0.6}, {2});

    const auto x1 = sim.Observable(ObsId::PauliX, {}, {q[1]});
    const auto y2 = sim.Observable(ObsId::PauliY, {}, {q[2]});
    const auto z0 = sim.Observable(ObsId::PauliZ, {}, {q[0]});
    const auto h3 = sim.Observable(ObsId::Hadamard, {}, {q[3]});
    const std::vector<cd> herm{{0.5, 0.0}, {0.2, -0.3}, {0.0, 0.1}, {-0.4, 0.0}, {0.2, 0.3}, {1.0, 0.0},
                               {0.3, 0.0}, {0.0, -0.2}, {0.0, -0.1}, {0.3, 0.0}, {-0.7, 0.0}, {0.1, 0.1},
                               {-0.4, 0.0}, {0.0, 0.2}, {0.1, -0.1}, {0.2, 0.0}};
    const auto hm = sim.Observable(ObsId::Hermitian, herm, {q[0], q[3]});
    const auto t = sim.TensorObservable({z0, x1});
    const auto ham = sim.HamiltonianObservable({0.3, -1.2, 0.8}, {t, y2, hm});
    // the same observables in the oracle's spec form
    std::vector<double> cdata;
    for (const cd &x : herm) {
        cdata.push_back(x.real());
        cdata.push_back(x.imag());
    }
    const struct {
        ObsIdType key;
        const char *spec;
        const char *what;
    } cases[] = {{x1, "named PauliX 1", "X1"},
                 {y2, "named PauliY 2", "Y2"},
                 {z0, "named PauliZ 0", "Z0"},
                 {h3, "named Hadamard 3", "H3"},
                 {hm, "herm 2 0 3 0", "Hermitian on 0, 3"},
                 {t, "prod 2 named PauliZ 0 named PauliX 1", "Z0 X1"},
                 {ham, "ham 3 0.3 prod 2 named PauliZ 0 named PauliX 1 -1.2 named PauliY 2 0.8 herm 2 0 3 0",
                  "Hamiltonian"}};
    for (const auto &c : cases) {
        double e_ref = 0.0, v_ref = 0.0;
        orc_expval_obs(m.o, c.spec, cdata.data(), nullptr, &e_ref);
        orc_var_obs(m.o, c.spec, cdata.data(), nullptr, &v_ref);
        expect(close(sim.Expval(c.key), e_ref, 1e-12), std::string("Expval ") + c.what);
        expect(close(sim.Var(c.key), v_ref, 1e-12), std::string("Var ") + c.what);
    }

    // probabilities
    std::vector<double> pall(16), p0(1), p2(4), pref(16), p2ref(4);
    DataView<double, 1> vall(pall), v0(p0), v2(p2);
    sim.Probs(vall);
    orc_probs(m.o, nullptr, -1, pref.data());
    bool same = true;
    for (size_t i = 0; i < 16; i++) {
        same = same && close(pall[i], pref[i], 1e-13);
    }
    expect(same, "Probs vs oracle");
    sim.PartialProbs(v0, std::vector<QubitIdType>{});
    expect(close(p0[0], 1.0, 1e-12), "PartialProbs over no wires");
    sim.PartialProbs(v2, {q[3], q[1]});
    const int64_t w31[2] = {3, 1};
    orc_probs(m.o, w31, 2, p2ref.data());
    same = true;
    for (size_t i = 0; i < 4; i++) {
        same = same && close(p2[i], p2ref[i], 1e-13);
    }
    expect(same, "PartialProbs({3, 1}) vs oracle");

    // seeded shots: the device's samples are the oracle's samples
    const int64_t shots = 1000;
    sim.SetDeviceShots(static_cast<size_t>(shots));
    std::mt19937 gen(77), twin(77);
    sim.SetDevicePRNG(&gen);
    std::vector<double> smp(static_cast<size_t>(shots) * n);
    const size_t sz[2] = {static_cast<size_t>(shots), n}, sd[2] = {n, 1};
    DataView<double, 2> sv(smp.data(), 0, sz, sd);
    sim.Sample(sv);
    const auto ref_samples = m.samples(shots, twin());
    same = true;
    for (size_t i = 0; i < smp.size(); i++) {
        same = same && smp[i] == static_cast<double>(ref_samples[i]);
    }
    expect(same, "Sample equals the oracle's samples for the same seed");

    std::vector<double> part(static_cast<size_t>(shots) * 2);
    const size_t psz[2] = {static_cast<size_t>(shots), 2}, psd[2] = {2, 1};
    DataView<double, 2> pv(part.data(), 0, psz, psd);
    sim.PartialSample(pv, {q[2], q[0]});
    const auto ref2 = m.samples(shots, twin());
    same = true;
    for (size_t s = 0; s < static_cast<size_t>(shots); s++) {
        same = same && part[2 * s] == static_cast<double>(ref2[s * n + 2]) &&
               part[2 * s + 1] == static_cast<double>(ref2[s * n + 0]);
    }
    expect(same, "PartialSample picks the wires of the oracle's samples");

    std::vector<double> eig(16);
    std::vector<int64_t> cnt(16);
    DataView<double, 1> ev(eig);
    DataView<int64_t, 1> cv(cnt);
    sim.Counts(ev, cv);
    const auto ref3 = m.samples(shots, twin());
    std::vector<int64_t> cref(16, 0);
    for (size_t s = 0; s < static_cast<size_t>(shots); s++) {
        size_t idx = 0;
        for (size_t w = 0; w < n; w++) {
            idx = (idx << 1) | static_cast<size_t>(ref3[s * n + w]);
        }
        cref[idx]++;
    }
    expect(cnt == cref && eig[5] == 5.0, "Counts from the oracle's samples");

    std::vector<double> eig2(4);
    std::vector<int64_t> cnt2(4);
    DataView<double, 1> ev2(eig2);
    DataView<int64_t, 1> cv2(cnt2);
    sim.PartialCounts(ev2, cv2, {q[1], q[3]});
    const auto ref4 = m.samples(shots, twin());
    std::vector<int64_t> cref2(4, 0);
    for (size_t s = 0; s < static_cast<size_t>(shots); s++) {
        cref2[static_cast<size_t>(ref4[s * n + 1] * 2 + ref4[s * n + 3])]++;
    }
    expect(cnt2 == cref2, "PartialCounts from the oracle's samples");

    sim.PartialProbs(v2, {q[3], q[1]});
    const auto ref5 = m.samples(shots, twin());
    std::vector<double> pshot(4, 0.0);
    for (size_t s = 0; s < static_cast<size_t>(shots); s++) {
        pshot[static_cast<size_t>(ref5[s * n + 3] * 2 + ref5[s * n + 1])] += 1.0;
    }
    same = true;
    for (size_t i = 0; i < 4; i++) {
        same = same && close(p2[i], pshot[i] / static_cast<double>(shots), 1e-15);
    }
    expect(same, "shot-based PartialProbs from the oracle's samples");

    // shot-based Z0 X1: the state rotated by H on wire 1, sampled with the seed
    const double e_shots = sim.Expval(t);
    {
        Mirror rot(n);
        orc_sv_set_state(rot.o, m.state().data());
        rot.gate("Hadamard", {}, {1});
        const auto r = rot.samples(shots, twin());
        double acc = 0.0;
        for (size_t s = 0; s < static_cast<size_t>(shots); s++) {
            acc += (r[s * n + 0] != 0 ? -1.0 : 1.0) * (r[s * n + 1] != 0 ? -1.0 : 1.0);
        }
        expect(close(e_shots, acc / static_cast<double>(shots), 1e-14), "shot-based Expval(Z0 X1) from samples");
    }
    // shot-based values of every observable within five standard errors
    std::mt19937 free_gen(5);
    sim.SetDevicePRNG(&free_gen);
    sim.SetDeviceShots(20000);
    auto sigma = [&](const char *spec) { // standard error of a 20000-shot mean
        double v = 0.0;
        orc_var_obs(m.o, spec, cdata.data(), nullptr, &v);
        return std::sqrt(std::max(v, 1e-4) / 20000.0);
    };
    for (const auto &c : cases) {
        double e_ref = 0.0;
        orc_expval_obs(m.o, c.spec, cdata.data(), nullptr, &e_ref);
        const double e = sim.Expval(c.key);
        // a Hamiltonian is sampled term by term: at most the sum of the terms' errors
        const double bound = 5.0 * (c.key == ham ? 0.3 * sigma(cases[5].spec) + 1.2 * sigma(cases[1].spec) +
                                                       0.8 * sigma(cases[4].spec)
                                                 : sigma(c.spec));
        expect(std::abs(e - e_ref) <= bound, std::string("shot-based Expval ") + c.what);
    }
    const double v_shots = sim.Var(x1);
    double vx = 0.0;
    orc_var_obs(m.o, "named PauliX 1", nullptr, nullptr, &vx);
    expect(std::abs(v_shots - vx) < 0.05, "shot-based Var X1");
    sim.SetDeviceShots(0);

    // errors (Test_LightningMeasures.cpp:44-209)
    LightningGB300Simulator empty;
    expect(throws_with([&] { empty.Observable(ObsId::PauliX, {}, {1}); }, "Invalid number of wires"),
           "observable on a device without qubits");
    empty.AllocateQubit();
    expect(throws_with([&] { empty.Observable(ObsId::PauliX, {}, {1}); }, "Invalid given wires"),
           "observable on an unknown qubit");
    expect(throws_with([&] { empty.Observable(static_cast<ObsId>(10), {}, {0}); },
                       "The given observable is not supported by the simulator"),
           "unsupported observable id");
    expect(throws_with([&] { empty.Expval(9); }, "Invalid key for cached observables"), "unknown observable key");
    std::vector<cd> wrong(3);
    DataView<cd, 1> wv(wrong);
    expect(throws_with([&] { empty.State(wv); }, "Invalid size for the pre-allocated state vector"),
           "State with a wrong buffer");
}

// ---- mid-circuit measurements (Test_LightningMeasures.cpp:88-199) ----
void mid_circuit() {
    LightningGB300Simulator sim;
    const auto q = sim.AllocateQubit();
    sim.NamedOperation("PauliX", {}, {q});
    expect(*sim.Measure(q), "measure |1>");

    LightningGB300Simulator p0, p1, bad;
    const auto a = p0.AllocateQubit(), b = p1.AllocateQubit(), c = bad.AllocateQubit();
    p0.NamedOperation("Hadamard", {}, {a});
    p1.NamedOperation("Hadamard", {}, {b});
    bad.NamedOperation("Hadamard", {}, {c});
    expect(!*p0.Measure(a, 0), "postselect 0");
    expect(*p1.Measure(b, 1), "postselect 1");
    expect(throws_with([&] { bad.Measure(c, 2); }, "Invalid postselect value"), "postselect 2");
    const auto s1 = device_state(p1);
    expect(std::abs(s1[1]) > 1.0 - 1e-12 && std::abs(s1[0]) == 0.0, "collapsed onto |1>");

    // outcome drawn from the device's generator: a collapse onto one branch
    LightningGB300Simulator two;
    std::mt19937 gen(3);
    two.SetDevicePRNG(&gen);
    const auto qs = two.AllocateQubits(2);
    two.NamedOperation("Hadamard", {}, {qs[0]});
    two.NamedOperation("CNOT", {}, {qs[0], qs[1]});
    const bool r = *two.Measure(qs[0]);
    const auto st = device_state(two);
    expect(std::abs(std::abs(st[r ? 3 : 0]) - 1.0) < 1e-12, "Bell pair collapses onto |00> or |11>");
}

// ---- adjoint gradient of the recorded tape (Test_LightningGradient.cpp) ----
void gradients() {
    const double pi = std::acos(-1.0);
    {
        LightningGB300Simulator sim;
        std::vector<DataView<double, 1>> none;
        sim.AllocateQubits(0);
        sim.Gradient(none, {});
    }
    {
        LightningGB300Simulator sim;
        std::vector<double> buf(1);
        std::vector<DataView<double, 1>> g;
        g.emplace_back(buf);
        const auto q = sim.AllocateQubit();
        sim.StartTapeRecording();
        sim.NamedOperation("RX", {-pi / 7}, {q});
        const auto z = sim.Observable(ObsId::PauliZ, {}, {q});
        sim.Var(z);
        expect(throws_with([&] { sim.Gradient(g, {0}); }, "Unsupported measurements to compute gradient"),
               "gradient of a variance");
        sim.StopTapeRecording();
    }
    {
        LightningGB300Simulator sim;
        std::vector<double> buf(1);
        std::vector<DataView<double, 1>> g;
        g.emplace_back(buf);
        const auto q = sim.AllocateQubit();
        sim.StartTapeRecording();
        sim.NamedOperation("RX", {-pi / 7}, {q});
        const auto z = sim.Observable(ObsId::PauliZ, {}, {q});
        sim.Expval(z);
        sim.Gradient(g, {0});
        expect(close(buf[0], -std::sin(-pi / 7), 1e-12), "d<Z>/dRX");
        buf[0] = 0.0;
        sim.Gradient(g, {});
        expect(close(buf[0], -std::sin(-pi / 7), 1e-12), "d<Z>/dRX, all parameters");
        sim.StopTapeRecording();
    }
    {
        // RX then a fixed unitary, <Y> (Test_LightningGradient.cpp:321-359)
        LightningGB300Simulator sim;
        std::vector<double> buf(1);
        std::vector<DataView<double, 1>> g;
        g.emplace_back(buf);
        const std::vector<cd> u{{-0.6709485262524046, -0.6304426335363695},
                                {-0.14885403153998722, 0.3608498832392019},
                                {-0.2376311670004963, 0.3096798175687841},
                                {-0.8818365947322423, -0.26456390390903695}};
        const auto q = sim.AllocateQubits(1);
        sim.StartTapeRecording();
        sim.NamedOperation("RX", {-pi / 7}, {q[0]});
        sim.MatrixOperation(u, {q[0]});
        const auto y = sim.Observable(ObsId::PauliY, {}, {q[0]});
        sim.Expval(y);
        sim.Gradient(g, {0});
        expect(close(buf[0], -0.8611041863, 1e-9), "gradient through a QubitUnitary");
        sim.StopTapeRecording();
    }
    {
        // two observables (Test_LightningGradient.cpp:361-426)
        LightningGB300Simulator sim;
        std::vector<double> b0(4), b1(4);
        std::vector<DataView<double, 1>> g;
        g.emplace_back(b0);
        g.emplace_back(b1);
        const auto q = sim.AllocateQubits(2);
        sim.StartTapeRecording();
        sim.NamedOperation("RY", {0.1}, {q[0]});
        sim.NamedOperation("RX", {0.3}, {q[0]});
        sim.NamedOperation("RY", {0.2}, {q[1]});
        sim.NamedOperation("RX", {0.4}, {q[1]});
        const auto z0 = sim.Observable(ObsId::PauliZ, {}, {q[0]});
        const auto z1 = sim.Observable(ObsId::PauliZ, {}, {q[1]});
        sim.Expval(z0);
        sim.Expval(z1);
        sim.Gradient(g, {});
        const double e0[4] = {-0.09537451, -0.29404384, 0.0, 0.0}, e1[4] = {0.0, 0.0, -0.18298657, -0.3816559};
        bool ok = true;
        for (int i = 0; i < 4; i++) {
            ok = ok && close(b0[static_cast<size_t>(i)], e0[i], 1e-7) && close(b1[static_cast<size_t>(i)], e1[i], 1e-7);
        }
        expect(ok, "gradients of two observables");
        const auto info = sim.CacheManagerInfo();
        expect(std::get<0>(info) == 4 && std::get<1>(info) == 2 && std::get<2>(info) == 4, "tape counts");
        sim.StopTapeRecording();
    }
    {
        // a larger tape against the oracle's adjoint Jacobian
        const size_t n = 4;
        LightningGB300Simulator sim;
        const auto q = sim.AllocateQubits(n);
        std::mt19937_64 rng(99);
        std::uniform_real_distribution<double> ang(0.0, 6.283185307179586);
        std::vector<std::string> names;
        std::vector<double> params;
        std::vector<int> nparams, nwires, ncw;
        std::vector<int64_t> wires, cwires, matsz;
        std::vector<uint8_t> inv, cvals;
        sim.StartTapeRecording();
        for (int layer = 0; layer < 3; layer++) {
            for (size_t i = 0; i < n; i++) {
                for (const char *r : {"RZ", "RY", "RZ"}) { // Rot as the three rotations the adjoint method takes
                    const double a = ang(rng);
                    sim.NamedOperation(r, {a}, {q[i]});
                    names.emplace_back(r);
                    params.push_back(a);
                    nparams.push_back(1);
                    wires.push_back(static_cast<int64_t>(i));
                    nwires.push_back(1);
                }
            }
            for (size_t i = 0; i < n; i++) {
                const double a = ang(rng);
                const int64_t w0 = static_cast<int64_t>(i), w1 = static_cast<int64_t>((i + 1) % n);
                sim.NamedOperation("IsingXY", {a}, {q[static_cast<size_t>(w0)], q[static_cast<size_t>(w1)]});
                names.emplace_back("IsingXY");
                params.push_back(a);
                nparams.push_back(1);
                wires.insert(wires.end(), {w0, w1});
                nwires.push_back(2);
            }
            const double a = ang(rng);
            sim.NamedOperation("CRY", {a}, {q[0], q[2]});
            names.emplace_back("CRY");
            params.push_back(a);
            nparams.push_back(1);
            wires.insert(wires.end(), {0, 2});
            nwires.push_back(2);
        }
        const auto z0 = sim.Observable(ObsId::PauliZ, {}, {q[0]});
        const auto x2 = sim.Observable(ObsId::PauliX, {}, {q[2]});
        const auto y3 = sim.Observable(ObsId::PauliY, {}, {q[3]});
        const auto zx = sim.TensorObservable({z0, x2});
        const auto h = sim.HamiltonianObservable({0.7, -0.4}, {zx, y3});
        sim.Expval(h);
        sim.Expval(y3);
        const size_t np = params.size();
        std::vector<double> b0(np), b1(np);
        std::vector<DataView<double, 1>> g;
        g.emplace_back(b0);
        g.emplace_back(b1);
        sim.Gradient(g, {});
        sim.StopTapeRecording();

        std::vector<const char *> cn;
        for (const auto &s : names) {
            cn.push_back(s.c_str());
        }
        inv.assign(names.size(), 0);
        matsz.assign(names.size(), 0);
        ncw.assign(names.size(), 0);
        std::vector<int64_t> tp(np);
        std::iota(tp.begin(), tp.end(), int64_t{0});
        const char *specs[2] = {"ham 2 0.7 prod 2 named PauliZ 0 named PauliX 2 -0.4 named PauliY 3",
                                "named PauliY 3"};
        Mirror zero(n);
        std::vector<double> jref(2 * np);
        const int rc = orc_adjoint(zero.o, static_cast<int>(names.size()), cn.data(), params.data(), nparams.data(),
                                   wires.data(), nwires.data(), inv.data(), nullptr, matsz.data(), nullptr,
                                   ncw.data(), nullptr, 2, specs, nullptr, nullptr, tp.data(),
                                   static_cast<int>(np), 1, jref.data());
        expect(rc == 0, "oracle adjoint ran");
        double worst = 0.0;
        for (size_t i = 0; i < np; i++) {
            worst = std::max({worst, std::abs(b0[i] - jref[i]), std::abs(b1[i] - jref[np + i])});
        }
        std::printf("gradient: 2 observables x %zu parameters, max |diff| vs oracle %.3e\n", np, worst);
        expect(worst < 1e-12, "tape gradient vs the oracle's adjoint Jacobian");
    }
}

// ---- keyword arguments and Metropolis samples ----
void kwargs_and_mcmc() {
    LightningGB300Simulator sim("{'mcmc': True, 'num_burnin': 200, 'kernel_name': 'NonZeroRandom'}");
    expect(sim.mcmc() && sim.num_burnin() == 200 && sim.kernel_name() == "NonZeroRandom", "device kwargs");
    LightningGB300Simulator plain;
    expect(!plain.mcmc() && plain.num_burnin() == 100 && plain.kernel_name() == "Local", "default kwargs");
    const auto q = sim.AllocateQubits(3);
    sim.NamedOperation("Hadamard", {}, {q[0]});
    sim.NamedOperation("CNOT", {}, {q[0], q[2]});
    std::mt19937 gen(11);
    sim.SetDevicePRNG(&gen);
    const auto s = sim.GenerateSamplesMetropolis(500);
    bool bell = s.size() == 1500;
    for (size_t i = 0; bell && i < 500; i++) {
        bell = s[3 * i] == s[3 * i + 2] && s[3 * i + 1] == 0;
    }
    expect(bell, "Metropolis samples stay on the support of the state");
}
} // namespace

int main() {
    qubits_and_tape();
    gates();
    measurements();
    mid_circuit();
    gradients();
    kwargs_and_mcmc();
    if (failures != 0) {
        std::printf("%d check(s) failed\n", failures);
        return 1;
    }
    std::printf("PASS\n");
    return 0;
}
