// Host-only parts of the Catalyst device and the C++ layer, on the CPU: the
// device keyword parser, the strided DataView, the qubit map, the subsystem
// purity behind qubit release, and the Hermitian eigen-decomposition behind
// shot-based Hermitian measurements.  Prints "PASS" and exits 0 when every
// check holds.
#include "pl_gb300_catalyst.hpp"

#include <cmath>
#include <cstdio>
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

void kwargs() {
    expect(parse_kwargs("").empty(), "empty kwargs");
    expect(parse_kwargs("{shots : 1000}") == parse_kwargs("shots : 1000"), "braces are optional");
    expect(parse_kwargs("shots : 1000") == parse_kwargs("'shots':'1000'"), "quotes are optional");
    auto a = parse_kwargs("{'mcmc': True, 'num_burnin': 200, 'kernel_name': 'Local'}");
    expect(a.size() == 3 && a["mcmc"] == "True" && a["num_burnin"] == "200" && a["kernel_name"] == "Local",
           "three items");
    auto b = parse_kwargs("backend : gb300,{'folder': \"('a', 'b')\", 'x': 1}");
    expect(b.size() == 3 && b["backend"] == "gb300" && b["folder"] == "('a', 'b')" && b["x"] == "1",
           "a quoted value with commas and parentheses");
}

void dataview() {
    // a 3 x 2 view with row stride 4 and offset 1 over 13 doubles
    std::vector<double> buf(13);
    for (size_t i = 0; i < buf.size(); i++) {
        buf[i] = static_cast<double>(i);
    }
    const size_t sizes[2] = {3, 2}, strides[2] = {4, 1};
    DataView<double, 2> v(buf.data(), 1, sizes, strides);
    std::vector<double> seen(v.begin(), v.end());
    expect(v.size() == 6 && seen == std::vector<double>{1, 2, 5, 6, 9, 10}, "strided row-major iteration");
    expect(v(2, 1) == 10.0, "element access");
    v(1, 0) = -1.0;
    expect(buf[5] == -1.0, "writes reach the buffer");
    std::vector<int64_t> one{4, 5, 6};
    DataView<int64_t, 1> w(one);
    int64_t sum = 0;
    for (auto it = w.begin(); it != w.end(); ++it) {
        sum += *it;
    }
    expect(w.size() == 3 && sum == 15 && w(1) == 5, "vector view");
}

void qubit_map() {
    QubitMap m;
    const auto ids = m.allocate_range(0, 3);
    expect(ids == std::vector<QubitIdType>{0, 1, 2} && m.size() == 3, "allocate a range");
    m.release(1);
    expect(m.size() == 2 && !m.valid(1) && m.free_wires().count(1) == 1, "release marks the wire free");
    const auto w = m.pop_free();
    expect(w.has_value() && *w == 1 && m.free_wires().empty(), "the free wire is taken again");
    const auto id = m.allocate(*w);
    expect(id == 3 && m.wire(3) == 1, "program ids are never reused");
    m.release(0);
    m.remap({{1, 0}, {2, 1}});
    expect(m.wire(3) == 0 && m.wire(2) == 1, "remap after a reduction");
    const auto live = m.live_by_wire();
    expect(live.size() == 2 && live[0].second == 3 && live[1].second == 2, "live qubits by wire");
    bool threw = false;
    try {
        m.release(9);
    } catch (const LightningException &) {
        threw = true;
    }
    expect(threw, "releasing an unknown id throws");
}

void purity() {
    // |+> (x) |1> (x) (|0> + i|1>)/sqrt(2): every subset is pure
    const double s = std::sqrt(0.5);
    std::vector<cd> prod(8);
    for (size_t i = 0; i < 8; i++) {
        const bool b0 = (i >> 2) & 1U, b1 = (i >> 1) & 1U, b2 = i & 1U;
        prod[i] = b1 ? s * s * (b2 ? cd(0, 1) : cd(1, 0)) * (b0 ? 1.0 : 1.0) : 0.0;
    }
    expect(std::abs(subsystem_purity(prod, 3, {1}) - 1.0) < 1e-14, "product state: one wire pure");
    expect(std::abs(subsystem_purity(prod, 3, {0, 2}) - 1.0) < 1e-14, "product state: two wires pure");
    // Bell pair on wires 0, 2 with wire 1 in |0>: each half is maximally mixed
    std::vector<cd> bell(8);
    bell[0] = s;
    bell[5] = s;
    expect(std::abs(subsystem_purity(bell, 3, {2}) - 0.5) < 1e-14, "Bell pair: purity 1/2");
    expect(std::abs(subsystem_purity(bell, 3, {1}) - 1.0) < 1e-14, "spectator wire is pure");
    expect(std::abs(subsystem_purity(bell, 3, {0, 1}) - 0.5) < 1e-14, "the larger part by its complement");
    // unnormalised input is normalised first
    for (auto &x : bell) {
        x *= 3.0;
    }
    expect(std::abs(subsystem_purity(bell, 3, {0}) - 0.5) < 1e-14, "unnormalised input");
}

void eigh() {
    std::mt19937_64 rng(7);
    std::normal_distribution<double> g(0.0, 1.0);
    double worst = 0.0;
    for (const size_t dim : {1U, 2U, 4U, 8U, 16U, 32U}) {
        for (int trial = 0; trial < 3; trial++) {
            std::vector<cd> a(dim * dim);
            for (size_t i = 0; i < dim; i++) {
                for (size_t j = i; j < dim; j++) {
                    const cd x = i == j ? cd(g(rng), 0.0) : cd(g(rng), g(rng));
                    a[i * dim + j] = x;
                    a[j * dim + i] = std::conj(x);
                }
            }
            if (trial == 2 && dim >= 4) { // a degenerate spectrum: P = Z (x) I (x) ...
                for (size_t i = 0; i < dim; i++) {
                    for (size_t j = 0; j < dim; j++) {
                        a[i * dim + j] = i == j ? cd(i < dim / 2 ? 1.0 : -1.0, 0.0) : cd(0.0, 0.0);
                    }
                }
            }
            std::vector<double> w;
            std::vector<cd> v;
            detail::hermitian_eigh(a, dim, w, v);
            double scale = 0.0;
            for (const cd &x : a) {
                scale = std::max(scale, std::abs(x));
            }
            for (size_t i = 0; i < dim; i++) {
                for (size_t j = 0; j < dim; j++) {
                    cd rec = 0.0, gram = 0.0;
                    for (size_t k = 0; k < dim; k++) {
                        rec += v[i * dim + k] * w[k] * std::conj(v[j * dim + k]);
                        gram += std::conj(v[k * dim + i]) * v[k * dim + j];
                    }
                    worst = std::max({worst, std::abs(rec - a[i * dim + j]) / scale,
                                      std::abs(gram - (i == j ? 1.0 : 0.0))});
                }
            }
            for (size_t k = 1; k < dim; k++) {
                expect(w[k - 1] <= w[k], "eigenvalues ascending");
            }
        }
    }
    std::printf("hermitian_eigh: worst residual %.3e\n", worst);
    expect(worst < 1e-12, "A = V diag(w) V^H with V unitary");
}
} // namespace

int main() {
    kwargs();
    dataview();
    qubit_map();
    purity();
    eigh();
    if (failures != 0) {
        std::printf("%d check(s) failed\n", failures);
        return 1;
    }
    std::printf("PASS\n");
    return 0;
}
