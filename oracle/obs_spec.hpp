// Test infrastructure: parser for the observable spec strings described in
// oracle_api.h.  Shared by the LM restatement (lm_oracle.cpp) and the shim
// over the reference headers (ref_shim.cpp); each supplies a Builder with
//   Obs named(std::string, std::size_t wire)
//   Obs herm(std::vector<std::complex<double>>, std::vector<std::size_t>)
//   Obs prod(std::vector<Obs>)
//   Obs ham(std::vector<double>, std::vector<Obs>)
//   Obs sparse(data, indices, indptr, wires)
#pragma once
#include <complex>
#include <cstdint>
#include <cstdlib>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

namespace orc_spec {

template <class Builder> struct Parser {
    using Obs = decltype(std::declval<Builder &>().named(std::string{}, 0));
    Builder &b;
    const double *cdata;
    const int64_t *idata;
    std::istringstream in;

    Parser(Builder &builder, const char *spec, const double *cd,
           const int64_t *id)
        : b(builder), cdata(cd), idata(id), in(spec) {}

    std::string tok() {
        std::string t;
        if (!(in >> t)) {
            throw std::runtime_error("observable spec ended early");
        }
        return t;
    }
    long long integer() { return std::stoll(tok()); }
    double real() { return std::strtod(tok().c_str(), nullptr); }

    Obs parse() {
        const std::string kind = tok();
        if (kind == "named") {
            std::string name = tok();
            auto w = static_cast<std::size_t>(integer());
            return b.named(name, w);
        }
        if (kind == "herm") {
            auto k = static_cast<std::size_t>(integer());
            std::vector<std::size_t> wires(k);
            for (auto &w : wires) {
                w = static_cast<std::size_t>(integer());
            }
            auto off = static_cast<std::size_t>(integer());
            const std::size_t dim = std::size_t{1} << k;
            std::vector<std::complex<double>> m(dim * dim);
            for (std::size_t i = 0; i < dim * dim; i++) {
                m[i] = {cdata[2 * (off + i)], cdata[2 * (off + i) + 1]};
            }
            return b.herm(std::move(m), std::move(wires));
        }
        if (kind == "prod") {
            auto m = integer();
            std::vector<Obs> obs;
            for (long long i = 0; i < m; i++) {
                obs.push_back(parse());
            }
            return b.prod(std::move(obs));
        }
        if (kind == "ham") {
            auto m = integer();
            std::vector<double> coeffs;
            std::vector<Obs> obs;
            for (long long i = 0; i < m; i++) {
                coeffs.push_back(real());
                obs.push_back(parse());
            }
            return b.ham(std::move(coeffs), std::move(obs));
        }
        if (kind == "sparse") {
            auto k = static_cast<std::size_t>(integer());
            std::vector<std::size_t> wires(k);
            for (auto &w : wires) {
                w = static_cast<std::size_t>(integer());
            }
            auto nnz = static_cast<std::size_t>(integer());
            auto off_d = static_cast<std::size_t>(integer());
            auto off_i = static_cast<std::size_t>(integer());
            auto off_p = static_cast<std::size_t>(integer());
            std::vector<std::complex<double>> data(nnz);
            std::vector<std::size_t> indices(nnz);
            for (std::size_t i = 0; i < nnz; i++) {
                data[i] = {cdata[2 * (off_d + i)], cdata[2 * (off_d + i) + 1]};
                indices[i] = static_cast<std::size_t>(idata[off_i + i]);
            }
            const std::size_t nptr = (std::size_t{1} << k) + 1;
            std::vector<std::size_t> indptr(nptr);
            for (std::size_t i = 0; i < nptr; i++) {
                indptr[i] = static_cast<std::size_t>(idata[off_p + i]);
            }
            return b.sparse(std::move(data), std::move(indices),
                            std::move(indptr), std::move(wires));
        }
        throw std::runtime_error("unknown observable kind: " + kind);
    }
};

} // namespace orc_spec
