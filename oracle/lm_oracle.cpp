// ORACLE — test infrastructure only.  C API (oracle_api.h, prefix orc_) over
// the LM restatement in lm_oracle.hpp.
#define ORC_PREFIX orc_
#include "oracle_api.h"

#include "lm_oracle.hpp"
#include "obs_spec.hpp"

#include <cstring>
#include <variant>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

thread_local std::string g_err;

struct Handle {
    bool dbl;
    std::variant<orc::StateVec<float>, orc::StateVec<double>> sv;
    Handle(int n, bool d)
        : dbl(d), sv(d ? std::variant<orc::StateVec<float>, orc::StateVec<double>>(
                             std::in_place_index<1>, static_cast<size_t>(n))
                       : std::variant<orc::StateVec<float>, orc::StateVec<double>>(
                             std::in_place_index<0>, static_cast<size_t>(n))) {}
};

template <class F> int guard(F &&f) {
    try {
        f();
        return 0;
    } catch (const std::exception &e) {
        g_err = e.what();
        return 1;
    }
}

std::vector<size_t> vec(const int64_t *p, int n) {
    std::vector<size_t> v;
    for (int i = 0; i < n; i++) {
        v.push_back(static_cast<size_t>(p[i]));
    }
    return v;
}
std::vector<bool> bvec(const uint8_t *p, int n) {
    std::vector<bool> v;
    for (int i = 0; i < n; i++) {
        v.push_back(p[i] != 0);
    }
    return v;
}
template <class T> std::vector<orc::C<T>> cvec(const double *p, size_t n) {
    std::vector<orc::C<T>> v(n);
    for (size_t i = 0; i < n; i++) {
        v[i] = {static_cast<T>(p[2 * i]), static_cast<T>(p[2 * i + 1])};
    }
    return v;
}

template <class T> struct Builder {
    using O = orc::ObsPtr<T>;
    O named(const std::string &name, size_t w) {
        auto o = std::make_shared<orc::NamedObs<T>>();
        o->name = name;
        o->wires = {w};
        return o;
    }
    O herm(std::vector<std::complex<double>> m, std::vector<size_t> wires) {
        auto o = std::make_shared<orc::HermObs<T>>();
        for (auto &x : m) {
            o->m.emplace_back(static_cast<T>(x.real()), static_cast<T>(x.imag()));
        }
        o->wires = std::move(wires);
        return o;
    }
    O prod(std::vector<O> obs) {
        auto o = std::make_shared<orc::ProdObs<T>>();
        o->obs = std::move(obs);
        return o;
    }
    O ham(std::vector<double> coeffs, std::vector<O> obs) {
        auto o = std::make_shared<orc::HamObs<T>>();
        for (auto c : coeffs) {
            o->coeffs.push_back(static_cast<T>(c));
        }
        o->obs = std::move(obs);
        return o;
    }
    O sparse(std::vector<std::complex<double>> data, std::vector<size_t> indices,
             std::vector<size_t> indptr, std::vector<size_t> wires) {
        auto o = std::make_shared<orc::SparseObs<T>>();
        for (auto &x : data) {
            o->data.emplace_back(static_cast<T>(x.real()), static_cast<T>(x.imag()));
        }
        o->indices = std::move(indices);
        o->indptr = std::move(indptr);
        o->wires = std::move(wires);
        return o;
    }
};

template <class T>
orc::ObsPtr<T> parse_obs(const char *spec, const double *cdata, const int64_t *idata) {
    Builder<T> b;
    orc_spec::Parser<Builder<T>> p(b, spec, cdata, idata);
    return p.parse();
}

template <class F> int with_sv(void *h, F &&f) {
    return guard([&] {
        auto *hd = static_cast<Handle *>(h);
        if (hd->dbl) {
            f(std::get<1>(hd->sv));
        } else {
            f(std::get<0>(hd->sv));
        }
    });
}

template <class T>
std::vector<orc::Op<T>> parse_ops(int nops, const char **names, const double *params, const int *nparams,
                                  const int64_t *wires, const int *nwires, const uint8_t *inverses,
                                  const double *mats, const int64_t *mat_sizes, const int64_t *cwires,
                                  const int *ncwires, const uint8_t *cvals) {
    std::vector<orc::Op<T>> ops(static_cast<size_t>(nops));
    size_t ip = 0, iw = 0, im = 0, ic = 0;
    for (int k = 0; k < nops; k++) {
        auto &op = ops[static_cast<size_t>(k)];
        op.name = names[k];
        for (int i = 0; i < nparams[k]; i++) {
            op.params.push_back(static_cast<T>(params[ip++]));
        }
        for (int i = 0; i < nwires[k]; i++) {
            op.wires.push_back(static_cast<size_t>(wires[iw++]));
        }
        op.inverse = inverses[k] != 0;
        op.matrix = cvec<T>(mats + 2 * im, static_cast<size_t>(mat_sizes[k]));
        im += static_cast<size_t>(mat_sizes[k]);
        for (int i = 0; i < ncwires[k]; i++) {
            op.cwires.push_back(static_cast<size_t>(cwires[ic]));
            op.cvals.push_back(cvals[ic] != 0);
            ic++;
        }
    }
    return ops;
}

} // namespace

extern "C" {

const char *orc_last_error(void) { return g_err.c_str(); }

void *orc_sv_new(int num_qubits, int is_double) {
    try {
        return new Handle(num_qubits, is_double != 0);
    } catch (const std::exception &e) {
        g_err = e.what();
        return nullptr;
    }
}
void orc_sv_free(void *sv) { delete static_cast<Handle *>(sv); }

int orc_sv_set_state(void *h, const void *data) {
    return with_sv(h, [&](auto &sv) {
        std::memcpy(sv.data.data(), data, sv.len() * sizeof(sv.data[0]));
    });
}
int orc_sv_get_state(void *h, void *out) {
    return with_sv(h, [&](auto &sv) {
        std::memcpy(out, sv.data.data(), sv.len() * sizeof(sv.data[0]));
    });
}
int orc_sv_apply(void *h, const char *name, const int64_t *cw, const uint8_t *cv,
                 int ncw, const int64_t *w, int nw, int inverse,
                 const double *params, int np) {
    return with_sv(h, [&](auto &sv) {
        using T = typename std::decay_t<decltype(sv.data[0])>::value_type;
        std::vector<T> ps;
        for (int i = 0; i < np; i++) {
            ps.push_back(static_cast<T>(params[i]));
        }
        orc::apply_named<T>(sv.ptr(), sv.n, name, vec(cw, ncw), bvec(cv, ncw),
                            vec(w, nw), inverse != 0, ps);
    });
}
int orc_sv_apply_matrix(void *h, const double *mat, const int64_t *cw,
                        const uint8_t *cv, int ncw, const int64_t *w, int nw,
                        int inverse) {
    return with_sv(h, [&](auto &sv) {
        using T = typename std::decay_t<decltype(sv.data[0])>::value_type;
        const size_t dim = size_t{1} << nw;
        orc::apply_matrix<T>(sv.ptr(), sv.n, cvec<T>(mat, dim * dim), vec(cw, ncw),
                             bvec(cv, ncw), vec(w, nw), inverse != 0);
    });
}
int orc_sv_apply_sparse(void *h, const int64_t *indptr, const int64_t *indices,
                        const double *data, int64_t nnz, const int64_t *cw,
                        const uint8_t *cv, int ncw, const int64_t *w, int nw) {
    return with_sv(h, [&](auto &sv) {
        using T = typename std::decay_t<decltype(sv.data[0])>::value_type;
        const size_t dim = size_t{1} << nw;
        orc::apply_sparse<T>(sv.ptr(), sv.n, vec(indptr, static_cast<int>(dim + 1)),
                             vec(indices, static_cast<int>(nnz)),
                             cvec<T>(data, static_cast<size_t>(nnz)), vec(cw, ncw),
                             bvec(cv, ncw), vec(w, nw));
    });
}
int orc_sv_apply_pauli_rot(void *h, const int64_t *w, int nw, int inverse,
                           double angle, const char *word) {
    return with_sv(h, [&](auto &sv) {
        using T = typename std::decay_t<decltype(sv.data[0])>::value_type;
        orc::apply_pauli_rot<T>(sv.ptr(), sv.n, vec(w, nw), inverse != 0,
                                static_cast<T>(angle), word);
    });
}
int orc_sv_apply_generator(void *h, const char *name, const int64_t *cw,
                           const uint8_t *cv, int ncw, const int64_t *w, int nw,
                           int adj, double *scale_out) {
    (void)adj;
    return with_sv(h, [&](auto &sv) {
        using T = typename std::decay_t<decltype(sv.data[0])>::value_type;
        *scale_out = static_cast<double>(orc::apply_generator<T>(
            sv.ptr(), sv.n, name, vec(cw, ncw), bvec(cv, ncw), vec(w, nw)));
    });
}
int orc_sv_collapse(void *h, int64_t wire, int branch) {
    return with_sv(h, [&](auto &sv) {
        orc::collapse(sv, static_cast<size_t>(wire), branch != 0);
    });
}
int orc_sv_normalize(void *h) {
    return with_sv(h, [&](auto &sv) { orc::normalize(sv); });
}
int orc_sv_set_basis_state(void *h, const int64_t *bits, const int64_t *w, int nw) {
    // StateVectorLQubit.hpp:928-963
    return with_sv(h, [&](auto &sv) {
        size_t index = 0;
        for (int k = 0; k < nw; k++) {
            index |= static_cast<size_t>(bits[k]) << (sv.n - 1 - static_cast<size_t>(w[k]));
        }
        ORC_CHECK(index < sv.len(), "Invalid index");
        std::fill(sv.data.begin(), sv.data.end(), 0.0);
        sv.data[index] = {1.0, 0.0};
    });
}
int orc_probs(void *h, const int64_t *w, int nw, double *out) {
    return with_sv(h, [&](auto &sv) {
        std::vector<size_t> wires;
        if (nw < 0) {
            wires.resize(sv.n);
            std::iota(wires.begin(), wires.end(), 0);
        } else {
            wires = vec(w, nw);
        }
        const auto p = orc::probs(sv, wires);
        for (size_t i = 0; i < p.size(); i++) {
            out[i] = static_cast<double>(p[i]);
        }
    });
}
int orc_expval_named(void *h, const char *name, const int64_t *w, int nw, double *out) {
    return with_sv(h, [&](auto &sv) {
        *out = static_cast<double>(orc::expval_named(sv, name, vec(w, nw)));
    });
}
int orc_expval_matrix(void *h, const double *mat, const int64_t *w, int nw, double *out) {
    return with_sv(h, [&](auto &sv) {
        using T = typename std::decay_t<decltype(sv.data[0])>::value_type;
        const size_t dim = size_t{1} << nw;
        *out = static_cast<double>(orc::expval_matrix<T>(sv, cvec<T>(mat, dim * dim), vec(w, nw)));
    });
}
int orc_var_named(void *h, const char *name, const int64_t *w, int nw, double *out) {
    // MeasurementsLQubit.hpp:444-458
    return with_sv(h, [&](auto &sv) {
        using T = typename std::decay_t<decltype(sv.data[0])>::value_type;
        orc::NamedObs<T> o;
        o.name = name;
        o.wires = vec(w, nw);
        *out = static_cast<double>(orc::var_obs<T>(sv, o));
    });
}
int orc_var_matrix(void *h, const double *mat, const int64_t *w, int nw, double *out) {
    return with_sv(h, [&](auto &sv) {
        using T = typename std::decay_t<decltype(sv.data[0])>::value_type;
        const size_t dim = size_t{1} << nw;
        orc::HermObs<T> o;
        o.m = cvec<T>(mat, dim * dim);
        o.wires = vec(w, nw);
        *out = static_cast<double>(orc::var_obs<T>(sv, o));
    });
}
int orc_expval_sparse(void *h, const int64_t *indptr, int64_t nptr,
                      const int64_t *indices, const double *data, int64_t nnz,
                      double *out) {
    return with_sv(h, [&](auto &sv) {
        using T = typename std::decay_t<decltype(sv.data[0])>::value_type;
        *out = static_cast<double>(orc::expval_sparse<T>(
            sv, vec(indptr, static_cast<int>(nptr)), vec(indices, static_cast<int>(nnz)),
            cvec<T>(data, static_cast<size_t>(nnz))));
    });
}
int orc_expval_obs(void *h, const char *spec, const double *cdata,
                   const int64_t *idata, double *out) {
    return with_sv(h, [&](auto &sv) {
        using T = typename std::decay_t<decltype(sv.data[0])>::value_type;
        auto o = parse_obs<T>(spec, cdata, idata);
        *out = static_cast<double>(orc::expval_obs<T>(sv, *o));
    });
}
int orc_var_obs(void *h, const char *spec, const double *cdata,
                const int64_t *idata, double *out) {
    return with_sv(h, [&](auto &sv) {
        using T = typename std::decay_t<decltype(sv.data[0])>::value_type;
        auto o = parse_obs<T>(spec, cdata, idata);
        *out = static_cast<double>(orc::var_obs<T>(sv, *o));
    });
}
int orc_samples(void *h, const int64_t *w, int nw, int64_t shots, uint64_t seed,
                int64_t *out) {
    return with_sv(h, [&](auto &sv) {
        std::vector<size_t> wires;
        if (nw < 0) {
            wires.resize(sv.n);
            std::iota(wires.begin(), wires.end(), 0);
        } else {
            wires = vec(w, nw);
        }
        const auto s = orc::samples(sv, wires, static_cast<size_t>(shots),
                                    static_cast<size_t>(seed));
        for (size_t i = 0; i < s.size(); i++) {
            out[i] = static_cast<int64_t>(s[i]);
        }
    });
}
int orc_mcmc_samples(void *h, const char *kernel, int64_t burnin, int64_t shots,
                     uint64_t seed, int64_t *out) {
    return with_sv(h, [&](auto &sv) {
        const auto s = orc::mcmc_samples(sv, std::string(kernel), static_cast<size_t>(burnin),
                                         static_cast<size_t>(shots), static_cast<size_t>(seed));
        for (size_t i = 0; i < s.size(); i++) {
            out[i] = static_cast<int64_t>(s[i]);
        }
    });
}
int orc_adjoint(void *h, int nops, const char **names, const double *params,
                const int *nparams, const int64_t *wires, const int *nwires,
                const uint8_t *inverses, const double *mats,
                const int64_t *mat_sizes, const int64_t *cwires,
                const int *ncwires, const uint8_t *cvals, int nobs,
                const char **obs_specs, const double *cdata,
                const int64_t *idata, const int64_t *trainable, int ntp,
                int apply_ops, double *jac_out) {
    return with_sv(h, [&](auto &sv) {
        using T = typename std::decay_t<decltype(sv.data[0])>::value_type;
        const auto ops = parse_ops<T>(nops, names, params, nparams, wires, nwires, inverses, mats,
                                      mat_sizes, cwires, ncwires, cvals);
        std::vector<orc::ObsPtr<T>> obs;
        for (int i = 0; i < nobs; i++) {
            obs.push_back(parse_obs<T>(obs_specs[i], cdata, idata));
        }
        std::vector<size_t> tp = vec(trainable, ntp);
        std::vector<T> jac;
        orc::adjoint_jacobian<T>(jac, sv, ops, obs, tp, apply_ops != 0);
        for (size_t i = 0; i < jac.size(); i++) {
            jac_out[i] = static_cast<double>(jac[i]);
        }
    });
}
int orc_vjp(void *h, int nops, const char **names, const double *params,
            const int *nparams, const int64_t *wires, const int *nwires,
            const uint8_t *inverses, const double *mats,
            const int64_t *mat_sizes, const int64_t *cwires,
            const int *ncwires, const uint8_t *cvals, const double *dy,
            const int64_t *trainable, int ntp, int apply_ops, double *out) {
    return with_sv(h, [&](auto &sv) {
        using T = typename std::decay_t<decltype(sv.data[0])>::value_type;
        const auto ops = parse_ops<T>(nops, names, params, nparams, wires, nwires, inverses, mats,
                                      mat_sizes, cwires, ncwires, cvals);
        const std::vector<std::complex<T>> cot = cvec<T>(dy, sv.len());
        std::vector<std::complex<T>> w;
        orc::vjp<T>(w, sv, ops, cot, vec(trainable, ntp), apply_ops != 0);
        for (size_t i = 0; i < w.size(); i++) {
            out[2 * i] = static_cast<double>(w[i].real());
            out[2 * i + 1] = static_cast<double>(w[i].imag());
        }
    });
}
int orc_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

} // extern "C"
