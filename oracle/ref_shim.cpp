// ORACLE PIN — test infrastructure only.
//
// C API (oracle_api.h, prefix ref_) over the reference's OWN lightning.qubit
// C++ classes.  This file holds no reference code: it is compiled against the
// reference's headers and sources where they lie (see build_oracle.py), and
// the resulting oracle/_ref/libplref.so is used only here, in this container,
// to pin the restatement in lm_oracle.hpp and to generate the golden fixtures
// under tests/golden/.
//
// Entry points used (reference paths, relative to the project root):
//   StateVectorLQubitManaged      pennylane_lightning/core/simulators/lightning_qubit/StateVectorLQubitManaged.hpp
//   Measurements                  .../lightning_qubit/measurements/MeasurementsLQubit.hpp
//   NamedObs/HermitianObs/...     .../lightning_qubit/observables/ObservablesLQubit.hpp
//   AdjointJacobian               .../lightning_qubit/algorithms/AdjointJacobianLQubit.hpp
//   VectorJacobianProduct         .../lightning_qubit/algorithms/VectorJacobianProduct.hpp
//   OpsData / JacobianData        pennylane_lightning/core/algorithms/JacobianData.hpp
#define ORC_PREFIX ref_
#include "oracle_api.h"
#include "obs_spec.hpp"

#include "AdjointJacobianLQubit.hpp"
#include "JacobianData.hpp"
#include "MeasurementsLQubit.hpp"
#include "ObservablesLQubit.hpp"
#include "StateVectorLQubitManaged.hpp"
#include "VectorJacobianProduct.hpp"

#include <cstring>
#include <numeric>
#include <span>
#include <variant>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {
using namespace Pennylane::LightningQubit;
using namespace Pennylane::LightningQubit::Measures;
using namespace Pennylane::LightningQubit::Observables;
using namespace Pennylane::LightningQubit::Algorithms;
using Pennylane::Algorithms::JacobianData;
using Pennylane::Algorithms::OpsData;
using Pennylane::Observables::Observable;

thread_local std::string g_err;

template <class T> using SV = StateVectorLQubitManaged<T>;

struct Handle {
    bool dbl;
    std::variant<SV<float>, SV<double>> sv;
    Handle(int n, bool d)
        : dbl(d),
          sv(d ? std::variant<SV<float>, SV<double>>(std::in_place_index<1>,
                                                    static_cast<std::size_t>(n))
               : std::variant<SV<float>, SV<double>>(std::in_place_index<0>,
                                                    static_cast<std::size_t>(n))) {}
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

std::vector<std::size_t> vec(const int64_t *p, int n) {
    std::vector<std::size_t> v;
    for (int i = 0; i < n; i++) {
        v.push_back(static_cast<std::size_t>(p[i]));
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
template <class T> std::vector<std::complex<T>> cvec(const double *p, std::size_t n) {
    std::vector<std::complex<T>> v(n);
    for (std::size_t i = 0; i < n; i++) {
        v[i] = {static_cast<T>(p[2 * i]), static_cast<T>(p[2 * i + 1])};
    }
    return v;
}

template <class T> struct Builder {
    using O = std::shared_ptr<Observable<SV<T>>>;
    O named(const std::string &name, std::size_t w) {
        return std::make_shared<NamedObs<SV<T>>>(name, std::vector<std::size_t>{w});
    }
    O herm(std::vector<std::complex<double>> m, std::vector<std::size_t> wires) {
        std::vector<std::complex<T>> mm;
        for (auto &x : m) {
            mm.emplace_back(static_cast<T>(x.real()), static_cast<T>(x.imag()));
        }
        return std::make_shared<HermitianObs<SV<T>>>(mm, wires);
    }
    O prod(std::vector<O> obs) { return TensorProdObs<SV<T>>::create(obs); }
    O ham(std::vector<double> coeffs, std::vector<O> obs) {
        std::vector<T> c;
        for (auto x : coeffs) {
            c.push_back(static_cast<T>(x));
        }
        return std::make_shared<Hamiltonian<SV<T>>>(c, obs);
    }
    O sparse(std::vector<std::complex<double>> data, std::vector<std::size_t> indices,
             std::vector<std::size_t> indptr, std::vector<std::size_t> wires) {
        std::vector<std::complex<T>> d;
        for (auto &x : data) {
            d.emplace_back(static_cast<T>(x.real()), static_cast<T>(x.imag()));
        }
        return std::make_shared<SparseHamiltonian<SV<T>>>(d, indices, indptr, wires);
    }
};
template <class T>
auto parse_obs(const char *spec, const double *cdata, const int64_t *idata) {
    Builder<T> b;
    orc_spec::Parser<Builder<T>> p(b, spec, cdata, idata);
    return p.parse();
}

template <class SVT>
OpsData<SVT> make_ops(int nops, const char **names, const double *params, const int *nparams,
                      const int64_t *wires, const int *nwires, const uint8_t *inverses, const double *mats,
                      const int64_t *mat_sizes, const int64_t *cwires, const int *ncwires, const uint8_t *cvals) {
    using T = typename SVT::PrecisionT;
    std::vector<std::string> on;
    std::vector<std::vector<T>> op;
    std::vector<std::vector<std::size_t>> ow, ocw;
    std::vector<bool> oi;
    std::vector<std::vector<std::complex<T>>> om;
    std::vector<std::vector<bool>> ocv;
    std::size_t ip = 0, iw = 0, im = 0, ic = 0;
    for (int k = 0; k < nops; k++) {
        on.emplace_back(names[k]);
        std::vector<T> p;
        for (int i = 0; i < nparams[k]; i++) {
            p.push_back(static_cast<T>(params[ip++]));
        }
        op.push_back(p);
        std::vector<std::size_t> w;
        for (int i = 0; i < nwires[k]; i++) {
            w.push_back(static_cast<std::size_t>(wires[iw++]));
        }
        ow.push_back(w);
        oi.push_back(inverses[k] != 0);
        om.push_back(cvec<T>(mats + 2 * im, static_cast<std::size_t>(mat_sizes[k])));
        im += static_cast<std::size_t>(mat_sizes[k]);
        std::vector<std::size_t> cw;
        std::vector<bool> cv;
        for (int i = 0; i < ncwires[k]; i++) {
            cw.push_back(static_cast<std::size_t>(cwires[ic]));
            cv.push_back(cvals[ic] != 0);
            ic++;
        }
        ocw.push_back(cw);
        ocv.push_back(cv);
    }
    return OpsData<SVT>{on, op, ow, oi, om, ocw, ocv};
}

} // namespace

extern "C" {

const char *ref_last_error(void) { return g_err.c_str(); }
void *ref_sv_new(int num_qubits, int is_double) {
    try {
        return new Handle(num_qubits, is_double != 0);
    } catch (const std::exception &e) {
        g_err = e.what();
        return nullptr;
    }
}
void ref_sv_free(void *sv) { delete static_cast<Handle *>(sv); }
int ref_sv_set_state(void *h, const void *data) {
    return with_sv(h, [&](auto &sv) {
        std::memcpy(sv.getData(), data, sv.getLength() * sizeof(sv.getData()[0]));
    });
}
int ref_sv_get_state(void *h, void *out) {
    return with_sv(h, [&](auto &sv) {
        std::memcpy(out, sv.getData(), sv.getLength() * sizeof(sv.getData()[0]));
    });
}
int ref_sv_apply(void *h, const char *name, const int64_t *cw, const uint8_t *cv,
                 int ncw, const int64_t *w, int nw, int inverse,
                 const double *params, int np) {
    return with_sv(h, [&](auto &sv) {
        using T = typename std::decay_t<decltype(sv)>::PrecisionT;
        std::vector<T> ps;
        for (int i = 0; i < np; i++) {
            ps.push_back(static_cast<T>(params[i]));
        }
        if (ncw > 0) {
            sv.applyOperation(name, vec(cw, ncw), bvec(cv, ncw), vec(w, nw),
                              inverse != 0, ps);
        } else {
            sv.applyOperation(name, vec(w, nw), inverse != 0, ps);
        }
    });
}
int ref_sv_apply_matrix(void *h, const double *mat, const int64_t *cw,
                        const uint8_t *cv, int ncw, const int64_t *w, int nw,
                        int inverse) {
    return with_sv(h, [&](auto &sv) {
        using T = typename std::decay_t<decltype(sv)>::PrecisionT;
        const std::size_t dim = std::size_t{1} << nw;
        auto m = cvec<T>(mat, dim * dim);
        if (ncw > 0) {
            sv.applyControlledMatrix(m, vec(cw, ncw), bvec(cv, ncw), vec(w, nw),
                                     inverse != 0);
        } else {
            sv.applyMatrix(m, vec(w, nw), inverse != 0);
        }
    });
}
int ref_sv_apply_sparse(void *h, const int64_t *indptr, const int64_t *indices,
                        const double *data, int64_t nnz, const int64_t *cw,
                        const uint8_t *cv, int ncw, const int64_t *w, int nw) {
    return with_sv(h, [&](auto &sv) {
        using T = typename std::decay_t<decltype(sv)>::PrecisionT;
        const std::size_t dim = std::size_t{1} << nw;
        auto ip = vec(indptr, static_cast<int>(dim + 1));
        auto ix = vec(indices, static_cast<int>(nnz));
        auto d = cvec<T>(data, static_cast<std::size_t>(nnz));
        if (ncw > 0) {
            sv.applyControlledSparseMatrix(ip.data(), ix.data(), d.data(), vec(cw, ncw),
                                           bvec(cv, ncw), vec(w, nw), false);
        } else {
            sv.applySparseMatrix(ip.data(), ix.data(), d.data(), vec(w, nw), false);
        }
    });
}
int ref_sv_apply_pauli_rot(void *h, const int64_t *w, int nw, int inverse,
                           double angle, const char *word) {
    return with_sv(h, [&](auto &sv) {
        using T = typename std::decay_t<decltype(sv)>::PrecisionT;
        sv.applyPauliRot(vec(w, nw), inverse != 0, {static_cast<T>(angle)}, word);
    });
}
int ref_sv_apply_generator(void *h, const char *name, const int64_t *cw,
                           const uint8_t *cv, int ncw, const int64_t *w, int nw,
                           int adj, double *scale_out) {
    return with_sv(h, [&](auto &sv) {
        if (ncw > 0) {
            *scale_out = static_cast<double>(sv.applyGenerator(
                name, vec(cw, ncw), bvec(cv, ncw), vec(w, nw), adj != 0));
        } else {
            *scale_out = static_cast<double>(sv.applyGenerator(name, vec(w, nw), adj != 0));
        }
    });
}
int ref_sv_collapse(void *h, int64_t wire, int branch) {
    return with_sv(h, [&](auto &sv) {
        sv.collapse(static_cast<std::size_t>(wire), branch != 0);
    });
}
int ref_sv_normalize(void *h) {
    return with_sv(h, [&](auto &sv) { sv.normalize(); });
}
int ref_sv_set_basis_state(void *h, const int64_t *bits, const int64_t *w, int nw) {
    return with_sv(h, [&](auto &sv) { sv.setBasisState(vec(bits, nw), vec(w, nw)); });
}
int ref_probs(void *h, const int64_t *w, int nw, double *out) {
    return with_sv(h, [&](auto &sv) {
        Measurements<std::decay_t<decltype(sv)>> m(sv);
        std::vector<std::size_t> wires;
        if (nw < 0) {
            wires.resize(sv.getNumQubits());
            std::iota(wires.begin(), wires.end(), 0);
        } else {
            wires = vec(w, nw);
        }
        auto p = m.probs(wires);
        for (std::size_t i = 0; i < p.size(); i++) {
            out[i] = static_cast<double>(p[i]);
        }
    });
}
int ref_expval_named(void *h, const char *name, const int64_t *w, int nw, double *out) {
    return with_sv(h, [&](auto &sv) {
        Measurements<std::decay_t<decltype(sv)>> m(sv);
        *out = static_cast<double>(m.expval(std::string(name), vec(w, nw)));
    });
}
int ref_expval_matrix(void *h, const double *mat, const int64_t *w, int nw, double *out) {
    return with_sv(h, [&](auto &sv) {
        using T = typename std::decay_t<decltype(sv)>::PrecisionT;
        Measurements<std::decay_t<decltype(sv)>> m(sv);
        const std::size_t dim = std::size_t{1} << nw;
        *out = static_cast<double>(m.expval(cvec<T>(mat, dim * dim), vec(w, nw)));
    });
}
int ref_var_named(void *h, const char *name, const int64_t *w, int nw, double *out) {
    return with_sv(h, [&](auto &sv) {
        Measurements<std::decay_t<decltype(sv)>> m(sv);
        *out = static_cast<double>(m.var(std::string(name), vec(w, nw)));
    });
}
int ref_var_matrix(void *h, const double *mat, const int64_t *w, int nw, double *out) {
    return with_sv(h, [&](auto &sv) {
        using T = typename std::decay_t<decltype(sv)>::PrecisionT;
        Measurements<std::decay_t<decltype(sv)>> m(sv);
        const std::size_t dim = std::size_t{1} << nw;
        *out = static_cast<double>(m.var(cvec<T>(mat, dim * dim), vec(w, nw)));
    });
}
int ref_expval_sparse(void *h, const int64_t *indptr, int64_t nptr,
                      const int64_t *indices, const double *data, int64_t nnz,
                      double *out) {
    return with_sv(h, [&](auto &sv) {
        using T = typename std::decay_t<decltype(sv)>::PrecisionT;
        Measurements<std::decay_t<decltype(sv)>> m(sv);
        auto ip = vec(indptr, static_cast<int>(nptr));
        auto ix = vec(indices, static_cast<int>(nnz));
        auto d = cvec<T>(data, static_cast<std::size_t>(nnz));
        *out = static_cast<double>(m.expval(ip.data(), static_cast<std::size_t>(nptr),
                                            ix.data(), d.data(),
                                            static_cast<std::size_t>(nnz)));
    });
}
int ref_expval_obs(void *h, const char *spec, const double *cdata,
                   const int64_t *idata, double *out) {
    return with_sv(h, [&](auto &sv) {
        using T = typename std::decay_t<decltype(sv)>::PrecisionT;
        Measurements<std::decay_t<decltype(sv)>> m(sv);
        auto o = parse_obs<T>(spec, cdata, idata);
        *out = static_cast<double>(m.expval(*o));
    });
}
int ref_var_obs(void *h, const char *spec, const double *cdata,
                const int64_t *idata, double *out) {
    return with_sv(h, [&](auto &sv) {
        using T = typename std::decay_t<decltype(sv)>::PrecisionT;
        Measurements<std::decay_t<decltype(sv)>> m(sv);
        auto o = parse_obs<T>(spec, cdata, idata);
        *out = static_cast<double>(m.var(*o));
    });
}
int ref_samples(void *h, const int64_t *w, int nw, int64_t shots, uint64_t seed,
                int64_t *out) {
    return with_sv(h, [&](auto &sv) {
        Measurements<std::decay_t<decltype(sv)>> m(sv);
        m.setSeed(static_cast<std::size_t>(seed));
        std::vector<std::size_t> wires;
        if (nw < 0) {
            wires.resize(sv.getNumQubits());
            std::iota(wires.begin(), wires.end(), 0);
        } else {
            wires = vec(w, nw);
        }
        auto s = m.generate_samples(wires, static_cast<std::size_t>(shots));
        for (std::size_t i = 0; i < s.size(); i++) {
            out[i] = static_cast<int64_t>(s[i]);
        }
    });
}
int ref_mcmc_samples(void *h, const char *kernel, int64_t burnin, int64_t shots,
                     uint64_t seed, int64_t *out) {
    return with_sv(h, [&](auto &sv) {
        Measurements<std::decay_t<decltype(sv)>> m(sv);
        m.setSeed(static_cast<std::size_t>(seed));
        auto s = m.generate_samples_metropolis(std::string(kernel), static_cast<std::size_t>(burnin),
                                               static_cast<std::size_t>(shots));
        for (std::size_t i = 0; i < s.size(); i++) {
            out[i] = static_cast<int64_t>(s[i]);
        }
    });
}
int ref_adjoint(void *h, int nops, const char **names, const double *params,
                const int *nparams, const int64_t *wires, const int *nwires,
                const uint8_t *inverses, const double *mats,
                const int64_t *mat_sizes, const int64_t *cwires,
                const int *ncwires, const uint8_t *cvals, int nobs,
                const char **obs_specs, const double *cdata,
                const int64_t *idata, const int64_t *trainable, int ntp,
                int apply_ops, double *jac_out) {
    return with_sv(h, [&](auto &sv) {
        using SVT = std::decay_t<decltype(sv)>;
        using T = typename SVT::PrecisionT;
        const OpsData<SVT> ops = make_ops<SVT>(nops, names, params, nparams, wires, nwires, inverses, mats,
                                               mat_sizes, cwires, ncwires, cvals);
        std::vector<std::shared_ptr<Observable<SVT>>> obs;
        for (int i = 0; i < nobs; i++) {
            obs.push_back(parse_obs<T>(obs_specs[i], cdata, idata));
        }
        std::vector<std::size_t> tp = vec(trainable, ntp);
        std::vector<T> jac(obs.size() * tp.size(), T{0});
        JacobianData<SVT> jd{ops.getTotalNumParams(), sv.getLength(), sv.getData(),
                             obs, ops, tp};
        AdjointJacobian<SVT> adj;
        adj.adjointJacobian(std::span{jac}, jd, sv, apply_ops != 0);
        for (std::size_t i = 0; i < jac.size(); i++) {
            jac_out[i] = static_cast<double>(jac[i]);
        }
    });
}
int ref_vjp(void *h, int nops, const char **names, const double *params,
            const int *nparams, const int64_t *wires, const int *nwires,
            const uint8_t *inverses, const double *mats,
            const int64_t *mat_sizes, const int64_t *cwires,
            const int *ncwires, const uint8_t *cvals, const double *dy,
            const int64_t *trainable, int ntp, int apply_ops, double *out) {
    return with_sv(h, [&](auto &sv) {
        using SVT = std::decay_t<decltype(sv)>;
        using T = typename SVT::PrecisionT;
        const OpsData<SVT> ops = make_ops<SVT>(nops, names, params, nparams, wires, nwires, inverses, mats,
                                               mat_sizes, cwires, ncwires, cvals);
        const std::vector<std::complex<T>> cot = cvec<T>(dy, sv.getLength());
        std::vector<std::size_t> tp = vec(trainable, ntp);
        std::vector<std::complex<T>> w(tp.size());
        JacobianData<SVT> jd{ops.getTotalNumParams(), sv.getLength(), sv.getData(), {}, ops, tp};
        VectorJacobianProduct<SVT> v;
        v(std::span{w}, jd, std::span<const std::complex<T>>{cot}, apply_ops != 0);
        for (std::size_t i = 0; i < w.size(); i++) {
            out[2 * i] = static_cast<double>(w[i].real());
            out[2 * i + 1] = static_cast<double>(w[i].imag());
        }
    });
}
int ref_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

} // extern "C"
