// A CPU test double of the C ABI entry points (include/pl_gb300.h) that the
// Catalyst device (include/pl_gb300_catalyst.hpp) calls, answered by the CPU
// oracle (liboracle.so).  It is linked only into the CPU build of
// tests/cpp/test_catalyst_device.cpp, so the device's host logic (qubit map,
// register growth and reduction, tape, observable cache, shot handling) runs
// without a GPU; the GPU build of the same program links the real
// libplgb300.so.  Test infrastructure: nothing in the backend links it.
#include "pl_gb300.h"

#include "oracle_api.h"

#include <algorithm>
#include <complex>
#include <cstdio>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

struct plgb_sv {
    void *o;
    int n;
};
struct plgb_obs {
    enum Kind { Named, Herm, Prod, Ham } kind;
    std::string name;
    std::vector<int64_t> wires;
    std::vector<double> matrix; // interleaved, 4^k complex entries
    std::vector<plgb_obs> children;
    std::vector<double> coeffs;
};
struct plgb_ops {
    std::vector<std::string> names;
    std::vector<double> params, mats;
    std::vector<int> nparams, nwires, ncwires;
    std::vector<int64_t> wires, matsz, cwires;
    std::vector<uint8_t> inverses, cvals;
};

namespace {
thread_local std::string g_err;
int status(int rc) {
    if (rc != 0) {
        g_err = orc_last_error();
        return PLGB_ERR_INVALID;
    }
    return PLGB_OK;
}
int fail(const std::string &m) {
    g_err = m;
    return PLGB_ERR_INVALID;
}
using cd = std::complex<double>;
std::vector<cd> state_of(const plgb_sv *s) {
    std::vector<cd> v(size_t{1} << s->n);
    orc_sv_get_state(s->o, v.data());
    return v;
}
void spec_of(const plgb_obs &o, std::string &out, std::vector<double> &cdata) {
    char buf[64];
    switch (o.kind) {
    case plgb_obs::Named:
        out += "named " + o.name + " " + std::to_string(o.wires.at(0)) + " ";
        break;
    case plgb_obs::Herm:
        out += "herm " + std::to_string(o.wires.size()) + " ";
        for (const auto w : o.wires) {
            out += std::to_string(w) + " ";
        }
        out += std::to_string(cdata.size() / 2) + " ";
        cdata.insert(cdata.end(), o.matrix.begin(), o.matrix.end());
        break;
    case plgb_obs::Prod:
        out += "prod " + std::to_string(o.children.size()) + " ";
        for (const auto &c : o.children) {
            spec_of(c, out, cdata);
        }
        break;
    case plgb_obs::Ham:
        out += "ham " + std::to_string(o.children.size()) + " ";
        for (size_t i = 0; i < o.children.size(); i++) {
            std::snprintf(buf, sizeof(buf), "%.17g ", o.coeffs[i]);
            out += buf;
            spec_of(o.children[i], out, cdata);
        }
        break;
    }
}
void wires_of(const plgb_obs &o, std::vector<int64_t> &out) {
    if (o.kind == plgb_obs::Named || o.kind == plgb_obs::Herm) {
        for (const auto w : o.wires) {
            if (std::find(out.begin(), out.end(), w) == out.end()) {
                out.push_back(w);
            }
        }
    }
    for (const auto &c : o.children) {
        wires_of(c, out);
    }
}
} // namespace

extern "C" {
const char *plgb_last_error(void) { return g_err.c_str(); }
const char *plgb_gate_name(int) { return nullptr; }

int plgb_sv_create(int num_qubits, int precision, plgb_sv **out) {
    if (precision != 128) {
        return fail("the CPU test double holds complex128 registers only");
    }
    auto *s = new plgb_sv{orc_sv_new(num_qubits, 1), num_qubits};
    std::vector<cd> zero(size_t{1} << num_qubits);
    zero[0] = 1.0;
    orc_sv_set_state(s->o, zero.data());
    *out = s;
    return PLGB_OK;
}
int plgb_sv_clone(const plgb_sv *src, plgb_sv **out) {
    auto *s = new plgb_sv{orc_sv_new(src->n, 1), src->n};
    orc_sv_set_state(s->o, state_of(src).data());
    *out = s;
    return PLGB_OK;
}
int plgb_sv_destroy(plgb_sv *sv) {
    if (sv != nullptr) {
        orc_sv_free(sv->o);
        delete sv;
    }
    return PLGB_OK;
}
int plgb_sv_num_qubits(const plgb_sv *sv, int *out) {
    *out = sv->n;
    return PLGB_OK;
}
int plgb_sv_length(const plgb_sv *sv, uint64_t *out) {
    *out = uint64_t{1} << sv->n;
    return PLGB_OK;
}
int plgb_sv_set_basis_state(plgb_sv *sv, const int64_t *bits, const int64_t *wires, int nw) {
    return status(orc_sv_set_basis_state(sv->o, bits, wires, nw));
}
int plgb_sv_set_state_vector(plgb_sv *sv, const void *host_state, uint64_t len, const int64_t *wires, int nw) {
    if (len != (uint64_t{1} << nw)) {
        return fail("Inconsistent state and wires dimensions.");
    }
    const auto *sub = static_cast<const cd *>(host_state);
    std::vector<cd> full(size_t{1} << sv->n);
    for (uint64_t j = 0; j < len; j++) {
        size_t idx = 0;
        for (int m = 0; m < nw; m++) {
            if ((j >> (nw - 1 - m)) & 1U) {
                idx |= size_t{1} << (sv->n - 1 - wires[m]);
            }
        }
        full[idx] = sub[j];
    }
    return status(orc_sv_set_state(sv->o, full.data()));
}
int plgb_sv_update_data(plgb_sv *sv, const void *host_data, uint64_t len) {
    if (len != (uint64_t{1} << sv->n)) {
        return fail("The size of provided data must be equal to the size of the state vector");
    }
    return status(orc_sv_set_state(sv->o, host_data));
}
int plgb_sv_get_state(const plgb_sv *sv, void *host_out, uint64_t len) {
    if (len != (uint64_t{1} << sv->n)) {
        return fail("size mismatch");
    }
    return status(orc_sv_get_state(sv->o, host_out));
}
int plgb_sv_apply_operation(plgb_sv *sv, const char *name, const int64_t *wires, int nw, int inverse,
                            const double *params, int np) {
    return status(orc_sv_apply(sv->o, name, nullptr, nullptr, 0, wires, nw, inverse, params, np));
}
int plgb_sv_apply_controlled_operation(plgb_sv *sv, const char *name, const int64_t *cwires, const uint8_t *cvals,
                                       int ncw, const int64_t *wires, int nw, int inverse, const double *params,
                                       int np) {
    return status(orc_sv_apply(sv->o, name, cwires, cvals, ncw, wires, nw, inverse, params, np));
}
int plgb_sv_apply_matrix(plgb_sv *sv, const double *matrix, const int64_t *wires, int nw, int inverse) {
    return status(orc_sv_apply_matrix(sv->o, matrix, nullptr, nullptr, 0, wires, nw, inverse));
}
int plgb_sv_apply_controlled_matrix(plgb_sv *sv, const double *matrix, const int64_t *cwires, const uint8_t *cvals,
                                    int ncw, const int64_t *wires, int nw, int inverse) {
    return status(orc_sv_apply_matrix(sv->o, matrix, cwires, cvals, ncw, wires, nw, inverse));
}
int plgb_sv_apply_pauli_rot(plgb_sv *sv, const int64_t *wires, int nw, int inverse, double angle, const char *word) {
    return status(orc_sv_apply_pauli_rot(sv->o, wires, nw, inverse, angle, word));
}
int plgb_sv_collapse(plgb_sv *sv, int64_t wire, int branch) { return status(orc_sv_collapse(sv->o, wire, branch)); }
int plgb_sv_normalize(plgb_sv *sv) { return status(orc_sv_normalize(sv->o)); }

int plgb_meas_probs(plgb_sv *sv, const int64_t *wires, int nw, double *out) {
    return status(orc_probs(sv->o, wires, nw, out));
}
int plgb_meas_expval_obs(plgb_sv *sv, const plgb_obs *obs, double *out) {
    std::string spec;
    std::vector<double> cdata;
    spec_of(*obs, spec, cdata);
    return status(orc_expval_obs(sv->o, spec.c_str(), cdata.data(), nullptr, out));
}
int plgb_meas_var_obs(plgb_sv *sv, const plgb_obs *obs, double *out) {
    std::string spec;
    std::vector<double> cdata;
    spec_of(*obs, spec, cdata);
    return status(orc_var_obs(sv->o, spec.c_str(), cdata.data(), nullptr, out));
}
int plgb_meas_generate_samples(plgb_sv *sv, const int64_t *wires, int nw, int64_t shots, uint64_t seed,
                               int64_t *out) {
    return status(orc_samples(sv->o, wires, nw, shots, seed, out));
}
int plgb_meas_generate_mcmc_samples(plgb_sv *sv, const char *kernelname, int64_t num_burnin, int64_t num_shots,
                                    uint64_t seed, int64_t *out) {
    return status(orc_mcmc_samples(sv->o, kernelname, num_burnin, num_shots, seed, out));
}

int plgb_obs_named(const char *name, const int64_t *wires, int nw, plgb_obs **out) {
    if (nw != 1) {
        return fail("the CPU test double takes one-wire named observables");
    }
    *out = new plgb_obs{plgb_obs::Named, name, {wires[0]}, {}, {}, {}};
    return PLGB_OK;
}
int plgb_obs_hermitian(const double *matrix, const int64_t *wires, int nw, plgb_obs **out) {
    const size_t count = size_t{2} << (2 * nw);
    *out = new plgb_obs{plgb_obs::Herm, "Hermitian", {wires, wires + nw}, {matrix, matrix + count}, {}, {}};
    return PLGB_OK;
}
int plgb_obs_tensor_prod(plgb_obs *const *obs, int n, plgb_obs **out) {
    auto *o = new plgb_obs{plgb_obs::Prod, "TensorProd", {}, {}, {}, {}};
    for (int i = 0; i < n; i++) {
        o->children.push_back(*obs[i]);
    }
    *out = o;
    return PLGB_OK;
}
int plgb_obs_hamiltonian(const double *coeffs, plgb_obs *const *obs, int n, plgb_obs **out) {
    auto *o = new plgb_obs{plgb_obs::Ham, "Hamiltonian", {}, {}, {}, {coeffs, coeffs + n}};
    for (int i = 0; i < n; i++) {
        o->children.push_back(*obs[i]);
    }
    *out = o;
    return PLGB_OK;
}
int plgb_obs_destroy(plgb_obs *obs) {
    delete obs;
    return PLGB_OK;
}
int plgb_obs_wires(const plgb_obs *obs, int64_t *wires, int cap, int *nw) {
    std::vector<int64_t> w;
    wires_of(*obs, w);
    *nw = static_cast<int>(w.size());
    for (int i = 0; i < cap && i < *nw; i++) {
        wires[i] = w[static_cast<size_t>(i)];
    }
    return PLGB_OK;
}
int plgb_obs_repr(const plgb_obs *obs, char *buf, size_t len) {
    std::snprintf(buf, len, "%s", obs->name.c_str());
    return PLGB_OK;
}

int plgb_ops_create(int nops, const char *const *names, const double *params, const int *nparams,
                    const int64_t *wires, const int *nwires, const uint8_t *inverses, const double *mats,
                    const int64_t *mat_sizes, const int64_t *cwires, const int *ncwires, const uint8_t *cvals,
                    plgb_ops **out) {
    auto *o = new plgb_ops;
    size_t np = 0, nw = 0, nm = 0, nc = 0;
    for (int k = 0; k < nops; k++) {
        o->names.emplace_back(names[k]);
        np += static_cast<size_t>(nparams[k]);
        nw += static_cast<size_t>(nwires[k]);
        nm += static_cast<size_t>(mat_sizes[k]);
        nc += static_cast<size_t>(ncwires[k]);
    }
    o->params.assign(params, params + np);
    o->nparams.assign(nparams, nparams + nops);
    o->wires.assign(wires, wires + nw);
    o->nwires.assign(nwires, nwires + nops);
    o->inverses.assign(inverses, inverses + nops);
    o->mats.assign(mats, mats + 2 * nm);
    o->matsz.assign(mat_sizes, mat_sizes + nops);
    o->cwires.assign(cwires, cwires + nc);
    o->ncwires.assign(ncwires, ncwires + nops);
    o->cvals.assign(cvals, cvals + nc);
    *out = o;
    return PLGB_OK;
}
int plgb_ops_destroy(plgb_ops *ops) {
    delete ops;
    return PLGB_OK;
}
int plgb_adjoint_jacobian(plgb_sv *sv, plgb_obs *const *obs, int nobs, const plgb_ops *ops, const int64_t *trainable,
                          int ntp, int apply_ops, double *jac_out) {
    std::vector<std::string> specs(static_cast<size_t>(nobs));
    std::vector<double> cdata;
    for (int i = 0; i < nobs; i++) {
        spec_of(*obs[i], specs[static_cast<size_t>(i)], cdata);
    }
    std::vector<const char *> sp, nm;
    for (const auto &s : specs) {
        sp.push_back(s.c_str());
    }
    for (const auto &s : ops->names) {
        nm.push_back(s.c_str());
    }
    // the oracle's sweep modifies the register it is given: run it on a copy
    plgb_sv *copy = nullptr;
    plgb_sv_clone(sv, &copy);
    const int rc = orc_adjoint(copy->o, static_cast<int>(nm.size()), nm.data(), ops->params.data(),
                               ops->nparams.data(), ops->wires.data(), ops->nwires.data(), ops->inverses.data(),
                               ops->mats.data(), ops->matsz.data(), ops->cwires.data(), ops->ncwires.data(),
                               ops->cvals.data(), nobs, sp.data(), cdata.data(), nullptr, trainable, ntp, apply_ops,
                               jac_out);
    plgb_sv_destroy(copy);
    return status(rc);
}
}
