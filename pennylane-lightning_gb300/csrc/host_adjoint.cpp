// Adjoint Jacobian on the GPU.
//
// Algorithm: arXiv:2009.02823 backward sweep exactly as
// pennylane_lightning/core/simulators/lightning_qubit/algorithms/
// AdjointJacobianLQubit.hpp:225-491 orders it (same op loop, trainable-
// parameter bookkeeping, generator scaling and [obs][param] layout).
//
// Differences in method (same results):
//   * H|lambda> for a Pauli-sum observable is accumulated group by group
//     (one pass per bit-flip mask, no per-term state copies);
//   * for generators that are Pauli words (possibly with a projector on the
//     control / target subspace: RX, RY, RZ, PhaseShift, Ising XX/YY/ZZ,
//     MultiRZ, CRX/CRY/CRZ, ControlledPhaseShift, GlobalPhase and their
//     controlled forms) Im<H lambda| G |lambda> is evaluated by one transition
//     kernel that reads both states once, instead of copy + apply + dot;
//   * other generators take the reference's route through a scratch state mu.
#include "fusion.hpp"
#include "host.hpp"

#include <algorithm>
#include <optional>

namespace plgb {

namespace {

struct PauliGen {
    u64 x{0}, yz{0};
    int ny4{0};
    u64 pmask{0}, pval{0};
    double scale{0};
};

// Returns the generator of `op` as projector x Pauli word, if it is one.
std::optional<PauliGen> pauli_generator(const OpRec &op, int n) {
    auto bit = [&](int64_t w) -> u64 {
        if (w < 0 || w >= n) {
            throw PLError("wire index out of range");
        }
        return u64{1} << (n - 1 - w);
    };
    PauliGen g;
    std::vector<int64_t> wires = op.wires;
    for (size_t i = 0; i < op.cwires.size(); i++) {
        g.pmask |= bit(op.cwires[i]);
        if (op.cvals[i]) {
            g.pval |= bit(op.cwires[i]);
        }
    }
    std::string base = op.name;
    if (base == "CRX" || base == "CRY" || base == "CRZ" || base == "ControlledPhaseShift") {
        if (wires.size() != 2 || !op.cwires.empty()) {
            return std::nullopt;
        }
        g.pmask |= bit(wires[0]);
        g.pval |= bit(wires[0]);
        wires.erase(wires.begin());
        base = base == "CRX" ? "RX" : base == "CRY" ? "RY" : base == "CRZ" ? "RZ" : "PhaseShift";
    }
    if (base == "RX" && wires.size() == 1) {
        g.x = bit(wires[0]);
        g.scale = -0.5;
    } else if (base == "RY" && wires.size() == 1) {
        g.x = g.yz = bit(wires[0]);
        g.ny4 = 1;
        g.scale = -0.5;
    } else if (base == "RZ" && wires.size() == 1) {
        g.yz = bit(wires[0]);
        g.scale = -0.5;
    } else if (base == "PhaseShift" && wires.size() == 1) {
        g.pmask |= bit(wires[0]);
        g.pval |= bit(wires[0]);
        g.scale = 1.0;
    } else if (base == "IsingXX" && wires.size() == 2) {
        g.x = bit(wires[0]) | bit(wires[1]);
        g.scale = -0.5;
    } else if (base == "IsingYY" && wires.size() == 2) {
        g.x = g.yz = bit(wires[0]) | bit(wires[1]);
        g.ny4 = 2;
        g.scale = -0.5;
    } else if (base == "IsingZZ" && wires.size() == 2) {
        g.yz = bit(wires[0]) | bit(wires[1]);
        g.scale = -0.5;
    } else if (base == "MultiRZ" && !wires.empty()) {
        for (auto w : wires) {
            g.yz |= bit(w);
        }
        g.scale = -0.5;
    } else if (base == "GlobalPhase") {
        g.scale = -1.0;
    } else {
        return std::nullopt;
    }
    if (g.x & g.pmask) {
        return std::nullopt;
    }
    return g;
}

} // namespace

template <class T>
std::vector<double> Adjoint<T>::jacobian(StateVector<T> &sv, const std::vector<ObsPtr> &obs, const OpsList &opsl,
                                         const std::vector<int64_t> &tp, bool apply_ops, bool consume,
                                         int fused_tile_bits) {
    const auto &ops = opsl.ops;
    const size_t nobs = obs.size();
    const size_t ntp = tp.size();
    std::vector<double> jac(nobs * ntp, 0.0);
    if (ntp == 0 || nobs == 0) {
        return jac;
    }
    for (size_t i = 1; i < ntp; i++) {
        PLGB_REQUIRE(tp[i] > tp[i - 1], "trainable parameter indices must be sorted and unique");
    }
    const size_t num_param_ops = opsl.num_par_ops();
    PLGB_REQUIRE(tp.back() < static_cast<int64_t>(num_param_ops), "trainable parameter index out of range");
    const int n = sv.num_qubits();

    // lambda: the caller's register when it may be consumed, else a copy
    std::optional<StateVector<T>> own;
    if (!consume) {
        own.emplace(sv); // same stream
    }
    StateVector<T> &lambda = consume ? sv : *own;
    if (apply_ops) {
        for (const auto &op : ops) {
            lambda.apply_op(op, op.inverse);
        }
    }
    std::vector<std::unique_ptr<StateVector<T>>> hl;
    for (size_t h = 0; h < nobs; h++) {
        hl.emplace_back(std::make_unique<StateVector<T>>(n, lambda.stream()));
        Measure<T>::apply_obs_into(lambda, *hl.back(), *obs[h]);
    }
    // ---- fused sweep: the reverse program (reduction, then U^dagger, per
    // operation, last to first) compiled into two-register tile passes
    if (fused_tile_bits > 0 && nobs == 1) {
        std::vector<Prim<T>> prims;
        std::vector<double> slot_scale(ntp, 0.0);
        bool ok = true;
        size_t tpn = ntp - 1;
        size_t curp = num_param_ops - 1;
        auto it = tp.rbegin();
        for (long op_idx = static_cast<long>(ops.size()) - 1; op_idx >= 0 && ok; op_idx--) {
            const auto &op = ops[static_cast<size_t>(op_idx)];
            PLGB_REQUIRE(op.params.size() <= 1,
                         "The operation is not supported using the adjoint differentiation method");
            if (op.name == "StatePrep" || op.name == "BasisState") {
                continue;
            }
            if (it == tp.rend()) {
                break;
            }
            if (!op.params.empty()) {
                if (static_cast<int64_t>(curp) == *it) {
                    const auto pg = pauli_generator(op, n);
                    if (!pg) {
                        ok = false;
                        break;
                    }
                    Prim<T> r;
                    r.kind = Prim<T>::Reduce;
                    r.rx = pg->x;
                    r.ryz = pg->yz;
                    r.rny4 = pg->ny4;
                    r.rpm = pg->pmask;
                    r.rpv = pg->pval;
                    r.rslot = static_cast<int>(tpn);
                    slot_scale[tpn] = -2.0 * pg->scale * (op.inverse ? -1.0 : 1.0);
                    prims.push_back(std::move(r));
                    tpn--;
                    ++it;
                }
                curp--;
            }
            auto p = lambda.lower_op(op, !op.inverse);
            prims.insert(prims.end(), std::make_move_iterator(p.begin()), std::make_move_iterator(p.end()));
        }
        if (ok) {
            // two tiles of 2^t amplitudes per CTA must fit 200 KiB of shared memory
            const int tmax = sizeof(T) == 8 ? 12 : 13;
            const int t = std::max(1, std::min({fused_tile_bits, n, tmax}));
            auto prog = compile_fused<T>(n, prims, t, true);
            const int G = adj_grid_capacity(sizeof(cx<T>) << t);
            double *d_part = static_cast<double *>(dev_alloc((static_cast<size_t>(G) + 1) * ntp * sizeof(double)));
            struct Guard {
                double *p;
                ~Guard() { dev_free(p); }
            } guard{d_part};
            double *d_out = d_part + static_cast<size_t>(G) * ntp;
            cuda_check(cudaMemsetAsync(d_part, 0, static_cast<size_t>(G) * ntp * sizeof(double), lambda.stream()),
                       "memset");
            run_fused_adjoint<T>(lambda, *hl[0], *prog, d_part, G);
            launch_adj_sum(lambda.stream(), d_part, static_cast<int>(ntp), G, d_out);
            std::vector<double> r(ntp);
            cuda_check(cudaMemcpyAsync(r.data(), d_out, ntp * sizeof(double), cudaMemcpyDeviceToHost,
                                       lambda.stream()), "D2H");
            lambda.synchronize();
            std::vector<double> out(ntp);
            for (size_t p = 0; p < ntp; p++) {
                out[p] = static_cast<double>(static_cast<T>(slot_scale[p] * r[p]));
            }
            return out;
        }
        // a generator that is not a Pauli word: the op-by-op sweep below
        // starts from the untouched registers
    }

    std::unique_ptr<StateVector<T>> mu;
    // Pauli-generator results stay on the device (two doubles per
    // [param][obs]); one copy at the end instead of a sync per parameter
    double *d_res = nullptr;
    d_res = static_cast<double *>(dev_alloc(2 * nobs * ntp * sizeof(double)));
    struct ResGuard {
        double *p;
        ~ResGuard() { dev_free(p); }
    } res_guard{d_res};
    std::vector<char> on_device(nobs * ntp, 0);
    std::vector<double> dev_scale(nobs * ntp, 0.0);

    size_t tp_num = ntp - 1;
    size_t cur = num_param_ops - 1;
    auto tp_it = tp.rbegin();
    double *red = lambda.scratch_red();
    for (long op_idx = static_cast<long>(ops.size()) - 1; op_idx >= 0; op_idx--) {
        const auto &op = ops[static_cast<size_t>(op_idx)];
        PLGB_REQUIRE(op.params.size() <= 1, "The operation is not supported using the adjoint differentiation method");
        if (op.name == "StatePrep" || op.name == "BasisState") {
            continue;
        }
        if (tp_it == tp.rend()) {
            break;
        }
        if (!op.params.empty()) {
            if (static_cast<int64_t>(cur) == *tp_it) {
                const auto pg = pauli_generator(op, n);
                if (pg) {
                    const double scale = pg->scale * (op.inverse ? -1.0 : 1.0);
                    for (size_t h = 0; h < nobs; h++) {
                        const size_t slot = tp_num * nobs + h;
                        reduce_pauli_transition<T>(lambda.stream(), hl[h]->data(), lambda.data(), lambda.length(),
                                                   pg->x, pg->yz, pg->ny4, pg->pmask, pg->pval, red,
                                                   d_res + 2 * slot);
                        on_device[slot] = 1;
                        dev_scale[slot] = -2.0 * scale;
                    }
                } else {
                    if (!mu) {
                        mu = std::make_unique<StateVector<T>>(lambda);
                    } else {
                        mu->copy_from(lambda);
                    }
                    const double scale =
                        mu->apply_generator(op.name, op.cwires, op.cvals, op.wires) * (op.inverse ? -1.0 : 1.0);
                    for (size_t h = 0; h < nobs; h++) {
                        const cd ip = hl[h]->inner(*mu);
                        jac[tp_num * nobs + h] = -2.0 * scale * ip.imag();
                    }
                }
                tp_num--;
                ++tp_it;
            }
            cur--;
        }
        lambda.apply_op(op, !op.inverse);
        for (size_t h = 0; h < nobs; h++) {
            hl[h]->apply_op(op, !op.inverse);
        }
    }
    {
        std::vector<double> r(2 * nobs * ntp);
        cuda_check(cudaMemcpyAsync(r.data(), d_res, r.size() * sizeof(double), cudaMemcpyDeviceToHost,
                                   lambda.stream()), "D2H");
        lambda.synchronize();
        for (size_t k = 0; k < nobs * ntp; k++) {
            if (on_device[k]) {
                jac[k] = dev_scale[k] * r[2 * k + 1];
            }
        }
    }
    // Transpose [param][obs] -> [obs][param] (AdjointJacobianLQubit.hpp:487-490)
    std::vector<double> out(jac.size());
    for (size_t p = 0; p < ntp; p++) {
        for (size_t h = 0; h < nobs; h++) {
            out[h * ntp + p] = static_cast<double>(static_cast<T>(jac[p * nobs + h]));
        }
    }
    lambda.synchronize();
    return out;
}

template <class T>
std::vector<cd> Adjoint<T>::vjp(StateVector<T> &sv, const OpsList &opsl, const std::complex<T> *dy,
                                const std::vector<int64_t> &tp) {
    const auto &ops = opsl.ops;
    const size_t ntp = tp.size();
    std::vector<cd> out(ntp, cd{0, 0});
    if (ntp == 0) {
        return out;
    }
    for (size_t i = 1; i < ntp; i++) {
        PLGB_REQUIRE(tp[i] > tp[i - 1], "trainable parameter indices must be sorted and unique");
    }
    const size_t num_param_ops = opsl.num_par_ops();
    PLGB_REQUIRE(tp.back() < static_cast<int64_t>(num_param_ops), "trainable parameter index out of range");
    const int n = sv.num_qubits();
    StateVector<T> lambda(sv); // same stream
    StateVector<T> mu(n, lambda.stream());
    mu.update_data(dy, lambda.length());
    std::unique_ptr<StateVector<T>> mu_d;
    double *red = lambda.scratch_red();
    double *d_res = nullptr;
    d_res = static_cast<double *>(dev_alloc(2 * ntp * sizeof(double)));
    struct Guard {
        double *p;
        ~Guard() { dev_free(p); }
    } guard{d_res};
    std::vector<double> scale(ntp, 0.0);
    std::vector<char> on_device(ntp, 0);
    size_t tpn = ntp - 1;
    size_t curp = num_param_ops - 1;
    auto it = tp.rbegin();
    for (long op_idx = static_cast<long>(ops.size()) - 1; op_idx >= 0; op_idx--) {
        const auto &op = ops[static_cast<size_t>(op_idx)];
        PLGB_REQUIRE(op.params.size() <= 1, "The operation is not supported using the adjoint differentiation method");
        if (op.name == "StatePrep" || op.name == "BasisState") {
            continue;
        }
        if (it == tp.rend()) {
            break;
        }
        if (!op.params.empty()) {
            if (static_cast<int64_t>(curp) == *it) {
                const auto pg = pauli_generator(op, n);
                if (pg) {
                    // <mu| P G |lambda> by the transition kernel
                    reduce_pauli_transition<T>(lambda.stream(), mu.data(), lambda.data(), lambda.length(), pg->x,
                                               pg->yz, pg->ny4, pg->pmask, pg->pval, red, d_res + 2 * tpn);
                    on_device[tpn] = 1;
                    scale[tpn] = pg->scale * (op.inverse ? -1.0 : 1.0);
                } else {
                    if (!mu_d) {
                        mu_d = std::make_unique<StateVector<T>>(mu);
                    } else {
                        mu_d->copy_from(mu);
                    }
                    const double sc =
                        mu_d->apply_generator(op.name, op.cwires, op.cvals, op.wires) * (op.inverse ? -1.0 : 1.0);
                    const cd ip = mu_d->inner(lambda);
                    out[tpn] = cd{0.0, sc} * ip;
                }
                tpn--;
                ++it;
            }
            curp--;
        }
        lambda.apply_op(op, !op.inverse);
        mu.apply_op(op, !op.inverse);
    }
    std::vector<double> r(2 * ntp);
    cuda_check(cudaMemcpyAsync(r.data(), d_res, r.size() * sizeof(double), cudaMemcpyDeviceToHost, lambda.stream()),
               "D2H");
    lambda.synchronize();
    for (size_t k = 0; k < ntp; k++) {
        if (on_device[k]) {
            out[k] = cd{0.0, scale[k]} * cd{r[2 * k], r[2 * k + 1]};
        }
        out[k] = cd{static_cast<T>(out[k].real()), static_cast<T>(out[k].imag())};
    }
    return out;
}

template struct Adjoint<float>;
template struct Adjoint<double>;

} // namespace plgb
