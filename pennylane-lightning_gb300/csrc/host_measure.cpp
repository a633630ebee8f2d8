// Measurements and observables on the GPU state vector.
//
// Reference: pennylane_lightning/core/simulators/lightning_qubit/measurements/
// MeasurementsLQubit.hpp, MeasurementKernels.hpp (alias sampler :308-381),
// core/observables/Observables.hpp and LQ/observables/ObservablesLQubit.hpp.
//
// Difference in method (same results): an observable that is a weighted sum
// of Pauli words is not applied term by term to state copies (the
// reference's HamiltonianApplyInPlace, ObservablesLQubit.hpp:156-251, costs
// ~7 state sweeps and a state-sized buffer per term).  Terms are grouped by
// their bit-flip mask and each group is evaluated in ONE read of the state.
#include "host.hpp"

#include <algorithm>
#include <cmath>
#include <limits>
#include <map>
#include <sstream>
#include <stack>

namespace plgb {

std::vector<int64_t> ObsNode::all_wires() const {
    std::vector<int64_t> w;
    if (kind == Prod || kind == Ham) {
        for (auto &c : children) {
            auto cw = c->all_wires();
            for (auto x : cw) {
                if (std::find(w.begin(), w.end(), x) == w.end()) {
                    w.push_back(x);
                }
            }
        }
        return w;
    }
    return wires;
}

std::string ObsNode::repr() const {
    std::ostringstream os;
    switch (kind) {
    case Named:
        os << name << "[";
        for (size_t i = 0; i < wires.size(); i++) {
            os << (i ? ", " : "") << wires[i];
        }
        os << "]";
        break;
    case Herm:
        os << "Hermitian";
        break;
    case Prod:
        for (size_t i = 0; i < children.size(); i++) {
            os << (i ? " @ " : "") << children[i]->repr();
        }
        break;
    case Ham:
        os << "Hamiltonian: { 'coeffs' : [";
        for (size_t i = 0; i < coeffs.size(); i++) {
            os << (i ? ", " : "") << coeffs[i];
        }
        os << "], 'observables' : [";
        for (size_t i = 0; i < children.size(); i++) {
            os << (i ? ", " : "") << children[i]->repr();
        }
        os << "]}";
        break;
    case Sparse:
        os << "SparseHamiltonian";
        break;
    }
    return os.str();
}

// ---------------------------------------------------------------------------
// Pauli compilation
// ---------------------------------------------------------------------------
static bool pauli_factor(const std::string &name, char &c) {
    if (name == "PauliX") {
        c = 'X';
    } else if (name == "PauliY") {
        c = 'Y';
    } else if (name == "PauliZ") {
        c = 'Z';
    } else if (name == "Identity") {
        c = 'I';
    } else {
        return false;
    }
    return true;
}

// Accumulate obs (times `coeff`) into `out`; false if obs is not a Pauli sum.
static bool compile_rec(const ObsNode &o, int n, double coeff, PauliSum &out) {
    if (o.kind == ObsNode::Named) {
        char c;
        if (!pauli_factor(o.name, c) || o.wires.size() != 1) {
            return false;
        }
        PauliSum::Term t{coeff, 0, 0, 0};
        const int64_t w = o.wires[0];
        if (w < 0 || w >= n) {
            throw PLError("wire index out of range");
        }
        const u64 b = u64{1} << (n - 1 - w);
        if (c == 'X' || c == 'Y') {
            t.x |= b;
        }
        if (c == 'Y' || c == 'Z') {
            t.yz |= b;
        }
        if (c == 'Y') {
            t.ny4 = 1;
        }
        out.terms.push_back(t);
        return true;
    }
    if (o.kind == ObsNode::Prod) {
        PauliSum::Term t{coeff, 0, 0, 0};
        u64 used = 0;
        for (auto &ch : o.children) {
            PauliSum sub;
            if (!compile_rec(*ch, n, 1.0, sub) || sub.terms.size() != 1) {
                return false;
            }
            const auto &s = sub.terms[0];
            const u64 touched = s.x | s.yz;
            if (touched & used) {
                return false; // overlapping factors: leave to the general path
            }
            used |= touched;
            t.x |= s.x;
            t.yz |= s.yz;
            t.ny4 = (t.ny4 + s.ny4) & 3;
            t.c *= s.c;
        }
        out.terms.push_back(t);
        return true;
    }
    if (o.kind == ObsNode::Ham) {
        for (size_t i = 0; i < o.children.size(); i++) {
            if (!compile_rec(*o.children[i], n, coeff * o.coeffs[i], out)) {
                return false;
            }
        }
        return true;
    }
    return false;
}

bool compile_pauli(const ObsNode &obs, int n, PauliSum &out) {
    out.terms.clear();
    return compile_rec(obs, n, 1.0, out);
}

std::vector<PauliGroup> group_pauli(const PauliSum &ps) {
    std::map<u64, std::vector<const PauliSum::Term *>> by_x;
    for (auto &t : ps.terms) {
        by_x[t.x].push_back(&t);
    }
    std::vector<PauliGroup> groups;
    for (auto &kv : by_x) {
        for (size_t start = 0; start < kv.second.size(); start += kMaxTermsPerGroup) {
            PauliGroup g{};
            g.x = kv.first;
            g.hb = kv.first ? 63 - __builtin_clzll(kv.first) : 0;
            const size_t end = std::min(kv.second.size(), start + kMaxTermsPerGroup);
            g.nterms = static_cast<int>(end - start);
            for (size_t i = start; i < end; i++) {
                const auto *t = kv.second[i];
                g.t[i - start] = PauliTerm{t->c, t->yz, t->ny4, 0};
            }
            groups.push_back(g);
        }
    }
    return groups;
}

// Every flip-mask group of a Pauli sum applied in one sweep per chunk of at
// most kApplyMaxGroups groups / kApplyMaxTerms terms (launch_pauli_apply):
// dst = sum_t c_t P_t psi.  Coefficients are split into double-float pairs
// here.
template <class T>
void pauli_sum_into(const cx<T> *psi, StateVector<T> &dst, const std::vector<PauliGroup> &groups) {
    struct Chunk {
        size_t g0, g1, t0, t1;
    };
    std::vector<PauliGroupHdr> hdr;
    std::vector<PauliTermDF> terms;
    std::vector<Chunk> chunks;
    Chunk cur{0, 0, 0, 0};
    for (size_t g = 0; g < groups.size(); g++) {
        const auto &G = groups[g];
        const size_t nt = static_cast<size_t>(G.nterms);
        if (cur.g1 > cur.g0 && (cur.g1 - cur.g0 == static_cast<size_t>(kApplyMaxGroups) ||
                                terms.size() + nt - cur.t0 > static_cast<size_t>(kApplyMaxTerms))) {
            chunks.push_back(cur);
            cur = Chunk{g, g, terms.size(), terms.size()};
        }
        PauliGroupHdr h{};
        h.x = G.x;
        h.tbegin = static_cast<int>(terms.size() - cur.t0);
        for (size_t t = 0; t < nt; t++) {
            PauliTermDF tm{};
            tm.yz = G.t[t].yz;
            tm.chi = static_cast<float>(G.t[t].coeff);
            tm.clo = static_cast<float>(G.t[t].coeff - static_cast<double>(tm.chi));
            tm.ny4 = G.t[t].ny4;
            terms.push_back(tm);
        }
        h.tend = static_cast<int>(terms.size() - cur.t0);
        hdr.push_back(h);
        cur.g1 = g + 1;
        cur.t1 = terms.size();
    }
    if (cur.g1 > cur.g0) {
        chunks.push_back(cur);
    }
    PLGB_REQUIRE(!chunks.empty(), "Pauli sum without terms");
    auto bufs = dst.scratch().carve({hdr.size() * sizeof(PauliGroupHdr), terms.size() * sizeof(PauliTermDF)});
    auto *d_hdr = reinterpret_cast<PauliGroupHdr *>(bufs[0]);
    auto *d_terms = reinterpret_cast<PauliTermDF *>(bufs[1]);
    cuda_check(cudaMemcpyAsync(d_hdr, hdr.data(), hdr.size() * sizeof(PauliGroupHdr), cudaMemcpyHostToDevice,
                               dst.stream()), "H2D");
    cuda_check(cudaMemcpyAsync(d_terms, terms.data(), terms.size() * sizeof(PauliTermDF), cudaMemcpyHostToDevice,
                               dst.stream()), "H2D");
    for (size_t c = 0; c < chunks.size(); c++) {
        const auto &ch = chunks[c];
        launch_pauli_apply<T>(dst.stream(), psi, dst.data(), dst.length(), d_hdr + ch.g0,
                              static_cast<int>(ch.g1 - ch.g0), d_terms + ch.t0, static_cast<int>(ch.t1 - ch.t0),
                              c == 0);
    }
}

// ---------------------------------------------------------------------------
// Observable application (Observable::applyInPlace)
// ---------------------------------------------------------------------------
template <class T> void Measure<T>::apply_obs(StateVector<T> &sv, const ObsNode &o) {
    switch (o.kind) {
    case ObsNode::Named: // Observables.hpp:172-174
        sv.apply_operation(o.name, o.wires, false, {});
        return;
    case ObsNode::Herm: // Observables.hpp:286-288
        sv.apply_matrix(o.mat.data(), o.wires, false);
        return;
    case ObsNode::Prod: // Observables.hpp:414-418
        for (auto &c : o.children) {
            apply_obs(sv, *c);
        }
        return;
    case ObsNode::Ham: {
        PauliSum ps;
        StateVector<T> src(sv);
        if (compile_pauli(o, sv.num_qubits(), ps) && !ps.terms.empty()) {
            pauli_sum_into<T>(src.data(), sv, group_pauli(ps));
            sv.synchronize();
            return;
        }
        // general path: res = sum_t c_t (O_t psi)
        StateVector<T> tmp(sv);
        cuda_check(cudaMemsetAsync(sv.data(), 0, sv.length() * sizeof(cx<T>), sv.stream()), "memset");
        for (size_t t = 0; t < o.children.size(); t++) {
            tmp.copy_from(src);
            apply_obs(tmp, *o.children[t]);
            sv.scale_add(tmp, cd{o.coeffs[t], 0.0});
        }
        sv.synchronize();
        return;
    }
    case ObsNode::Sparse: { // ObservablesLQubit.hpp:426-435
        PLGB_REQUIRE(static_cast<int>(o.wires.size()) == sv.num_qubits(),
                     "SparseH wire count does not match state-vector size");
        StateVector<T> src(sv);
        const int64_t nnz = static_cast<int64_t>(o.sp_data.size());
        const auto bufs = sv.scratch().carve({o.sp_indptr.size() * sizeof(long long),
                                              static_cast<size_t>(nnz) * sizeof(long long),
                                              static_cast<size_t>(nnz) * sizeof(cx<T>)});
        long long *dip = reinterpret_cast<long long *>(bufs[0]);
        long long *dix = reinterpret_cast<long long *>(bufs[1]);
        cx<T> *dval = reinterpret_cast<cx<T> *>(bufs[2]);
        std::vector<cx<T>> vals(static_cast<size_t>(nnz));
        for (size_t i = 0; i < vals.size(); i++) {
            vals[i] = cx<T>{static_cast<T>(o.sp_data[i].real()), static_cast<T>(o.sp_data[i].imag())};
        }
        cuda_check(cudaMemcpyAsync(dip, o.sp_indptr.data(), o.sp_indptr.size() * sizeof(long long),
                                   cudaMemcpyHostToDevice, sv.stream()), "H2D");
        cuda_check(cudaMemcpyAsync(dix, o.sp_indices.data(), static_cast<size_t>(nnz) * sizeof(long long),
                                   cudaMemcpyHostToDevice, sv.stream()), "H2D");
        cuda_check(cudaMemcpyAsync(dval, vals.data(), vals.size() * sizeof(cx<T>), cudaMemcpyHostToDevice,
                                   sv.stream()), "H2D");
        launch_csr_apply<T>(sv.stream(), src.data(), sv.data(), sv.length(), dip, dix, dval);
        sv.synchronize();
        return;
    }
    }
}

template <class T>
void Measure<T>::apply_obs_into(const StateVector<T> &src, StateVector<T> &dst, const ObsNode &o) {
    PLGB_REQUIRE(src.num_qubits() == dst.num_qubits(), "observable: register sizes differ");
    PauliSum ps;
    if (o.kind != ObsNode::Sparse && o.kind != ObsNode::Herm && compile_pauli(o, src.num_qubits(), ps) &&
        !ps.terms.empty()) {
        src.synchronize();
        pauli_sum_into<T>(src.data(), dst, group_pauli(ps));
        dst.synchronize();
        return;
    }
    dst.copy_from(src);
    apply_obs(dst, o);
}

// ---------------------------------------------------------------------------
template <class T>
std::vector<double> Measure<T>::probs(StateVector<T> &sv, const std::vector<int64_t> &wires, bool all_wires) {
    // MeasurementsLQubit.hpp:90-163
    const int n = sv.num_qubits();
    if (!all_wires && wires.empty()) {
        return {1.0};
    }
    bool ordered = all_wires;
    if (!all_wires && static_cast<int>(wires.size()) == n) {
        ordered = true;
        for (size_t k = 0; k < wires.size(); k++) {
            ordered = ordered && wires[k] == static_cast<int64_t>(k);
        }
    }
    const u64 N = sv.length();
    if (ordered) {
        sv.scratch().ensure_mat(N * sizeof(T));
        T *dp = static_cast<T *>(sv.scratch().mat);
        launch_probs_all<T>(sv.stream(), sv.data(), N, dp);
        std::vector<T> hp(N);
        cuda_check(cudaMemcpyAsync(hp.data(), dp, N * sizeof(T), cudaMemcpyDeviceToHost, sv.stream()), "D2H");
        sv.synchronize();
        return std::vector<double>(hp.begin(), hp.end());
    }
    std::vector<int64_t> s(wires);
    std::sort(s.begin(), s.end());
    PLGB_REQUIRE(std::adjacent_find(s.begin(), s.end()) == s.end(), "wires must be unique");
    PLGB_REQUIRE(wires.size() <= 30, "marginal probabilities over at most 30 wires");
    // every entry summed in the reference's order in the working precision
    // (bit-exact, so seeded samples of a wire subset equal the reference's)
    const int k = static_cast<int>(wires.size());
    const size_t D = size_t{1} << k;
    MarginalGeom g{};
    g.k = k;
    u64 wmask = 0;
    for (int m = 0; m < k; m++) {
        g.wb[m] = sv.bit_of(wires[static_cast<size_t>(m)]);
        wmask |= u64{1} << g.wb[m];
    }
    g.cmask = (N - 1) & ~wmask;
    sv.scratch().ensure_mat(D * sizeof(T));
    T *dp = static_cast<T *>(sv.scratch().mat);
    launch_probs_marginal_serial<T>(sv.stream(), sv.data(), g, dp);
    std::vector<T> hp(D);
    cuda_check(cudaMemcpyAsync(hp.data(), dp, D * sizeof(T), cudaMemcpyDeviceToHost, sv.stream()), "D2H");
    sv.synchronize();
    return std::vector<double>(hp.begin(), hp.end());
}

template <class T>
double Measure<T>::expval_named(StateVector<T> &sv, const std::string &name, const std::vector<int64_t> &wires) {
    // MeasurementsLQubit.hpp:247-305
    if (name == "Identity") {
        return 1.0;
    }
    int kind = name == "PauliX" ? 0 : name == "PauliY" ? 1 : name == "PauliZ" ? 2 : name == "Hadamard" ? 3 : -1;
    PLGB_REQUIRE(kind >= 0, "Expval does not exist for named observable " + name);
    PLGB_REQUIRE(wires.size() == 1, "named expval takes one wire");
    const int b = sv.bit_of(wires[0]);
    reduce_expval1<T>(sv.stream(), sv.data(), sv.length(), b, kind, sv.scratch_red(),
                      sv.scratch_red() + 2 * kReduceBlocks);
    cuda_check(cudaMemcpyAsync(sv.host_out(), sv.scratch_red() + 2 * kReduceBlocks, sizeof(double),
                               cudaMemcpyDeviceToHost, sv.stream()), "D2H");
    sv.synchronize();
    return sv.host_out()[0];
}

template <class T>
double Measure<T>::expval_matrix(StateVector<T> &sv, const cd *mat, const std::vector<int64_t> &wires) {
    // MeasurementsLQubit.hpp:213-238
    const size_t k = wires.size();
    PLGB_REQUIRE(k >= 1, "Number of wires must be larger than 0");
    std::vector<int64_t> s(wires);
    std::sort(s.begin(), s.end());
    PLGB_REQUIRE(std::adjacent_find(s.begin(), s.end()) == s.end(), "wires must be unique");
    const size_t D = size_t{1} << k;
    if (k <= 5) {
        std::vector<int> tb;
        for (auto w : wires) {
            tb.push_back(sv.bit_of(w));
        }
        GroupGeom g{};
        std::vector<int> ins(tb);
        std::sort(ins.begin(), ins.end());
        g.nins = static_cast<int>(ins.size());
        for (int i = 0; i < g.nins; i++) {
            g.ins[i] = ins[static_cast<size_t>(i)];
        }
        g.ngroups = sv.length() >> g.nins;
        LocalOffsets lo{};
        for (size_t j = 0; j < D; j++) {
            u64 o = 0;
            for (size_t m = 0; m < k; m++) {
                if ((j >> (k - 1 - m)) & 1U) {
                    o |= u64{1} << tb[m];
                }
            }
            lo.off[j] = o;
        }
        std::vector<cx<T>> m(D * D);
        for (size_t i = 0; i < D * D; i++) {
            m[i] = cx<T>{static_cast<T>(mat[i].real()), static_cast<T>(mat[i].imag())};
        }
        sv.scratch().ensure_mat(D * D * sizeof(cx<T>));
        cx<T> *dm = static_cast<cx<T> *>(sv.scratch().mat);
        cuda_check(cudaMemcpyAsync(dm, m.data(), D * D * sizeof(cx<T>), cudaMemcpyHostToDevice, sv.stream()), "H2D");
        reduce_expval_matrix<T>(sv.stream(), sv.data(), g, static_cast<int>(k), lo, dm, sv.scratch_red(),
                                sv.scratch_red() + 2 * kReduceBlocks);
        cuda_check(cudaMemcpyAsync(sv.host_out(), sv.scratch_red() + 2 * kReduceBlocks, sizeof(double),
                                   cudaMemcpyDeviceToHost, sv.stream()), "D2H");
        sv.synchronize();
        return sv.host_out()[0];
    }
    StateVector<T> bra(sv);
    bra.apply_matrix(mat, wires, false);
    return bra.inner(sv).real();
}

template <class T>
double Measure<T>::expval_sparse(StateVector<T> &sv, const int64_t *indptr, int64_t nptr, const int64_t *indices,
                                 const cd *data, int64_t nnz) {
    // MeasurementsLQubit.hpp:322-338
    PLGB_REQUIRE(static_cast<u64>(nptr - 1) == sv.length(), "Statevector and Hamiltonian have incompatible sizes.");
    const auto bufs = sv.scratch().carve({static_cast<size_t>(nptr) * sizeof(long long),
                                          static_cast<size_t>(nnz) * sizeof(long long),
                                          static_cast<size_t>(nnz) * sizeof(cx<T>)});
    long long *dip = reinterpret_cast<long long *>(bufs[0]);
    long long *dix = reinterpret_cast<long long *>(bufs[1]);
    cx<T> *dval = reinterpret_cast<cx<T> *>(bufs[2]);
    std::vector<cx<T>> vals(static_cast<size_t>(nnz));
    for (size_t i = 0; i < vals.size(); i++) {
        vals[i] = cx<T>{static_cast<T>(data[i].real()), static_cast<T>(data[i].imag())};
    }
    cuda_check(cudaMemcpyAsync(dip, indptr, static_cast<size_t>(nptr) * sizeof(long long), cudaMemcpyHostToDevice,
                               sv.stream()), "H2D");
    cuda_check(cudaMemcpyAsync(dix, indices, static_cast<size_t>(nnz) * sizeof(long long), cudaMemcpyHostToDevice,
                               sv.stream()), "H2D");
    cuda_check(cudaMemcpyAsync(dval, vals.data(), vals.size() * sizeof(cx<T>), cudaMemcpyHostToDevice, sv.stream()),
               "H2D");
    reduce_expval_csr<T>(sv.stream(), sv.data(), sv.length(), dip, dix, dval, sv.scratch_red(),
                         sv.scratch_red() + 2 * kReduceBlocks);
    cuda_check(cudaMemcpyAsync(sv.host_out(), sv.scratch_red() + 2 * kReduceBlocks, sizeof(double),
                               cudaMemcpyDeviceToHost, sv.stream()), "D2H");
    sv.synchronize();
    return sv.host_out()[0];
}

template <class T>
double Measure<T>::var_sparse(StateVector<T> &sv, const int64_t *indptr, int64_t nptr, const int64_t *indices,
                              const cd *data, int64_t nnz) {
    // MeasurementsLQubit.hpp:615-636
    ObsNode o;
    o.kind = ObsNode::Sparse;
    o.wires.resize(static_cast<size_t>(sv.num_qubits()));
    for (size_t i = 0; i < o.wires.size(); i++) {
        o.wires[i] = static_cast<int64_t>(i);
    }
    o.sp_indptr.assign(indptr, indptr + nptr);
    o.sp_indices.assign(indices, indices + nnz);
    o.sp_data.assign(data, data + nnz);
    return var_obs(sv, o);
}

// <psi| sum_t c_t P_t |psi> by passes (launch_pauli_pass): the words are
// packed, in order of their flip masks, into passes of at most kPassTerms
// words whose flip bits together leave at least four of the tile's local
// bits for the lowest index bits (coalesced tile loads); one read of the
// state per pass.  Each word's sum is scaled by its coefficient on the host
// and added in word order (deterministic).
template <class T> double pauli_expval_passes(StateVector<T> &sv, const PauliSum &ps) {
    const int n = sv.num_qubits();
    const int t = std::min(n, kPassMaxTileBits);
    struct W {
        double coef;
        const PauliSum::Term *term;
    };
    std::vector<W> words;
    PauliSum wide; // words with more flip bits than a tile holds: one sweep per flip mask
    for (const auto &tm : ps.terms) {
        if (__builtin_popcountll(tm.x) > t) {
            wide.terms.push_back(tm);
            continue;
        }
        const int par = __builtin_popcountll(tm.x & tm.yz) & 1;
        const bool odd = (tm.ny4 & 1) != 0;
        if (tm.x != 0 && par != (odd ? 1 : 0)) {
            continue; // purely imaginary on every pair: no real part
        }
        double coef = tm.c;
        if (tm.x != 0) {
            coef = (tm.ny4 == 0 || tm.ny4 == 1) ? 2.0 * tm.c : -2.0 * tm.c;
        } else if (tm.ny4 != 0) {
            coef = tm.ny4 == 2 ? -tm.c : 0.0; // i^ny on a diagonal word: real part only
        }
        if (coef != 0.0) {
            words.push_back({coef, &tm});
        }
    }
    // Passes: groups of at most kPassTerms words whose flip bits together
    // leave the tile at least its 2 lowest other bits (4 consecutive
    // amplitudes per group of copies, whole 32-byte sectors).  Up to 512 words: each pass starts from
    // the open word with the most flip bits and adds the words that widen its
    // flip set least (diagonal words widen nothing); larger sums are grouped
    // in flip-mask order.
    std::vector<std::pair<size_t, size_t>> passes; // [begin, end) of words
    const int lim = std::max(1, t - 2);
    if (words.size() <= 512) {
        std::vector<W> ordered;
        ordered.reserve(words.size());
        std::vector<char> used(words.size(), 0);
        size_t left = words.size();
        while (left > 0) {
            size_t seed = words.size();
            for (size_t i = 0; i < words.size(); i++) {
                if (!used[i] && (seed == words.size() || __builtin_popcountll(words[i].term->x) >
                                                             __builtin_popcountll(words[seed].term->x))) {
                    seed = i;
                }
            }
            const size_t b0 = ordered.size();
            u64 U = words[seed].term->x;
            const int cap = std::max(lim, __builtin_popcountll(U));
            used[seed] = 1;
            ordered.push_back(words[seed]);
            left--;
            while (left > 0 && ordered.size() - b0 < static_cast<size_t>(kPassTerms)) {
                size_t best = words.size();
                int best_add = 64;
                for (size_t i = 0; i < words.size(); i++) {
                    if (used[i]) {
                        continue;
                    }
                    const u64 nu = U | words[i].term->x;
                    const int add = __builtin_popcountll(nu) - __builtin_popcountll(U);
                    if (__builtin_popcountll(nu) <= cap && add < best_add) {
                        best = i;
                        best_add = add;
                    }
                }
                if (best == words.size()) {
                    break;
                }
                used[best] = 1;
                U |= words[best].term->x;
                ordered.push_back(words[best]);
                left--;
            }
            passes.emplace_back(b0, ordered.size());
        }
        words.swap(ordered);
    } else {
        std::stable_sort(words.begin(), words.end(), [](const W &a, const W &b) { return a.term->x < b.term->x; });
        size_t b = 0;
        u64 U = 0;
        for (size_t i = 0; i < words.size(); i++) {
            const u64 nu = U | words[i].term->x;
            const int cap = std::max(lim, __builtin_popcountll(words[i].term->x));
            if (i > b && (i - b == static_cast<size_t>(kPassTerms) || __builtin_popcountll(nu) > cap)) {
                passes.emplace_back(b, i);
                b = i;
                U = words[i].term->x;
            } else {
                U = nu;
            }
        }
        if (b < words.size()) {
            passes.emplace_back(b, words.size());
        }
    }
    const std::vector<PauliGroup> wide_groups = group_pauli(wide);
    if (passes.empty() && wide_groups.empty()) {
        return 0.0;
    }
    const u64 N = sv.length();
    const size_t max_grid = static_cast<size_t>(LaunchGeom::sm_count()) * 8;
    const size_t nout = passes.size() * kPassTerms + wide_groups.size();
    const auto bufs = sv.scratch().carve({std::max<size_t>(max_grid * kPassTerms, kReduceBlocks) * sizeof(double),
                                         nout * sizeof(double)});
    double *partials = reinterpret_cast<double *>(bufs[0]);
    double *outs = reinterpret_cast<double *>(bufs[1]);
    for (size_t pi = 0; pi < passes.size(); pi++) {
        PauliPass pp{};
        pp.t = t;
        u64 U = 0;
        for (size_t i = passes[pi].first; i < passes[pi].second; i++) {
            U |= words[i].term->x;
        }
        u64 L = U;
        for (int b = 0; b < n && __builtin_popcountll(L) < t; b++) {
            L |= u64{1} << b;
        }
        int nl = 0;
        for (int b = 0; b < n; b++) {
            if ((L >> b) & 1u) {
                pp.lbit[nl++] = b;
            } else {
                pp.glob[pp.nglob++] = b;
            }
        }
        pp.ntiles = N >> t;
        auto gather = [&](u64 m) {
            unsigned out = 0;
            for (int q = 0; q < t; q++) {
                if ((m >> pp.lbit[q]) & 1u) {
                    out |= 1u << q;
                }
            }
            return out;
        };
        pp.nterms = static_cast<int>(passes[pi].second - passes[pi].first);
        for (int w = 0; w < pp.nterms; w++) {
            const auto *tm = words[passes[pi].first + static_cast<size_t>(w)].term;
            PauliPassTerm &pt = pp.term[w];
            pt.yz = tm->yz;
            pt.x = gather(tm->x);
            pt.yzl = gather(tm->yz);
            pt.hb = pt.x ? 31 - __builtin_clz(pt.x) : 0;
            pt.im = (tm->ny4 & 1) != 0 ? 1 : 0;
            if (t == kPassMaxTileBits) {
                const unsigned lo = (1u << pt.hb) - 1u;
                pt.srm = 0;
                for (unsigned r = 0; r < (pt.x ? 4u : 8u); r++) {
                    const unsigned k = r << 9;
                    const unsigned j = pt.x ? (((k >> pt.hb) << (pt.hb + 1)) | (k & lo)) : k;
                    if (pt.x) {
                        pt.jr[r] = static_cast<unsigned short>(j);
                    }
                    pt.srm |= (static_cast<unsigned>(__builtin_popcount(j & pt.yzl)) & 1u) << r;
                }
            }
        }
        const int grid = launch_pauli_pass<T>(sv.stream(), sv.data(), pp, partials);
        launch_finalize_pass(sv.stream(), partials, grid, outs + pi * kPassTerms);
    }
    for (size_t g = 0; g < wide_groups.size(); g++) {
        reduce_pauli_group<T>(sv.stream(), sv.data(), N, wide_groups[g], partials,
                              outs + passes.size() * kPassTerms + g);
    }
    std::vector<double> h(nout);
    cuda_check(cudaMemcpyAsync(h.data(), outs, h.size() * sizeof(double), cudaMemcpyDeviceToHost, sv.stream()),
               "D2H");
    sv.synchronize();
    double total = 0.0;
    for (size_t pi = 0; pi < passes.size(); pi++) {
        for (size_t i = passes[pi].first; i < passes[pi].second; i++) {
            total += words[i].coef * h[pi * kPassTerms + (i - passes[pi].first)];
        }
    }
    for (size_t g = 0; g < wide_groups.size(); g++) {
        total += h[passes.size() * kPassTerms + g]; // coefficients applied in the sweep
    }
    return total;
}

template <class T> double Measure<T>::expval_obs(StateVector<T> &sv, const ObsNode &obs) {
    // MeasurementsLQubit.hpp:372-394
    PauliSum ps;
    if (compile_pauli(obs, sv.num_qubits(), ps)) {
        return pauli_expval_passes(sv, ps);
    }
    if (obs.kind == ObsNode::Named && obs.wires.size() == 1 &&
        (obs.name == "Hadamard" || obs.name == "Identity")) {
        return expval_named(sv, obs.name, obs.wires);
    }
    if (obs.kind == ObsNode::Herm && obs.wires.size() <= 5) {
        return expval_matrix(sv, obs.mat.data(), obs.wires);
    }
    StateVector<T> bra(sv);
    apply_obs(bra, obs);
    return bra.inner(sv).real();
}

template <class T> double Measure<T>::var_obs(StateVector<T> &sv, const ObsNode &obs) {
    // MeasurementsLQubit.hpp:420-442 calculateObsVar
    StateVector<T> bra(sv);
    apply_obs(bra, obs);
    const double ms = bra.inner(bra).real();
    const double sm = bra.inner(sv).real();
    return static_cast<double>(static_cast<T>(ms) - static_cast<T>(std::pow(static_cast<T>(sm), 2)));
}

// ---------------------------------------------------------------------------
// Sampling: the alias method of MeasurementKernels.hpp:308-381 restated
// (DiscreteRandomVariable), driven by std::mt19937 seeded as
// MeasurementsBase::setSeed does, over probabilities computed on the GPU.
// The draw sequence must match the reference for exact integer parity.
// ---------------------------------------------------------------------------
namespace {
template <class T> struct AliasTable {
    static constexpr size_t none = std::numeric_limits<size_t>::max();
    std::mt19937 &gen;
    size_t n;
    std::vector<std::pair<double, size_t>> buckets;
    mutable std::uniform_real_distribution<T> dist{0.0, 1.0};
    AliasTable(std::mt19937 &g, const std::vector<T> &p) : gen(g), n(p.size()), buckets(p.size(), {0.0, none}) {
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
            const size_t i = over.top();
            over.pop();
            const size_t j = under.top();
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
    size_t draw() const {
        const auto idx = static_cast<size_t>(dist(gen) * n);
        if (dist(gen) >= buckets[idx].first && buckets[idx].second != none) {
            return buckets[idx].second;
        }
        return idx;
    }
};
} // namespace

template <class T>
std::vector<int64_t> Measure<T>::samples(StateVector<T> &sv, const std::vector<int64_t> &wires, int64_t shots,
                                         uint64_t seed) {
    // MeasurementsLQubit.hpp:646-679
    PLGB_REQUIRE(shots >= 0, "number of shots must be non-negative");
    const auto pd = probs(sv, wires, false);
    std::vector<T> p(pd.size());
    for (size_t i = 0; i < p.size(); i++) {
        p[i] = static_cast<T>(pd[i]);
    }
    std::mt19937 rng;
    rng.seed(static_cast<std::mt19937::result_type>(seed));
    AliasTable<T> drv(rng, p);
    const size_t nw = wires.size();
    std::vector<int64_t> out(static_cast<size_t>(shots) * nw);
    for (int64_t s = 0; s < shots; s++) {
        const size_t idx = drv.draw();
        for (size_t j = 0; j < nw; j++) {
            out[static_cast<size_t>(s) * nw + (nw - 1 - j)] = static_cast<int64_t>((idx >> j) & 1U);
        }
    }
    return out;
}

// Metropolis-Hastings sampling (generate_mcmc_samples): MeasurementsLQubit.hpp
// :551-594 generate_samples_metropolis, :740-770 metropolis_step, transition
// kernels TransitionKernels.hpp:37-163.  The reference's kernel_factory
// builds the non-zero-random kernel for the type Local (every name but
// "NonZeroRandom") and the local bit-flip kernel for NonZeroRandom; this
// keeps that mapping.  The random numbers do not depend on the state, so they
// are drawn here from std::mt19937 in the reference's order (proposal draws,
// then the acceptance draw, per step) and the device runs the chain
// (kernels_mcmc.cu).
template <class T>
std::vector<int64_t> Measure<T>::mcmc_samples(StateVector<T> &sv, const std::string &kernel, int64_t burnin,
                                              int64_t shots, uint64_t seed) {
    PLGB_REQUIRE(burnin >= 0 && shots >= 0, "MCMC sampling: burn-in and shots must be non-negative");
    const int n = sv.num_qubits();
    const u64 N = sv.length();
    const u64 steps = static_cast<u64>(burnin) + static_cast<u64>(shots);
    std::vector<int64_t> out(static_cast<size_t>(shots) * static_cast<size_t>(n));
    std::mt19937 rng;
    rng.seed(static_cast<std::mt19937::result_type>(seed));
    std::uniform_real_distribution<T> distrib(0.0, 1.0);
    const bool nonzero_kernel = kernel != "NonZeroRandom";
    std::vector<T> ran(steps);
    cudaStream_t st = sv.stream();
    const T eps = std::numeric_limits<T>::epsilon();
    if (nonzero_kernel) {
        const u64 nchunks = (N + kMcmcChunk - 1) / kMcmcChunk;
        auto b0 = sv.scratch().carve({nchunks * sizeof(unsigned)});
        launch_nz_count<T>(st, sv.data(), N, eps, nchunks, reinterpret_cast<unsigned *>(b0[0]));
        std::vector<unsigned> counts(nchunks);
        cuda_check(cudaMemcpyAsync(counts.data(), b0[0], nchunks * sizeof(unsigned), cudaMemcpyDeviceToHost, st),
                   "D2H");
        sv.synchronize();
        std::vector<u64> prefix(nchunks + 1, 0);
        for (u64 c = 0; c < nchunks; c++) {
            prefix[c + 1] = prefix[c] + counts[c];
        }
        const u64 nnz = prefix[nchunks];
        PLGB_REQUIRE(nnz > 0, "MCMC sampling: the state has no non-zero amplitude");
        std::uniform_int_distribution<size_t> d_nz(0, static_cast<size_t>(nnz - 1));
        std::vector<u64> rank(steps);
        for (u64 s = 0; s < steps; s++) {
            rank[s] = d_nz(rng);
            ran[s] = distrib(rng);
        }
        const size_t nout = static_cast<size_t>(shots) * static_cast<size_t>(n);
        auto b = sv.scratch().carve({(nchunks + 1) * sizeof(u64), steps * sizeof(u64), steps * sizeof(T),
                                     steps * sizeof(u64), steps * sizeof(T), static_cast<size_t>(shots) * sizeof(u64),
                                     nout * sizeof(long long)});
        u64 *d_prefix = reinterpret_cast<u64 *>(b[0]);
        u64 *d_rank = reinterpret_cast<u64 *>(b[1]);
        T *d_ran = reinterpret_cast<T *>(b[2]);
        u64 *d_tidx = reinterpret_cast<u64 *>(b[3]);
        T *d_tplog = reinterpret_cast<T *>(b[4]);
        u64 *d_idx = reinterpret_cast<u64 *>(b[5]);
        long long *d_out = reinterpret_cast<long long *>(b[6]);
        cuda_check(cudaMemcpyAsync(d_prefix, prefix.data(), prefix.size() * sizeof(u64), cudaMemcpyHostToDevice, st),
                   "H2D");
        if (steps > 0) {
            cuda_check(cudaMemcpyAsync(d_rank, rank.data(), steps * sizeof(u64), cudaMemcpyHostToDevice, st), "H2D");
            cuda_check(cudaMemcpyAsync(d_ran, ran.data(), steps * sizeof(T), cudaMemcpyHostToDevice, st), "H2D");
            launch_nz_select<T>(st, sv.data(), N, eps, d_prefix, nchunks, d_rank, steps, d_tidx, d_tplog);
            launch_mcmc_chain_nz<T>(st, sv.data(), d_tidx, d_tplog, d_ran, steps, static_cast<u64>(burnin), d_idx);
        }
        launch_index_bits(st, d_idx, static_cast<u64>(shots), n, d_out);
        if (nout > 0) {
            cuda_check(cudaMemcpyAsync(out.data(), d_out, nout * sizeof(long long), cudaMemcpyDeviceToHost, st), "D2H");
        }
        sv.synchronize();
        return out;
    }
    // the reference tests bits of the index truncated to 32 bits
    PLGB_REQUIRE(n <= 32, "MCMC sampling with the local kernel: at most 32 qubits");
    std::uniform_int_distribution<size_t> dist_site(0, static_cast<size_t>(n - 1)), dist_bin(0, 1);
    std::vector<unsigned char> site(steps), value(steps);
    for (u64 s = 0; s < steps; s++) {
        site[s] = static_cast<unsigned char>(dist_site(rng));
        value[s] = static_cast<unsigned char>(dist_bin(rng));
        ran[s] = distrib(rng);
    }
    const size_t nout = static_cast<size_t>(shots) * static_cast<size_t>(n);
    auto b = sv.scratch().carve({steps, steps, steps * sizeof(T), static_cast<size_t>(shots) * sizeof(u64),
                                 nout * sizeof(long long)});
    auto *d_site = reinterpret_cast<unsigned char *>(b[0]);
    auto *d_value = reinterpret_cast<unsigned char *>(b[1]);
    T *d_ran = reinterpret_cast<T *>(b[2]);
    u64 *d_idx = reinterpret_cast<u64 *>(b[3]);
    long long *d_out = reinterpret_cast<long long *>(b[4]);
    if (steps > 0) {
        cuda_check(cudaMemcpyAsync(d_site, site.data(), steps, cudaMemcpyHostToDevice, st), "H2D");
        cuda_check(cudaMemcpyAsync(d_value, value.data(), steps, cudaMemcpyHostToDevice, st), "H2D");
        cuda_check(cudaMemcpyAsync(d_ran, ran.data(), steps * sizeof(T), cudaMemcpyHostToDevice, st), "H2D");
        launch_mcmc_chain_local<T>(st, sv.data(), d_site, d_value, d_ran, steps, static_cast<u64>(burnin), d_idx);
    }
    launch_index_bits(st, d_idx, static_cast<u64>(shots), n, d_out);
    if (nout > 0) {
        cuda_check(cudaMemcpyAsync(out.data(), d_out, nout * sizeof(long long), cudaMemcpyDeviceToHost, st), "D2H");
    }
    sv.synchronize();
    return out;
}

template struct Measure<float>;
template struct Measure<double>;

} // namespace plgb
