// Dense-block fusion: a gate sequence merged into dense 2^k x 2^k blocks on
// at most k wires, each applied as one dense kernel (one HBM pass).
//
// Greedy, in program order.  Open blocks act on disjoint bit sets (so they
// commute).  A gate whose touched bits, together with those of the open
// blocks it meets, fit in k bits joins them: the blocks are joined by a
// tensor product, widened by identities to the gate's other bits, and the
// gate's action is multiplied in on the left.  Otherwise the blocks it meets
// are emitted and the gate opens a new block.  Primitives with no dense form
// here (Pauli rotations, projections) close the blocks they meet and pass
// through unchanged; global scalings multiply into the next block.
// Matrices are composed in complex128 and rounded to the register's
// precision once per block.
//
// A block's local index bit q is bit bits[q] of the amplitude index (bits
// ascending); it is emitted with targets in descending order (first target
// = most significant local bit, the DenseK convention).  For complex64,
// blocks on four or more bits are widened to six bits with identities so
// that they run on the tensor-core kernel (kernels_tc.cu).
#include "host.hpp"

#include <algorithm>
#include <complex>
#include <type_traits>
#include <vector>

namespace plgb {

namespace {

using C2 = std::complex<double>;

struct Block {
    std::vector<int> bits; // ascending
    std::vector<C2> m;     // row-major, dim 2^bits.size()
    size_t order{0};       // creation order (emission order among open blocks)
};

// local index (over `bits`) of the global bits set in `mask`
unsigned local_mask(const std::vector<int> &bits, u64 mask) {
    unsigned out = 0;
    for (size_t q = 0; q < bits.size(); q++) {
        if ((mask >> bits[q]) & 1u) {
            out |= 1u << q;
        }
    }
    return out;
}

// position of global bit b in `bits`
int local_index(const std::vector<int> &bits, int b) {
    for (size_t q = 0; q < bits.size(); q++) {
        if (bits[q] == b) {
            return static_cast<int>(q);
        }
    }
    throw PLError("dense-block fusion: bit outside the block");
}

template <class T> C2 c2(cx<T> v) { return C2(static_cast<double>(v.x), static_cast<double>(v.y)); }

// The 2x2 matrix of a Pair primitive in its mode (kernels_gates.cu k_1q).
template <class T> void pair_matrix(const Prim<T> &p, C2 (&m)[4]) {
    switch (p.mode) {
    case M1_DENSE: m[0] = c2(p.m[0]); m[1] = c2(p.m[1]); m[2] = c2(p.m[2]); m[3] = c2(p.m[3]); break;
    case M1_REAL: m[0] = p.m[0].x; m[1] = p.m[1].x; m[2] = p.m[2].x; m[3] = p.m[3].x; break;
    case M1_RXF:
        m[0] = m[3] = p.m[0].x;
        m[1] = m[2] = C2(0, p.m[1].y);
        break;
    case M1_DIAG: m[0] = c2(p.m[0]); m[1] = m[2] = 0; m[3] = c2(p.m[3]); break;
    case M1_PHASE1: m[0] = 1; m[1] = m[2] = 0; m[3] = c2(p.m[3]); break;
    case M1_SWAP: m[0] = m[3] = 0; m[1] = m[2] = 1; break;
    case M1_ANTI: m[0] = m[3] = 0; m[1] = c2(p.m[1]); m[2] = c2(p.m[2]); break;
    default: m[0] = 1; m[1] = m[2] = 0; m[3] = -1; break; // M1_NEG1
    }
}

// whether the primitive has a dense form here
template <class T> bool densifiable(const Prim<T> &p) {
    switch (p.kind) {
    case Prim<T>::Pair:
    case Prim<T>::Dense2:
    case Prim<T>::DenseK:
    case Prim<T>::DiagK:
    case Prim<T>::Parity:
    case Prim<T>::Scale: return true;
    default: return false;
    }
}

// Apply primitive p to the local vector v (dimension 2^bits.size(); the
// primitive's touched bits are among `bits`).
template <class T> void apply_local(const Prim<T> &p, const std::vector<int> &bits, std::vector<C2> &v) {
    const unsigned D = static_cast<unsigned>(v.size());
    const unsigned cm = local_mask(bits, p.cmask), cv = local_mask(bits, p.cval);
    switch (p.kind) {
    case Prim<T>::Pair: {
        C2 m[4];
        pair_matrix(p, m);
        u64 tm = 0;
        for (int b : p.tbits) {
            tm |= u64{1} << b;
        }
        const unsigned lt = local_mask(bits, tm), l0 = local_mask(bits, p.o0), l1 = local_mask(bits, p.o1);
        for (unsigned j = 0; j < D; j++) {
            if ((j & lt) != 0 || (j & cm) != cv) {
                continue;
            }
            const C2 a = v[j | l0], b = v[j | l1];
            v[j | l0] = m[0] * a + m[1] * b;
            v[j | l1] = m[2] * a + m[3] * b;
        }
        return;
    }
    case Prim<T>::Dense2:
    case Prim<T>::DenseK: {
        const size_t k = p.tbits.size();
        const unsigned Dk = 1u << k;
        std::vector<unsigned> off(Dk);
        u64 tm = 0;
        for (int b : p.tbits) {
            tm |= u64{1} << b;
        }
        for (unsigned j = 0; j < Dk; j++) {
            u64 o = 0;
            for (size_t b = 0; b < k; b++) {
                if ((j >> (k - 1 - b)) & 1u) {
                    o |= u64{1} << p.tbits[b];
                }
            }
            off[j] = local_mask(bits, o);
        }
        const unsigned lt = local_mask(bits, tm);
        std::vector<C2> in(Dk);
        for (unsigned j = 0; j < D; j++) {
            if ((j & lt) != 0 || (j & cm) != cv) {
                continue;
            }
            for (unsigned c = 0; c < Dk; c++) {
                in[c] = v[j | off[c]];
            }
            for (unsigned r = 0; r < Dk; r++) {
                C2 acc = 0;
                for (unsigned c = 0; c < Dk; c++) {
                    acc += c2(p.m[r * Dk + c]) * in[c];
                }
                v[j | off[r]] = acc;
            }
        }
        return;
    }
    case Prim<T>::DiagK: {
        const size_t k = p.tbits.size();
        std::vector<int> pos(k);
        for (size_t b = 0; b < k; b++) {
            pos[b] = local_index(bits, p.tbits[b]);
        }
        for (unsigned j = 0; j < D; j++) {
            if ((j & cm) != cv) {
                continue;
            }
            unsigned t = 0;
            for (size_t b = 0; b < k; b++) {
                t = (t << 1) | ((j >> pos[b]) & 1u);
            }
            v[j] *= c2(p.m[t]);
        }
        return;
    }
    case Prim<T>::Parity: {
        const unsigned pm = local_mask(bits, p.pmask);
        for (unsigned j = 0; j < D; j++) {
            if ((j & cm) != cv) {
                if (p.zero_outside) {
                    v[j] = 0;
                }
                continue;
            }
            v[j] *= (__builtin_popcount(j & pm) & 1) ? c2(p.m[1]) : c2(p.m[0]);
        }
        return;
    }
    case Prim<T>::Scale: {
        for (unsigned j = 0; j < D; j++) {
            if ((j & cm) == cv) {
                v[j] *= c2(p.m[0]);
            }
        }
        return;
    }
    default: throw PLError("dense-block fusion: primitive without a dense form");
    }
}

// M <- widened to `nb` (a superset of blk.bits), identity on the new bits
void widen(Block &blk, const std::vector<int> &nb) {
    if (nb == blk.bits) {
        return;
    }
    const unsigned Dn = 1u << nb.size(), Do = 1u << blk.bits.size();
    std::vector<unsigned> pos(blk.bits.size());
    for (size_t q = 0; q < blk.bits.size(); q++) {
        pos[q] = static_cast<unsigned>(local_index(nb, blk.bits[q]));
    }
    unsigned oldmask = 0;
    for (unsigned p : pos) {
        oldmask |= 1u << p;
    }
    auto project = [&](unsigned j) { // new local index -> old local index
        unsigned o = 0;
        for (size_t q = 0; q < pos.size(); q++) {
            o |= ((j >> pos[q]) & 1u) << q;
        }
        return o;
    };
    std::vector<C2> m(static_cast<size_t>(Dn) * Dn, C2(0));
    for (unsigned r = 0; r < Dn; r++) {
        for (unsigned c = 0; c < Dn; c++) {
            if ((r & ~oldmask) != (c & ~oldmask)) {
                continue; // identity on the new bits
            }
            m[static_cast<size_t>(r) * Dn + c] = blk.m[static_cast<size_t>(project(r)) * Do + project(c)];
        }
    }
    blk.bits = nb;
    blk.m.swap(m);
}

// A <- A (x) B (disjoint bit sets)
void join(Block &a, const Block &b) {
    std::vector<int> nb(a.bits);
    nb.insert(nb.end(), b.bits.begin(), b.bits.end());
    std::sort(nb.begin(), nb.end());
    Block bw = b;
    widen(a, nb);
    widen(bw, nb);
    const unsigned D = 1u << nb.size();
    std::vector<C2> m(static_cast<size_t>(D) * D, C2(0));
    for (unsigned r = 0; r < D; r++) {
        for (unsigned k = 0; k < D; k++) {
            const C2 x = a.m[static_cast<size_t>(r) * D + k];
            if (x == C2(0)) {
                continue;
            }
            for (unsigned c = 0; c < D; c++) {
                m[static_cast<size_t>(r) * D + c] += x * bw.m[static_cast<size_t>(k) * D + c];
            }
        }
    }
    a.m.swap(m);
    a.order = std::min(a.order, b.order);
}

template <class T> Prim<T> emit_block(const Block &b, int n, int min_tc_bits) {
    Block blk = b;
    // complex64 blocks of four or more bits: widened to six for the
    // tensor-core kernel
    if (std::is_same_v<T, float> && static_cast<int>(blk.bits.size()) >= min_tc_bits && blk.bits.size() < 6 &&
        n >= 12) {
        std::vector<int> nb(blk.bits);
        for (int q = 0; q < n && nb.size() < 6; q++) {
            if (std::find(nb.begin(), nb.end(), q) == nb.end()) {
                nb.push_back(q);
            }
        }
        std::sort(nb.begin(), nb.end());
        widen(blk, nb);
    }
    const size_t k = blk.bits.size();
    const unsigned D = 1u << k;
    Prim<T> p;
    p.tbits.assign(blk.bits.rbegin(), blk.bits.rend()); // first target = most significant local bit
    p.m.resize(static_cast<size_t>(D) * D);
    for (size_t i = 0; i < p.m.size(); i++) {
        p.m[i] = cx<T>{static_cast<T>(blk.m[i].real()), static_cast<T>(blk.m[i].imag())};
    }
    if (k == 1) {
        p.kind = Prim<T>::Pair;
        p.mode = M1_DENSE;
        p.o0 = 0;
        p.o1 = u64{1} << blk.bits[0];
    } else {
        p.kind = k == 2 ? Prim<T>::Dense2 : Prim<T>::DenseK;
    }
    return p;
}

} // namespace

template <class T> std::vector<Prim<T>> fuse_dense_blocks(const std::vector<Prim<T>> &prims, int n, int kmax) {
    PLGB_REQUIRE(kmax >= 1 && kmax <= 6, "dense-block fusion: block width must be 1 to 6 wires");
    constexpr int kMinTcBits = 4;
    std::vector<Block> open;
    std::vector<Prim<T>> out;
    size_t counter = 0;
    C2 scalar(1.0);
    auto remove = [&](const std::vector<size_t> &idx) {
        std::vector<Block> keep;
        for (size_t i = 0; i < open.size(); i++) {
            if (std::find(idx.begin(), idx.end(), i) == idx.end()) {
                keep.push_back(std::move(open[i]));
            }
        }
        open.swap(keep);
    };
    auto emit_blocks = [&](std::vector<size_t> idx) {
        std::sort(idx.begin(), idx.end(), [&](size_t a, size_t b) { return open[a].order < open[b].order; });
        for (size_t i : idx) {
            Block &b = open[i];
            if (scalar != C2(1.0)) {
                for (auto &x : b.m) {
                    x *= scalar;
                }
                scalar = 1.0;
            }
            out.push_back(emit_block<T>(b, n, kMinTcBits));
        }
        remove(idx);
    };
    for (const Prim<T> &p : prims) {
        const u64 q = p.touched();
        if (p.kind == Prim<T>::Scale && p.cmask == 0) {
            scalar *= c2(p.m[0]); // a global phase: into the next block emitted
            continue;
        }
        std::vector<size_t> meet;
        u64 uni = q;
        for (size_t i = 0; i < open.size(); i++) {
            u64 bm = 0;
            for (int b : open[i].bits) {
                bm |= u64{1} << b;
            }
            if (bm & q) {
                meet.push_back(i);
                uni |= bm;
            }
        }
        if (!densifiable(p) || __builtin_popcountll(q) > kmax) {
            emit_blocks(meet);
            out.push_back(p);
            continue;
        }
        if (__builtin_popcountll(uni) > kmax) {
            emit_blocks(meet);
            meet.clear();
            uni = q;
        }
        // join the met blocks and widen to the gate's bits
        Block nb;
        nb.order = counter++;
        nb.m.assign(1, C2(1.0));
        for (size_t i : meet) {
            join(nb, open[i]);
        }
        std::vector<int> bits;
        for (u64 r = uni; r; r &= r - 1) {
            bits.push_back(__builtin_ctzll(r));
        }
        widen(nb, bits);
        // gate on the left: every column of M gets the gate's action
        const unsigned D = 1u << bits.size();
        std::vector<C2> col(D);
        for (unsigned c = 0; c < D; c++) {
            for (unsigned r = 0; r < D; r++) {
                col[r] = nb.m[static_cast<size_t>(r) * D + c];
            }
            apply_local(p, bits, col);
            for (unsigned r = 0; r < D; r++) {
                nb.m[static_cast<size_t>(r) * D + c] = col[r];
            }
        }
        remove(meet);
        open.push_back(std::move(nb));
    }
    std::vector<size_t> all(open.size());
    for (size_t i = 0; i < all.size(); i++) {
        all[i] = i;
    }
    emit_blocks(all);
    if (scalar != C2(1.0)) {
        Prim<T> s;
        s.kind = Prim<T>::Scale;
        s.m = {cx<T>{static_cast<T>(scalar.real()), static_cast<T>(scalar.imag())}};
        out.push_back(s);
    }
    return out;
}

template std::vector<Prim<float>> fuse_dense_blocks<float>(const std::vector<Prim<float>> &, int, int);
template std::vector<Prim<double>> fuse_dense_blocks<double>(const std::vector<Prim<double>> &, int, int);


template <class T> std::shared_ptr<const BlockProgram<T>> prepare_blocks(std::vector<Prim<T>> prims, int n) {
    auto prog = std::make_shared<BlockProgram<T>>();
    prog->tc.assign(prims.size(), -1);
    if constexpr (std::is_same_v<T, float>) {
        std::vector<unsigned short> host;
        const size_t words = tc_a_image_bytes() / sizeof(unsigned short);
        for (size_t i = 0; i < prims.size(); i++) {
            const Prim<T> &p = prims[i];
            TcGeom g{};
            if (p.kind == Prim<T>::DenseK && p.tbits.size() == 6 && p.cmask == 0 && tc_geom_for(n, p.tbits.data(), g)) {
                prog->tc[i] = static_cast<int>(prog->geom.size());
                prog->geom.push_back(g);
                host.resize(host.size() + words);
                tc_build_a_image(p.m.data(), g, host.data() + host.size() - words);
            }
        }
        if (!prog->geom.empty()) {
            prog->images = dev_alloc(host.size() * sizeof(unsigned short));
            cuda_check(cudaMemcpy(prog->images, host.data(), host.size() * sizeof(unsigned short),
                                  cudaMemcpyHostToDevice),
                       "H2D block matrix images");
        }
    }
    prog->prims = std::move(prims);
    return prog;
}

template <class T> void run_blocks(StateVector<T> &sv, const BlockProgram<T> &prog) {
    bool any_tc = false;
    int *derr = nullptr;
    for (size_t i = 0; i < prog.prims.size(); i++) {
        if constexpr (std::is_same_v<T, float>) {
            if (prog.tc[i] >= 0 && tc_dense_enabled()) {
                if (!any_tc) {
                    derr = sv.scratch().ensure_flag();
                    cuda_check(cudaMemsetAsync(derr, 0, sizeof(int), sv.stream()), "clear error word");
                    any_tc = true;
                }
                const auto *img = static_cast<const unsigned short *>(prog.images) +
                                  static_cast<size_t>(prog.tc[i]) * (tc_a_image_bytes() / sizeof(unsigned short));
                launch_dense6_tc(sv.stream(), sv.data(), prog.geom[static_cast<size_t>(prog.tc[i])], img, derr);
                continue;
            }
        }
        sv.run_prim(prog.prims[i]);
    }
    if (any_tc) {
        int herr = 0;
        cuda_check(cudaMemcpyAsync(&herr, derr, sizeof(int), cudaMemcpyDeviceToHost, sv.stream()), "D2H error word");
        sv.synchronize();
        PLGB_REQUIRE(herr == 0, "tensor-core dense block: a CTA timed out waiting for its MMAs");
    }
}

template std::shared_ptr<const BlockProgram<float>> prepare_blocks<float>(std::vector<Prim<float>>, int);
template std::shared_ptr<const BlockProgram<double>> prepare_blocks<double>(std::vector<Prim<double>>, int);
template void run_blocks<float>(StateVector<float> &, const BlockProgram<float> &);
template void run_blocks<double>(StateVector<double> &, const BlockProgram<double> &);

} // namespace plgb
