// State vector, gate dispatch and generators on the GPU.
//
// Gate semantics follow pennylane_lightning/core/simulators/lightning_qubit/
// gates/cpu_kernels/GateImplementationsLM.hpp ("LM" below); coefficients are
// formed on the host in the working precision T with the same formulas, then
// each gate is lowered to one of the streaming kernels of kernels_gates.cu.
#include "host.hpp"
#include "kernels_tc.hpp"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <unordered_map>

namespace plgb {

// ---------------------------------------------------------------------------
int LaunchGeom::sm_count() {
    static int sms = [] {
        int dev = 0, v = 0;
        if (cudaGetDevice(&dev) != cudaSuccess ||
            cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || v <= 0) {
            return 152;
        }
        return v;
    }();
    return sms;
}

static std::atomic<unsigned long long> g_launches{0};
void note_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }
unsigned long long launch_count() { return g_launches.load(std::memory_order_relaxed); }

static thread_local std::string g_last_error;
void set_last_error(const std::string &msg) { g_last_error = msg; }
const char *last_error() { return g_last_error.c_str(); }

// ---- device / pinned buffers: cudaMalloc, or the thread's reuse pool
namespace {
thread_local ReusePool *tl_pool = nullptr;
size_t pool_bucket(size_t bytes) {
    size_t c = 256;
    while (c < bytes) {
        c <<= 1;
    }
    return c;
}
} // namespace

ReusePool::~ReusePool() {
    recycle();
    for (int k = 0; k < 2; k++) {
        for (auto &kv : free_[k]) {
            k ? cudaFreeHost(kv.second) : cudaFree(kv.second);
        }
    }
}
void *ReusePool::take(size_t bytes, bool pinned) {
    const size_t cap = pool_bucket(bytes);
    auto &fl = free_[pinned ? 1 : 0];
    void *p = nullptr;
    auto it = fl.find(cap);
    if (it != fl.end()) {
        p = it->second;
        fl.erase(it);
        held_ -= cap;
    } else if (pinned) {
        cuda_check(cudaMallocHost(&p, cap), "cudaMallocHost(pool)");
    } else {
        cuda_check(cudaMalloc(&p, cap), "cudaMalloc(pool)");
    }
    out_[p] = Buf{cap, pinned};
    return p;
}
bool ReusePool::give(void *p) {
    auto it = out_.find(p);
    if (it == out_.end()) {
        return false;
    }
    pending_.emplace_back(p, it->second);
    out_.erase(it);
    return true;
}
void ReusePool::recycle() {
    for (auto &pb : pending_) {
        if (held_ + pb.second.cap > cap_bytes) {
            pb.second.pinned ? cudaFreeHost(pb.first) : cudaFree(pb.first);
        } else {
            free_[pb.second.pinned ? 1 : 0].emplace(pb.second.cap, pb.first);
            held_ += pb.second.cap;
        }
    }
    pending_.clear();
}
ReuseScope::ReuseScope(ReusePool &pool) : prev_(tl_pool) { tl_pool = &pool; }
ReuseScope::~ReuseScope() { tl_pool = prev_; }

namespace {
std::atomic<unsigned long long> g_dev_allocs{0};
}
void count_device_allocation() { g_dev_allocs.fetch_add(1, std::memory_order_relaxed); }
unsigned long long device_allocation_count() { return g_dev_allocs.load(std::memory_order_relaxed); }

void *dev_alloc(size_t bytes) {
    count_device_allocation();
    if (tl_pool) {
        return tl_pool->take(bytes, false);
    }
    void *p = nullptr;
    cuda_check(cudaMalloc(&p, bytes), "cudaMalloc");
    return p;
}
void dev_free(void *p) {
    if (!p || (tl_pool && tl_pool->give(p))) {
        return;
    }
    cudaFree(p);
}
void *pinned_alloc(size_t bytes) {
    if (tl_pool) {
        return tl_pool->take(bytes, true);
    }
    void *p = nullptr;
    cuda_check(cudaMallocHost(&p, bytes), "cudaMallocHost");
    return p;
}
void pinned_free(void *p) {
    if (!p || (tl_pool && tl_pool->give(p))) {
        return;
    }
    cudaFreeHost(p);
}

void DeviceScratch::ensure_mat(size_t bytes) {
    if (bytes <= mat_bytes) {
        return;
    }
    if (mat) {
        dev_free(mat);
        mat = nullptr;
    }
    mat = dev_alloc(bytes);
    mat_bytes = bytes;
}
std::vector<char *> DeviceScratch::carve(std::initializer_list<size_t> sizes) {
    size_t total = 0;
    for (auto sz : sizes) {
        total += align_up(sz);
    }
    ensure_mat(total + 256);
    std::vector<char *> out;
    char *p = static_cast<char *>(mat);
    for (auto sz : sizes) {
        out.push_back(p);
        p += align_up(sz);
    }
    return out;
}

int *DeviceScratch::ensure_flag() {
    if (!flag) {
        flag = static_cast<int *>(dev_alloc(sizeof(int)));
    }
    return flag;
}
DeviceScratch::~DeviceScratch() {
    dev_free(red);
    pinned_free(host_out);
    dev_free(mat);
    dev_free(flag);
}

static const char *kGateNames[] = {
    "Identity", "PauliX", "PauliY", "PauliZ", "Hadamard", "S", "SX", "T", "PhaseShift", "RX", "RY", "RZ", "Rot",
    "CNOT", "CY", "CZ", "SWAP", "IsingXX", "IsingXY", "IsingYY", "IsingZZ", "ControlledPhaseShift", "CRX", "CRY",
    "CRZ", "CRot", "SingleExcitation", "SingleExcitationMinus", "SingleExcitationPlus", "PSWAP", "Toffoli", "CSWAP",
    "DoubleExcitation", "DoubleExcitationMinus", "DoubleExcitationPlus", "MultiRZ", "GlobalPhase", "PCPhase"};

const char *gate_name_of(int code) {
    constexpr int k = static_cast<int>(sizeof(kGateNames) / sizeof(kGateNames[0]));
    return code >= 0 && code < k ? kGateNames[code] : nullptr;
}
int gate_code_count() { return static_cast<int>(sizeof(kGateNames) / sizeof(kGateNames[0])); }
int gate_param_count(const std::string &name) {
    if (name == "Rot" || name == "CRot") {
        return 3;
    }
    if (name == "PCPhase") {
        return 2;
    }
    static const char *kNoParam[] = {"Identity", "PauliX", "PauliY", "PauliZ", "Hadamard", "S", "SX", "T", "CNOT",
                                     "CY", "CZ", "SWAP", "Toffoli", "CSWAP"};
    for (auto *g : kNoParam) {
        if (name == g) {
            return 0;
        }
    }
    return 1;
}

bool is_named_gate(const std::string &name) {
    for (auto *g : kGateNames) {
        if (name == g) {
            return true;
        }
    }
    return false;
}

size_t OpsList::num_par_ops() const {
    size_t k = 0;
    for (const auto &o : ops) {
        k += o.params.empty() ? 0 : 1;
    }
    return k;
}

// ---------------------------------------------------------------------------
// construction
// ---------------------------------------------------------------------------
template <class T> void StateVector<T>::alloc_(bool zero) {
    PLGB_REQUIRE(n_ >= 0 && n_ <= 40, "number of qubits out of range");
    N_ = u64{1} << n_;
    if (owns_) {
        d_ = static_cast<CT *>(dev_alloc(N_ * sizeof(CT)));
        if (zero) {
            cuda_check(cudaMemsetAsync(d_, 0, N_ * sizeof(CT), s_), "memset");
        }
    }
    scratch_.red = static_cast<double *>(dev_alloc(sizeof(double) * (kReduceBlocks * 2 + 8)));
    scratch_.host_out = static_cast<double *>(pinned_alloc(sizeof(double) * 8));
}

template <class T> StateVector<T>::StateVector(int num_qubits, cudaStream_t stream) : n_(num_qubits) {
    if (stream) {
        s_ = stream;
    } else {
        cuda_check(cudaStreamCreateWithFlags(&s_, cudaStreamNonBlocking), "cudaStreamCreate");
        owns_stream_ = true;
    }
    alloc_(false);
    reset();
}

template <class T> StateVector<T>::StateVector(int num_qubits, LowerOnly) : n_(num_qubits) {
    PLGB_REQUIRE(n_ >= 0 && n_ <= 40, "number of qubits out of range");
    N_ = u64{1} << n_;
    owns_ = false;
}

template <class T> StateVector<T>::StateVector(CT *external, int num_qubits, cudaStream_t stream) : n_(num_qubits) {
    owns_ = false;
    d_ = external;
    if (stream) {
        s_ = stream;
    } else {
        cuda_check(cudaStreamCreateWithFlags(&s_, cudaStreamNonBlocking), "cudaStreamCreate");
        owns_stream_ = true;
    }
    alloc_(false);
}

template <class T> StateVector<T>::StateVector(const StateVector &o) : n_(o.n_), s_(o.s_) {
    alloc_(false);
    cuda_check(cudaMemcpyAsync(d_, o.d_, N_ * sizeof(CT), cudaMemcpyDeviceToDevice, s_), "copy");
}

template <class T> StateVector<T>::~StateVector() {
    if (owns_ && d_) {
        cudaStreamSynchronize(s_);
        dev_free(d_);
    }
    if (owns_stream_) {
        cudaStreamDestroy(s_);
    }
}


template <class T> void StateVector<T>::synchronize() const {
    cuda_check(cudaStreamSynchronize(s_), "stream synchronize");
}

template <class T> int StateVector<T>::bit_of(int64_t wire) const {
    PLGB_REQUIRE(wire >= 0 && wire < n_, "wire index out of range");
    return n_ - 1 - static_cast<int>(wire);
}

template <class T>
void StateVector<T>::check_wires_(const std::vector<int64_t> &wires, const std::vector<int64_t> &cwires) const {
    std::vector<int64_t> all(wires);
    all.insert(all.end(), cwires.begin(), cwires.end());
    for (auto w : all) {
        PLGB_REQUIRE(w >= 0 && w < n_, "wire index out of range");
    }
    std::sort(all.begin(), all.end());
    PLGB_REQUIRE(std::adjacent_find(all.begin(), all.end()) == all.end(),
                 "`controlled_wires` and `target wires` must be disjoint.");
}

template <class T>
GroupGeom StateVector<T>::geom_(const std::vector<int> &target_bits, const std::vector<int64_t> &cwires,
                                const std::vector<bool> &cvals) const {
    PLGB_REQUIRE(cwires.size() == cvals.size(),
                 "`controlled_wires` must have the same size as `controlled_values`.");
    GroupGeom g{};
    std::vector<int> ins(target_bits);
    g.cval = 0;
    for (size_t i = 0; i < cwires.size(); i++) {
        const int b = bit_of(cwires[i]);
        ins.push_back(b);
        if (cvals[i]) {
            g.cval |= u64{1} << b;
        }
    }
    std::sort(ins.begin(), ins.end());
    PLGB_REQUIRE(static_cast<int>(ins.size()) <= PLGB_MAX_INS && static_cast<int>(ins.size()) <= n_,
                 "too many wires for the register");
    g.nins = static_cast<int>(ins.size());
    for (int i = 0; i < g.nins; i++) {
        g.ins[i] = ins[static_cast<size_t>(i)];
    }
    g.ngroups = N_ >> g.nins;
    return g;
}

// ---------------------------------------------------------------------------
// state management
// ---------------------------------------------------------------------------
template <class T> void StateVector<T>::set_basis_state_index(u64 index) {
    PLGB_REQUIRE(index < N_, "Invalid index");
    cuda_check(cudaMemsetAsync(d_, 0, N_ * sizeof(CT), s_), "memset");
    const CT one{1, 0};
    cuda_check(cudaMemcpyAsync(d_ + index, &one, sizeof(CT), cudaMemcpyHostToDevice, s_), "set basis");
    synchronize(); // `one` lives on this stack frame
}
template <class T> void StateVector<T>::reset() { set_basis_state_index(0); }

template <class T>
void StateVector<T>::set_basis_state(const std::vector<int64_t> &bits, const std::vector<int64_t> &wires) {
    PLGB_REQUIRE(bits.size() == wires.size(), "state and wires must have the same length");
    u64 index = 0;
    for (size_t k = 0; k < wires.size(); k++) {
        PLGB_REQUIRE(bits[k] == 0 || bits[k] == 1, "basis state entries must be 0 or 1");
        index |= static_cast<u64>(bits[k]) << bit_of(wires[k]);
    }
    set_basis_state_index(index);
}

template <class T>
void StateVector<T>::set_state_vector(const std::complex<T> *host_state, u64 len, const std::vector<int64_t> &wires) {
    // StateVectorLQubit.hpp:971-1036: the sub-state is written onto the
    // subspace where every other wire is |0>; the binding resets first.
    PLGB_REQUIRE(len == (u64{1} << wires.size()), "Inconsistent state and wires dimensions.");
    check_wires_(wires, {});
    if (wires.size() == static_cast<size_t>(n_)) {
        bool ordered = true;
        for (size_t i = 0; i < wires.size(); i++) {
            ordered = ordered && wires[i] == static_cast<int64_t>(i);
        }
        if (ordered) {
            update_data(host_state, len);
            return;
        }
    }
    const auto bufs = scratch_.carve({len * sizeof(CT), len * sizeof(u64)});
    CT *dsub = reinterpret_cast<CT *>(bufs[0]);
    u64 *dloc = reinterpret_cast<u64 *>(bufs[1]);
    std::vector<u64> loc(len);
    const size_t k = wires.size();
    for (u64 j = 0; j < len; j++) {
        u64 idx = 0;
        for (size_t m = 0; m < k; m++) {
            if ((j >> (k - 1 - m)) & 1U) {
                idx |= u64{1} << bit_of(wires[m]);
            }
        }
        loc[j] = idx;
    }
    cuda_check(cudaMemcpyAsync(dsub, host_state, len * sizeof(CT), cudaMemcpyHostToDevice, s_), "H2D");
    cuda_check(cudaMemcpyAsync(dloc, loc.data(), len * sizeof(u64), cudaMemcpyHostToDevice, s_), "H2D");
    launch_scatter_sub<T>(s_, d_, dsub, len, dloc);
    synchronize();
}

template <class T> void StateVector<T>::update_data(const std::complex<T> *host, u64 len) {
    PLGB_REQUIRE(len == N_, "The given data size does not match the state vector size");
    cuda_check(cudaMemcpyAsync(d_, host, N_ * sizeof(CT), cudaMemcpyHostToDevice, s_), "H2D");
    synchronize();
}
template <class T> void StateVector<T>::get_state(std::complex<T> *host_out, u64 len) const {
    PLGB_REQUIRE(len >= N_, "Output array is too small");
    cuda_check(cudaMemcpyAsync(host_out, d_, N_ * sizeof(CT), cudaMemcpyDeviceToHost, s_), "D2H");
    synchronize();
}
template <class T> void StateVector<T>::copy_from(const StateVector &o) {
    PLGB_REQUIRE(o.N_ == N_, "state vectors have different sizes");
    if (o.s_ != s_) {
        o.synchronize();
    }
    cuda_check(cudaMemcpyAsync(d_, o.d_, N_ * sizeof(CT), cudaMemcpyDeviceToDevice, s_), "D2D");
}

template <class T> double StateVector<T>::norm2() const {
    reduce_norm2<T>(s_, d_, N_, scratch_.red, scratch_.red + 2 * kReduceBlocks);
    cuda_check(cudaMemcpyAsync(scratch_.host_out, scratch_.red + 2 * kReduceBlocks, sizeof(double),
                               cudaMemcpyDeviceToHost, s_),
               "D2H");
    synchronize();
    return scratch_.host_out[0];
}
template <class T> cd StateVector<T>::inner(const StateVector &ket) const {
    if (ket.s_ != s_) {
        ket.synchronize();
    }
    reduce_inner<T>(s_, d_, ket.d_, N_, scratch_.red, scratch_.red + 2 * kReduceBlocks);
    cuda_check(cudaMemcpyAsync(scratch_.host_out, scratch_.red + 2 * kReduceBlocks, 2 * sizeof(double),
                               cudaMemcpyDeviceToHost, s_),
               "D2H");
    synchronize();
    return {scratch_.host_out[0], scratch_.host_out[1]};
}

template <class T> void StateVector<T>::normalize() {
    // StateVectorLQubit.hpp:905-921
    const T norm = static_cast<T>(std::sqrt(norm2()));
    PLGB_REQUIRE(!(norm < std::numeric_limits<T>::epsilon() * 1e2),
                 "Vector has norm close to zero and cannot be normalized");
    const T inv = T(1.) / norm;
    launch_scale<T>(s_, d_, N_, CT{inv, 0}, 0, 0);
}

template <class T> void StateVector<T>::collapse(int64_t wire, bool branch) {
    // StateVectorLQubit.hpp:881-898: zero the other branch, renormalize
    const u64 m = u64{1} << bit_of(wire);
    launch_zero_outside<T>(s_, d_, N_, m, branch ? m : 0);
    normalize();
}

template <class T> void StateVector<T>::scale_add(const StateVector &x, cd factor) {
    if (x.s_ != s_) {
        x.synchronize();
    }
    launch_axpy<T>(s_, d_, x.d_, N_, CT{static_cast<T>(factor.real()), static_cast<T>(factor.imag())});
}

// ---------------------------------------------------------------------------
// primitives: emitted into the fusion sink when one is set, launched otherwise
// ---------------------------------------------------------------------------
template <class T> u64 Prim<T>::touched() const {
    u64 t = cmask | pmask | my | mz | rx | ryz | rpm;
    for (int b : tbits) {
        t |= u64{1} << b;
    }
    return t;
}
template <class T> bool Prim<T>::diagonal() const {
    return kind == DiagK || kind == Parity || kind == Scale ||
           (kind == Pair && (mode == M1_DIAG || mode == M1_PHASE1 || mode == M1_NEG1));
}

template <class T> void StateVector<T>::emit_(Prim<T> &&p) {
    if (sink_) {
        sink_->push_back(std::move(p));
    } else {
        run_prim(p);
    }
}

template <class T> static void set_controls(Prim<T> &p, const StateVector<T> &sv, const std::vector<int64_t> &cw,
                                            const std::vector<bool> &cv) {
    PLGB_REQUIRE(cw.size() == cv.size(), "`controlled_wires` must have the same size as `controlled_values`.");
    for (size_t i = 0; i < cw.size(); i++) {
        const int b = sv.bit_of(cw[i]);
        p.cbits.push_back(b);
        p.cmask |= u64{1} << b;
        if (cv[i]) {
            p.cval |= u64{1} << b;
        }
    }
}

template <class T> void StateVector<T>::run_prim(const Prim<T> &p) {
    auto geom = [&](const std::vector<int> &tb) {
        GroupGeom g{};
        std::vector<int> ins(tb);
        ins.insert(ins.end(), p.cbits.begin(), p.cbits.end());
        std::sort(ins.begin(), ins.end());
        PLGB_REQUIRE(static_cast<int>(ins.size()) <= PLGB_MAX_INS && static_cast<int>(ins.size()) <= n_,
                     "too many wires for the register");
        g.nins = static_cast<int>(ins.size());
        for (int i = 0; i < g.nins; i++) {
            g.ins[i] = ins[static_cast<size_t>(i)];
        }
        g.cval = p.cval;
        g.ngroups = N_ >> g.nins;
        return g;
    };
    switch (p.kind) {
    case Prim<T>::Pair: {
        Mat1<T> m{};
        for (size_t i = 0; i < 4 && i < p.m.size(); i++) {
            m.m[i] = p.m[i];
        }
        const GroupGeom g = geom(p.tbits);
        if (g.ngroups > 0) {
            launch_1q<T>(s_, d_, g, p.o0, p.o1, p.mode, m);
        }
        return;
    }
    case Prim<T>::Dense2: {
        Mat2<T> m{};
        for (size_t i = 0; i < 16; i++) {
            m.m[i] = p.m[i];
        }
        launch_2q<T>(s_, d_, geom(p.tbits), p.tbits[0], p.tbits[1], false, m);
        return;
    }
    case Prim<T>::DenseK: {
        const size_t k = p.tbits.size();
        const size_t D = size_t{1} << k;
        if constexpr (std::is_same_v<T, float>) {
            // complex64, six targets, no controls: the tensor-core kernel
            TcGeom tg{};
            if (k == 6 && p.cmask == 0 && tc_dense_enabled() && tc_geom_for(n_, p.tbits.data(), tg)) {
                std::vector<unsigned short> img(tc_a_image_bytes() / sizeof(unsigned short));
                tc_build_a_image(p.m.data(), tg, img.data());
                const auto bufs = scratch_.carve({tc_a_image_bytes()});
                int *derr = scratch_.ensure_flag();
                cuda_check(cudaMemcpyAsync(bufs[0], img.data(), tc_a_image_bytes(), cudaMemcpyHostToDevice, s_),
                           "H2D matrix image");
                cuda_check(cudaMemsetAsync(derr, 0, sizeof(int), s_), "clear error word");
                launch_dense6_tc(s_, d_, tg, reinterpret_cast<const unsigned short *>(bufs[0]), derr);
                int herr = 0;
                cuda_check(cudaMemcpyAsync(&herr, derr, sizeof(int), cudaMemcpyDeviceToHost, s_), "D2H error word");
                synchronize(); // the scratch image is reused by the next call
                PLGB_REQUIRE(herr == 0, "tensor-core dense block: a CTA timed out waiting for its MMAs");
                return;
            }
        }
        LocalOffsets lo{};
        std::vector<u64> loc(D);
        for (size_t j = 0; j < D; j++) {
            u64 o = 0;
            for (size_t b = 0; b < k; b++) {
                if ((j >> (k - 1 - b)) & 1U) {
                    o |= u64{1} << p.tbits[b];
                }
            }
            loc[j] = o;
            if (j < 32) {
                lo.off[j] = o;
            }
        }
        const size_t mbytes = D * D * sizeof(CT);
        const auto bufs = scratch_.carve({mbytes, D * sizeof(u64)});
        CT *dm = reinterpret_cast<CT *>(bufs[0]);
        u64 *dloc = reinterpret_cast<u64 *>(bufs[1]);
        cuda_check(cudaMemcpyAsync(dm, p.m.data(), mbytes, cudaMemcpyHostToDevice, s_), "H2D matrix");
        cuda_check(cudaMemcpyAsync(dloc, loc.data(), D * sizeof(u64), cudaMemcpyHostToDevice, s_), "H2D offsets");
        launch_kq<T>(s_, d_, geom(p.tbits), static_cast<int>(k), lo, dm, dloc);
        synchronize(); // the scratch matrix is reused by the next call
        return;
    }
    case Prim<T>::DiagK: {
        const size_t k = p.tbits.size();
        if (k == 2) {
            Mat2<T> m{};
            m.m[0] = p.m[0];
            m.m[5] = p.m[1];
            m.m[10] = p.m[2];
            m.m[15] = p.m[3];
            launch_2q<T>(s_, d_, geom(p.tbits), p.tbits[0], p.tbits[1], true, m);
            return;
        }
        TBits tb{};
        for (size_t b = 0; b < k; b++) {
            tb.b[b] = p.tbits[b];
        }
        scratch_.ensure_mat(p.m.size() * sizeof(CT));
        CT *dd = static_cast<CT *>(scratch_.mat);
        cuda_check(cudaMemcpyAsync(dd, p.m.data(), p.m.size() * sizeof(CT), cudaMemcpyHostToDevice, s_), "H2D diag");
        launch_diag<T>(s_, d_, N_, p.cmask, p.cval, static_cast<int>(k), tb, dd);
        synchronize();
        return;
    }
    case Prim<T>::Parity:
        launch_parity<T>(s_, d_, N_, p.pmask, p.cmask, p.cval, p.m[0], p.m[1], p.zero_outside);
        return;
    case Prim<T>::Scale:
        launch_scale<T>(s_, d_, N_, p.m[0], p.cmask, p.cval);
        return;
    case Prim<T>::PauliRot:
        launch_pauli_rot<T>(s_, d_, n_, p.pmask, p.my, p.mz, p.c, p.m[0]);
        return;
    case Prim<T>::ZeroOut:
        if (p.cmask) {
            launch_zero_outside<T>(s_, d_, N_, p.cmask, p.cval);
        }
        return;
    }
}

template <class T>
void StateVector<T>::prim_pair(const std::vector<int> &ins_bits, u64 o0, u64 o1, const std::vector<int64_t> &cwires,
                               const std::vector<bool> &cvals, int mode, const Mat1<T> &m) {
    Prim<T> p;
    p.kind = Prim<T>::Pair;
    p.mode = mode;
    p.tbits = ins_bits;
    p.o0 = o0;
    p.o1 = o1;
    set_controls(p, *this, cwires, cvals);
    p.m.assign(m.m, m.m + 4);
    emit_(std::move(p));
}

template <class T>
void StateVector<T>::prim_1q(int64_t wire, const std::vector<int64_t> &cwires, const std::vector<bool> &cvals,
                             int mode, const Mat1<T> &m) {
    const int b = bit_of(wire);
    prim_pair({b}, 0, u64{1} << b, cwires, cvals, mode, m);
}

template <class T>
void StateVector<T>::prim_dense(const std::vector<int64_t> &wires, const std::vector<int64_t> &cwires,
                                const std::vector<bool> &cvals, const std::vector<CT> &mat) {
    const size_t k = wires.size();
    PLGB_REQUIRE(k >= 1, "Number of wires must be larger than 0");
    PLGB_REQUIRE(mat.size() == (size_t{1} << (2 * k)),
                 "The size of matrix does not match with the given number of wires");
    check_wires_(wires, cwires);
    if (k == 1) {
        Mat1<T> m{};
        for (int i = 0; i < 4; i++) {
            m.m[i] = mat[static_cast<size_t>(i)];
        }
        prim_1q(wires[0], cwires, cvals, M1_DENSE, m);
        return;
    }
    PLGB_REQUIRE(k <= 12, "dense matrices act on at most 12 wires");
    Prim<T> p;
    p.kind = k == 2 ? Prim<T>::Dense2 : Prim<T>::DenseK;
    for (auto w : wires) {
        p.tbits.push_back(bit_of(w));
    }
    set_controls(p, *this, cwires, cvals);
    p.m = mat;
    emit_(std::move(p));
}

template <class T>
void StateVector<T>::prim_diag(const std::vector<int64_t> &wires, const std::vector<int64_t> &cwires,
                               const std::vector<bool> &cvals, const std::vector<CT> &diag) {
    const size_t k = wires.size();
    PLGB_REQUIRE(k >= 1 && k <= 16, "diagonal gates act on 1..16 wires");
    check_wires_(wires, cwires);
    Prim<T> p;
    p.kind = Prim<T>::DiagK;
    for (auto w : wires) {
        p.tbits.push_back(bit_of(w));
    }
    set_controls(p, *this, cwires, cvals);
    p.m = diag;
    emit_(std::move(p));
}

template <class T>
void StateVector<T>::prim_zero_outside(const std::vector<int64_t> &cwires, const std::vector<bool> &cvals) {
    if (cwires.empty()) {
        return;
    }
    Prim<T> p;
    p.kind = Prim<T>::ZeroOut;
    set_controls(p, *this, cwires, cvals);
    emit_(std::move(p));
}

template <class T> std::vector<Prim<T>> StateVector<T>::lower_op(const OpRec &op, bool inverse) {
    std::vector<Prim<T>> out;
    auto *saved = sink_;
    sink_ = &out;
    try {
        apply_op(op, inverse);
    } catch (...) {
        sink_ = saved;
        throw;
    }
    sink_ = saved;
    return out;
}

// ---------------------------------------------------------------------------
// named gates
// ---------------------------------------------------------------------------
template <class T> static Mat1<T> m1(cx<T> a, cx<T> b, cx<T> c, cx<T> d) { return Mat1<T>{{a, b, c, d}}; }
template <class T> static cx<T> C(T re, T im) { return cx<T>{re, im}; }
template <class T> static cx<T> cexp_i(T angle) { return cx<T>{std::cos(angle), std::sin(angle)}; }
template <class T> static constexpr T invsqrt2() {
    return static_cast<T>(0.7071067811865475244008443621048490392848359376884740L);
}

// getRot (pennylane_lightning/core/gates/Gates.hpp:389-399)
template <class T> static std::vector<cx<T>> rot_matrix(T phi, T theta, T omega) {
    const T c = std::cos(theta / 2);
    const T s = std::sin(theta / 2);
    const T p{phi + omega};
    const T m{phi - omega};
    return {cx<T>{std::cos(p / 2) * c, -std::sin(p / 2) * c}, cx<T>{-std::cos(m / 2) * s, -std::sin(m / 2) * s},
            cx<T>{std::cos(m / 2) * s, -std::sin(m / 2) * s}, cx<T>{std::cos(p / 2) * c, std::sin(p / 2) * c}};
}
template <class T> static std::vector<cx<T>> dagger(const std::vector<cx<T>> &m, size_t dim) {
    std::vector<cx<T>> r(m.size());
    for (size_t i = 0; i < dim; i++) {
        for (size_t j = 0; j < dim; j++) {
            r[j * dim + i] = conj(m[i * dim + j]);
        }
    }
    return r;
}

template <class T>
void StateVector<T>::global_phase_(const std::vector<int64_t> &cw, const std::vector<bool> &cv, bool inverse,
                                   T angle) {
    // LM:2046-2111 applyNCGlobalPhase
    const CT phase = cexp_i<T>(inverse ? angle : -angle);
    if (cw.size() == 1 && cv[0]) {
        // phase shift on the control wire by -angle
        const T a = -angle;
        const CT s = inverse ? cexp_i<T>(-a) : cexp_i<T>(a);
        prim_1q(cw[0], {}, {}, M1_PHASE1, m1<T>(C<T>(1, 0), C<T>(0, 0), C<T>(0, 0), s));
        return;
    }
    if (n_ == 1 && cw.size() == 1 && !cv[0]) {
        const CT s = inverse ? cexp_i<T>(-angle) : cexp_i<T>(angle);
        prim_1q(cw[0], {}, {}, M1_PHASE1, m1<T>(C<T>(1, 0), C<T>(0, 0), C<T>(0, 0), s));
        Prim<T> p;
        p.kind = Prim<T>::Scale;
        p.m = {phase};
        emit_(std::move(p));
        return;
    }
    Prim<T> p;
    p.kind = Prim<T>::Scale;
    set_controls(p, *this, cw, cv);
    p.m = {phase};
    emit_(std::move(p));
}

template <class T>
void StateVector<T>::apply_named_(const std::string &name, std::vector<int64_t> cw, std::vector<bool> cv,
                                  std::vector<int64_t> wires, bool inverse, const std::vector<double> &params) {
    PLGB_REQUIRE(cw.size() == cv.size(), "`controlled_wires` must have the same size as `controlled_values`.");
    auto P = [&](size_t i) -> T {
        PLGB_REQUIRE(params.size() > i, "missing gate parameter for " + name);
        return static_cast<T>(params[i]);
    };
    auto need = [&](size_t k) { PLGB_REQUIRE(wires.size() == k, "wrong number of wires for gate " + name); };
    auto lift = [&](size_t nc) {
        PLGB_REQUIRE(wires.size() > nc, "wrong number of wires for gate " + name);
        for (size_t i = 0; i < nc; i++) {
            cw.push_back(wires[i]);
            cv.push_back(true);
        }
        wires.erase(wires.begin(), wires.begin() + static_cast<long>(nc));
    };
    if (name == "Identity") {
        return;
    }
    std::string base = name;
    if (name == "CNOT" || name == "CY" || name == "CZ" || name == "CRX" || name == "CRY" || name == "CRZ" ||
        name == "CRot" || name == "ControlledPhaseShift") {
        need(2);
        PLGB_REQUIRE(cw.empty(), "gate " + name + " takes no extra controls");
        lift(1);
        base = name == "CNOT" ? "PauliX" : name == "CY" ? "PauliY" : name == "CZ" ? "PauliZ"
             : name == "CRX" ? "RX" : name == "CRY" ? "RY" : name == "CRZ" ? "RZ" : name == "CRot" ? "Rot"
             : "PhaseShift";
    } else if (name == "CSWAP") {
        need(3);
        PLGB_REQUIRE(cw.empty(), "gate CSWAP takes no extra controls");
        lift(1);
        base = "SWAP";
    } else if (name == "Toffoli") {
        need(3);
        PLGB_REQUIRE(cw.empty(), "gate Toffoli takes no extra controls");
        lift(2);
        base = "PauliX";
    }
    check_wires_(wires, cw);
    const cx<T> Z0{0, 0}, O1{1, 0};
    const T isq = invsqrt2<T>();
    auto pair_bits = [&](int64_t w_hi, int64_t w_lo, int p0, int p1, std::vector<int> &ins, u64 &o0, u64 &o1) {
        // local 2-bit pattern p (bit1 = first wire) -> offsets
        const int bh = bit_of(w_hi), bl = bit_of(w_lo);
        ins = {bh, bl};
        auto off = [&](int p) { return ((p & 2) ? (u64{1} << bh) : 0) | ((p & 1) ? (u64{1} << bl) : 0); };
        o0 = off(p0);
        o1 = off(p1);
    };

    if (base == "PauliX") { // LM:705-734 swap
        need(1);
        prim_1q(wires[0], cw, cv, M1_SWAP, Mat1<T>{});
    } else if (base == "PauliY") { // LM:762-800: v0' = -i v1, v1' = i v0
        need(1);
        prim_1q(wires[0], cw, cv, M1_ANTI, m1<T>(Z0, C<T>(0, -1), C<T>(0, 1), Z0));
    } else if (base == "PauliZ") { // LM:820-855
        need(1);
        prim_1q(wires[0], cw, cv, M1_NEG1, Mat1<T>{});
    } else if (base == "Hadamard") { // LM:857-890
        need(1);
        prim_1q(wires[0], cw, cv, M1_REAL, m1<T>(C<T>(isq, 0), C<T>(isq, 0), C<T>(isq, 0), C<T>(-isq, 0)));
    } else if (base == "S") { // LM:892-925
        need(1);
        prim_1q(wires[0], cw, cv, M1_PHASE1, m1<T>(O1, Z0, Z0, inverse ? C<T>(0, -1) : C<T>(0, 1)));
    } else if (base == "T") { // LM:927-958
        need(1);
        prim_1q(wires[0], cw, cv, M1_PHASE1, m1<T>(O1, Z0, Z0, C<T>(isq, inverse ? -isq : isq)));
    } else if (base == "SX") { // LM:960-1000 (= 1/2 [[1+i, 1-i], [1-i, 1+i]], dagger if inverse)
        need(1);
        const T h = T(0.5);
        const cx<T> p{h, inverse ? -h : h}, q{h, inverse ? h : -h};
        prim_1q(wires[0], cw, cv, M1_DENSE, m1<T>(p, q, q, p));
    } else if (base == "PhaseShift") { // LM:1001-1031
        need(1);
        const T a = P(0);
        const CT s = inverse ? cexp_i<T>(-a) : cexp_i<T>(a);
        prim_1q(wires[0], cw, cv, M1_PHASE1, m1<T>(O1, Z0, Z0, s));
    } else if (base == "RX") { // LM:1063-1095
        need(1);
        const T a = P(0);
        const T c = std::cos(a / 2);
        const T js = inverse ? -std::sin(-a / 2) : std::sin(-a / 2);
        prim_1q(wires[0], cw, cv, M1_RXF, m1<T>(C<T>(c, 0), C<T>(0, js), C<T>(0, js), C<T>(c, 0)));
    } else if (base == "RY") { // LM:1126-1158
        need(1);
        const T a = P(0);
        const T c = std::cos(a / 2);
        const T s = inverse ? -std::sin(a / 2) : std::sin(a / 2);
        prim_1q(wires[0], cw, cv, M1_REAL, m1<T>(C<T>(c, 0), C<T>(-s, 0), C<T>(s, 0), C<T>(c, 0)));
    } else if (base == "RZ") { // LM:1190-1220
        need(1);
        const T a = P(0);
        const CT first{std::cos(a / 2), -std::sin(a / 2)};
        const CT second{std::cos(a / 2), std::sin(a / 2)};
        prim_1q(wires[0], cw, cv, M1_DIAG,
                m1<T>(inverse ? conj(first) : first, Z0, Z0, inverse ? conj(second) : second));
    } else if (base == "Rot") { // LM:1262-1301
        need(1);
        std::vector<CT> m;
        bool dag = false;
        if (name == "Rot" && !cw.empty()) {
            m = rot_matrix<T>(P(0), P(1), P(2)); // applyNCRot: conj-transpose when inverse
            dag = inverse;
        } else {
            m = inverse ? rot_matrix<T>(-P(2), -P(1), -P(0)) : rot_matrix<T>(P(0), P(1), P(2));
        }
        if (dag) {
            m = dagger<T>(m, 2);
        }
        prim_1q(wires[0], cw, cv, M1_DENSE, m1<T>(m[0], m[1], m[2], m[3]));
    } else if (base == "SWAP") { // LM:1388-1426: swap |01>, |10>
        need(2);
        std::vector<int> ins;
        u64 o0, o1;
        pair_bits(wires[0], wires[1], 1, 2, ins, o0, o1);
        prim_pair(ins, o0, o1, cw, cv, M1_SWAP, Mat1<T>{});
    } else if (base == "IsingXX" || base == "IsingYY") { // LM:1429-1467, 1507-1545
        need(2);
        const T a = P(0);
        const T cr = std::cos(a / 2);
        const T sj = inverse ? -std::sin(a / 2) : std::sin(a / 2);
        const CT c{cr, 0};
        const CT mis{0, -sj}, pis{0, sj};
        std::vector<CT> m(16, Z0);
        m[0] = m[5] = m[10] = m[15] = c;
        if (base == "IsingXX") {
            m[3] = m[6] = m[9] = m[12] = mis;
        } else {
            m[3] = m[12] = pis;
            m[6] = m[9] = mis;
        }
        prim_dense(wires, cw, cv, m);
    } else if (base == "IsingXY") { // LM:1469-1505: [[c, i s],[i s, c]] on |01>,|10>
        need(2);
        const T a = P(0);
        const T cr = std::cos(a / 2);
        const T sj = inverse ? -std::sin(a / 2) : std::sin(a / 2);
        std::vector<int> ins;
        u64 o0, o1;
        pair_bits(wires[0], wires[1], 1, 2, ins, o0, o1);
        prim_pair(ins, o0, o1, cw, cv, M1_RXF, m1<T>(C<T>(cr, 0), C<T>(0, sj), C<T>(0, sj), C<T>(cr, 0)));
    } else if (base == "IsingZZ") { // LM:1547-1575
        need(2);
        const T a = P(0);
        const CT first{std::cos(a / 2), -std::sin(a / 2)};
        const CT second{std::cos(a / 2), std::sin(a / 2)};
        const CT s0 = inverse ? conj(first) : first, s1 = inverse ? conj(second) : second;
        prim_diag(wires, cw, cv, {s0, s1, s1, s0});
    } else if (base == "SingleExcitation") { // LM:1613-1644: rotation on |01>,|10>
        need(2);
        const T a = P(0);
        const T c = std::cos(a / 2);
        const T s = inverse ? -std::sin(a / 2) : std::sin(a / 2);
        std::vector<int> ins;
        u64 o0, o1;
        pair_bits(wires[0], wires[1], 1, 2, ins, o0, o1);
        prim_pair(ins, o0, o1, cw, cv, M1_REAL, m1<T>(C<T>(c, 0), C<T>(-s, 0), C<T>(s, 0), C<T>(c, 0)));
    } else if (base == "SingleExcitationMinus" || base == "SingleExcitationPlus") { // LM:1646-1710
        need(2);
        const T a = P(0);
        const T c = std::cos(a / 2);
        const T s = inverse ? -std::sin(a / 2) : std::sin(a / 2);
        const bool minus = base == "SingleExcitationMinus";
        const CT e = minus ? (inverse ? cexp_i<T>(a / 2) : cexp_i<T>(-a / 2))
                           : (inverse ? cexp_i<T>(-a / 2) : cexp_i<T>(a / 2));
        std::vector<CT> m(16, Z0);
        m[0] = e;
        m[5] = C<T>(c, 0);
        m[6] = C<T>(-s, 0);
        m[9] = C<T>(s, 0);
        m[10] = C<T>(c, 0);
        m[15] = e;
        prim_dense(wires, cw, cv, m);
    } else if (base == "PSWAP") { // LM:1742-1770
        need(2);
        const T a = P(0);
        const CT ph = cexp_i<T>(inverse ? -a : a);
        std::vector<int> ins;
        u64 o0, o1;
        pair_bits(wires[0], wires[1], 1, 2, ins, o0, o1);
        prim_pair(ins, o0, o1, cw, cv, M1_ANTI, m1<T>(Z0, ph, ph, Z0));
    } else if (base == "DoubleExcitation" || base == "DoubleExcitationMinus" ||
               base == "DoubleExcitationPlus") { // LM:1798-1985
        need(4);
        const T a = P(0);
        const T cr = std::cos(a / 2);
        const T sj = inverse ? -std::sin(a / 2) : std::sin(a / 2);
        std::vector<int> ins;
        for (auto w : wires) {
            ins.push_back(bit_of(w));
        }
        auto off = [&](int p) {
            u64 o = 0;
            for (int m = 0; m < 4; m++) {
                if ((p >> (3 - m)) & 1) {
                    o |= u64{1} << ins[static_cast<size_t>(m)];
                }
            }
            return o;
        };
        if (base != "DoubleExcitation") {
            const bool minus = base == "DoubleExcitationMinus";
            const CT e = minus ? (inverse ? cexp_i<T>(a / 2) : cexp_i<T>(-a / 2))
                               : (inverse ? cexp_i<T>(-a / 2) : cexp_i<T>(a / 2));
            std::vector<CT> d(16, e);
            d[3] = O1;
            d[12] = O1;
            prim_diag(wires, cw, cv, d);
        }
        prim_pair(ins, off(3), off(12), cw, cv, M1_REAL,
                  m1<T>(C<T>(cr, 0), C<T>(-sj, 0), C<T>(sj, 0), C<T>(cr, 0)));
    } else if (base == "MultiRZ") { // LM:1989-2043
        PLGB_REQUIRE(!wires.empty(), "MultiRZ needs at least one wire");
        const T a = P(0);
        const CT first{std::cos(a / 2), -std::sin(a / 2)};
        const CT second{std::cos(a / 2), std::sin(a / 2)};
        Prim<T> p;
        p.kind = Prim<T>::Parity;
        for (auto w : wires) {
            p.pmask |= u64{1} << bit_of(w);
        }
        set_controls(p, *this, cw, cv);
        p.m = {inverse ? conj(first) : first, inverse ? conj(second) : second};
        emit_(std::move(p));
    } else if (base == "GlobalPhase") {
        global_phase_(cw, cv, inverse, P(0));
    } else if (base == "PCPhase") { // LM:2114-2162
        PLGB_REQUIRE(!wires.empty(), "PCPhase needs at least one wire");
        const T a = P(0);
        const auto dim = static_cast<u64>(std::llround(static_cast<double>(P(1))));
        PLGB_REQUIRE(dim <= N_, "The dimension of the PCPhase gate must be a positive integer and less than or "
                                "equal to statevector size.");
        const T ph = inverse ? -a : a;
        const CT up{std::cos(ph), std::sin(ph)};
        const CT lo = conj(up);
        const size_t md = size_t{1} << wires.size();
        std::vector<CT> d(md);
        for (size_t i = 0; i < md; i++) {
            d[i] = i < dim ? up : lo;
        }
        prim_diag(wires, cw, cv, d);
    } else {
        throw PLError("Gate " + name + " is not supported by the GB300 backend");
    }
}

template <class T>
void StateVector<T>::apply_operation(const std::string &name, const std::vector<int64_t> &wires, bool inverse,
                                     const std::vector<double> &params) {
    apply_named_(name, {}, {}, wires, inverse, params);
}

template <class T>
void StateVector<T>::apply_controlled_operation(const std::string &name, const std::vector<int64_t> &cwires,
                                                const std::vector<bool> &cvals, const std::vector<int64_t> &wires,
                                                bool inverse, const std::vector<double> &params) {
    // StateVectorLQubit.hpp:404-424
    check_wires_(wires, cwires);
    PLGB_REQUIRE(cwires.size() == cvals.size(), "`controlled_wires` must have the same size as `controlled_values`.");
    static const char *controlled[] = {"PauliX", "PauliY", "PauliZ", "Hadamard", "S", "SX", "T", "PhaseShift", "RX",
                                       "RY", "RZ", "Rot", "SWAP", "IsingXX", "IsingXY", "IsingYY", "IsingZZ",
                                       "SingleExcitation", "SingleExcitationMinus", "SingleExcitationPlus",
                                       "DoubleExcitation", "DoubleExcitationMinus", "DoubleExcitationPlus",
                                       "MultiRZ", "GlobalPhase", "PSWAP", "PCPhase"};
    bool ok = false;
    for (auto *c : controlled) {
        ok = ok || name == c;
    }
    PLGB_REQUIRE(ok, "Controlled gate " + name + " is not supported");
    apply_named_(name, cwires, cvals, wires, inverse, params);
}

template <class T>
void StateVector<T>::apply_matrix(const cd *mat, const std::vector<int64_t> &wires, bool inverse,
                                  const std::vector<int64_t> &cwires, const std::vector<bool> &cvals) {
    PLGB_REQUIRE(!wires.empty(), "Number of wires must be larger than 0");
    const size_t dim = size_t{1} << wires.size();
    std::vector<CT> m(dim * dim);
    for (size_t i = 0; i < dim * dim; i++) {
        m[i] = CT{static_cast<T>(mat[i].real()), static_cast<T>(mat[i].imag())};
    }
    if (inverse) {
        m = dagger<T>(m, dim);
    }
    prim_dense(wires, cwires, cvals, m);
}

template <class T>
void StateVector<T>::apply_sparse_matrix(const int64_t *indptr, const int64_t *indices, const cd *data, int64_t nnz,
                                         const std::vector<int64_t> &wires, const std::vector<int64_t> &cwires,
                                         const std::vector<bool> &cvals) {
    // applyNCMultiQubitSparseOp (LM:505-560): a local CSR operator on `wires`.
    PLGB_REQUIRE(!wires.empty(), "Number of wires must be larger than 0");
    const size_t k = wires.size();
    PLGB_REQUIRE(k <= 12, "sparse local operators act on at most 12 wires");
    const size_t D = size_t{1} << k;
    std::vector<CT> m(D * D, CT{0, 0});
    for (size_t r = 0; r < D; r++) {
        for (int64_t p = indptr[r]; p < indptr[r + 1]; p++) {
            PLGB_REQUIRE(p < nnz && indices[p] >= 0 && static_cast<size_t>(indices[p]) < D, "bad CSR data");
            const CT v{static_cast<T>(data[p].real()), static_cast<T>(data[p].imag())};
            CT &e = m[r * D + static_cast<size_t>(indices[p])];
            e = e + v;
        }
    }
    prim_dense(wires, cwires, cvals, m);
}

template <class T>
void StateVector<T>::apply_pauli_rot(const std::vector<int64_t> &wires, bool inverse, double angle_d,
                                     const std::string &word) {
    // LM:577-629
    PLGB_REQUIRE(wires.size() == word.size(), "wires and word have incompatible dimensions.");
    check_wires_(wires, {});
    const T angle = static_cast<T>(angle_d);
    if (std::all_of(word.begin(), word.end(), [](char c) { return c == 'Z'; })) {
        apply_named_("MultiRZ", {}, {}, wires, inverse, {angle_d});
        return;
    }
    u64 mxy = 0, my = 0, mz = 0;
    for (size_t i = 0; i < wires.size(); i++) {
        const u64 b = u64{1} << bit_of(wires[i]);
        const char c = word[i];
        PLGB_REQUIRE(c == 'X' || c == 'Y' || c == 'Z' || c == 'I', "Pauli word letters must be I, X, Y or Z");
        if (c != 'Z') {
            mxy |= b;
        }
        if (c == 'Y') {
            my |= b;
        }
        if (c == 'Z') {
            mz |= b;
        }
    }
    const T c = std::cos(angle / 2);
    const T sn = std::sin(angle / 2);
    // s = (inverse ? i : -i) * sin(angle/2)
    const CT s = inverse ? CT{0, sn} : CT{0, -sn};
    Prim<T> p;
    p.kind = Prim<T>::PauliRot;
    p.pmask = mxy;
    p.my = my;
    p.mz = mz;
    p.c = c;
    p.m = {s};
    emit_(std::move(p));
}

// ---------------------------------------------------------------------------
// generators (LM:2165-2940, PauliGenerator.hpp:27-57)
// ---------------------------------------------------------------------------
template <class T>
double StateVector<T>::apply_generator(const std::string &name, const std::vector<int64_t> &cwires_in,
                                       const std::vector<bool> &cvals_in, const std::vector<int64_t> &wires_in) {
    std::vector<int64_t> cw(cwires_in), wires(wires_in);
    std::vector<bool> cv(cvals_in);
    PLGB_REQUIRE(cw.size() == cv.size(), "`controlled_wires` must have the same size as `controlled_values`.");
    std::string base = name;
    if (name == "CRX" || name == "CRY" || name == "CRZ" || name == "ControlledPhaseShift") {
        PLGB_REQUIRE(wires.size() == 2, "wrong number of wires for generator " + name);
        PLGB_REQUIRE(cw.empty(), "generator " + name + " takes no extra controls");
        cw.push_back(wires[0]);
        cv.push_back(true);
        wires.erase(wires.begin());
        base = name == "CRX" ? "RX" : name == "CRY" ? "RY" : name == "CRZ" ? "RZ" : "PhaseShift";
    }
    check_wires_(wires, cw);
    auto need = [&](size_t k) { PLGB_REQUIRE(wires.size() == k, "wrong number of wires for generator " + name); };
    const CT Z0{0, 0}, O1{1, 0}, I{0, 1}, mI{0, -1}, M1{-1, 0};
    if (base == "GlobalPhase") {
        prim_zero_outside(cw, cv);
        return -1.0;
    }
    if (base == "MultiRZ") {
        Prim<T> p;
        p.kind = Prim<T>::Parity;
        for (auto w : wires) {
            p.pmask |= u64{1} << bit_of(w);
        }
        set_controls(p, *this, cw, cv);
        p.m = {O1, M1};
        p.zero_outside = true;
        emit_(std::move(p));
        return -0.5;
    }
    prim_zero_outside(cw, cv);
    if (base == "RX") {
        need(1);
        prim_1q(wires[0], cw, cv, M1_SWAP, Mat1<T>{});
        return -0.5;
    }
    if (base == "RY") {
        need(1);
        prim_1q(wires[0], cw, cv, M1_ANTI, m1<T>(Z0, mI, I, Z0));
        return -0.5;
    }
    if (base == "RZ") {
        need(1);
        prim_1q(wires[0], cw, cv, M1_NEG1, Mat1<T>{});
        return -0.5;
    }
    if (base == "PhaseShift") {
        need(1);
        prim_1q(wires[0], cw, cv, M1_DIAG, m1<T>(Z0, Z0, Z0, O1));
        return 1.0;
    }
    // two- and four-wire generators as (non-unitary) local matrices
    auto mat = [&](size_t k, std::initializer_list<std::pair<int, CT>> entries, bool identity_rest) {
        const size_t D = size_t{1} << k;
        std::vector<CT> m(D * D, Z0);
        if (identity_rest) {
            for (size_t i = 0; i < D; i++) {
                m[i * D + i] = O1;
            }
        }
        for (auto &e : entries) {
            const size_t r = static_cast<size_t>(e.first) / D;
            m[r * D + r] = identity_rest ? Z0 : m[r * D + r];
        }
        for (auto &e : entries) {
            m[static_cast<size_t>(e.first)] = e.second;
        }
        return m;
    };
    if (base == "IsingXX") {
        need(2);
        prim_dense(wires, cw, cv, mat(2, {{3, O1}, {6, O1}, {9, O1}, {12, O1}}, false));
        return -0.5;
    }
    if (base == "IsingXY") {
        need(2);
        prim_dense(wires, cw, cv, mat(2, {{6, O1}, {9, O1}}, false));
        return 0.5;
    }
    if (base == "IsingYY") {
        need(2);
        prim_dense(wires, cw, cv, mat(2, {{3, M1}, {6, O1}, {9, O1}, {12, M1}}, false));
        return -0.5;
    }
    if (base == "IsingZZ") {
        need(2);
        prim_dense(wires, cw, cv, mat(2, {{0, O1}, {5, M1}, {10, M1}, {15, O1}}, false));
        return -0.5;
    }
    if (base == "SingleExcitation") {
        need(2);
        prim_dense(wires, cw, cv, mat(2, {{6, mI}, {9, I}}, false));
        return -0.5;
    }
    if (base == "SingleExcitationMinus") {
        need(2);
        prim_dense(wires, cw, cv, mat(2, {{0, O1}, {6, mI}, {9, I}, {15, O1}}, false));
        return -0.5;
    }
    if (base == "SingleExcitationPlus") {
        need(2);
        prim_dense(wires, cw, cv, mat(2, {{0, M1}, {6, mI}, {9, I}, {15, M1}}, false));
        return -0.5;
    }
    if (base == "PSWAP") {
        need(2);
        prim_dense(wires, cw, cv, mat(2, {{6, O1}, {9, O1}}, false));
        return 1.0;
    }
    if (base == "DoubleExcitation") {
        need(4);
        prim_dense(wires, cw, cv, mat(4, {{3 * 16 + 12, mI}, {12 * 16 + 3, I}}, false));
        return -0.5;
    }
    if (base == "DoubleExcitationMinus") {
        need(4);
        prim_dense(wires, cw, cv, mat(4, {{3 * 16 + 12, mI}, {12 * 16 + 3, I}}, true));
        return -0.5;
    }
    if (base == "DoubleExcitationPlus") {
        need(4);
        prim_dense(wires, cw, cv, mat(4, {{3 * 16 + 12, I}, {12 * 16 + 3, mI}}, true));
        return 0.5;
    }
    throw PLError("Generator of " + name + " is not supported");
}

// StateVectorLQubit.hpp:431-482: a known name dispatches by name, anything
// else is applied through its matrix.
template <class T> void StateVector<T>::apply_op(const OpRec &op, bool inverse) {
    if (is_named_gate(op.name)) {
        if (op.cwires.empty()) {
            apply_named_(op.name, {}, {}, op.wires, inverse, op.params);
        } else {
            apply_named_(op.name, op.cwires, op.cvals, op.wires, inverse, op.params);
        }
        return;
    }
    PLGB_REQUIRE(!op.matrix.empty(), "operation " + op.name + " has neither a known name nor a matrix");
    apply_matrix(op.matrix.data(), op.wires, inverse, op.cwires, op.cvals);
}

template struct Prim<float>;
template struct Prim<double>;
template class StateVector<float>;
template class StateVector<double>;

} // namespace plgb
