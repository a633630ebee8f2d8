// extern "C" boundary (include/pl_gb300.h) over the C++ host layer.
#include "pl_gb300.h"

#include "batch.hpp"
#include "fused.hpp"
#include "host.hpp"
#include "kernels_tc.hpp"

#include <algorithm>
#include <atomic>
#include <cstring>
#include <map>
#include <mutex>
#include <tuple>
#include <sstream>
#include <variant>

using namespace plgb;

struct plgb_sv {
    int precision;
    std::unique_ptr<StateVector<float>> f;
    std::unique_ptr<StateVector<double>> d;
    // deferred gate calls (lazy fusion): their primitives, run as fused tile
    // passes by the next call that reads or rewrites the state
    bool lazy{false};
    std::vector<plgb::Prim<float>> pend_f;
    std::vector<plgb::Prim<double>> pend_d;
};
struct plgb_obs {
    ObsPtr node;
};
struct plgb_batch {
    int precision;
    std::unique_ptr<BatchEngine<float>> f;
    std::unique_ptr<BatchEngine<double>> d;
};
struct plgb_ops {
    OpsList list;
    // compiled fused programs, keyed by (num_qubits, precision, tile bits)
    std::map<std::tuple<int, int, int>, std::shared_ptr<FusedProgram<float>>> prog_f;
    std::map<std::tuple<int, int, int>, std::shared_ptr<FusedProgram<double>>> prog_d;
    // dense-block programs, keyed by (num_qubits, precision, block width)
    std::map<std::tuple<int, int, int>, std::shared_ptr<const BlockProgram<float>>> blk_f;
    std::map<std::tuple<int, int, int>, std::shared_ptr<const BlockProgram<double>>> blk_d;
    std::mutex mu;
};

namespace {

int fail(int code, const std::string &msg) {
    set_last_error(msg);
    return code;
}

template <class F> int guard(F &&f) {
    try {
        f();
        return PLGB_OK;
    } catch (const PLError &e) {
        return fail(PLGB_ERR_INVALID, e.what());
    } catch (const std::bad_alloc &) {
        return fail(PLGB_ERR_CUDA, "out of memory");
    } catch (const std::runtime_error &e) {
        const std::string w = e.what();
        return fail(w.find("cuda") != std::string::npos || w.find("CUDA") != std::string::npos ||
                            w.find("launch") != std::string::npos || w.find("cudaMalloc") != std::string::npos
                        ? PLGB_ERR_CUDA
                        : PLGB_ERR_INTERNAL,
                    w);
    } catch (const std::exception &e) {
        return fail(PLGB_ERR_INTERNAL, e.what());
    }
}

void need(const void *p, const char *what) {
    if (p == nullptr) {
        throw PLError(std::string("null pointer: ") + what);
    }
}

// Lazy fusion of per-gate calls (the call pattern of lightning.qubit's
// Python device, one binding call per gate): a gate call validates and
// lowers the gate at once (errors surface at that call) and queues its
// primitives; the next call that reads or rewrites the state first runs the
// queue, as fused register-tile passes when it holds at least
// kLazyFuseMin primitives on a register of at least 2^9 amplitudes, else
// primitive by primitive.  Registers below g_lazy_min_qubits apply each gate
// at its call: their kernels are shorter than a binding call, so launching
// at once overlaps the caller's per-gate cost, while a fused program adds
// its compilation to the read (measured on 12-16 qubit config-0 circuits;
// from 17 qubits on the fused program is ahead).
std::atomic<int> g_lazy_fusion{1};
std::atomic<int> g_lazy_min_qubits{17};
constexpr size_t kLazyFuseMin = 16;
// Complex64 registers from 22 qubits on run fused gate lists as dense blocks
// of up to six wires (six-wire blocks on the tensor cores) instead of tile
// passes: measured faster on the config-0, -1 and -3 circuits at 22, 26 and
// 29 qubits (1.2-1.7x).  Switched off with the tensor cores
// (plgb_set_tc_dense(0)).
constexpr int kC64BlocksMinQubits = 22;
template <class T> bool blocks_preferred(const StateVector<T> &s) {
    return std::is_same_v<T, float> && s.num_qubits() >= kC64BlocksMinQubits && tc_dense_enabled();
}

// the operation list as dense blocks of at most block_wires wires, the block
// program cached on the ops object per (register size, precision, width);
// returns the number of blocks
template <class T> int apply_ops_blocks(StateVector<T> &s, plgb_ops *ops, int block_wires) {
    std::shared_ptr<const BlockProgram<T>> prog;
    {
        std::lock_guard<std::mutex> lk(ops->mu);
        const auto key = std::make_tuple(s.num_qubits(), static_cast<int>(sizeof(T)), block_wires);
        auto &cache = [&]() -> auto & {
            if constexpr (std::is_same_v<T, double>) {
                return ops->blk_d;
            } else {
                return ops->blk_f;
            }
        }();
        auto it = cache.find(key);
        if (it == cache.end()) {
            std::vector<Prim<T>> prims;
            for (const auto &op : ops->list.ops) {
                auto p = s.lower_op(op, op.inverse);
                prims.insert(prims.end(), std::make_move_iterator(p.begin()), std::make_move_iterator(p.end()));
            }
            auto blocks =
                prepare_blocks<T>(fuse_dense_blocks<T>(prims, s.num_qubits(), block_wires), s.num_qubits());
            it = cache.emplace(key, std::move(blocks)).first;
        }
        prog = it->second;
    }
    run_blocks<T>(s, *prog);
    return static_cast<int>(prog->prims.size());
}

template <class T> void run_pending(StateVector<T> &s, std::vector<Prim<T>> &pend) {
    if (pend.empty()) {
        return;
    }
    std::vector<Prim<T>> prims;
    prims.swap(pend); // the queue is empty whatever happens next
    if (blocks_preferred(s) && prims.size() >= kLazyFuseMin) {
        run_blocks<T>(s, *prepare_blocks<T>(fuse_dense_blocks<T>(prims, s.num_qubits(), 6), s.num_qubits()));
    } else if (s.num_qubits() >= kMinRegTileBits && prims.size() >= kLazyFuseMin) {
        s.apply_prims_fused(prims, sizeof(T) == 8 ? 11 : 12);
    } else {
        for (const auto &p : prims) {
            s.run_prim(p);
        }
    }
}
void flush_sv(plgb_sv *sv) {
    if (sv->precision == 128) {
        run_pending(*sv->d, sv->pend_d);
    } else {
        run_pending(*sv->f, sv->pend_f);
    }
}

template <class F> int with_sv(plgb_sv *sv, F &&f) {
    return guard([&] {
        need(sv, "state vector");
        flush_sv(sv);
        if (sv->precision == 128) {
            f(*sv->d);
        } else {
            f(*sv->f);
        }
    });
}
// Queries of the register's shape: no need to run the queue.
template <class F> int with_sv_meta(plgb_sv *sv, F &&f) {
    return guard([&] {
        need(sv, "state vector");
        if (sv->precision == 128) {
            f(*sv->d);
        } else {
            f(*sv->f);
        }
    });
}
// A gate call: queued when the handle is lazy, applied at once otherwise.
template <class F> int with_sv_gate(plgb_sv *sv, F &&f) {
    return guard([&] {
        need(sv, "state vector");
        const int nq = sv->precision == 128 ? sv->d->num_qubits() : sv->f->num_qubits();
        if (!sv->lazy || nq < g_lazy_min_qubits.load()) {
            flush_sv(sv);
            if (sv->precision == 128) {
                f(*sv->d);
            } else {
                f(*sv->f);
            }
            return;
        }
        if (sv->precision == 128) {
            auto &s = *sv->d;
            auto prims = s.capture_prims([&] { f(s); });
            sv->pend_d.insert(sv->pend_d.end(), std::make_move_iterator(prims.begin()),
                              std::make_move_iterator(prims.end()));
        } else {
            auto &s = *sv->f;
            auto prims = s.capture_prims([&] { f(s); });
            sv->pend_f.insert(sv->pend_f.end(), std::make_move_iterator(prims.begin()),
                              std::make_move_iterator(prims.end()));
        }
    });
}

std::vector<int64_t> vec(const int64_t *p, int n) {
    if (n > 0) {
        need(p, "wires");
    }
    return n > 0 ? std::vector<int64_t>(p, p + n) : std::vector<int64_t>{};
}
std::vector<bool> bvec(const uint8_t *p, int n) {
    std::vector<bool> v;
    if (n > 0) {
        need(p, "control values");
    }
    for (int i = 0; i < n; i++) {
        v.push_back(p[i] != 0);
    }
    return v;
}
std::vector<cd> cmat(const double *p, size_t n) {
    need(p, "matrix");
    std::vector<cd> m(n);
    for (size_t i = 0; i < n; i++) {
        m[i] = {p[2 * i], p[2 * i + 1]};
    }
    return m;
}
std::vector<double> dvec(const double *p, int n) {
    if (n > 0) {
        need(p, "params");
    }
    return n > 0 ? std::vector<double>(p, p + n) : std::vector<double>{};
}

int copy_text(const std::string &s, char *buf, size_t len) {
    if (!buf || len == 0) {
        return fail(PLGB_ERR_INVALID, "null buffer");
    }
    const size_t k = std::min(len - 1, s.size());
    std::memcpy(buf, s.data(), k);
    buf[k] = '\0';
    return s.size() + 1 > len ? fail(PLGB_ERR_INVALID, "buffer too small") : PLGB_OK;
}

} // namespace

extern "C" {

const char *plgb_last_error(void) { return last_error(); }

int plgb_device_count(int *out) {
    return guard([&] {
        need(out, "out");
        int c = 0;
        if (cudaGetDeviceCount(&c) != cudaSuccess) {
            c = 0;
        }
        *out = c;
    });
}

int plgb_kernel_launches(uint64_t *out) {
    return guard([&] {
        need(out, "out");
        *out = launch_count();
    });
}
int plgb_device_allocations(uint64_t *out) {
    return guard([&] {
        need(out, "out");
        *out = device_allocation_count();
    });
}

int plgb_backend_info(char *buf, size_t len) {
    return copy_text("{\"NAME\": \"lightning.gb300\", \"ARCH\": \"sm_103a\", \"REFERENCE\": \"lightning.qubit\"}", buf,
                     len);
}

int plgb_runtime_info(char *buf, size_t len) {
    std::ostringstream os;
    int dev = -1, rt = 0, drv = 0, count = 0;
    cudaRuntimeGetVersion(&rt);
    cudaDriverGetVersion(&drv);
    if (cudaGetDeviceCount(&count) != cudaSuccess) {
        count = 0;
    }
    os << "{\"cuda_runtime\": " << rt << ", \"cuda_driver\": " << drv << ", \"device_count\": " << count;
    if (count > 0 && cudaGetDevice(&dev) == cudaSuccess) {
        cudaDeviceProp p{};
        if (cudaGetDeviceProperties(&p, dev) == cudaSuccess) {
            os << ", \"device\": \"" << p.name << "\", \"sm\": " << p.major << p.minor
               << ", \"multiprocessors\": " << p.multiProcessorCount << ", \"global_mem\": " << p.totalGlobalMem;
        }
    }
    os << ", \"compiled_for\": \"sm_103a\", \"cuda_compiled\": " << CUDART_VERSION << "}";
    return copy_text(os.str(), buf, len);
}

// ---- state vector ---------------------------------------------------------
int plgb_sv_create(int num_qubits, int precision, plgb_sv **out) {
    return guard([&] {
        need(out, "out");
        PLGB_REQUIRE(precision == 64 || precision == 128, "precision must be 64 or 128");
        PLGB_REQUIRE(num_qubits >= 0 && num_qubits <= 36, "num_qubits must be in [0, 36]");
        int count = 0;
        if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) {
            throw std::runtime_error("CUDA: no GPU available (the GB300 backend has no CPU fallback)");
        }
        auto h = std::make_unique<plgb_sv>();
        h->precision = precision;
        h->lazy = g_lazy_fusion.load() != 0;
        if (precision == 128) {
            h->d = std::make_unique<StateVector<double>>(num_qubits);
        } else {
            h->f = std::make_unique<StateVector<float>>(num_qubits);
        }
        *out = h.release();
    });
}

int plgb_sv_create_raw(void *device_data, int num_qubits, int precision, plgb_sv **out) {
    return guard([&] {
        need(out, "out");
        need(device_data, "device data");
        PLGB_REQUIRE(precision == 64 || precision == 128, "precision must be 64 or 128");
        auto h = std::make_unique<plgb_sv>();
        h->precision = precision;
        h->lazy = g_lazy_fusion.load() != 0;
        if (precision == 128) {
            h->d = std::make_unique<StateVector<double>>(static_cast<cx<double> *>(device_data), num_qubits);
        } else {
            h->f = std::make_unique<StateVector<float>>(static_cast<cx<float> *>(device_data), num_qubits);
        }
        *out = h.release();
    });
}

int plgb_sv_clone(const plgb_sv *src, plgb_sv **out) {
    return guard([&] {
        need(src, "source");
        need(out, "out");
        flush_sv(const_cast<plgb_sv *>(src));
        auto h = std::make_unique<plgb_sv>();
        h->precision = src->precision;
        h->lazy = src->lazy;
        if (src->precision == 128) {
            h->d = std::make_unique<StateVector<double>>(src->d->num_qubits());
            h->d->copy_from(*src->d);
        } else {
            h->f = std::make_unique<StateVector<float>>(src->f->num_qubits());
            h->f->copy_from(*src->f);
        }
        *out = h.release();
    });
}

int plgb_sv_destroy(plgb_sv *sv) {
    return guard([&] { delete sv; });
}
int plgb_sv_num_qubits(const plgb_sv *sv, int *out) {
    return with_sv_meta(const_cast<plgb_sv *>(sv), [&](auto &s) {
        need(out, "out");
        *out = s.num_qubits();
    });
}
int plgb_sv_precision(const plgb_sv *sv, int *out) {
    return guard([&] {
        need(sv, "sv");
        need(out, "out");
        *out = sv->precision;
    });
}
int plgb_sv_length(const plgb_sv *sv, uint64_t *out) {
    return with_sv_meta(const_cast<plgb_sv *>(sv), [&](auto &s) {
        need(out, "out");
        *out = s.length();
    });
}
int plgb_sv_device_ptr(plgb_sv *sv, void **out) {
    return with_sv(sv, [&](auto &s) {
        need(out, "out");
        *out = s.data();
    });
}
int plgb_sv_synchronize(plgb_sv *sv) {
    return with_sv(sv, [&](auto &s) { s.synchronize(); });
}
int plgb_sv_stream(plgb_sv *sv, void **out) {
    return with_sv(sv, [&](auto &s) {
        need(out, "out");
        *out = static_cast<void *>(s.stream());
    });
}
int plgb_sv_reset(plgb_sv *sv) {
    return with_sv(sv, [&](auto &s) { s.reset(); });
}
int plgb_sv_set_basis_state(plgb_sv *sv, const int64_t *bits, const int64_t *wires, int nw) {
    return with_sv(sv, [&](auto &s) { s.set_basis_state(vec(bits, nw), vec(wires, nw)); });
}
int plgb_sv_set_state_vector(plgb_sv *sv, const void *host_state, uint64_t len, const int64_t *wires, int nw) {
    return with_sv(sv, [&](auto &s) {
        need(host_state, "state");
        using T = std::remove_reference_t<decltype(*s.data())>;
        using R = decltype(T{}.x);
        s.reset();
        s.set_state_vector(static_cast<const std::complex<R> *>(host_state), len, vec(wires, nw));
    });
}
int plgb_sv_update_data(plgb_sv *sv, const void *host_data, uint64_t len) {
    return with_sv(sv, [&](auto &s) {
        need(host_data, "data");
        using T = std::remove_reference_t<decltype(*s.data())>;
        using R = decltype(T{}.x);
        s.update_data(static_cast<const std::complex<R> *>(host_data), len);
    });
}
int plgb_sv_get_state(const plgb_sv *sv, void *host_out, uint64_t len) {
    return with_sv(const_cast<plgb_sv *>(sv), [&](auto &s) {
        need(host_out, "out");
        using T = std::remove_reference_t<decltype(*s.data())>;
        using R = decltype(T{}.x);
        s.get_state(static_cast<std::complex<R> *>(host_out), len);
    });
}
int plgb_sv_apply_operation(plgb_sv *sv, const char *name, const int64_t *wires, int nw, int inverse,
                            const double *params, int np) {
    return with_sv_gate(sv, [&](auto &s) {
        need(name, "name");
        s.apply_operation(name, vec(wires, nw), inverse != 0, dvec(params, np));
    });
}
int plgb_sv_apply_controlled_operation(plgb_sv *sv, const char *name, const int64_t *cwires, const uint8_t *cvals,
                                       int ncw, const int64_t *wires, int nw, int inverse, const double *params,
                                       int np) {
    return with_sv_gate(sv, [&](auto &s) {
        need(name, "name");
        s.apply_controlled_operation(name, vec(cwires, ncw), bvec(cvals, ncw), vec(wires, nw), inverse != 0,
                                     dvec(params, np));
    });
}
int plgb_sv_apply_matrix(plgb_sv *sv, const double *matrix, const int64_t *wires, int nw, int inverse) {
    return with_sv_gate(sv, [&](auto &s) {
        PLGB_REQUIRE(nw >= 1 && nw <= 12, "Number of wires must be larger than 0 (and at most 12)");
        const auto m = cmat(matrix, size_t{1} << (2 * nw));
        s.apply_matrix(m.data(), vec(wires, nw), inverse != 0);
    });
}
int plgb_sv_apply_controlled_matrix(plgb_sv *sv, const double *matrix, const int64_t *cwires, const uint8_t *cvals,
                                    int ncw, const int64_t *wires, int nw, int inverse) {
    return with_sv_gate(sv, [&](auto &s) {
        PLGB_REQUIRE(nw >= 1 && nw <= 12, "Number of wires must be larger than 0 (and at most 12)");
        const auto m = cmat(matrix, size_t{1} << (2 * nw));
        s.apply_matrix(m.data(), vec(wires, nw), inverse != 0, vec(cwires, ncw), bvec(cvals, ncw));
    });
}
int plgb_sv_apply_sparse_matrix(plgb_sv *sv, const int64_t *indptr, const int64_t *indices, const double *data,
                                int64_t nnz, const int64_t *cwires, const uint8_t *cvals, int ncw,
                                const int64_t *wires, int nw) {
    return with_sv(sv, [&](auto &s) {
        need(indptr, "indptr");
        PLGB_REQUIRE(nw >= 1 && nw <= 12, "Number of wires must be larger than 0 (and at most 12)");
        const auto d = cmat(nnz > 0 ? data : reinterpret_cast<const double *>(indptr), static_cast<size_t>(nnz));
        s.apply_sparse_matrix(indptr, indices, d.data(), nnz, vec(wires, nw), vec(cwires, ncw), bvec(cvals, ncw));
    });
}
int plgb_sv_apply_pauli_rot(plgb_sv *sv, const int64_t *wires, int nw, int inverse, double angle, const char *word) {
    return with_sv(sv, [&](auto &s) {
        need(word, "word");
        s.apply_pauli_rot(vec(wires, nw), inverse != 0, angle, word);
    });
}
int plgb_sv_apply_generator(plgb_sv *sv, const char *name, const int64_t *cwires, const uint8_t *cvals, int ncw,
                            const int64_t *wires, int nw, int adj, double *scale_out) {
    (void)adj;
    return with_sv(sv, [&](auto &s) {
        need(name, "name");
        need(scale_out, "scale_out");
        *scale_out = s.apply_generator(name, vec(cwires, ncw), bvec(cvals, ncw), vec(wires, nw));
    });
}
int plgb_sv_collapse(plgb_sv *sv, int64_t wire, int branch) {
    return with_sv(sv, [&](auto &s) { s.collapse(wire, branch != 0); });
}
int plgb_sv_normalize(plgb_sv *sv) {
    return with_sv(sv, [&](auto &s) { s.normalize(); });
}

// ---- measurements ------------------------------------------------------------
int plgb_meas_probs(plgb_sv *sv, const int64_t *wires, int nw, double *out) {
    return with_sv(sv, [&](auto &s) {
        need(out, "out");
        using T = decltype(s.data()->x);
        const auto p = Measure<T>::probs(s, nw < 0 ? std::vector<int64_t>{} : vec(wires, nw), nw < 0);
        std::memcpy(out, p.data(), p.size() * sizeof(double));
    });
}
int plgb_meas_expval_named(plgb_sv *sv, const char *name, const int64_t *wires, int nw, double *out) {
    return with_sv(sv, [&](auto &s) {
        need(out, "out");
        need(name, "name");
        using T = decltype(s.data()->x);
        *out = Measure<T>::expval_named(s, name, vec(wires, nw));
    });
}
int plgb_meas_expval_matrix(plgb_sv *sv, const double *matrix, const int64_t *wires, int nw, double *out) {
    return with_sv(sv, [&](auto &s) {
        need(out, "out");
        PLGB_REQUIRE(nw >= 1 && nw <= 12, "Number of wires must be larger than 0 (and at most 12)");
        using T = decltype(s.data()->x);
        const auto m = cmat(matrix, size_t{1} << (2 * nw));
        *out = Measure<T>::expval_matrix(s, m.data(), vec(wires, nw));
    });
}
int plgb_batch_create(int precision, plgb_batch **out) {
    return guard([&] {
        need(out, "out");
        PLGB_REQUIRE(precision == 64 || precision == 128, "precision must be 64 or 128");
        auto b = std::make_unique<plgb_batch>();
        b->precision = precision;
        if (precision == 128) {
            b->d = std::make_unique<BatchEngine<double>>();
        } else {
            b->f = std::make_unique<BatchEngine<float>>();
        }
        *out = b.release();
    });
}
int plgb_batch_destroy(plgb_batch *b) {
    delete b;
    return PLGB_OK;
}
int plgb_batch_configure(plgb_batch *b, int tile_bits, int64_t wave_bytes, int threads) {
    return guard([&] {
        need(b, "batch");
        PLGB_REQUIRE(tile_bits == 0 || (tile_bits >= 9 && tile_bits <= 12), "tile_bits must be 0 or in 9..12");
        PLGB_REQUIRE(wave_bytes >= 0 && threads >= 0, "wave_bytes and threads must be non-negative");
        auto cfg = [&](auto &e) {
            e.set_tile_bits(tile_bits);
            e.set_wave_bytes(wave_bytes > 0 ? static_cast<size_t>(wave_bytes) : size_t{8} << 30);
            e.set_threads(threads);
        };
        b->precision == 128 ? cfg(*b->d) : cfg(*b->f);
    });
}
int plgb_batch_run(plgb_batch *b, int ncirc, const int32_t *num_qubits, const int64_t *op_offsets,
                   const int32_t *op_codes, const int32_t *op_wires, const double *op_params, const uint8_t *op_inverse,
                   const int64_t *obs_offsets, const int64_t *term_offsets, const double *term_coeffs,
                   const uint64_t *term_x, const uint64_t *term_y, const uint64_t *term_z, double *out) {
    return guard([&] {
        need(b, "batch");
        BatchInput in;
        in.ncirc = ncirc;
        in.num_qubits = num_qubits;
        in.op_offsets = op_offsets;
        in.op_codes = op_codes;
        in.op_wires = op_wires;
        in.op_params = op_params;
        in.op_inverse = op_inverse;
        in.obs_offsets = obs_offsets;
        in.term_offsets = term_offsets;
        in.term_coeffs = term_coeffs;
        in.term_x = term_x;
        in.term_y = term_y;
        in.term_z = term_z;
        if (ncirc > 0) {
            need(obs_offsets, "obs_offsets");
            if (obs_offsets[ncirc] > 0) {
                need(out, "out");
            }
        }
        b->precision == 128 ? b->d->run(in, out) : b->f->run(in, out);
    });
}
int plgb_batch_adjoint(plgb_batch *b, int ncirc, const int32_t *num_qubits, const int64_t *op_offsets,
                       const int32_t *op_codes, const int32_t *op_wires, const double *op_params,
                       const uint8_t *op_inverse, const int64_t *obs_offsets, const int64_t *term_offsets,
                       const double *term_coeffs, const uint64_t *term_x, const uint64_t *term_y,
                       const uint64_t *term_z, double *values, double *jac) {
    return guard([&] {
        need(b, "batch");
        BatchInput in;
        in.ncirc = ncirc;
        in.num_qubits = num_qubits;
        in.op_offsets = op_offsets;
        in.op_codes = op_codes;
        in.op_wires = op_wires;
        in.op_params = op_params;
        in.op_inverse = op_inverse;
        in.obs_offsets = obs_offsets;
        in.term_offsets = term_offsets;
        in.term_coeffs = term_coeffs;
        in.term_x = term_x;
        in.term_y = term_y;
        in.term_z = term_z;
        if (ncirc > 0) {
            need(values, "values");
            need(jac, "jac");
        }
        b->precision == 128 ? b->d->run_adjoint(in, values, jac) : b->f->run_adjoint(in, values, jac);
    });
}
int plgb_batch_stats(const plgb_batch *b, char *buf, size_t len) {
    std::string js;
    const int rc = guard([&] {
        need(b, "batch");
        js = b->precision == 128 ? b->d->stats_json() : b->f->stats_json();
    });
    return rc != PLGB_OK ? rc : copy_text(js, buf, len);
}
const char *plgb_gate_name(int code) { return gate_name_of(code); }
int plgb_set_tile_variant(int precision, int occ) {
    if (precision != 64 && precision != 128) {
        set_last_error("precision must be 64 or 128");
        return -1;
    }
    return set_tile_variant_occ(precision, occ != 0) ? 1 : 0;
}
int plgb_set_lazy_fusion(int on) { return g_lazy_fusion.exchange(on != 0 ? 1 : 0); }
int plgb_set_lazy_min_qubits(int q) { return q < 1 ? -1 : g_lazy_min_qubits.exchange(q); }
int plgb_sv_set_lazy(plgb_sv *sv, int on) {
    return with_sv(sv, [&](auto &) { sv->lazy = on != 0; }); // runs the queue first
}
int plgb_set_tc_dense(int on) { return set_tc_dense_enabled(on != 0) ? 1 : 0; }
int plgb_set_c128_fp64_passes(int on) {
    const bool prev = c128_fp64_passes();
    set_c128_fp64_passes(on != 0);
    return prev ? 1 : 0;
}

int plgb_meas_expval_matrix_noalloc(plgb_sv *sv, const double *matrix, const int64_t *wires, int nw, double *out) {
    // no host containers on the success path: the matrix and wires are read
    // in place (noalloc.cu).  Gates queued on a lazy handle are not run here:
    // running them compiles and uploads a fused program, which allocates.
    return with_sv_meta(sv, [&](auto &s) {
        PLGB_REQUIRE(sv->pend_d.empty() && sv->pend_f.empty(),
                     "plgb_meas_expval_matrix_noalloc: gates are queued on this state vector and running them "
                     "allocates device memory; run them first (plgb_sv_synchronize)");
        need(out, "out");
        need(matrix, "matrix");
        if (nw > 0) {
            need(wires, "wires");
        }
        *out = expval_matrix_noalloc(s, matrix, wires, nw);
    });
}
int plgb_meas_expval_sparse(plgb_sv *sv, const int64_t *indptr, int64_t nptr, const int64_t *indices,
                            const double *data, int64_t nnz, double *out) {
    return with_sv(sv, [&](auto &s) {
        need(out, "out");
        need(indptr, "indptr");
        using T = decltype(s.data()->x);
        const auto d = cmat(data, static_cast<size_t>(nnz));
        *out = Measure<T>::expval_sparse(s, indptr, nptr, indices, d.data(), nnz);
    });
}
int plgb_meas_var_sparse(plgb_sv *sv, const int64_t *indptr, int64_t nptr, const int64_t *indices,
                         const double *data, int64_t nnz, double *out) {
    return with_sv(sv, [&](auto &s) {
        need(out, "out");
        need(indptr, "indptr");
        using T = decltype(s.data()->x);
        const auto d = cmat(data, static_cast<size_t>(nnz));
        *out = Measure<T>::var_sparse(s, indptr, nptr, indices, d.data(), nnz);
    });
}
int plgb_meas_expval_obs(plgb_sv *sv, const plgb_obs *obs, double *out) {
    return with_sv(sv, [&](auto &s) {
        need(obs, "observable");
        need(out, "out");
        using T = decltype(s.data()->x);
        *out = Measure<T>::expval_obs(s, *obs->node);
    });
}
int plgb_meas_var_obs(plgb_sv *sv, const plgb_obs *obs, double *out) {
    return with_sv(sv, [&](auto &s) {
        need(obs, "observable");
        need(out, "out");
        using T = decltype(s.data()->x);
        *out = Measure<T>::var_obs(s, *obs->node);
    });
}
int plgb_meas_var_named(plgb_sv *sv, const char *name, const int64_t *wires, int nw, double *out) {
    return with_sv(sv, [&](auto &s) {
        need(out, "out");
        need(name, "name");
        using T = decltype(s.data()->x);
        ObsNode o;
        o.kind = ObsNode::Named;
        o.name = name;
        o.wires = vec(wires, nw);
        *out = Measure<T>::var_obs(s, o);
    });
}
int plgb_meas_var_matrix(plgb_sv *sv, const double *matrix, const int64_t *wires, int nw, double *out) {
    return with_sv(sv, [&](auto &s) {
        need(out, "out");
        PLGB_REQUIRE(nw >= 1 && nw <= 12, "Number of wires must be larger than 0 (and at most 12)");
        using T = decltype(s.data()->x);
        ObsNode o;
        o.kind = ObsNode::Herm;
        o.mat = cmat(matrix, size_t{1} << (2 * nw));
        o.wires = vec(wires, nw);
        *out = Measure<T>::var_obs(s, o);
    });
}
int plgb_meas_generate_samples(plgb_sv *sv, const int64_t *wires, int nw, int64_t shots, uint64_t seed,
                               int64_t *out) {
    return with_sv(sv, [&](auto &s) {
        need(out, "out");
        using T = decltype(s.data()->x);
        std::vector<int64_t> w;
        if (nw < 0) {
            for (int i = 0; i < s.num_qubits(); i++) {
                w.push_back(i);
            }
        } else {
            w = vec(wires, nw);
        }
        const auto r = Measure<T>::samples(s, w, shots, seed);
        std::memcpy(out, r.data(), r.size() * sizeof(int64_t));
    });
}

int plgb_meas_generate_mcmc_samples(plgb_sv *sv, const char *kernelname, int64_t num_burnin, int64_t num_shots,
                                    uint64_t seed, int64_t *out) {
    return with_sv(sv, [&](auto &s) {
        need(kernelname, "kernelname");
        need(out, "out");
        using T = decltype(s.data()->x);
        const auto r = Measure<T>::mcmc_samples(s, std::string(kernelname), num_burnin, num_shots, seed);
        if (!r.empty()) {
            std::memcpy(out, r.data(), r.size() * sizeof(int64_t));
        }
    });
}

// ---- observables --------------------------------------------------------------
int plgb_obs_named(const char *name, const int64_t *wires, int nw, plgb_obs **out) {
    return guard([&] {
        need(name, "name");
        need(out, "out");
        const std::string n(name);
        PLGB_REQUIRE(is_named_gate(n), "unknown observable name " + n);
        auto o = std::make_shared<ObsNode>();
        o->kind = ObsNode::Named;
        o->name = n;
        o->wires = vec(wires, nw);
        *out = new plgb_obs{o};
    });
}
int plgb_obs_hermitian(const double *matrix, const int64_t *wires, int nw, plgb_obs **out) {
    return guard([&] {
        need(out, "out");
        PLGB_REQUIRE(nw >= 1 && nw <= 12, "Hermitian observables act on 1..12 wires");
        auto o = std::make_shared<ObsNode>();
        o->kind = ObsNode::Herm;
        o->mat = cmat(matrix, size_t{1} << (2 * nw));
        o->wires = vec(wires, nw);
        *out = new plgb_obs{o};
    });
}
int plgb_obs_tensor_prod(plgb_obs *const *obs, int n, plgb_obs **out) {
    return guard([&] {
        need(out, "out");
        PLGB_REQUIRE(n >= 1, "a tensor product needs at least one observable");
        auto o = std::make_shared<ObsNode>();
        o->kind = ObsNode::Prod;
        std::vector<int64_t> seen;
        for (int i = 0; i < n; i++) {
            need(obs[i], "observable");
            for (auto w : obs[i]->node->all_wires()) {
                PLGB_REQUIRE(std::find(seen.begin(), seen.end(), w) == seen.end(),
                             "All wires in observables must be disjoint.");
                seen.push_back(w);
            }
            o->children.push_back(obs[i]->node);
        }
        *out = new plgb_obs{o};
    });
}
int plgb_obs_hamiltonian(const double *coeffs, plgb_obs *const *obs, int n, plgb_obs **out) {
    return guard([&] {
        need(out, "out");
        auto o = std::make_shared<ObsNode>();
        o->kind = ObsNode::Ham;
        for (int i = 0; i < n; i++) {
            need(obs[i], "observable");
            o->children.push_back(obs[i]->node);
            o->coeffs.push_back(coeffs[i]);
        }
        *out = new plgb_obs{o};
    });
}
int plgb_obs_sparse_hamiltonian(const double *data, const int64_t *indices, int64_t nnz, const int64_t *indptr,
                                int64_t nptr, const int64_t *wires, int nw, plgb_obs **out) {
    return guard([&] {
        need(out, "out");
        need(indptr, "indptr");
        auto o = std::make_shared<ObsNode>();
        o->kind = ObsNode::Sparse;
        o->sp_data = cmat(data, static_cast<size_t>(nnz));
        o->sp_indices.assign(indices, indices + nnz);
        o->sp_indptr.assign(indptr, indptr + nptr);
        o->wires = vec(wires, nw);
        *out = new plgb_obs{o};
    });
}
int plgb_obs_destroy(plgb_obs *obs) {
    return guard([&] { delete obs; });
}
int plgb_obs_wires(const plgb_obs *obs, int64_t *wires, int cap, int *nw) {
    return guard([&] {
        need(obs, "observable");
        need(nw, "nw");
        const auto w = obs->node->all_wires();
        *nw = static_cast<int>(w.size());
        for (int i = 0; i < cap && i < static_cast<int>(w.size()); i++) {
            wires[i] = w[static_cast<size_t>(i)];
        }
    });
}
int plgb_obs_repr(const plgb_obs *obs, char *buf, size_t len) {
    if (!obs) {
        return fail(PLGB_ERR_INVALID, "null observable");
    }
    return copy_text(obs->node->repr(), buf, len);
}

// ---- algorithms -------------------------------------------------------------------
int plgb_ops_create(int nops, const char *const *names, const double *params, const int *nparams,
                    const int64_t *wires, const int *nwires, const uint8_t *inverses, const double *mats,
                    const int64_t *mat_sizes, const int64_t *cwires, const int *ncwires, const uint8_t *cvals,
                    plgb_ops **out) {
    return guard([&] {
        need(out, "out");
        auto h = std::make_unique<plgb_ops>();
        size_t ip = 0, iw = 0, im = 0, ic = 0;
        for (int k = 0; k < nops; k++) {
            OpRec op;
            op.name = names[k];
            for (int i = 0; i < nparams[k]; i++) {
                op.params.push_back(params[ip++]);
            }
            for (int i = 0; i < nwires[k]; i++) {
                op.wires.push_back(wires[iw++]);
            }
            op.inverse = inverses[k] != 0;
            const auto ms = static_cast<size_t>(mat_sizes ? mat_sizes[k] : 0);
            if (ms > 0) {
                op.matrix = cmat(mats + 2 * im, ms);
                im += ms;
            }
            const int nc = ncwires ? ncwires[k] : 0;
            for (int i = 0; i < nc; i++) {
                op.cwires.push_back(cwires[ic]);
                op.cvals.push_back(cvals[ic] != 0);
                ic++;
            }
            h->list.ops.push_back(std::move(op));
        }
        *out = h.release();
    });
}
int plgb_ops_destroy(plgb_ops *ops) {
    return guard([&] { delete ops; });
}
int plgb_ops_num_par_ops(const plgb_ops *ops, int *out) {
    return guard([&] {
        need(ops, "ops");
        need(out, "out");
        *out = static_cast<int>(ops->list.num_par_ops());
    });
}
int plgb_sv_apply_operations(plgb_sv *sv, plgb_ops *ops, int tile_bits, int *passes_out) {
    return with_sv(sv, [&](auto &s) {
        need(ops, "ops");
        using T = decltype(s.data()->x);
        if (tile_bits > 0 && blocks_preferred(s)) {
            PLGB_REQUIRE(tile_bits <= 14, "tile_bits must be in 1..14");
            const int nb = apply_ops_blocks<T>(s, ops, 6);
            if (passes_out) {
                *passes_out = nb;
            }
            return;
        }
        if (tile_bits <= 0) {
            for (const auto &op : ops->list.ops) {
                s.apply_op(op, op.inverse);
            }
            if (passes_out) {
                *passes_out = static_cast<int>(ops->list.ops.size());
            }
            return;
        }
        PLGB_REQUIRE(tile_bits <= 14, "tile_bits must be in 1..14");
        std::shared_ptr<FusedProgram<T>> prog;
        {
            std::lock_guard<std::mutex> lk(ops->mu);
            const auto key = std::make_tuple(s.num_qubits(), static_cast<int>(sizeof(T)), tile_bits);
            auto &cache = [&]() -> auto & {
                if constexpr (std::is_same_v<T, double>) {
                    return ops->prog_d;
                } else {
                    return ops->prog_f;
                }
            }();
            auto it = cache.find(key);
            if (it == cache.end()) {
                std::vector<Prim<T>> prims;
                for (const auto &op : ops->list.ops) {
                    auto p = s.lower_op(op, op.inverse);
                    prims.insert(prims.end(), std::make_move_iterator(p.begin()), std::make_move_iterator(p.end()));
                }
                it = cache.emplace(key, compile_fused<T>(s.num_qubits(), prims, tile_bits)).first;
            }
            prog = it->second;
        }
        run_fused<T>(s, *prog);
        if (passes_out) {
            const auto st = fused_stats<T>(*prog);
            *passes_out = static_cast<int>(st.passes + st.unfused);
        }
    });
}

int plgb_sv_apply_operations_blocks(plgb_sv *sv, plgb_ops *ops, int block_wires, int *blocks_out) {
    return with_sv(sv, [&](auto &s) {
        need(ops, "ops");
        using T = decltype(s.data()->x);
        PLGB_REQUIRE(block_wires >= 1 && block_wires <= 6, "block_wires must be in 1..6");
        const int nb = apply_ops_blocks<T>(s, ops, block_wires);
        if (blocks_out) {
            *blocks_out = nb;
        }
    });
}

int plgb_ops_fusion_plan(const plgb_ops *ops, int num_qubits, int precision, int tile_bits, char *buf, size_t len) {
    std::string js;
    const int rc = guard([&] {
        need(ops, "ops");
        PLGB_REQUIRE(precision == 64 || precision == 128, "precision must be 64 or 128");
        PLGB_REQUIRE(tile_bits >= 1 && tile_bits <= 14, "tile_bits must be in 1..14");
        auto plan = [&](auto tag) {
            using T = decltype(tag);
            StateVector<T> reg(num_qubits, LowerOnly{});
            std::vector<Prim<T>> prims;
            for (const auto &op : ops->list.ops) {
                auto p = reg.lower_op(op, op.inverse);
                prims.insert(prims.end(), std::make_move_iterator(p.begin()), std::make_move_iterator(p.end()));
            }
            js = fused_plan_json<T>(*compile_fused<T>(num_qubits, prims, tile_bits, false));
        };
        if (precision == 128) {
            plan(double{});
        } else {
            plan(float{});
        }
    });
    if (rc != PLGB_OK) {
        return rc;
    }
    return copy_text(js, buf, len);
}

int plgb_ops_block_plan(const plgb_ops *ops, int num_qubits, int precision, int block_wires, int with_matrices,
                        char *buf, size_t len) {
    std::string js;
    const int rc = guard([&] {
        need(ops, "ops");
        PLGB_REQUIRE(precision == 64 || precision == 128, "precision must be 64 or 128");
        PLGB_REQUIRE(block_wires >= 1 && block_wires <= 6, "block_wires must be in 1..6");
        auto plan = [&](auto tag) {
            using T = decltype(tag);
            StateVector<T> reg(num_qubits, LowerOnly{});
            std::vector<Prim<T>> prims;
            for (const auto &op : ops->list.ops) {
                auto p = reg.lower_op(op, op.inverse);
                prims.insert(prims.end(), std::make_move_iterator(p.begin()), std::make_move_iterator(p.end()));
            }
            const auto blocks = fuse_dense_blocks<T>(prims, num_qubits, block_wires);
            js = "[";
            char tmp[64];
            for (size_t i = 0; i < blocks.size(); i++) {
                const auto &p = blocks[i];
                js += i ? ",{" : "{";
                js += "\"kind\": " + std::to_string(static_cast<int>(p.kind)) + ", \"targets\": [";
                for (size_t b = 0; b < p.tbits.size(); b++) {
                    js += (b ? ", " : "") + std::to_string(p.tbits[b]);
                }
                js += "]";
                if (with_matrices && p.cmask == 0 &&
                    (p.kind == Prim<T>::Pair || p.kind == Prim<T>::Dense2 || p.kind == Prim<T>::DenseK)) {
                    js += ", \"matrix\": [";
                    for (size_t m = 0; m < p.m.size(); m++) {
                        std::snprintf(tmp, sizeof(tmp), "%s[%.17g, %.17g]", m ? ", " : "",
                                      static_cast<double>(p.m[m].x), static_cast<double>(p.m[m].y));
                        js += tmp;
                    }
                    js += "]";
                }
                js += "}";
            }
            js += "]";
        };
        if (precision == 128) {
            plan(double{});
        } else {
            plan(float{});
        }
    });
    if (rc != PLGB_OK) {
        return rc;
    }
    return copy_text(js, buf, len);
}

int plgb_adjoint_jacobian(plgb_sv *sv, plgb_obs *const *obs, int nobs, const plgb_ops *ops, const int64_t *trainable,
                          int ntp, int apply_ops, double *jac_out) {
    return with_sv(sv, [&](auto &s) {
        need(ops, "ops");
        need(jac_out, "jac_out");
        using T = decltype(s.data()->x);
        std::vector<ObsPtr> ob;
        for (int i = 0; i < nobs; i++) {
            need(obs[i], "observable");
            ob.push_back(obs[i]->node);
        }
        const auto j = Adjoint<T>::jacobian(s, ob, ops->list, vec(trainable, ntp), apply_ops != 0);
        std::memcpy(jac_out, j.data(), j.size() * sizeof(double));
    });
}
int plgb_vjp(plgb_sv *sv, const plgb_ops *ops, const double *dy, const int64_t *trainable, int ntp, double *out) {
    return with_sv(sv, [&](auto &s) {
        need(ops, "ops");
        need(dy, "dy");
        need(out, "out");
        using T = decltype(s.data()->x);
        std::vector<std::complex<T>> d(s.length());
        for (size_t i = 0; i < d.size(); i++) {
            d[i] = std::complex<T>(static_cast<T>(dy[2 * i]), static_cast<T>(dy[2 * i + 1]));
        }
        const auto w = Adjoint<T>::vjp(s, ops->list, d.data(), vec(trainable, ntp));
        for (size_t k = 0; k < w.size(); k++) {
            out[2 * k] = w[k].real();
            out[2 * k + 1] = w[k].imag();
        }
    });
}
int plgb_adjoint_jacobian_inplace(plgb_sv *sv, plgb_obs *const *obs, int nobs, const plgb_ops *ops,
                                  const int64_t *trainable, int ntp, double *jac_out) {
    return with_sv(sv, [&](auto &s) {
        need(ops, "ops");
        need(jac_out, "jac_out");
        using T = decltype(s.data()->x);
        std::vector<ObsPtr> ob;
        for (int i = 0; i < nobs; i++) {
            need(obs[i], "observable");
            ob.push_back(obs[i]->node);
        }
        const auto j = Adjoint<T>::jacobian(s, ob, ops->list, vec(trainable, ntp), false, true);
        std::memcpy(jac_out, j.data(), j.size() * sizeof(double));
    });
}

} // extern "C"
