// Batch engine: many independent circuits, each on its own state vector,
// run together (batch.cpp, kernels_batch.cu).
//
// Every circuit is compiled into fused tile passes (host_fusion.cpp); pass k
// of every circuit that has one runs in ONE persistent launch over the tiles
// of all those registers ("one launch per fused layer").  Registers below
// 9 qubits run padded to 9 idle-extended qubits so that every tile fits the
// register-blocked kernel.  Expectation values of Pauli sums are reduced per
// (register, flip-mask group) with a work split that depends only on the
// register size, so a circuit's results are bit-identical whatever else is
// in the batch.
#pragma once

#include "df.cuh"
#include "fused.hpp"
#include "host.hpp"

#include <map>
#include <mutex>

namespace plgb {

// one register's share of a batched tile-pass launch
template <class T> struct BatchTileItem {
    cx<T> *sv;
    const TileOp<T> *ops;
    const DiagForm<T> *forms;
    const cx<T> *tables;
    const StageDesc *stages;
    u64 tile_begin; // first global tile index of this item in the launch
    TilePassDesc desc;
};

// one (register, flip-mask group) reduction of a batched expectation value
template <class T> struct BatchRedItem {
    const cx<T> *sv;
    const PauliGroup *group;
    u64 work;      // amplitudes (x == 0) or pairs (x != 0)
    u64 block_begin;
    int df;        // complex128 register held as double-float pairs
};

constexpr u64 kBatchRedChunk = 4096; // amplitudes or pairs per reduction block

template <class T>
void launch_tile_reg_batch(cudaStream_t s, int t, const BatchTileItem<T> *items, int nitems, u64 total_tiles,
                           int max_ops);
template <class T> void launch_batch_set_one(cudaStream_t s, cx<T> *const *svs, int n);
template <class T>
void launch_pauli_batch(cudaStream_t s, const BatchRedItem<T> *items, int nitems, u64 total_blocks, double *partials,
                        double *item_sums);

// Packed input of a batch (all arrays in host memory).
struct BatchInput {
    int ncirc{0};
    const int32_t *num_qubits{nullptr};   // [ncirc]
    const int64_t *op_offsets{nullptr};   // [ncirc + 1]
    const int32_t *op_codes{nullptr};     // gate-name codes (gate_name_of)
    const int32_t *op_wires{nullptr};     // 4 per op, -1 = unused
    const double *op_params{nullptr};     // 3 per op
    const uint8_t *op_inverse{nullptr};   // optional, 1 per op
    const int64_t *obs_offsets{nullptr};  // [ncirc + 1] observables per circuit
    const int64_t *term_offsets{nullptr}; // [nobs + 1] Pauli terms per observable
    const double *term_coeffs{nullptr};
    const uint64_t *term_x{nullptr}; // wire masks (bit w = wire w) of the X, Y, Z letters
    const uint64_t *term_y{nullptr};
    const uint64_t *term_z{nullptr};
};

const char *gate_name_of(int code); // nullptr past the end
int gate_code_count();
int gate_param_count(const std::string &name);

struct BatchStats {
    int ncirc{0}, waves{0}, launches{0}, max_passes{0}, padded{0}, fallback{0};
    bool df{false};
    double compile_ms{0}, device_ms{0}, total_ms{0}, pack_ms{0}, program_bytes{0};
    std::map<int, int> tile_bits; // register size -> tile bits used
    std::vector<double> wave_done_ms; // completion time of each wave, from the start of run()
    std::vector<int> wave_of;         // wave index of each circuit
    std::vector<double> done_ms;      // when each circuit's results were ready, from the start of the run
};

template <class T> class BatchEngine {
  public:
    BatchEngine();
    ~BatchEngine();
    BatchEngine(const BatchEngine &) = delete;
    BatchEngine &operator=(const BatchEngine &) = delete;

    // Run every circuit from |0...0> and write one expectation value per
    // observable (in input order) to out.
    void run(const BatchInput &in, double *out);

    // Adjoint requests: per circuit, <O> for each of its observables and the
    // Jacobian d<O>/d(parameter of each parametric gate) (the in-place
    // adjoint sweep).  Circuits run concurrently on host threads with their
    // own streams, within the engine's memory budget (three registers each).
    // values: one per observable; jac: per circuit, observable-major rows of
    // its parametric-gate count.
    void run_adjoint(const BatchInput &in, double *values, double *jac);

    // Tile size for a register of n qubits: fixed, or measured once per n
    // (autotune) over the candidates the register kernel supports.
    void set_tile_bits(int t) { fixed_tile_bits_ = t; }
    void set_wave_bytes(size_t b) { wave_bytes_ = b; }
    void set_threads(int k) { threads_ = k; }
    const BatchStats &stats() const { return stats_; }
    std::string stats_json() const;
    cudaStream_t stream() const { return s_; }

  private:
    int tile_bits_for(int n);
    void *grow(void *&buf, size_t &cap, size_t need, bool pinned);

    cudaStream_t s_{nullptr};
    cudaEvent_t ev0_{nullptr}, ev1_{nullptr};
    cudaEvent_t wev0_[2]{}, wev1_[2]{}, ev_run0_{nullptr}; // per staging set; start of a run's device work
    int fixed_tile_bits_{0};
    size_t wave_bytes_{size_t{8} << 30};
    int threads_{0};
    std::map<int, int> tuned_;
    std::mutex mu_;
    // grow-only device / pinned host arenas
    void *d_states_{nullptr}, *d_prog_{nullptr}, *d_items_{nullptr}, *d_red_{nullptr};
    size_t c_states_{0}, c_prog_{0}, c_items_{0}, c_red_{0};
    // pinned staging, two sets: wave k packs into set k % 2
    void *h_prog_[2]{}, *h_items_[2]{}, *h_out_[2]{};
    size_t ch_prog_[2]{}, ch_items_[2]{}, ch_out_[2]{};
    BatchStats stats_;
    // run_adjoint workers' buffer pools, kept between calls (a serving lane
    // calls it once per request); worker k uses adj_pools_[k]
    std::vector<std::unique_ptr<ReusePool>> adj_pools_;
};

} // namespace plgb
