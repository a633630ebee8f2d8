// Batch engine host side (batch.hpp).
//
// run(): circuits are lowered and compiled into fused tile passes on a pool
// of host threads, then executed in waves that fit a device-memory budget.
// Within a wave all registers sit in one device arena and all compiled
// programs in another (one host->device copy each); pass k of every circuit
// runs as one persistent launch per tile size, the expectation values as one
// batched reduction; one device->host copy returns the sums.
#include "batch.hpp"
#include "fusion.hpp"

#include <algorithm>
#include <atomic>
#include <condition_variable>
#include <chrono>
#include <cstring>
#include <thread>
#include <type_traits>

namespace plgb {

namespace {

constexpr int kBatchMinQubits = kMinRegTileBits; // smaller registers run padded
constexpr int kBatchMaxQubits = 30;
constexpr int kMaxWiresPerOp = 4;

double ms_since(std::chrono::steady_clock::time_point t0) {
    return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
}

template <class T> struct Compiled {
    int n{0};     // register size as given
    int ne{0};    // register size run (>= 9)
    int t{0};     // tile bits
    bool fast{false}; // every segment is a register-kernel tile pass of size t
    std::shared_ptr<FusedProgram<T>> prog;
    std::vector<std::vector<PauliGroup>> obs_groups; // per observable
    std::string error;
};

// a small config-0-like circuit used to time tile sizes for one register size
template <class T> std::vector<Prim<T>> tuning_circuit(int n) {
    StateVector<T> reg(n, LowerOnly{});
    std::vector<Prim<T>> prims;
    for (int layer = 0; layer < 4; layer++) {
        for (int q = 0; q < n; q++) {
            for (const char *g : {"RX", "RY", "RZ"}) {
                OpRec r;
                r.name = g;
                r.wires = {q};
                r.params = {0.1 + 0.01 * (q + 7 * layer)};
                auto p = reg.lower_op(r, false);
                prims.insert(prims.end(), std::make_move_iterator(p.begin()), std::make_move_iterator(p.end()));
            }
        }
        for (int q = 0; q < n; q++) {
            OpRec r;
            r.name = "CNOT";
            r.wires = {q, (q + 1) % n};
            auto p = reg.lower_op(r, false);
            prims.insert(prims.end(), std::make_move_iterator(p.begin()), std::make_move_iterator(p.end()));
        }
    }
    return prims;
}

} // namespace

template <class T> BatchEngine<T>::BatchEngine() {
    cuda_check(cudaStreamCreateWithFlags(&s_, cudaStreamNonBlocking), "cudaStreamCreate");
    cuda_check(cudaEventCreate(&ev0_), "cudaEventCreate");
    cuda_check(cudaEventCreate(&ev1_), "cudaEventCreate");
    cuda_check(cudaEventCreate(&ev_run0_), "cudaEventCreate");
    for (int i = 0; i < 2; i++) {
        cuda_check(cudaEventCreate(&wev0_[i]), "cudaEventCreate");
        cuda_check(cudaEventCreate(&wev1_[i]), "cudaEventCreate");
    }
}

template <class T> BatchEngine<T>::~BatchEngine() {
    if (s_) {
        cudaStreamSynchronize(s_);
    }
    for (void *p : {d_states_, d_prog_, d_items_, d_red_}) {
        if (p) {
            cudaFree(p);
        }
    }
    for (int i = 0; i < 2; i++) {
        for (void *p : {h_prog_[i], h_items_[i], h_out_[i]}) {
            if (p) {
                cudaFreeHost(p);
            }
        }
        if (wev0_[i]) {
            cudaEventDestroy(wev0_[i]);
        }
        if (wev1_[i]) {
            cudaEventDestroy(wev1_[i]);
        }
    }
    if (ev_run0_) {
        cudaEventDestroy(ev_run0_);
    }
    if (ev0_) {
        cudaEventDestroy(ev0_);
    }
    if (ev1_) {
        cudaEventDestroy(ev1_);
    }
    if (s_) {
        cudaStreamDestroy(s_);
    }
}

template <class T> void *BatchEngine<T>::grow(void *&buf, size_t &cap, size_t need, bool pinned) {
    if (need <= cap && buf) {
        return buf;
    }
    cuda_check(cudaStreamSynchronize(s_), "cudaStreamSynchronize");
    if (buf) {
        pinned ? cudaFreeHost(buf) : cudaFree(buf);
        buf = nullptr;
        cap = 0;
    }
    const size_t want = std::max<size_t>(need + need / 4, 1 << 16);
    if (pinned) {
        cuda_check(cudaMallocHost(&buf, want), "cudaMallocHost(batch)");
    } else {
        count_device_allocation();
        cuda_check(cudaMalloc(&buf, want), "cudaMalloc(batch)");
    }
    cap = want;
    return buf;
}

template <class T> int BatchEngine<T>::tile_bits_for(int n) {
    if (fixed_tile_bits_ > 0) {
        return std::max(kMinRegTileBits, std::min({fixed_tile_bits_, n, 12}));
    }
    auto it = tuned_.find(n);
    if (it != tuned_.end()) {
        return it->second;
    }
    // Autotune: time the register kernel on a tuning circuit at every
    // candidate tile size this register supports; keep the fastest.
    // (timed on at most 20 qubits: the choice depends on the tile, not on
    // how many tiles there are)
    const int tmin = kMinRegTileBits, tmax = std::min(n, 12);
    int best = tmax;
    if (tmin < tmax) {
        const int nt = std::min(n, 20);
        const auto prims = tuning_circuit<T>(nt);
        StateVector<T> sv(nt);
        float best_ms = 1e30f;
        for (int t = tmin; t <= tmax; t++) {
            auto prog = compile_fused<T>(nt, prims, t, true);
            run_fused<T>(sv, *prog); // warm
            cuda_check(cudaEventRecord(ev0_, sv.stream()), "event");
            run_fused<T>(sv, *prog);
            run_fused<T>(sv, *prog);
            cuda_check(cudaEventRecord(ev1_, sv.stream()), "event");
            cuda_check(cudaEventSynchronize(ev1_), "event sync");
            float ms = 0;
            cuda_check(cudaEventElapsedTime(&ms, ev0_, ev1_), "event time");
            if (ms < best_ms * 0.97f) { // prefer the smaller tile unless clearly slower
                best_ms = ms;
                best = t;
            }
        }
    }
    tuned_[n] = best;
    return best;
}

template <class T> void BatchEngine<T>::run(const BatchInput &in, double *out) {
    std::lock_guard<std::mutex> lk(mu_);
    const auto t_start = std::chrono::steady_clock::now();
    // complex128 batches run their fused passes in double-float arithmetic
    // unless FP64 passes were requested
    const bool use_df = std::is_same_v<T, double> && !c128_fp64_passes();
    stats_ = BatchStats{};
    stats_.df = use_df;
    const int nc = in.ncirc;
    stats_.ncirc = nc;
    PLGB_REQUIRE(nc >= 0, "number of circuits must be non-negative");
    if (nc == 0) {
        return;
    }
    PLGB_REQUIRE(in.num_qubits && in.op_offsets && in.obs_offsets, "batch: missing circuit arrays");
    const int64_t nops_total = in.op_offsets[nc];
    PLGB_REQUIRE(in.op_offsets[0] == 0 && nops_total >= 0, "batch: op offsets must start at 0");
    PLGB_REQUIRE(nops_total == 0 || (in.op_codes && in.op_wires && in.op_params), "batch: missing op arrays");
    const int64_t nobs_total = in.obs_offsets[nc];
    PLGB_REQUIRE(in.obs_offsets[0] == 0 && nobs_total >= 0, "batch: observable offsets must start at 0");
    PLGB_REQUIRE(nobs_total == 0 || in.term_offsets, "batch: missing term offsets");
    const int64_t nterms_total = nobs_total ? in.term_offsets[nobs_total] : 0;
    PLGB_REQUIRE(nterms_total == 0 || (in.term_coeffs && in.term_x && in.term_y && in.term_z),
                 "batch: missing term arrays");
    for (int c = 0; c < nc; c++) {
        const int n = in.num_qubits[c];
        PLGB_REQUIRE(n >= 1 && n <= kBatchMaxQubits, "batch: number of qubits must be in 1..30");
        PLGB_REQUIRE(in.op_offsets[c + 1] >= in.op_offsets[c], "batch: op offsets must not decrease");
        PLGB_REQUIRE(in.obs_offsets[c + 1] >= in.obs_offsets[c], "batch: observable offsets must not decrease");
    }

    // tile sizes first (autotuning runs on the device, one register size at a time)
    std::map<int, int> tsel;
    for (int c = 0; c < nc; c++) {
        const int ne = std::max(in.num_qubits[c], kBatchMinQubits);
        if (!tsel.count(ne)) {
            tsel[ne] = tile_bits_for(ne);
        }
    }
    stats_.tile_bits = tsel;

    // ---- lower + compile on a pool of host threads, one wave at a time
    std::vector<Compiled<T>> comp(static_cast<size_t>(nc));
    std::atomic<int> next{0};
    int comp_hi = 0;
    auto worker = [&]() {
        for (int c = next++; c < comp_hi; c = next++) {
            Compiled<T> &cc = comp[static_cast<size_t>(c)];
            try {
                cc.n = in.num_qubits[c];
                cc.ne = std::max(cc.n, kBatchMinQubits);
                cc.t = tsel.at(cc.ne);
                StateVector<T> reg(cc.ne, LowerOnly{});
                std::vector<Prim<T>> prims;
                OpRec rec;
                for (int64_t o = in.op_offsets[c]; o < in.op_offsets[c + 1]; o++) {
                    const char *name = gate_name_of(in.op_codes[o]);
                    PLGB_REQUIRE(name != nullptr, "batch: unknown gate code");
                    rec.name = name;
                    rec.wires.clear();
                    for (int k = 0; k < kMaxWiresPerOp; k++) {
                        const int w = in.op_wires[kMaxWiresPerOp * o + k];
                        if (w >= 0) {
                            PLGB_REQUIRE(w < cc.n, "batch: wire index out of range");
                            rec.wires.push_back(w);
                        }
                    }
                    rec.params.assign(in.op_params + 3 * o, in.op_params + 3 * o + 3);
                    rec.inverse = in.op_inverse ? in.op_inverse[o] != 0 : false;
                    auto p = reg.lower_op(rec, rec.inverse);
                    prims.insert(prims.end(), std::make_move_iterator(p.begin()), std::make_move_iterator(p.end()));
                }
                cc.prog = compile_fused<T>(cc.ne, prims, cc.t, false, true);
                cc.fast = true;
                for (const auto &seg : cc.prog->segs) {
                    if (!seg.tile || !seg.reg || seg.desc.t != cc.t) {
                        cc.fast = false;
                    }
                }
                if (!cc.fast) { // runs on its own, with its program in device memory
                    cc.prog = compile_fused<T>(cc.ne, prims, cc.t, true);
                }
                for (int64_t ob = in.obs_offsets[c]; ob < in.obs_offsets[c + 1]; ob++) {
                    PauliSum ps;
                    for (int64_t tm = in.term_offsets[ob]; tm < in.term_offsets[ob + 1]; tm++) {
                        const u64 X = in.term_x[tm], Y = in.term_y[tm], Z = in.term_z[tm];
                        PLGB_REQUIRE(((X & Y) | (X & Z) | (Y & Z)) == 0, "batch: a wire has two Pauli letters");
                        PLGB_REQUIRE(cc.n >= 64 || ((X | Y | Z) >> cc.n) == 0, "batch: term wire out of range");
                        PauliSum::Term t{in.term_coeffs[tm], 0, 0, 0};
                        for (u64 r = X | Y | Z; r; r &= r - 1) {
                            const int w = __builtin_ctzll(r);
                            const u64 b = u64{1} << (cc.ne - 1 - w);
                            if ((X >> w) & 1U) {
                                t.x |= b;
                            } else if ((Y >> w) & 1U) {
                                t.x |= b;
                                t.yz |= b;
                                t.ny4 = (t.ny4 + 1) & 3;
                            } else {
                                t.yz |= b;
                            }
                        }
                        ps.terms.push_back(t);
                    }
                    cc.obs_groups.push_back(group_pauli(ps));
                }
            } catch (const std::exception &e) {
                cc.error = e.what();
            }
        }
    };
    auto compile_range = [&](int lo, int hi) {
        const auto t_comp = std::chrono::steady_clock::now();
        next = lo;
        comp_hi = hi;
        int nt = threads_ > 0 ? threads_ : static_cast<int>(std::thread::hardware_concurrency());
        nt = std::max(1, std::min({nt, 64, hi - lo}));
        std::vector<std::thread> pool;
        for (int i = 1; i < nt; i++) {
            pool.emplace_back(worker);
        }
        worker();
        for (auto &th : pool) {
            th.join();
        }
        for (int c = lo; c < hi; c++) {
            if (!comp[static_cast<size_t>(c)].error.empty()) {
                throw PLError(comp[static_cast<size_t>(c)].error);
            }
        }
        stats_.compile_ms += ms_since(t_comp);
    };

    // ---- waves of registers that fit the memory budget, planned from the
    // register sizes.  The host compiles and packs wave k+1 while the device
    // runs wave k: pinned staging buffers alternate between two sets, the
    // device arenas are reused in stream order.
    std::vector<std::pair<int, int>> wave_rng;
    stats_.wave_of.assign(static_cast<size_t>(nc), 0);
    for (int c0 = 0; c0 < nc;) {
        int c1 = c0;
        size_t sv_bytes = 0;
        while (c1 < nc) {
            const size_t b = align_up(sizeof(cx<T>) << std::max(in.num_qubits[c1], kBatchMinQubits));
            if (c1 > c0 && sv_bytes + b > wave_bytes_) {
                break;
            }
            sv_bytes += b;
            stats_.wave_of[static_cast<size_t>(c1)] = static_cast<int>(wave_rng.size());
            c1++;
        }
        wave_rng.emplace_back(c0, c1);
        c0 = c1;
    }
    const int nwaves = static_cast<int>(wave_rng.size());
    stats_.wave_done_ms.assign(static_cast<size_t>(nwaves), 0.0);
    float dev_ms_total = 0;

    struct WaveRun {
        int k{0}, set{0}, c0{0}, c1{0};
        std::vector<std::pair<int64_t, size_t>> obs_item; // (observable index, item index)
        size_t nred_items{0};
        double enqueue_ms{0};
    };
    auto prepare_and_enqueue = [&](int k) -> WaveRun {
        WaveRun W;
        W.k = k;
        W.set = k & 1;
        W.c0 = wave_rng[static_cast<size_t>(k)].first;
        W.c1 = wave_rng[static_cast<size_t>(k)].second;
        const int c0 = W.c0, c1 = W.c1, set = W.set;
        compile_range(c0, c1);
        // registers of this wave
        size_t sv_bytes = 0;
        std::vector<size_t> sv_off;
        for (int c = c0; c < c1; c++) {
            sv_off.push_back(sv_bytes);
            sv_bytes += align_up(sizeof(cx<T>) << comp[static_cast<size_t>(c)].ne);
        }
        const int wn = c1 - c0;
        grow(d_states_, c_states_, sv_bytes, false);
        char *states = static_cast<char *>(d_states_);

        // programs: one arena, 256-byte aligned blocks per circuit
        struct ProgOff {
            size_t ops, forms, tables, stages;
        };
        std::vector<ProgOff> po(static_cast<size_t>(wn));
        size_t pbytes = 0;
        for (int i = 0; i < wn; i++) {
            const auto &pr = *comp[static_cast<size_t>(c0 + i)].prog;
            if (!comp[static_cast<size_t>(c0 + i)].fast) { // runs its own uploaded program
                po[static_cast<size_t>(i)] = ProgOff{pbytes, pbytes, pbytes, pbytes};
                continue;
            }
            po[static_cast<size_t>(i)].ops = pbytes;
            pbytes += align_up(pr.h_ops.size() * sizeof(TileOp<T>));
            po[static_cast<size_t>(i)].forms = pbytes;
            pbytes += align_up(pr.h_forms.size() * sizeof(DiagForm<T>));
            po[static_cast<size_t>(i)].tables = pbytes;
            pbytes += align_up(pr.table_entries * sizeof(cx<T>));
            po[static_cast<size_t>(i)].stages = pbytes;
            pbytes += align_up(pr.h_stages.size() * sizeof(StageDesc));
        }
        pbytes = std::max<size_t>(pbytes, 256);
        const auto t_pack = std::chrono::steady_clock::now();
        stats_.program_bytes += static_cast<double>(pbytes);
        grow(h_prog_[set], ch_prog_[set], pbytes, true);
        grow(d_prog_, c_prog_, pbytes, false);
        char *hp = static_cast<char *>(h_prog_[set]);
        for (int i = 0; i < wn; i++) {
            const auto &pr = *comp[static_cast<size_t>(c0 + i)].prog;
            if (!comp[static_cast<size_t>(c0 + i)].fast) {
                continue;
            }
            const auto &o = po[static_cast<size_t>(i)];
            PLGB_REQUIRE(pr.h_recipes.empty() || !pr.h_factors.empty(), "batch: table recipe without factors");
            for (const auto &ch : pr.h_table_chunks) {
                PLGB_REQUIRE(ch[1] + ch[2] <= pr.h_tables.size() && ch[0] + ch[2] <= pr.table_entries,
                             "batch: table chunk out of range");
            }
            std::memcpy(hp + o.ops, pr.h_ops.data(), pr.h_ops.size() * sizeof(TileOp<T>));
            std::memcpy(hp + o.forms, pr.h_forms.data(), pr.h_forms.size() * sizeof(DiagForm<T>));
            for (const auto &ch : pr.h_table_chunks) { // tables materialised on the host
                std::memcpy(hp + o.tables + ch[0] * sizeof(cx<T>), pr.h_tables.data() + ch[1], ch[2] * sizeof(cx<T>));
            }
            std::memcpy(hp + o.stages, pr.h_stages.data(), pr.h_stages.size() * sizeof(StageDesc));
            if constexpr (std::is_same_v<T, double>) {
                if (use_df) { // the same tables re-encoded as double-float (same layout)
                    auto cdf = [](cx<double> v) { return cx<df>{df(v.x), df(v.y)}; };
                    auto *od = reinterpret_cast<TileOp<df> *>(hp + o.ops);
                    for (size_t k = 0; k < pr.h_ops.size(); k++) {
                        for (int m = 0; m < 16; m++) {
                            od[k].m[m] = cdf(pr.h_ops[k].m[m]);
                        }
                    }
                    auto *fd = reinterpret_cast<DiagForm<df> *>(hp + o.forms);
                    for (size_t k = 0; k < pr.h_forms.size(); k++) {
                        for (int m = 0; m < 16; m++) {
                            fd[k].tab[m] = cdf(pr.h_forms[k].tab[m]);
                        }
                    }
                    auto *td = reinterpret_cast<cx<df> *>(hp + o.tables);
                    for (const auto &ch : pr.h_table_chunks) {
                        for (size_t k = 0; k < ch[2]; k++) {
                            td[ch[0] + k] = cdf(pr.h_tables[ch[1] + k]);
                        }
                    }
                }
            }
        }
        char *dp = static_cast<char *>(d_prog_);
        // merged-diagonal tables described by their factors: expanded on the device
        std::vector<DevRecipe> recs;
        std::vector<TableFactor> facs;
        u64 rec_entries = 0;
        for (int i = 0; i < wn; i++) {
            const auto &pr = *comp[static_cast<size_t>(c0 + i)].prog;
            if (!comp[static_cast<size_t>(c0 + i)].fast) {
                continue;
            }
            const auto &o = po[static_cast<size_t>(i)];
            for (const auto &r : pr.h_recipes) {
                DevRecipe d{};
                d.dst = dp + o.tables + static_cast<size_t>(r.table_off) * sizeof(cx<T>);
                d.fac = reinterpret_cast<const TableFactor *>(facs.size()); // index, fixed below
                d.t = r.t;
                d.nfac = r.nfac;
                d.entry_begin = rec_entries;
                rec_entries += u64{1} << r.t;
                facs.insert(facs.end(), pr.h_factors.begin() + r.fac_begin,
                            pr.h_factors.begin() + r.fac_begin + r.nfac);
                recs.push_back(d);
            }
        }
        stats_.pack_ms += ms_since(t_pack);

        // launch plan: pass k of every fast circuit, grouped by tile size
        struct Launch {
            int t;
            size_t item0;
            int nitems;
            u64 tiles;
            int max_ops;
        };
        std::vector<BatchTileItem<T>> titems;
        std::vector<Launch> launches;
        int maxp = 0;
        for (int i = 0; i < wn; i++) {
            const auto &cc = comp[static_cast<size_t>(c0 + i)];
            if (cc.fast) {
                maxp = std::max(maxp, static_cast<int>(cc.prog->segs.size()));
            }
        }
        stats_.max_passes = std::max(stats_.max_passes, maxp);
        for (int k = 0; k < maxp; k++) {
            std::map<int, std::vector<int>> by_t;
            for (int i = 0; i < wn; i++) {
                const auto &cc = comp[static_cast<size_t>(c0 + i)];
                if (cc.fast && k < static_cast<int>(cc.prog->segs.size())) {
                    by_t[cc.t].push_back(i);
                }
            }
            for (auto &kv : by_t) {
                Launch L{kv.first, titems.size(), 0, 0, 0};
                for (int i : kv.second) {
                    const auto &cc = comp[static_cast<size_t>(c0 + i)];
                    const auto &o = po[static_cast<size_t>(i)];
                    BatchTileItem<T> it{};
                    it.sv = reinterpret_cast<cx<T> *>(states + sv_off[static_cast<size_t>(i)]);
                    it.ops = reinterpret_cast<const TileOp<T> *>(dp + o.ops);
                    it.forms = reinterpret_cast<const DiagForm<T> *>(dp + o.forms);
                    it.tables = reinterpret_cast<const cx<T> *>(dp + o.tables);
                    it.stages = reinterpret_cast<const StageDesc *>(dp + o.stages);
                    it.desc = cc.prog->segs[static_cast<size_t>(k)].desc;
                    it.tile_begin = L.tiles;
                    L.tiles += it.desc.ntiles;
                    L.max_ops = std::max(L.max_ops, it.desc.nops);
                    titems.push_back(it);
                    L.nitems++;
                }
                launches.push_back(L);
            }
        }

        // reductions: one item per (register, observable, flip-mask group)
        std::vector<PauliGroup> groups;
        std::vector<BatchRedItem<T>> ritems;
        auto &obs_item = W.obs_item;
        u64 rblocks = 0;
        for (int i = 0; i < wn; i++) {
            const auto &cc = comp[static_cast<size_t>(c0 + i)];
            const int64_t ob0 = in.obs_offsets[c0 + i];
            for (size_t ob = 0; ob < cc.obs_groups.size(); ob++) {
                for (const auto &g : cc.obs_groups[ob]) {
                    BatchRedItem<T> r{};
                    r.sv = reinterpret_cast<const cx<T> *>(states + sv_off[static_cast<size_t>(i)]);
                    r.group = reinterpret_cast<const PauliGroup *>(groups.size()); // index, fixed below
                    const u64 N = u64{1} << cc.ne;
                    r.work = g.x == 0 ? N : N >> 1;
                    r.block_begin = rblocks;
                    r.df = use_df && cc.fast ? 1 : 0;
                    rblocks += (r.work + kBatchRedChunk - 1) / kBatchRedChunk;
                    obs_item.emplace_back(ob0 + static_cast<int64_t>(ob), ritems.size());
                    ritems.push_back(r);
                    groups.push_back(g);
                }
            }
        }

        // one staging block: [tile items][set-one pointers][red items][groups][recipes][factors]
        const size_t b_titems = align_up(std::max<size_t>(1, titems.size()) * sizeof(BatchTileItem<T>));
        const size_t b_ptrs = align_up(static_cast<size_t>(wn) * sizeof(cx<T> *));
        const size_t b_ritems = align_up(std::max<size_t>(1, ritems.size()) * sizeof(BatchRedItem<T>));
        const size_t b_groups = align_up(std::max<size_t>(1, groups.size()) * sizeof(PauliGroup));
        const size_t b_recs = align_up(std::max<size_t>(1, recs.size()) * sizeof(DevRecipe));
        const size_t b_facs = align_up(std::max<size_t>(1, facs.size()) * sizeof(TableFactor));
        const size_t ibytes = b_titems + b_ptrs + b_ritems + b_groups + b_recs + b_facs;
        grow(h_items_[set], ch_items_[set], ibytes, true);
        grow(d_items_, c_items_, ibytes, false);
        char *hi = static_cast<char *>(h_items_[set]);
        char *di = static_cast<char *>(d_items_);
        auto *d_titems = reinterpret_cast<BatchTileItem<T> *>(di);
        auto *d_ptrs = reinterpret_cast<cx<T> **>(di + b_titems);
        auto *d_ritems = reinterpret_cast<BatchRedItem<T> *>(di + b_titems + b_ptrs);
        auto *d_groups = reinterpret_cast<PauliGroup *>(di + b_titems + b_ptrs + b_ritems);
        for (auto &r : ritems) {
            r.group = d_groups + reinterpret_cast<size_t>(r.group);
        }
        std::memcpy(hi, titems.data(), titems.size() * sizeof(BatchTileItem<T>));
        auto *h_ptrs = reinterpret_cast<cx<T> **>(hi + b_titems);
        for (int i = 0; i < wn; i++) {
            h_ptrs[i] = reinterpret_cast<cx<T> *>(states + sv_off[static_cast<size_t>(i)]);
        }
        std::memcpy(hi + b_titems + b_ptrs, ritems.data(), ritems.size() * sizeof(BatchRedItem<T>));
        std::memcpy(hi + b_titems + b_ptrs + b_ritems, groups.data(), groups.size() * sizeof(PauliGroup));
        auto *d_recs = reinterpret_cast<DevRecipe *>(di + b_titems + b_ptrs + b_ritems + b_groups);
        auto *d_facs = reinterpret_cast<TableFactor *>(di + b_titems + b_ptrs + b_ritems + b_groups + b_recs);
        for (auto &r : recs) {
            r.fac = d_facs + reinterpret_cast<size_t>(r.fac);
        }
        std::memcpy(hi + b_titems + b_ptrs + b_ritems + b_groups, recs.data(), recs.size() * sizeof(DevRecipe));
        std::memcpy(hi + b_titems + b_ptrs + b_ritems + b_groups + b_recs, facs.data(),
                    facs.size() * sizeof(TableFactor));

        const size_t nred = std::max<size_t>(1, ritems.size());
        grow(d_red_, c_red_, (rblocks + nred) * sizeof(double), false);
        grow(h_out_[set], ch_out_[set], nred * sizeof(double), true);
        W.nred_items = ritems.size();
        double *partials = static_cast<double *>(d_red_);
        double *item_sums = partials + rblocks;

        // ---- device work of the wave
        cuda_check(cudaEventRecord(wev0_[set], s_), "event");
        if (k == 0) {
            cuda_check(cudaEventRecord(ev_run0_, s_), "event");
            W.enqueue_ms = ms_since(t_start);
        }
        cuda_check(cudaMemcpyAsync(dp, hp, pbytes, cudaMemcpyHostToDevice, s_), "H2D programs");
        cuda_check(cudaMemcpyAsync(di, hi, ibytes, cudaMemcpyHostToDevice, s_), "H2D items");
        cuda_check(cudaMemsetAsync(states, 0, sv_bytes, s_), "memset registers");
        launch_expand_tables(s_, d_recs, static_cast<int>(recs.size()), rec_entries,
                             use_df ? 2 : (std::is_same_v<T, float> ? 0 : 1));
        stats_.launches += recs.empty() ? 0 : 1;
        if (use_df) { // registers stay double-float pairs from |0..0> to the reductions
            launch_batch_set_one<df>(s_, reinterpret_cast<cx<df> *const *>(d_ptrs), wn);
        } else {
            launch_batch_set_one<T>(s_, d_ptrs, wn);
        }
        stats_.launches += 1;
        for (const auto &L : launches) {
            if (use_df) {
                launch_tile_reg_batch<df>(s_, L.t, reinterpret_cast<const BatchTileItem<df> *>(d_titems + L.item0),
                                          L.nitems, L.tiles, L.max_ops);
            } else {
                launch_tile_reg_batch<T>(s_, L.t, d_titems + L.item0, L.nitems, L.tiles, L.max_ops);
            }
            stats_.launches++;
        }
        // circuits the batched kernel cannot take run pass by pass on their own
        for (int i = 0; i < wn; i++) {
            auto &cc = comp[static_cast<size_t>(c0 + i)];
            if (cc.fast) {
                continue;
            }
            stats_.fallback++;
            StateVector<T> view(reinterpret_cast<cx<T> *>(states + sv_off[static_cast<size_t>(i)]), cc.ne, s_);
            if (use_df) {
                view.reset(); // this register stays in doubles
            }
            const auto l0 = launch_count();
            run_fused<T>(view, *cc.prog);
            stats_.launches += static_cast<int>(launch_count() - l0);
        }
        if (!ritems.empty()) {
            launch_pauli_batch<T>(s_, d_ritems, static_cast<int>(ritems.size()), rblocks, partials, item_sums);
            stats_.launches += 2;
            cuda_check(cudaMemcpyAsync(h_out_[set], item_sums, ritems.size() * sizeof(double),
                                       cudaMemcpyDeviceToHost, s_),
                       "D2H sums");
        }
        cuda_check(cudaEventRecord(wev1_[set], s_), "event");
        return W;
    };
    double run0_ms = 0; // host time at which the device work of wave 0 was enqueued
    auto finish = [&](const WaveRun &W) {
        const int set = W.set, c0 = W.c0, c1 = W.c1, wn = c1 - c0;
        cuda_check(cudaEventSynchronize(wev1_[set]), "wave sync");
        float wms = 0;
        cuda_check(cudaEventElapsedTime(&wms, wev0_[set], wev1_[set]), "event time");
        dev_ms_total += wms;
        float done = 0;
        cuda_check(cudaEventElapsedTime(&done, ev_run0_, wev1_[set]), "event time");
        stats_.wave_done_ms[static_cast<size_t>(W.k)] = run0_ms + static_cast<double>(done);

        // observable sums in a fixed order
        const double *sums = static_cast<const double *>(h_out_[set]);
        const auto &obs_item = W.obs_item;
        int64_t ob_last = -1;
        for (const auto &oi : obs_item) {
            if (oi.first != ob_last) {
                out[oi.first] = 0.0;
                ob_last = oi.first;
            }
            out[oi.first] += sums[oi.second];
        }
        // observables without terms
        for (int i = 0; i < wn; i++) {
            for (int64_t ob = in.obs_offsets[c0 + i]; ob < in.obs_offsets[c0 + i + 1]; ob++) {
                if (in.term_offsets[ob + 1] == in.term_offsets[ob]) {
                    out[ob] = 0.0;
                }
            }
        }
        stats_.waves++;
    };
    WaveRun cur = prepare_and_enqueue(0);
    run0_ms = cur.enqueue_ms;
    for (int k = 1; k < nwaves; k++) {
        WaveRun nxt = prepare_and_enqueue(k);
        finish(cur);
        cur = std::move(nxt);
    }
    finish(cur);
    for (const auto &cc : comp) {
        stats_.padded += cc.ne != cc.n ? 1 : 0;
    }
    stats_.device_ms = dev_ms_total;
    stats_.done_ms.assign(static_cast<size_t>(nc), 0.0);
    for (int c = 0; c < nc; c++) {
        stats_.done_ms[static_cast<size_t>(c)] = stats_.wave_done_ms[static_cast<size_t>(stats_.wave_of[static_cast<size_t>(c)])];
    }
    stats_.total_ms = ms_since(t_start);
}

template <class T> void BatchEngine<T>::run_adjoint(const BatchInput &in, double *values, double *jac) {
    std::lock_guard<std::mutex> lk(mu_);
    const auto t_start = std::chrono::steady_clock::now();
    stats_ = BatchStats{};
    const int nc = in.ncirc;
    stats_.ncirc = nc;
    if (nc <= 0) {
        return;
    }
    PLGB_REQUIRE(in.num_qubits && in.op_offsets && in.obs_offsets && in.term_offsets, "batch: missing arrays");
    // per circuit: its parametric-op count and where its Jacobian rows start
    std::vector<int64_t> npar(static_cast<size_t>(nc), 0), jac_off(static_cast<size_t>(nc) + 1, 0);
    for (int c = 0; c < nc; c++) {
        const int n = in.num_qubits[c];
        PLGB_REQUIRE(n >= 1 && n <= kBatchMaxQubits, "batch: number of qubits must be in 1..30");
        for (int64_t o = in.op_offsets[c]; o < in.op_offsets[c + 1]; o++) {
            const char *name = gate_name_of(in.op_codes[o]);
            PLGB_REQUIRE(name != nullptr, "batch: unknown gate code");
            npar[static_cast<size_t>(c)] += gate_param_count(name) > 0 ? 1 : 0;
        }
        jac_off[static_cast<size_t>(c) + 1] =
            jac_off[static_cast<size_t>(c)] + npar[static_cast<size_t>(c)] * (in.obs_offsets[c + 1] - in.obs_offsets[c]);
    }
    std::mutex bmu;
    std::condition_variable bcv;
    size_t in_use = 0;
    int active = 0;
    std::atomic<int> next{0};
    std::vector<std::string> errors(static_cast<size_t>(nc));
    stats_.done_ms.assign(static_cast<size_t>(nc), 0.0);
    int dev = 0;
    cuda_check(cudaGetDevice(&dev), "cudaGetDevice");
    std::atomic<int> next_worker{0};
    auto worker = [&]() {
        cudaSetDevice(dev);
        // the request's registers, scratch and programs come from this
        // worker's pool: no device-wide wait in cudaFree between requests
        ReusePool &pool = *adj_pools_[static_cast<size_t>(next_worker++)];
        for (int c = next++; c < nc; c = next++) {
            const int n = in.num_qubits[c];
            const size_t need = size_t{3} * (sizeof(cx<T>) << n);
            {
                std::unique_lock<std::mutex> g(bmu);
                bcv.wait(g, [&] { return active == 0 || in_use + need <= wave_bytes_; });
                in_use += need;
                active++;
            }
            try {
                ReuseScope scope(pool);
                OpsList ops;
                for (int64_t o = in.op_offsets[c]; o < in.op_offsets[c + 1]; o++) {
                    OpRec r;
                    r.name = gate_name_of(in.op_codes[o]);
                    for (int k = 0; k < kMaxWiresPerOp; k++) {
                        const int w = in.op_wires[kMaxWiresPerOp * o + k];
                        if (w >= 0) {
                            PLGB_REQUIRE(w < n, "batch: wire index out of range");
                            r.wires.push_back(w);
                        }
                    }
                    r.params.assign(in.op_params + 3 * o, in.op_params + 3 * o + gate_param_count(r.name));
                    r.inverse = in.op_inverse ? in.op_inverse[o] != 0 : false;
                    ops.ops.push_back(std::move(r));
                }
                std::vector<ObsPtr> obs;
                for (int64_t ob = in.obs_offsets[c]; ob < in.obs_offsets[c + 1]; ob++) {
                    auto h = std::make_shared<ObsNode>();
                    h->kind = ObsNode::Ham;
                    for (int64_t tm = in.term_offsets[ob]; tm < in.term_offsets[ob + 1]; tm++) {
                        auto prod = std::make_shared<ObsNode>();
                        prod->kind = ObsNode::Prod;
                        for (int w = 0; w < n; w++) {
                            const char *letter = ((in.term_x[tm] >> w) & 1U)   ? "PauliX"
                                                 : ((in.term_y[tm] >> w) & 1U) ? "PauliY"
                                                 : ((in.term_z[tm] >> w) & 1U) ? "PauliZ"
                                                                                 : nullptr;
                            if (letter) {
                                auto f = std::make_shared<ObsNode>();
                                f->kind = ObsNode::Named;
                                f->name = letter;
                                f->wires = {w};
                                prod->children.push_back(f);
                            }
                        }
                        if (prod->children.empty()) {
                            auto f = std::make_shared<ObsNode>();
                            f->kind = ObsNode::Named;
                            f->name = "Identity";
                            f->wires = {0};
                            prod->children.push_back(f);
                        }
                        h->children.push_back(prod);
                        h->coeffs.push_back(in.term_coeffs[tm]);
                    }
                    obs.push_back(h);
                }
                StateVector<T> sv(n);
                std::vector<Prim<T>> prims;
                for (const auto &op : ops.ops) {
                    auto p = sv.lower_op(op, op.inverse);
                    prims.insert(prims.end(), std::make_move_iterator(p.begin()), std::make_move_iterator(p.end()));
                }
                const int t = n >= kMinRegTileBits ? tile_bits_for(n) : n;
                auto prog = compile_fused<T>(n, prims, t, true);
                run_fused<T>(sv, *prog);
                for (size_t k = 0; k < obs.size(); k++) {
                    values[in.obs_offsets[c] + static_cast<int64_t>(k)] = Measure<T>::expval_obs(sv, *obs[k]);
                }
                std::vector<int64_t> tp(static_cast<size_t>(npar[static_cast<size_t>(c)]));
                for (size_t k = 0; k < tp.size(); k++) {
                    tp[k] = static_cast<int64_t>(k);
                }
                const auto j = Adjoint<T>::jacobian(sv, obs, ops, tp, false, true);
                std::copy(j.begin(), j.end(), jac + jac_off[static_cast<size_t>(c)]);
                stats_.done_ms[static_cast<size_t>(c)] = ms_since(t_start);
            } catch (const std::exception &e) {
                errors[static_cast<size_t>(c)] = e.what();
            }
            // every register of the request synchronised its stream when it
            // was destroyed, and the results were copied back: its buffers
            // are idle
            pool.recycle();
            {
                std::lock_guard<std::mutex> g(bmu);
                in_use -= need;
                active--;
            }
            bcv.notify_all();
        }
    };
    // tile sizes are tuned on this thread first (they time kernels on the device)
    for (int c = 0; c < nc; c++) {
        if (in.num_qubits[c] >= kMinRegTileBits) {
            tile_bits_for(in.num_qubits[c]);
        }
    }
    int nt = threads_ > 0 ? threads_ : static_cast<int>(std::thread::hardware_concurrency());
    nt = std::max(1, std::min({nt, 8, nc}));
    while (static_cast<int>(adj_pools_.size()) < nt) {
        adj_pools_.push_back(std::make_unique<ReusePool>());
    }
    std::vector<std::thread> pool;
    for (int i = 1; i < nt; i++) {
        pool.emplace_back(worker);
    }
    worker();
    for (auto &th : pool) {
        th.join();
    }
    for (const auto &e : errors) {
        if (!e.empty()) {
            throw PLError(e);
        }
    }
    stats_.total_ms = ms_since(t_start);
}

template <class T> std::string BatchEngine<T>::stats_json() const {
    std::string js = "{\"circuits\": " + std::to_string(stats_.ncirc) + ", \"waves\": " + std::to_string(stats_.waves) +
                     ", \"launches\": " + std::to_string(stats_.launches) +
                     ", \"max_passes\": " + std::to_string(stats_.max_passes) +
                     ", \"padded\": " + std::to_string(stats_.padded) +
                     ", \"fallback\": " + std::to_string(stats_.fallback) +
                     ", \"double_float\": " + std::string(stats_.df ? "true" : "false") +
                     ", \"compile_ms\": " + std::to_string(stats_.compile_ms) +
                     ", \"device_ms\": " + std::to_string(stats_.device_ms) +
                     ", \"pack_ms\": " + std::to_string(stats_.pack_ms) +
                     ", \"program_bytes\": " + std::to_string(stats_.program_bytes) +
                     ", \"total_ms\": " + std::to_string(stats_.total_ms) + ", \"tile_bits\": {";
    bool first = true;
    for (const auto &kv : stats_.tile_bits) {
        js += (first ? "\"" : ", \"") + std::to_string(kv.first) + "\": " + std::to_string(kv.second);
        first = false;
    }
    js += "}, \"wave_done_ms\": [";
    for (size_t i = 0; i < stats_.wave_done_ms.size(); i++) {
        js += (i ? ", " : "") + std::to_string(stats_.wave_done_ms[i]);
    }
    js += "], \"wave_of\": [";
    for (size_t i = 0; i < stats_.wave_of.size(); i++) {
        js += (i ? ", " : "") + std::to_string(stats_.wave_of[i]);
    }
    js += "], \"done_ms\": [";
    for (size_t i = 0; i < stats_.done_ms.size(); i++) {
        js += (i ? ", " : "") + std::to_string(stats_.done_ms[i]);
    }
    return js + "]}";
}

template class BatchEngine<float>;
template class BatchEngine<double>;

} // namespace plgb
