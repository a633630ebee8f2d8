// The compiled form of a fused primitive list (host_fusion.cpp), shared by
// the single-register path and the batch engine (batch.cpp).
#pragma once

#include "fused.hpp"
#include "host.hpp"

#include <array>

namespace plgb {

template <class T> struct FusedProgram {
    struct Seg {
        bool tile{false};
        bool reg{false}; // register-blocked kernel
        TilePassDesc desc{};
        Prim<T> prim; // unfused segment
    };
    std::vector<Seg> segs;
    // device copies (compile_fused with upload)
    void *dev{nullptr};
    TileOp<T> *d_ops{nullptr};
    DiagForm<T> *d_forms{nullptr};
    cx<T> *d_tables{nullptr};
    StageDesc *d_stages{nullptr};
    // double-float copies of the op tables (complex128 programs whose every
    // pass runs on the register kernel; df_ok tells whether they exist)
    bool df_ok{false};  // df tables exist (every segment is a tile pass)
    bool df_reg{false}; // and every pass runs on the register kernel
    void *dev_df{nullptr};
    const void *d_ops_df{nullptr}, *d_forms_df{nullptr}, *d_tables_df{nullptr};
    // host copies (compile_fused without upload); indices in the segments'
    // descriptors are relative to these arrays
    std::vector<TileOp<T>> h_ops;
    std::vector<DiagForm<T>> h_forms;
    std::vector<cx<T>> h_tables;
    std::vector<StageDesc> h_stages;
    // recipe mode (compile_fused with recipes): h_tables stays empty; the
    // table area holds table_entries entries built from these on the device
    std::vector<TableRecipe> h_recipes;
    std::vector<TableFactor> h_factors;
    size_t table_entries{0};
    // h_tables chunks: (entry offset in the table area, offset in h_tables, count)
    std::vector<std::array<size_t, 3>> h_table_chunks;
    int n{0};
    size_t passes{0}, unfused{0}, prims{0};
    std::string plan; // JSON lines of the segments
    FusedProgram() = default;
    FusedProgram(const FusedProgram &) = delete;
    FusedProgram &operator=(const FusedProgram &) = delete;
    ~FusedProgram() {
        dev_free(dev);
        dev_free(dev_df);
    }
};

} // namespace plgb
