// Descriptors of the fused tile passes (kernels_fused.cu, host_fusion.cpp).
#pragma once

#include "kernels.hpp"

namespace plgb {

constexpr int kTileThreads = 256;
constexpr int kMaxTileBits = 14;
constexpr int kMaxMixedForms = 16;

enum TileKind : int {
    TK_PAIR = 0,    // two-amplitude update (Mode1), local targets, local/global controls
    TK_SROT = 1,    // scaled real rotation [[a,-b],[b,a]], one of a, b == 1; scale folded into the pass
    TK_DENSE2 = 2,  // dense 4x4 on two local bits
    TK_DIAGTAB = 3, // merged diagonal: local table x global scalar x local/global sign flips
    TK_PARITY = 4,  // parity phase on the full index (MultiRZ and its generator)
    TK_REDUCE = 5,  // adjoint sweep: Im <b| P G |a> over the tile into a parameter slot
};
constexpr int kMaxReducePerPass = 64; // reduction slots accumulated per CTA and pass

constexpr int kRegBits = 4;              // amplitudes per thread in register stages: 2^4
constexpr int kAdjRegBits = 3;           // two-register adjoint passes: 2^3 of each register
constexpr int kMaxOpsPerPass = 192;      // ops of a pass staged in shared memory per CTA
constexpr int kMinRegTileBits = 9;       // register kernel needs >= 32 threads
constexpr int kMaxDiagOpsPerPass = 48;   // merged diagonals evaluated per tile

struct TilePassDesc {
    int t;          // local bits in a tile
    int L;          // the lowest L bits are always local
    int H;          // number of further local bits
    int hb[kMaxTileBits];
    u64 ntiles;     // 2^(n - t)
    int op_begin, nops;
    double pass_scale; // product of the scalars factored out of rotations
    // register-blocked execution (t >= kMinRegTileBits): stages over the op list
    int stage_begin, nstages;
    int ndiag;      // merged-diagonal ops in the pass (prologue slots)
    int rslot_begin, nrslots; // reductions of the pass (adjoint programs): count in nrslots
};

// A stage of a register-blocked pass.  REG: ops [op_begin, op_begin+nops)
// run on amplitudes held in registers, register bit k being local bit rb[k]
// and thread-index bit m local bit tb[m].  SMEM: the ops run on the tile in
// shared memory (two-target ops).
struct StageDesc {
    int kind; // 0 = REG, 1 = SMEM
    int op_begin, nops;
    int rb[kRegBits];
    int tb[kMaxTileBits];
};

template <class T> struct TileOp {
    int kind{0};
    int mode{0};
    u32 lo0{0}, lo1{0};          // local offsets of the mixed amplitudes (DENSE2: first, second wire)
    int nlins{0};                // sorted local bits cleared when enumerating pairs (targets + local controls)
    int lins[12]{};
    u32 lcval{0};                // local control values
    u64 gcmask{0}, gcval{0};     // global control mask / values (tile-uniform)
    // DIAGTAB
    int has_table{0};
    int table_off{0};
    int gform_begin{0}, ngforms{0};
    int mform_begin{0}, nmforms{0};
    // PARITY (full index)
    u64 pmask{0}, cmask{0}, cval{0};
    int zero_outside{0};
    // register stages: target register bit, control predicates over the
    // register index and the thread index, slot of a merged diagonal
    // (TK_REDUCE in a register stage: tcmask = the flip as a register-slot
    // mask, tcval = merged diagonals before it in the pass)
    int rk{0};
    u32 rcmask{0}, rcval{0}, tcmask{0}, tcval{0};
    int diag_slot{0};
    // TK_REDUCE: lo1 = local flip mask, pmask = Y|Z mask, cmask/cval =
    // projector, mode = number of Y mod 4, result slot, and the square of
    // the rotation scales deferred to the store at this point
    int rslot{0};
    double rmul{1.0};
    cx<T> m[16]{};
};

// The fields of a TileOp that register stages and the tile prologue read,
// staged once per CTA and pass in shared memory (k_tile_reg*).
template <class T> struct RegOpS {
    int kind, mode, rk, diag_slot;
    u32 rcmask, rcval;
    int has_table, table_off;
    u64 gcmask, gcval;
    int ngforms, gform_begin, nmforms, mform_begin;
    cx<T> m[4];
};

// A diagonal factor on at most 4 bits: tab[k] with k = bits (first = MSB).
// For a mixed (global x local) form, bits[0] is the global bit and
// local_bit is the tile-local position of the other bit.
template <class T> struct DiagForm {
    int nb{0};
    int bits[4]{};
    int local_bit{0};
    cx<T> tab[16]{};
};

template <class T>
void launch_tile_pass(cudaStream_t s, cx<T> *sv, const TilePassDesc &d, const TileOp<T> *ops, const DiagForm<T> *forms,
                      const cx<T> *tables);
struct df;

// Adjoint sweep: the pass applied to two registers (lambda and H lambda),
// with its TK_REDUCE ops accumulated into partials[slot * G + CTA].
template <class T>
void launch_tile_pass_adj(cudaStream_t s, cx<T> *lam, cx<T> *hlam, const TilePassDesc &d, const TileOp<T> *ops,
                          const DiagForm<T> *forms, const cx<T> *tables, double *partials, int G);
int adj_grid_capacity(size_t tile_bytes_each);
// the same in double-float arithmetic (io as for launch_tile_pass_reg_df)
void launch_tile_pass_adj_df(cudaStream_t s, void *lam, void *hlam, int io, const TilePassDesc &d,
                             const TileOp<df> *ops, const DiagForm<df> *forms, const cx<df> *tables, double *partials,
                             int G);
void launch_adj_sum(cudaStream_t s, const double *partials, int nslots, int G, double *out);
// the same on the register-blocked kernel, for passes with register stages
// (kernels_adjoint_reg.cu)
template <class T>
void launch_tile_pass_reg_adj(cudaStream_t s, cx<T> *lam, cx<T> *hlam, const TilePassDesc &d, const TileOp<T> *ops,
                              const DiagForm<T> *forms, const cx<T> *tables, const StageDesc *stages,
                              double *partials, int G);
void launch_tile_pass_reg_adj_df(cudaStream_t s, void *lam, void *hlam, int io, const TilePassDesc &d,
                                 const TileOp<df> *ops, const DiagForm<df> *forms, const cx<df> *tables,
                                 const StageDesc *stages, double *partials, int G);

// A merged-diagonal table of 2^t entries described by its factors instead
// of its values (batch engine: expanded on the device).  Entry j is the
// product over factors of val[k], k = the bits of j at pos[0..nb) (first =
// most significant).
struct TableFactor {
    int nb;
    int pos[4];
    cx<double> val[16];
};
struct TableRecipe {
    int table_off; // entry offset in the program's table area
    int t;         // 2^t entries
    int fac_begin, nfac;
};
// one merged-diagonal table to expand on the device
struct DevRecipe {
    void *dst;          // first entry of the table in the program arena
    const TableFactor *fac;
    int t, nfac;
    u64 entry_begin;    // first global entry index of this table in the launch
};
// enc: 0 = complex64, 1 = complex128, 2 = complex128 as double-float pairs
void launch_expand_tables(cudaStream_t s, const DevRecipe *recipes, int nrec, u64 total_entries, int enc);

// Register-tile kernel variant per precision (64 or 128): false = up to 255
// registers per thread, true = at most 128 (twice the resident warps).
bool tile_variant_occ(int precision);
bool set_tile_variant_occ(int precision, bool occ);

// Complex128 passes in double-float arithmetic (df.cuh).  io: 0 = doubles in
// and out, 1 = doubles in / df out (first pass of a program), 2 = df in and
// out, 3 = df in / doubles out (last pass).
void launch_tile_pass_reg_df(cudaStream_t s, void *sv, int io, const TilePassDesc &d, const TileOp<df> *ops,
                             const DiagForm<df> *forms, const cx<df> *tables, const StageDesc *stages);

template <class T>
void launch_tile_pass_reg(cudaStream_t s, cx<T> *sv, const TilePassDesc &d, const TileOp<T> *ops,
                          const DiagForm<T> *forms, const cx<T> *tables, const StageDesc *stages);

// register-stage op codes (TileOp::mode when executed in registers)
enum RegMode : int { RM_SROT_A = 0, RM_SROT_B = 1, RM_SWAP = 2, RM_DENSE = 3 };

} // namespace plgb
