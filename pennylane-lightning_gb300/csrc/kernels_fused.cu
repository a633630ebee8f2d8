// Fused tile passes (sm_103a).
//
// A pass keeps a set of 2^t amplitude indices "local": the L lowest bits
// (contiguous runs of 2^L amplitudes, so every load and store is coalesced)
// plus H chosen higher bits.  Each CTA stages one tile — the 2^t amplitudes
// that share the remaining (global) bits — in shared memory, applies the
// pass's whole op list to it, and writes it back: one HBM read and one write
// per pass instead of one per gate.
//
// Ops whose mixing targets are local run on the tile (pair updates, scaled
// rotations, dense two-wire blocks); diagonal ops run for any bits: a merged
// diagonal multiplies by a per-pass table over the local index, folds
// factors that depend only on global bits into one scalar per tile (applied
// at the store), and turns local x global sign patterns (CZ across the tile
// boundary) into integer sign flips.  Scalars factored out of rotations are
// one constant per pass, also applied at the store.
#include "tile_smem.cuh"

namespace plgb {

template <class T>
__global__ void __launch_bounds__(kTileThreads) k_tile_pass(cx<T> *__restrict__ a, const TilePassDesc dp,
                                                           const TileOp<T> *__restrict__ ops,
                                                           const DiagForm<T> *__restrict__ forms,
                                                           const cx<T> *__restrict__ tables) {
    extern __shared__ unsigned char smraw[];
    cx<T> *tile = reinterpret_cast<cx<T> *>(smraw);
    __shared__ SmemDiag<T> sd;
    __shared__ TilePassDesc d; // indexed dynamically (hb[]): kept in shared memory
    if (threadIdx.x == 0) {
        d = dp;
    }
    __syncthreads();
    const u32 T_ = 1u << d.t;
    for (u64 g = blockIdx.x; g < d.ntiles; g += gridDim.x) {
        // tile base: g spread over the global bits (zeros at every local bit)
        u64 gbase = g << d.L;
        for (int m = 0; m < d.H; m++) {
            const int p = d.hb[m];
            gbase = ((gbase >> p) << (p + 1)) | (gbase & ((u64{1} << p) - 1));
        }
        for (u32 j = threadIdx.x; j < T_; j += blockDim.x) {
            tile[j] = a[gbase | local_offset(j, d)];
        }
        if (threadIdx.x == 0) {
            sd.tile_factor = cx<T>{1, 0};
        }
        __syncthreads();
        for (int oi = 0; oi < d.nops; oi++) {
            const TileOp<T> &op = ops[d.op_begin + oi];
            if ((gbase & op.gcmask) != op.gcval) {
                continue; // global controls not met: the op is the identity on this tile
            }
            if (op.kind == TK_DIAGTAB) {
                smem_diag_prepare<T>(op, gbase, forms, sd);
                __syncthreads();
            }
            smem_apply<T>(tile, op, d, gbase, tables, sd);
            __syncthreads();
        }
        const cx<T> f = sd.tile_factor;
        const cx<T> sf{f.x * d.pass_scale, f.y * d.pass_scale};
        for (u32 j = threadIdx.x; j < T_; j += blockDim.x) {
            a[gbase | local_offset(j, d)] = sf * tile[j];
        }
        __syncthreads();
    }
}

template <class T>
void launch_tile_pass(cudaStream_t s, cx<T> *sv, const TilePassDesc &d, const TileOp<T> *ops, const DiagForm<T> *forms,
                      const cx<T> *tables) {
    const size_t smem = sizeof(cx<T>) << d.t;
    static bool attr_set = false;
    if (!attr_set) {
        cuda_check(cudaFuncSetAttribute(k_tile_pass<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024),
                   "tile smem attribute");
        attr_set = true;
    }
    int per_sm = 1;
    cuda_check(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_tile_pass<T>, kTileThreads, smem),
               "tile occupancy");
    if (per_sm < 1) {
        throw std::runtime_error("tile pass: shared-memory tile too large for one CTA");
    }
    const u64 cap = static_cast<u64>(LaunchGeom::sm_count()) * static_cast<u64>(per_sm);
    const unsigned grid = static_cast<unsigned>(d.ntiles < cap ? d.ntiles : cap);
    k_tile_pass<T><<<grid, kTileThreads, smem, s>>>(sv, d, ops, forms, tables);
    cuda_check(cudaGetLastError(), "k_tile_pass launch");
    note_launch();
}

template void launch_tile_pass<float>(cudaStream_t, cx<float> *, const TilePassDesc &, const TileOp<float> *,
                                      const DiagForm<float> *, const cx<float> *);
template void launch_tile_pass<double>(cudaStream_t, cx<double> *, const TilePassDesc &, const TileOp<double> *,
                                       const DiagForm<double> *, const cx<double> *);

} // namespace plgb
